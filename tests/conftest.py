"""Shared fixtures.  Tests marked `gpu` need a GB300 and the built library; everything else runs on
CPU (the oracle, the deck and validation logic, the C-ABI's symbol table and host-only paths)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_DECKS = ["bm1_head", "bm2_head", "small_head", "large_head", "edge"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and libbude_gb300.so")


def load_golden(name):
    """(deck, FP32 golden energies, FP64 rerun energies) of a committed fixture."""
    from minibude_gb300.deck import read_deck
    d = os.path.join(GOLDEN, name)
    deck = read_deck(d)
    refs32 = np.fromfile(os.path.join(d, "ref_energies.f32"), "<f4")
    f64 = np.fromfile(os.path.join(d, "f64_energies.f64"), "<f8")
    return deck, refs32, f64


@pytest.fixture(scope="session")
def built_library():
    """Build (if stale) and load libbude_gb300.so."""
    from minibude_gb300 import build, capi
    build.build_library()
    return capi.lib()
