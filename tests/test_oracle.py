"""The oracle, pinned against the reference's golden vectors and its own compiled models (CPU)."""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN_DECKS, load_golden
from minibude_gb300 import SMALL, synthetic_deck, validate, validate_abs
from minibude_gb300.deck import ATOM_DTYPE


@pytest.mark.parametrize("name", GOLDEN_DECKS)
def test_oracle_matches_golden(name):
    deck, refs, f64 = load_golden(name)
    e = oracle.fasten_f32(deck)
    max_diff, failed = validate(e, refs)
    assert failed == [] and max_diff < 0.025, (max_diff, failed[:5])
    assert validate_abs(e, refs) < 0.025
    # FP32 oracle and the golden FP32 energies both sit close to the FP64 rerun.
    scale = np.maximum(np.abs(f64), 1.0)
    assert np.max(np.abs(e - f64) / scale) < 2e-4
    assert np.max(np.abs(refs - f64) / scale) < 2e-4


def test_bm1_readme_energies():
    # The first eight bm1 energies printed by the reference's README (README.md:125-132).
    deck, refs, _ = load_golden("bm1_head")
    e = oracle.fasten_f32(deck.head(8))
    readme = np.array([865.52, 25.07, 368.43, 14.67, 574.99, 707.35, 33.95, 135.59], np.float32)
    assert np.allclose(e, readme, atol=0.006)


def test_oracle_fast_build_matches_strict():
    deck, refs, _ = load_golden("small_head")
    a = oracle.fasten_f32(deck)
    b = oracle.fasten_f32(deck, fast=True)
    assert validate(b, a)[0] < 0.01


@pytest.mark.parametrize("n", [1, 5, 16, 17, 33])
def test_oracle_tail_poses(n):
    # Poses past a multiple of the group size are computed and equal the same poses in a full run.
    deck, _, _ = load_golden("small_head")
    full = oracle.fasten_f32(deck.head(64))
    part = oracle.fasten_f32(deck.head(n))
    assert np.array_equal(full[:n], part)


def test_oracle_thread_count_independent():
    deck, _, _ = load_golden("small_head")
    a = oracle.fasten_f32(deck.head(256), nthreads=1)
    b = oracle.fasten_f32(deck.head(256), nthreads=4)
    assert np.array_equal(a, b)


def test_oracle_rejects_bad_type():
    deck = synthetic_deck(SMALL, 0, 16)
    deck.ligand = deck.ligand.copy()
    deck.ligand["type"][3] = deck.ntypes
    with pytest.raises(ValueError):
        oracle.fasten_f32(deck)


def test_oracle_empty_ligand_gives_zero():
    deck = synthetic_deck(SMALL, 0, 16)
    deck.ligand = np.zeros(0, ATOM_DTYPE)
    assert np.array_equal(oracle.fasten_f32(deck), np.zeros(16, np.float32))


@pytest.mark.skipif(not oracle.reference_available(), reason="reference tree not built here")
def test_oracle_vs_reference_models():
    deck = synthetic_deck(SMALL, 7, 512)
    e = oracle.fasten_f32(deck)
    for ppwi in (1, 4, 16, 64):
        r = oracle.ref_omp_fasten(deck, ppwi)
        assert validate(e, r)[0] < 0.005
    s = oracle.ref_serial_fasten(deck.head(64))
    assert validate(e[:64], s)[0] < 0.005


@pytest.mark.parametrize("ppwi", [1, 2, 4, 8, 16, 32, 64, 128])
def test_flop_counts(ppwi):
    # The reference's count (src/main.cpp:359) is the PPWI-independent algorithmic count plus the
    # per-pair setup (10 per interaction, 2 per ligand atom) once per group of PPWI poses.
    from minibude_gb300.validate import algorithmic_flops, reference_formula_flops
    n, lig, pro = 65536, 26, 938
    ref = reference_formula_flops(n, lig, pro, ppwi)
    setup = (n / ppwi) * (2.0 * lig + 10.0 * lig * pro)
    assert ref == pytest.approx(algorithmic_flops(n, lig, pro) + setup, rel=1e-12)
    assert reference_formula_flops(n, lig, pro, 2 * ppwi) < ref


def test_oracle_nonfinite_poses_match_the_reference_serial_model():
    # NaN and infinite poses, overflowing squared distances, far and huge-angle poses: the oracle
    # gives NaN exactly where the reference's SerialBude<1> does and its energies elsewhere.
    deck, refs, f64 = load_golden("nonfinite")
    e = oracle.fasten_f32(deck)
    nan = np.isnan(refs)
    assert nan.sum() == 13
    assert np.array_equal(np.isnan(e), nan)
    max_diff, failed = validate(e[~nan], refs[~nan])
    assert failed == [] and max_diff < 0.025, (max_diff, failed[:5])
