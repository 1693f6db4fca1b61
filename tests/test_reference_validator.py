"""The reference's own driver judges the GB300 model's energies.

The GB300 model's energies of the bm1_head fixture (the first 1,024 poses of the reference's bm1
deck with its golden energies) are recorded on a GB300 (tests/golden/make_gb300_energies.py) for
each (PPWI, wgsize) the reference driver accepts for that pose count.  On the CPU, the reference's
unmodified src/main.cpp and src/bude.h are compiled with a replay model in the model slot
(tests/replay_model/fasten.hpp) and run on the deck with -p 1,8,16 -w 32,64: its evaluate() and
validate() (src/main.cpp:329-396) must report every run valid and exit 0.  A planted error in one
recording (on the CPU, in a temporary copy) must make it fail.  On a GB300, the model must still
produce the recorded energies, so the recordings cannot go stale."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, ROOT, load_golden

REC = os.path.join(GOLDEN, "bm1_head", "gb300")
RUNS = [(p, w) for p in (1, 8, 16) for w in (32, 64)]
REF = oracle.reference_root()
needs_ref = pytest.mark.skipif(not oracle.reference_tree_present(), reason="reference tree not present")


@pytest.fixture(scope="module")
def reference_driver(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("refdrv")
    src = tmp / "src"
    src.mkdir()
    os.symlink(os.path.join(REF, "src", "bude.h"), src / "bude.h")
    os.symlink(os.path.join(REF, "src", "main.cpp"), src / "main.cpp")
    (src / "cuda").mkdir()  # the slot `-DCUDA` selects in main.cpp's model chain
    os.symlink(os.path.join(ROOT, "tests", "replay_model", "fasten.hpp"), src / "cuda" / "fasten.hpp")
    exe = tmp / "replay-bude"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-DCUDA", str(src / "main.cpp"), "-o", str(exe)],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    return str(exe)


def run_driver(exe, replay_dir, cwd):
    env = dict(os.environ, BUDE_REPLAY_DIR=replay_dir)
    return subprocess.run([exe, "--deck", os.path.join(GOLDEN, "bm1_head"), "-p", "1,8,16", "-w", "32,64", "-i", "2"],
                          stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120, env=env, cwd=cwd)


@needs_ref
def test_reference_validator_accepts_the_recorded_gb300_energies(reference_driver, tmp_path):
    r = run_driver(reference_driver, REC, str(tmp_path))
    assert r.returncode == 0, r.stdout[-3000:]
    flags = re.findall(r"valid: (true|false)", r.stdout)
    assert flags == ["true"] * len(RUNS), r.stdout[-3000:]


@needs_ref
def test_reference_validator_rejects_a_planted_error(reference_driver, tmp_path):
    bad = tmp_path / "rec"
    shutil.copytree(REC, bad)
    e = np.fromfile(bad / "p8_w64.f32", "<f4")
    i = int(np.argmax(e))  # the largest (positive) energy: the signed-denominator rule checks it
    e[i] *= 1.001
    e.astype("<f4").tofile(bad / "p8_w64.f32")
    r = run_driver(reference_driver, str(bad), str(tmp_path))
    assert r.returncode != 0
    assert re.findall(r"valid: (true|false)", r.stdout).count("false") == 1


@pytest.mark.gpu
def test_recordings_are_the_models_current_output(built_library):
    import sys
    sys.path.insert(0, GOLDEN)
    from make_gb300_energies import model_energies
    from minibude_gb300 import validate
    from minibude_gb300.model import GpuContext
    deck, refs, _ = load_golden("bm1_head")
    with GpuContext(0) as ctx:
        for p, w in RUNS:
            got = model_energies(ctx, deck, p, w)
            rec = np.fromfile(os.path.join(REC, f"p{p}_w{w}.f32"), "<f4")
            # bit for bit on the same launch shape; another SM count may choose another protein split
            assert np.array_equal(got, rec) or validate(got, rec)[0] < 1e-3, (p, w)
            max_diff, failed = validate(got, refs)
            assert not failed and max_diff < 0.025
