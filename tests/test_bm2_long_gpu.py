"""bm2_long: the reference's 1,048,576-pose deck of the 2,672-atom protein against itself
(data/bm2_long/params.txt).  The reference ships it without poses.in and without reference
energies; gb300-makedeck regenerates the poses from the same inputs and the oracle's FP64 rerun
stands in for the missing energies on a sample of poses.  Also the chunked host-streaming
evaluation (bude_gpu_score_stream) against the one-shot evaluation."""
import gzip
import os
import subprocess

import numpy as np
import pytest

import oracle
from minibude_gb300 import Deck, build, read_deck
from minibude_gb300.model import GpuContext, PinnedBuffer

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "makedeck")
F64_TOL = 2e-4


@pytest.fixture(scope="module")
def bm2_long(tmp_path_factory):
    build.build_library()
    exe = build.build_makedeck()
    d = tmp_path_factory.mktemp("bm2_long")
    for name in ("by_atom.bhff", "bm2_protein.mol2"):
        with gzip.open(os.path.join(FIX, name + ".gz"), "rb") as g:
            (d / name).write_bytes(g.read())
    out = d / "deck"
    r = subprocess.run([exe, "-f", d / "by_atom.bhff", "-p", d / "bm2_protein.mol2", "-l", d / "bm2_protein.mol2",
                        "-o", out, "-n", "1048576", "--force", "--no-energies"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return read_deck(str(out), need_refs=False)


def test_bm2_long_deck_shape(bm2_long):
    assert bm2_long.natpro == 2672 and bm2_long.natlig == 2672 and bm2_long.nposes == 1 << 20
    assert len(np.unique(bm2_long.poses.T, axis=0)) == bm2_long.nposes  # distinct grid points


def test_bm2_long_streamed_equals_one_shot_and_fp64(bm2_long):
    with GpuContext(0) as ctx:
        ctx.upload(bm2_long)
        cfg, _ = ctx.autotune(max_ms=3000)
        ctx.run(cfg)
        full = ctx.download()
        # poses from pinned host memory, streamed in uneven chunks
        n = bm2_long.nposes
        pin_p, pin_e = PinnedBuffer((6, n)), PinnedBuffer((n,))
        try:
            pin_p.array[:] = bm2_long.poses
            for chunk in (100000, 1 << 18):
                pin_e.array[:] = np.nan
                ctx.score_stream(cfg, pin_p.array, pin_e.array, chunk=chunk)
                assert np.array_equal(pin_e.array, full), chunk
        finally:
            pin_p.free()
            pin_e.free()
        # pageable memory and a chunk larger than the deck work too
        e = np.full(n, np.nan, np.float32)
        ctx.score_stream(cfg, np.ascontiguousarray(bm2_long.poses), e, chunk=2 * n)
        assert np.array_equal(e, full)
    assert np.all(np.isfinite(full))
    idx = np.random.default_rng(5).choice(bm2_long.nposes, 48, replace=False)
    sub = Deck(bm2_long.protein, bm2_long.ligand, bm2_long.forcefield, np.ascontiguousarray(bm2_long.poses[:, idx]),
               None, len(idx), "bm2_long sample")
    f64 = oracle.fasten_f64(sub)
    err = np.abs(full[idx].astype(np.float64) - f64) / np.maximum(np.abs(f64), 1.0)
    assert err.max() < F64_TOL, err.max()


def test_stream_errors(built_library):
    from minibude_gb300.capi import BudeError
    from minibude_gb300.model import launch_cfg
    with GpuContext(0) as ctx:
        e = np.zeros(4, np.float32)
        with pytest.raises(BudeError):  # no deck uploaded
            ctx.score_stream(launch_cfg(4, 64), np.zeros((6, 4), np.float32), e)
