"""Batched ragged scoring (persistent CUDA-graph launch and one launch per ligand) against the oracle
and the single-deck path."""
import numpy as np
import pytest

import oracle
from conftest import load_golden
from minibude_gb300 import BatchSpec, synthetic_batch, validate
from minibude_gb300.capi import BUDE_ERR_ARG, BUDE_ERR_STATE, BUDE_ERR_TYPE, BudeError
from minibude_gb300.model import GpuContext, launch_cfg

pytestmark = pytest.mark.gpu
F64_TOL = 2e-4


def bm2_protein():
    deck, _, _ = load_golden("bm2_head")
    return deck.protein, deck.forcefield


def small_batch(seed=0, n=12, lo=12, hi=96, plo=50, phi=3000):
    protein, ff = bm2_protein()
    return synthetic_batch(BatchSpec("t", n, lo, hi, plo, phi), protein, ff, seed)


def oracle_batch(batch):
    e32 = np.concatenate([oracle.fasten_f32(batch.deck(l)) for l in range(batch.nligands)])
    e64 = np.concatenate([oracle.fasten_f64(batch.deck(l)) for l in range(batch.nligands)])
    return e32, e64


def assert_parity(got, want, f64):
    assert np.all(np.isfinite(got))
    max_diff, failed = validate(got, want)
    assert not failed and max_diff < 0.025, (max_diff, failed[:5])
    err = np.abs(got.astype(np.float64) - f64) / np.maximum(np.abs(f64), 1.0)
    assert err.max() < F64_TOL, err.max()


@pytest.fixture(scope="module")
def ctx(built_library):
    c = GpuContext(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def batch_and_refs():
    b = small_batch()
    return b, oracle_batch(b)


@pytest.mark.parametrize("ppwi,wgsize,unroll", [(16, 128, 1), (8, 128, 2), (4, 64, 4), (2, 96, 2), (1, 32, 1)])
def test_persistent_batch_matches_oracle(ctx, batch_and_refs, ppwi, wgsize, unroll):
    b, (e32, e64) = batch_and_refs
    ctx.upload_batch(b)
    ctx.run_batch(launch_cfg(ppwi, wgsize, 1, 64, unroll))
    got = ctx.download_batch()
    assert_parity(got, e32, e64)
    # the captured graph is relaunched: same bits
    ctx.run_batch(launch_cfg(ppwi, wgsize, 1, 64, unroll))
    assert np.array_equal(got, ctx.download_batch())


def test_persistent_equals_per_ligand_unsplit(ctx, batch_and_refs):
    # Without a protein split every launch shape sums each pose in the same order, so the
    # persistent kernel and one plain launch per ligand agree bit for bit.
    b, (e32, e64) = batch_and_refs
    ctx.upload_batch(b)
    ctx.run_batch(launch_cfg(8, 128, 1, 64, 2))
    persistent = ctx.download_batch()
    per_lig = []
    for l in range(b.nligands):
        ctx.upload(b.deck(l))
        ctx.run(launch_cfg(8, 128, 1, 64, 2))
        per_lig.append(ctx.download())
    assert np.array_equal(persistent, np.concatenate(per_lig))


def test_short_items_run_with_fewer_poses_per_thread(ctx):
    # An item that fits in P/4 or P/2 poses per thread (a ligand's last pose block) runs with that
    # many.  Pose counts around each boundary (P = 16, 64 threads: 256 / 512 / 1024 poses) give the
    # same bits as a launch with 2 poses per thread, and match the oracle.
    import dataclasses
    base = small_batch(seed=3, n=12, plo=50, phi=3000)
    counts = [1, 255, 256, 257, 511, 512, 513, 1023, 1024, 1025, 1024 + 256, 2048 + 700]
    rng = np.random.default_rng(4)
    poses = []
    for n in counts:
        p = np.empty((6, n), np.float32)
        p[:3] = rng.uniform(0, 2 * np.pi, (3, n))
        p[3:] = rng.uniform(-3, 3, (3, n))
        poses.append(p)
    b = dataclasses.replace(base, poses=poses)
    ctx.upload_batch(b)
    ctx.run_batch(launch_cfg(16, 64, 1, 64, 1))
    got = ctx.download_batch()
    ctx.run_batch(launch_cfg(2, 64, 1, 64, 1))
    assert np.array_equal(got, ctx.download_batch())
    ctx.run_batch(launch_cfg(16, 64, 3, 64, 2, cluster=0))
    split = ctx.download_batch()
    ctx.run_batch(launch_cfg(2, 32, 3, 64, 4, cluster=0))
    assert np.array_equal(split, ctx.download_batch())
    e32, e64 = oracle_batch(b)
    assert_parity(got, e32, e64)
    assert_parity(split, e32, e64)


@pytest.mark.parametrize("split,ppwi,wgsize", [(2, 8, 128), (5, 4, 64), (8, 16, 32), (64, 2, 64)])
def test_split_batch_matches_oracle_and_is_deterministic(ctx, batch_and_refs, split, ppwi, wgsize):
    # Protein slices per item (split 64 leaves some slices empty for the 2672-atom protein): parity
    # with the oracle, and the same bits for every pose shape with the same split and tile.
    b, (e32, e64) = batch_and_refs
    ctx.upload_batch(b)
    ctx.run_batch(launch_cfg(ppwi, wgsize, split, 64, 2, cluster=0))
    got = ctx.download_batch()
    assert_parity(got, e32, e64)
    ctx.run_batch(launch_cfg(ppwi, wgsize, split, 64, 2, cluster=0))
    assert np.array_equal(got, ctx.download_batch())
    ctx.run_batch(launch_cfg(4, 128, split, 64, 1, cluster=0))
    assert np.array_equal(got, ctx.download_batch())


def test_per_ligand_mode_matches_oracle(ctx, batch_and_refs):
    b, (e32, e64) = batch_and_refs
    ctx.upload_batch(b)
    ctx.run_batch(launch_cfg(8, 128, 1, 64, 2), per_ligand=True)
    assert_parity(ctx.download_batch(), e32, e64)


def test_batch_autotune_and_ragged_edges(ctx):
    # ligands with 1 atom and 1 pose, an empty pose list and the largest sizes in one batch
    protein, ff = bm2_protein()
    b = synthetic_batch(BatchSpec("edge", 5, 1, 96, 1, 1), protein, ff, 3)
    b.poses[2] = b.poses[2][:, :0]
    b.poses[4] = synthetic_batch(BatchSpec("x", 1, 5, 5, 1025, 1025), protein, ff, 4).poses[0]
    e32, e64 = oracle_batch(b)
    ctx.upload_batch(b)
    cfg, ms = ctx.autotune_batch(max_ms=500)
    assert ms > 0
    ctx.run_batch(cfg)
    assert_parity(ctx.download_batch(), e32, e64)


def test_batch_errors(ctx):
    b = small_batch(n=3)
    b.ligands[1] = b.ligands[1].copy()
    b.ligands[1]["type"][0] = 99
    with pytest.raises(BudeError) as ei:
        ctx.upload_batch(b)
    assert ei.value.code == BUDE_ERR_TYPE
    with pytest.raises(BudeError) as ei:
        ctx.run_batch(launch_cfg(8, 128))
    assert ei.value.code == BUDE_ERR_STATE
    ok = small_batch(n=3)
    ctx.upload_batch(ok)
    with pytest.raises(BudeError) as ei:
        ctx.run_batch(launch_cfg(3, 128))
    assert ei.value.code == BUDE_ERR_ARG
    # uploading a deck replaces the batch
    deck, _, _ = load_golden("small_head")
    ctx.upload(deck)
    with pytest.raises(BudeError):
        ctx.run_batch(launch_cfg(8, 128))


def test_batch_pose_limit(ctx):
    # Work items index poses with 32-bit integers: a batch of 2^31 poses is refused before any pose
    # is read (a one-pose buffer stands in for the poses; nothing reads past it).
    from minibude_gb300 import capi
    from minibude_gb300.model import _atoms, _ff
    b = small_batch(n=1)
    prot, ff, atoms = _atoms(b.protein), _ff(b.forcefield), _atoms(b.ligands[0])
    lig_off = np.array([0, atoms.size], np.int32)
    pose_off = np.array([0, 2 ** 31], np.int64)
    one = np.zeros(6, np.float32)
    rc = capi.lib().bude_gpu_upload_batch(ctx.handle, capi.ptr(prot), prot.size, capi.ptr(ff), ff.size, 1,
                                          capi.ptr(atoms), capi.ptr(lig_off), capi.ptr(one), 2 ** 31,
                                          capi.ptr(pose_off))
    assert rc == BUDE_ERR_ARG and "2^31" in capi.last_error()
    with pytest.raises(BudeError) as ei:
        ctx.run_batch(launch_cfg(8, 128))
    assert ei.value.code == BUDE_ERR_STATE


def _reshaped(b, seed, poses_shift=0):
    """A batch of the same ligand sizes with other coordinates; poses_shift moves poses between the
    first two ligands (same ligand count and total pose count, another shape)."""
    import dataclasses
    rng = np.random.default_rng(seed)
    ligs = []
    for l in b.ligands:
        m = l.copy()
        for k in ("x", "y", "z"):
            m[k] = m[k] + rng.normal(0, 0.3, len(m)).astype(np.float32)
        ligs.append(m)
    poses = [p + rng.normal(0, 0.05, p.shape).astype(np.float32) for p in b.poses]
    if poses_shift:
        moved = poses[0][:, :poses_shift]
        poses[0] = np.ascontiguousarray(poses[0][:, poses_shift:])
        poses[1] = np.ascontiguousarray(np.concatenate([poses[1], moved], axis=1))
    return dataclasses.replace(b, ligands=ligs, poses=poses)


def test_reupload_of_the_same_shape_and_of_another(ctx):
    # A batch of the same shape re-uses the uploaded batch's work items and captured graph; one
    # with the same ligand and pose totals but another split rebuilds them.  Either way the
    # energies equal those of a fresh context.
    a = small_batch(seed=5, n=6, plo=300, phi=2000)
    same = _reshaped(a, 1)
    other = _reshaped(a, 2, poses_shift=97)
    cfg = launch_cfg(8, 128, 2, 64, 2, cluster=0)
    ctx.upload_batch(a)
    ctx.run_batch(cfg)
    got = {}
    for name, b in (("same", same), ("other", other)):
        ctx.upload_batch(b)
        ctx.run_batch(cfg)
        got[name] = ctx.download_batch()
    with GpuContext(0) as fresh:
        for name, b in (("same", same), ("other", other)):
            fresh.upload_batch(b)
            fresh.run_batch(cfg)
            assert np.array_equal(got[name], fresh.download_batch()), name


def test_surrogate_items_follow_the_batch_shape(ctx):
    # Surrogate scores after a re-upload with the same totals but another per-ligand split equal
    # those of a fresh context with the same weights.
    a = small_batch(seed=8, n=5, plo=300, phi=1500)
    other = _reshaped(a, 3, poses_shift=129)
    protein, ff = bm2_protein()
    ctx.upload_batch(a)
    ctx.surrogate_init(protein, ff, seed=4)
    ctx.surrogate_score()
    ctx.upload_batch(other)
    ctx.surrogate_score()
    got = ctx.surrogate_download()
    with GpuContext(0) as fresh:
        fresh.upload_batch(other)
        fresh.surrogate_init(protein, ff, seed=4)
        fresh.surrogate_score()
        assert np.array_equal(got, fresh.surrogate_download())


def test_upload_from_pinned_arrays(ctx, batch_and_refs):
    # The array form of the batch upload, from a row-strided pinned buffer, and the download into
    # pinned memory give the energies of the object form.
    from minibude_gb300.model import PinnedBuffer
    b, (e32, e64) = batch_and_refs
    cfg = launch_cfg(8, 128, 1, 64, 2)
    ctx.upload_batch(b)
    ctx.run_batch(cfg)
    want = ctx.download_batch()
    block = b.pose_block()
    n = block.shape[1]
    pin_p, pin_e = PinnedBuffer((6, n + 3)), PinnedBuffer((n,))
    try:
        pin_p.array[:, :n] = block
        ctx.upload_batch_arrays(b.protein, b.forcefield, b.atoms(), b.ligand_offsets(), pin_p.array[:, :n],
                                b.pose_offsets())
        ctx.run_batch(cfg)
        got = ctx.download_batch(pin_e.array)
        assert np.array_equal(got, want)
        assert_parity(np.array(got), e32, e64)
    finally:
        pin_p.free()
        pin_e.free()
