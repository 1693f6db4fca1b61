"""The learned pre-screen: MLP forward and gradients against a plain PyTorch FP32 reference,
training behaviour, checkpoints, and the screening pipeline's invariants (the exact kernel computes
the energy of every pose it reports as rescored)."""
import numpy as np
import pytest

import surrogate_ref as ref
from minibude_gb300 import SMALL, BatchSpec, synthetic_batch, synthetic_deck
from minibude_gb300.capi import BUDE_ERR_ARG, BUDE_ERR_STATE, BudeError
from minibude_gb300.model import GpuContext, launch_cfg

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def small_protein():
    d = synthetic_deck(SMALL, 0, 1)
    return d.protein, d.forcefield


@pytest.fixture(scope="module")
def setup(built_library):
    protein, ff = small_protein()
    batch = synthetic_batch(BatchSpec("t", 10, 16, 64, 200, 600), protein, ff, 5)
    ctx = GpuContext(0)
    ctx.upload_batch(batch)
    ctx.surrogate_init(protein, ff, extent=11.0, spacing=0.4, seed=3)
    yield ctx, batch
    ctx.close()


def counts_of(batch, poses):
    lo = batch.pose_offsets()
    lig = np.searchsorted(lo, poses, side="right") - 1
    return np.array([len(batch.ligands[l]) for l in lig])


def test_forward_matches_torch(setup):
    ctx, batch = setup
    ctx.surrogate_score()
    got = ctx.surrogate_download()
    poses = np.arange(0, batch.total_poses, 37, dtype=np.int32)
    cnt = counts_of(batch, poses)
    X, types = ctx.surrogate_features(poses, int(cnt.sum()))
    P = ref.split(ctx.surrogate_params(), torch)
    with torch.no_grad():
        want = ref.pose_sums(torch, ref.row_outputs(torch, P, X, types), cnt).numpy()
    scale = np.maximum(np.abs(want), 1.0)
    assert np.max(np.abs(got[poses] - want) / scale) < 2e-2


def test_tcgen05_and_mma_sync_scorers_agree(setup):
    """The tensor-memory scorer and the warp-level one evaluate the same network, the first in FP16
    (weights, features, activations) and the second in BF16 as the training pass does.  Rounding
    an activation to BF16 moves it by up to 2^-9 of its value, and through the convex hard-swish
    that noise raises the BF16 chain's energies by a few tenths of a per cent on average."""
    ctx, batch = setup
    out = {}
    for kind in ("mma_sync", "tcgen05"):
        ctx.surrogate_set_scorer(kind)
        ctx.surrogate_score()
        out[kind] = ctx.surrogate_download()
    scale = np.maximum(np.abs(out["mma_sync"]), 1.0)
    assert np.all(np.isfinite(out["tcgen05"]))
    assert np.max(np.abs(out["tcgen05"] - out["mma_sync"]) / scale) < 1e-2
    with pytest.raises(ValueError):
        ctx.surrogate_set_scorer("wmma")


def poses_with_rows(batch, target, seed):
    """Pose indices whose ligands' atom counts sum to exactly `target` rows."""
    rng = np.random.default_rng(seed)
    all_cnt = counts_of(batch, np.arange(batch.total_poses))
    for _ in range(200):
        picked, rows = [], 0
        for p in rng.permutation(batch.total_poses):
            if rows + all_cnt[p] <= target:
                picked.append(p)
                rows += all_cnt[p]
            if rows == target:
                return np.array(picked, np.int32)
    raise AssertionError(f"no pose set of {target} rows")


def assert_gradient_matches_torch(ctx, batch, poses, labels):
    grads, pred = ctx.surrogate_gradient(poses, labels)
    cnt = counts_of(batch, poses)
    X, types = ctx.surrogate_features(poses, int(cnt.sum()))
    P = ref.split(ctx.surrogate_params(), torch, requires_grad=True)
    tp = ref.pose_sums(torch, ref.row_outputs(torch, P, X, types), cnt)
    L = ref.loss(torch, tp, labels[poses])
    L.backward()
    assert np.max(np.abs(pred - tp.detach().numpy()) / np.maximum(np.abs(tp.detach().numpy()), 1)) < 2e-2
    rels = {}
    for name, (o, s) in ref.OFF.items():
        g_gpu = grads[o:o + s]
        g_ref = P[name].grad.numpy().reshape(-1)
        if name == "emb":  # only the rows of types that occur
            used = np.unique(types)
            g_gpu = g_gpu.reshape(64, 16)[used].ravel()
            g_ref = g_ref.reshape(64, 16)[used].ravel()
        if name == "b4":
            g_gpu, g_ref = g_gpu[:1], g_ref[:1]
        rels[name] = float(np.linalg.norm(g_gpu - g_ref) / max(np.linalg.norm(g_ref), 1e-12))
    assert max(rels.values()) < 0.05, rels


def test_gradient_matches_torch_autograd(setup):
    ctx, batch = setup
    rng = np.random.default_rng(0)
    labels = rng.normal(50.0, 80.0, batch.total_poses).astype(np.float32)
    poses = rng.choice(batch.total_poses, 300, replace=False).astype(np.int32)
    assert_gradient_matches_torch(ctx, batch, poses, labels)


@pytest.mark.parametrize("rows", [256, 129, 127])
def test_gradient_at_tile_edges(setup, rows):
    """The training pass keeps its rows in 128-row tiles: whole tiles, one row into a second tile,
    and a single partial tile give the same gradients as the FP32 reference."""
    ctx, batch = setup
    labels = np.random.default_rng(1).normal(50.0, 80.0, batch.total_poses).astype(np.float32)
    poses = poses_with_rows(batch, rows, seed=rows)
    assert counts_of(batch, poses).sum() == rows
    assert_gradient_matches_torch(ctx, batch, poses, labels)


def test_gradient_of_one_pose(setup):
    ctx, batch = setup
    labels = np.random.default_rng(2).normal(50.0, 80.0, batch.total_poses).astype(np.float32)
    assert_gradient_matches_torch(ctx, batch, np.array([17], np.int32), labels)


def test_training_reduces_loss_deterministically_and_checkpoints(built_library, tmp_path):
    protein, ff = small_protein()
    batch = synthetic_batch(BatchSpec("t", 8, 16, 64, 400, 800), protein, ff, 9)
    params, losses = [], []
    for _ in range(2):
        with GpuContext(0) as ctx:
            ctx.upload_batch(batch)
            ctx.surrogate_init(protein, ff, seed=1)
            l1, _ = ctx.surrogate_train(1, batch_poses=512, lr=2e-3, seed=7)
            l2, ms = ctx.surrogate_train(6, batch_poses=512, lr=2e-3, seed=8)
            assert ms > 0 and l2 < l1
            params.append(ctx.surrogate_params())
            losses.append((l1, l2))
            ctx.surrogate_score()
            s1 = ctx.surrogate_download()
            ctx.surrogate_save(str(tmp_path / "w.bin"))
    # deterministic for a seed: the weights and the reported losses (read back after each step's
    # loss kernel has finished)
    assert np.array_equal(params[0], params[1]) and losses[0] == losses[1]
    with GpuContext(0) as ctx:
        ctx.upload_batch(batch)
        ctx.surrogate_init(protein, ff, seed=99)
        ctx.surrogate_load(str(tmp_path / "w.bin"))
        assert np.array_equal(ctx.surrogate_params(), params[0])
        ctx.surrogate_score()
        assert np.array_equal(ctx.surrogate_download(), s1)
        with pytest.raises(BudeError):
            ctx.surrogate_load(str(tmp_path / "missing.bin"))


def exact_energies(ctx, split=1):
    ctx.run_batch(launch_cfg(8, 128, split, 64, 2, cluster=0))
    return ctx.download_batch()


@pytest.mark.parametrize("split", [1, 4])
def test_screen_invariants(built_library, split):
    protein, ff = small_protein()
    batch = synthetic_batch(BatchSpec("t", 12, 16, 64, 300, 2000), protein, ff, 11)
    with GpuContext(0) as ctx:
        ctx.upload_batch(batch)
        exact = exact_energies(ctx, split)
        ctx.surrogate_init(protein, ff, seed=2)
        ctx.surrogate_train(4, batch_poses=1024, lr=2e-3, labels=exact, seed=3)
        ctx.surrogate_score()
        sur = ctx.surrogate_download()
        st = ctx.screen(launch_cfg(8, 128, split, 64, 2, cluster=0), top_frac=0.02, audit_frac=0.05, audit_tol=1e9,
                        seed=5)
        final, rescored, err = ctx.screen_download(batch.nligands)
        off = batch.pose_offsets()
        assert st["fallback_ligands"] == 0 and st["rescored_poses"] == rescored.sum()
        for l in range(batch.nligands):
            a, b = off[l], off[l + 1]
            n = b - a
            k = int(np.ceil(np.float32(0.02) * np.float32(n)))
            picks = np.argsort(sur[a:b], kind="stable")[:k]
            assert rescored[a:b][picks].all()
            assert rescored[a:b].sum() >= k
        # exact where rescored (same kernel, bit for bit), surrogate elsewhere
        assert np.array_equal(final[rescored], exact[rescored])
        assert np.array_equal(final[~rescored], sur[~rescored])
        # an impossible tolerance sends every ligand to the exhaustive fallback
        st = ctx.screen(launch_cfg(8, 128, split, 64, 2, cluster=0), audit_tol=-1.0)
        final, rescored, err = ctx.screen_download(batch.nligands)
        assert st["fallback_ligands"] == batch.nligands and rescored.all()
        assert np.array_equal(final, exact)


def test_screen_ties_pick_first_poses(built_library):
    # With every weight zero all surrogate scores tie: the picks are the first k poses of each
    # ligand, in pose order.
    protein, ff = small_protein()
    batch = synthetic_batch(BatchSpec("t", 4, 16, 32, 100, 300), protein, ff, 12)
    with GpuContext(0) as ctx:
        ctx.upload_batch(batch)
        ctx.surrogate_init(protein, ff, seed=2)
        ctx.surrogate_params(np.zeros(ref.NPARAMS, np.float32))
        ctx.screen(launch_cfg(8, 128), top_frac=0.1, audit_frac=0.0, audit_tol=1e9)
        _, rescored, _ = ctx.screen_download(batch.nligands)
        off = batch.pose_offsets()
        for l in range(batch.nligands):
            n = off[l + 1] - off[l]
            k = int(np.ceil(np.float32(0.1) * np.float32(n)))
            assert rescored[off[l]:off[l] + k].all() and not rescored[off[l] + k:off[l + 1]].any()


def test_surrogate_errors(built_library):
    protein, ff = small_protein()
    with GpuContext(0) as ctx:
        with pytest.raises(BudeError) as ei:
            ctx.surrogate_init(protein, ff, extent=100.0, spacing=0.1)
        assert ei.value.code == BUDE_ERR_ARG
        big_ff = np.concatenate([ff, ff, ff])
        with pytest.raises(BudeError):
            ctx.surrogate_init(protein, big_ff)  # 102 types > 64


def test_screen_result_belongs_to_its_batch(built_library):
    # A screen's result is downloadable until the next batch upload, even one of the same shape
    # (whose poses differ); screening that batch gives a result again.
    protein, ff = small_protein()
    a = synthetic_batch(BatchSpec("t", 6, 16, 40, 200, 600), protein, ff, 21)
    b = synthetic_batch(BatchSpec("t", 6, 16, 40, 200, 600), protein, ff, 22)
    cfg = launch_cfg(8, 128, 1, 64, 2, cluster=0)
    with GpuContext(0) as ctx:
        ctx.upload_batch(a)
        ctx.surrogate_init(protein, ff, seed=2)
        ctx.screen(cfg, top_frac=0.05, audit_frac=0.05, audit_tol=1e9, seed=1)
        fa, ra, _ = ctx.screen_download(a.nligands)
        ctx.upload_batch(a)  # the same batch again: still a new upload
        with pytest.raises(BudeError) as ei:
            ctx.screen_download(a.nligands)
        assert ei.value.code == BUDE_ERR_STATE
        ctx.screen(cfg, top_frac=0.05, audit_frac=0.05, audit_tol=1e9, seed=1)
        fa2, ra2, _ = ctx.screen_download(a.nligands)
        assert np.array_equal(fa, fa2) and np.array_equal(ra, ra2)
        ctx.upload_batch(b)
        with pytest.raises(BudeError):
            ctx.screen_download(b.nligands)
        ctx.screen(cfg, top_frac=0.05, audit_frac=0.05, audit_tol=1e9, seed=1)
        fb, _, _ = ctx.screen_download(b.nligands)
        assert not np.array_equal(fa, fb)


def test_screen_chunks_give_the_same_answer(built_library):
    # The ligand-chunk pipeline (rescoring beside the surrogate on a second stream) changes the
    # schedule, not the result; the audit sample has exactly ceil(audit_frac * n) poses.
    protein, ff = small_protein()
    batch = synthetic_batch(BatchSpec("t", 24, 16, 64, 300, 2000), protein, ff, 13)
    with GpuContext(0) as ctx:
        ctx.upload_batch(batch)
        ctx.surrogate_init(protein, ff, seed=2)
        ctx.surrogate_train(2, batch_poses=1024, lr=2e-3, seed=3)
        out = []
        for chunks in (1, 5):
            st = ctx.screen(launch_cfg(8, 128, 4, 64, 2, cluster=0), top_frac=0.02, audit_frac=0.05, audit_tol=1e9,
                            seed=5, chunks=chunks)
            out.append((st, ctx.screen_download(batch.nligands)))
        (st1, (f1, r1, e1)), (st5, (f5, r5, e5)) = out
        assert np.array_equal(f1, f5) and np.array_equal(r1, r5) and np.array_equal(e1, e5)
        off = batch.pose_offsets()
        want = 0
        for l in range(batch.nligands):
            n = int(off[l + 1] - off[l])
            k = min(n, int(np.ceil(np.float32(0.02) * np.float32(n))))
            want += k + min(n - k, int(np.ceil(np.float32(0.05) * np.float32(n))))
        assert st1["rescored_poses"] == st5["rescored_poses"] == want == r1.sum()


def test_screen_rescoring_shape_does_not_change_the_answer(built_library):
    # The shape of the exact rescoring (poses per thread, threads per block, unroll, stage size) is
    # free: every shape gives the same energies bit for bit; a shape the kernel does not have is
    # refused.
    from minibude_gb300.capi import BudeError, BudeLaunchCfg
    protein, ff = small_protein()
    batch = synthetic_batch(BatchSpec("t", 12, 16, 64, 3000, 9000), protein, ff, 17)
    exact = launch_cfg(8, 128, 4, 64, 2, cluster=0)
    with GpuContext(0) as ctx:
        ctx.upload_batch(batch)
        ctx.surrogate_init(protein, ff, seed=2)
        ctx.surrogate_train(2, batch_poses=1024, lr=2e-3, seed=3)
        base = None
        # (ppwi, wgsize, unroll, records per shared-memory stage; 0: the exact launch's 64)
        for p, w, u, t in ((0, 0, 0, 0), (8, 32, 4, 0), (4, 64, 2, 32), (16, 32, 1, 16), (2, 96, 2, 8)):
            ctx.screen(exact, audit_tol=1e9, seed=5, rescore_cfg=BudeLaunchCfg(p, w, 0, t, u, 0))
            got = ctx.screen_download(batch.nligands)
            if base is None:
                base = got
            assert all(np.array_equal(a, b) for a, b in zip(got, base)), (p, w, u, t)
        with pytest.raises(BudeError):
            ctx.screen(exact, rescore_cfg=BudeLaunchCfg(3, 32, 0, 0, 1, 0))
        with pytest.raises(BudeError):  # the stage must divide the exact launch's tile
            ctx.screen(exact, rescore_cfg=BudeLaunchCfg(8, 32, 0, 48, 1, 0))


def test_screen_ragged_ligands(built_library):
    # Ligands with 0, 1, 2, 50 and 3,000 poses in one screen: every count picks
    # ceil(top_frac * n) poses plus the audit, a one-pose ligand is rescored whole, and every
    # rescored energy is the batch kernel's.
    import dataclasses
    protein, ff = small_protein()
    base = synthetic_batch(BatchSpec("t", 5, 16, 64, 3000, 3000), protein, ff, 21)
    poses = [base.poses[0][:, :0], base.poses[1][:, :1], base.poses[2][:, :2], base.poses[3][:, :50], base.poses[4]]
    batch = dataclasses.replace(base, poses=[np.ascontiguousarray(p) for p in poses])
    exact = launch_cfg(8, 64, 4, 64, 2, cluster=0)
    with GpuContext(0) as ctx:
        ctx.upload_batch(batch)
        ctx.run_batch(exact)
        full = ctx.download_batch()
        ctx.surrogate_init(protein, ff, seed=6)
        st = ctx.screen(exact, top_frac=0.02, audit_frac=0.005, audit_tol=1e9, seed=2)
        final, rescored, err = ctx.screen_download(batch.nligands)
    off = batch.pose_offsets()
    want = 0
    for l in range(batch.nligands):
        n = int(off[l + 1] - off[l])
        k = min(n, int(np.ceil(np.float32(0.02) * np.float32(n))))
        a = min(n - k, int(np.ceil(np.float32(0.005) * np.float32(n))))
        assert rescored[off[l]:off[l + 1]].sum() == k + a, l
        want += k + a
    assert st["rescored_poses"] == want and rescored[off[1]]
    assert np.array_equal(final[rescored], full[rescored])
    assert np.all(np.isfinite(final))


def test_screen_from_c(built_library, tmp_path):
    # minibude_gb300/examples/screen_example.c drives batch upload, exhaustive scoring, surrogate
    # training and the screen through the C-ABI alone and checks its own results.
    import os
    import subprocess
    from minibude_gb300 import build
    exe = tmp_path / "screen_example"
    subprocess.run(["gcc", "-std=c11", "-Wall", f"-I{build.INCLUDE}",
                    os.path.join(build.PKG, "examples", "screen_example.c"), f"-L{build.PKG}", "-lbude_gb300",
                    f"-Wl,-rpath,{build.PKG}", "-lm", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatching energies" in r.stdout
