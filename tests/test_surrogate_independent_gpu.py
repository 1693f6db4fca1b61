"""The surrogate's inputs and optimiser against computations that share nothing with the GPU.

* Field features: the 13 protein-field channels of every (pose, ligand atom) row are rebuilt on
  the CPU from the protein and forcefield alone -- the channel formulas evaluated in float64 at
  every grid point, scaled to unit standard deviation, rounded to the FP16 texels, and sampled
  trilinearly at positions transformed on the CPU from the raw poses (clamped at the grid's faces).
  The tolerance per value is the BF16 rounding of the feature (2^-8 relative) plus the texture
  unit's 8-bit interpolation weights (3/256 of the spread of the 8 surrounding texels) plus 2e-3.
  The type-embedding and position features are checked the same way.
* Adam: two optimiser steps of bude_surrogate_train (lr, betas 0.9/0.999, eps 1e-8; the cosine
  schedule is at its start, so the rate is lr) against torch.optim.Adam on the gradients the
  library reports at the same parameters."""
import numpy as np
import pytest

from minibude_gb300 import SMALL, BatchSpec, synthetic_batch, synthetic_deck
from minibude_gb300.model import GpuContext

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

N_CH = 13


def small_protein():
    d = synthetic_deck(SMALL, 0, 1)
    return d.protein, d.forcefield


def cpu_field_grid(protein, ff, extent, spacing):
    """[n, n, n, 13] scaled channels (float64) on the grid over [-extent, extent]^3, indexed
    [ix, iy, iz]; and n."""
    f32 = np.float32
    n = int(np.ceil(f32(2.0) * f32(extent) / f32(spacing))) + 1
    axis = (f32(-extent) + np.arange(n, dtype=f32) * f32(spacing)).astype(np.float64)
    gx, gy, gz = np.meshgrid(axis, axis, axis, indexing="ij")
    pts = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], 1)
    t = protein["type"].astype(int)
    R = ff["radius"][t].astype(np.float64)
    q = ff["elsc"][t].astype(np.float64)
    hp = ff["hphb"][t].astype(np.float64)
    is_f = ff["hbtype"][t] == 70
    P = np.stack([protein["x"], protein["y"], protein["z"]], 1).astype(np.float64)
    c = np.zeros((len(pts), N_CH))
    c[:, 12] = 8.0
    sat = lambda v: np.clip(v, 0.0, 1.0)  # noqa: E731
    for a in range(0, len(pts), 1024):
        r = np.sqrt(((pts[a:a + 1024, None, :] - P[None]) ** 2).sum(-1))
        for k, probe in enumerate((1.0, 1.5, 2.0, 2.5)):
            c[a:a + 1024, k] = np.maximum(0.0, 1.0 - r / (probe + R)).sum(1)
        bb = r - (1.75 + R)
        s2, s4, s55, s1 = sat(1 - bb * 0.5), sat(1 - bb * 0.25), sat(1 - bb / 5.5), sat(1 - bb)
        c[a:a + 1024, 4] = (q * s2).sum(1)
        c[a:a + 1024, 5] = (q * s4).sum(1)
        c[a:a + 1024, 6] = (np.abs(q) * s2).sum(1)
        c[a:a + 1024, 7] = (np.abs(q) * s4).sum(1)
        c[a:a + 1024, 8] = (np.where(is_f, q, 0.0) * s4).sum(1)
        c[a:a + 1024, 9] = (np.where(hp < 0, hp, 0.0) * s55).sum(1)
        c[a:a + 1024, 10] = (np.where(hp > 0, hp, 0.0) * s1).sum(1)
        c[a:a + 1024, 11] = (np.where(hp < 0, hp, 0.0) * s1).sum(1)
        c[a:a + 1024, 12] = np.minimum(8.0, (r - R).min(1))
    c[:, 12] = np.maximum(c[:, 12], -3.0)
    var = (c ** 2).mean(0) - c.mean(0) ** 2
    scale = np.where(var > 1e-12, 1.0 / np.sqrt(np.maximum(var, 1e-300)), 1.0)
    texels = (c * scale).astype(np.float16).astype(np.float64)
    return texels.reshape(n, n, n, N_CH), n


def trilinear(texels, n, extent, spacing, pos):
    """Texture-style sample: texel i of an axis at coordinate i (+0.5 in texture space), clamped
    addressing; returns (value, spread of the 8 texels) per row and channel."""
    u = (pos + extent) / spacing
    i0 = np.floor(u).astype(int)
    a = u - i0
    lo = np.clip(i0, 0, n - 1)
    hi = np.clip(i0 + 1, 0, n - 1)
    val = np.zeros((len(pos), N_CH))
    corners = []
    for cx in (0, 1):
        for cy in (0, 1):
            for cz in (0, 1):
                ix = np.where(cx, hi[:, 0], lo[:, 0])
                iy = np.where(cy, hi[:, 1], lo[:, 1])
                iz = np.where(cz, hi[:, 2], lo[:, 2])
                w = (np.where(cx, a[:, 0], 1 - a[:, 0]) * np.where(cy, a[:, 1], 1 - a[:, 1]) *
                     np.where(cz, a[:, 2], 1 - a[:, 2]))
                t = texels[ix, iy, iz]
                corners.append(t)
                val += w[:, None] * t
    corners = np.stack(corners)
    return val, corners.max(0) - corners.min(0)


def pose_positions(batch, poses):
    """Ligand atom positions of the given batch poses, row by row (pose by pose), in float64."""
    off = batch.pose_offsets()
    out, types = [], []
    block = batch.pose_block().astype(np.float64)
    for p in poses:
        l = int(np.searchsorted(off, p, side="right") - 1)
        sx, sy, sz = np.sin(block[:3, p])
        cx, cy, cz = np.cos(block[:3, p])
        Rm = np.array([[cy * cz, sx * sy * cz - cx * sz, cx * sy * cz + sx * sz],
                       [cy * sz, sx * sy * sz + cx * cz, cx * sy * sz - sx * cz],
                       [-sy, sx * cy, cx * cy]])
        lig = batch.ligands[l]
        xyz = np.stack([lig["x"], lig["y"], lig["z"]], 1).astype(np.float64)
        out.append(xyz @ Rm.T + block[3:6, p])
        types.append(lig["type"])
    return np.concatenate(out), np.concatenate(types)


def bf16(x):
    return torch.tensor(np.asarray(x, np.float32)).to(torch.bfloat16).to(torch.float32).numpy().astype(np.float64)


@pytest.mark.parametrize("spacing", [1.25, 2.0])
def test_field_features_match_an_independent_cpu_grid(built_library, spacing):
    protein, ff = small_protein()
    extent = 11.0
    batch = synthetic_batch(BatchSpec("feat", 6, 16, 40, 40, 40), protein, ff, 21)
    # Two ligands pushed out of the grid on some axes, to exercise the clamped faces.
    block_poses = [p.copy() for p in batch.poses]
    block_poses[4][3, :] += 17.0
    block_poses[5][4, :] -= 25.0
    batch = batch.__class__(batch.protein, batch.forcefield, batch.ligands, block_poses, batch.name)
    poses = np.arange(batch.total_poses, dtype=np.int32)
    pos, types = pose_positions(batch, poses)
    with GpuContext(0) as ctx:
        ctx.upload_batch(batch)
        ctx.surrogate_init(protein, ff, extent=extent, spacing=spacing, seed=4)
        X, gtypes = ctx.surrogate_features(poses, len(pos))
        params = ctx.surrogate_params()
    X = X.astype(np.float64)
    assert np.array_equal(gtypes, types)
    # features 0..15: the BF16 type embedding
    emb = params[:64 * 16].reshape(64, 16)
    assert np.array_equal(X[:, :16], bf16(emb[types]))
    # features 16..18: the transformed position x 0.1
    want_xyz = pos * 0.1
    assert np.all(np.abs(X[:, 16:19] - want_xyz) <= 2.0 ** -8 * np.abs(want_xyz) + 1e-5)
    # features 19..31: the field channels
    texels, n = cpu_field_grid(protein, ff, extent, spacing)
    want, spread = trilinear(texels, n, extent, spacing, pos)
    tol = 2.0 ** -8 * np.abs(want) + 3.0 / 256.0 * spread + 2e-3
    err = np.abs(X[:, 19:] - want)
    assert np.all(err <= tol), (float((err - tol).max()), np.unravel_index(np.argmax(err - tol), err.shape))
    # the check has teeth: a CPU grid with the steric probe radii shifted by 0.25 A fails it
    texels_bad = texels.copy()
    texels_bad[..., :4] = texels[..., [1, 2, 3, 3]]
    bad, _ = trilinear(texels_bad, n, extent, spacing, pos)
    assert np.any(np.abs(X[:, 19:23] - bad[:, :4]) > tol[:, :4])


def test_adam_steps_match_torch_optim_adam(built_library):
    protein, ff = small_protein()
    batch = synthetic_batch(BatchSpec("adam", 4, 16, 40, 64, 64), protein, ff, 11)
    rng = np.random.default_rng(1)
    labels = rng.normal(0.0, 50.0, batch.total_poses).astype(np.float32)
    every = np.arange(batch.total_poses, dtype=np.int32)
    lr = 1e-3
    with GpuContext(0) as ctx:
        ctx.upload_batch(batch)
        ctx.surrogate_init(protein, ff, seed=5)
        ctx.surrogate_train(0, batch_poses=batch.total_poses, lr=lr, labels=labels, seed=1)  # sets b4, no step
        p0 = ctx.surrogate_params()
        g1, _ = ctx.surrogate_gradient(every, labels)
        ctx.surrogate_train(1, batch_poses=batch.total_poses, lr=lr, labels=labels, seed=1)  # Adam step t = 1
        p1 = ctx.surrogate_params()
        g2, _ = ctx.surrogate_gradient(every, labels)
        ctx.surrogate_train(1, batch_poses=batch.total_poses, lr=lr, labels=labels, seed=2)  # Adam step t = 2
        p2 = ctx.surrogate_params()
    w = torch.tensor(p0.copy(), requires_grad=True)
    opt = torch.optim.Adam([w], lr=lr, betas=(0.9, 0.999), eps=1e-8)
    want = []
    for g in (g1, g2):
        w.grad = torch.tensor(g)
        opt.step()
        want.append(w.detach().numpy().copy())
    # The training step sums the same gradient in another pose order, so compare where the gradient
    # stands well above its FP32 rounding; elsewhere (unused embedding rows: zero) nothing may move.
    for got, ref, g in ((p1, want[0], g1), (p2, want[1], g2)):
        big = np.abs(g) > 1e-4 * np.abs(g).max()
        assert big.sum() > 0.5 * len(g)
        assert np.allclose(got[big] - p0[big], ref[big] - p0[big], rtol=1e-3, atol=1e-3 * lr)
        zero = (g1 == 0) & (g2 == 0)
        assert np.array_equal(got[zero], p0[zero])
    assert not np.array_equal(p1, p0) and not np.array_equal(p2, p1)
