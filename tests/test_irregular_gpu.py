"""Non-finite and out-of-range inputs: every exact path against the oracle.

The reference's serial model (src/serial/fasten.hpp:98-124) propagates non-finite values: a NaN or
infinite pose angle or translation, a translation so large that x*x + y*y + z*z overflows in FP32
(|d| > ~1.8e19), or a forcefield whose radius sum is zero all give a NaN energy, while a far but
finite pose gives 0 and a huge finite angle an ordinary energy.  The GPU paths must give NaN at
exactly the oracle's NaN positions and match it (max_diff_% < 0.025, plus the FP64 bound
|e - e_fp64| <= 2e-4 * max(|e_fp64|, 1) where both are finite) everywhere else.

Irregular poses are planted at fixed positions, including both sides of the 32-pose boundaries
of the transform pass's bit mask."""
import dataclasses

import numpy as np
import pytest

import oracle
from conftest import load_golden
from minibude_gb300 import SMALL, BatchSpec, synthetic_batch, synthetic_deck, validate
from minibude_gb300.model import GpuContext, launch_cfg

pytestmark = pytest.mark.gpu
F64_TOL = 2e-4

# (pose index, field, value): fields 0-2 are the angles, 3-5 the translation.
PLANTED = [
    (1, 0, np.nan), (2, 1, np.inf), (3, 2, -np.inf), (4, 3, np.inf), (5, 4, -np.inf), (6, 5, np.nan),
    (7, 3, 1e30),    # d^2 overflows: NaN
    (8, 4, 2e19),    # d^2 overflows: NaN
    (9, 5, 1e19),    # far but finite: 0
    (10, 3, 1e12),   # far: 0
    (11, 0, 1e30),   # huge finite angle: an ordinary energy
    (12, 3, 3e11),   # just outside the regular-pose bound: 0
    (13, 4, 2.7e11),  # just inside it: 0
    (31, 3, np.nan), (32, 4, np.nan), (63, 5, 1e25), (64, 0, -np.inf),
]


def plant(poses, extra_last=True):
    p = poses.copy()
    for i, f, v in PLANTED:
        if i < p.shape[1]:
            p[f, i] = v
    if extra_last:
        p[3, -1] = np.nan
    return p


def irregular_deck(n=1000, seed=11):
    deck = synthetic_deck(SMALL, seed, n)
    deck.poses = np.ascontiguousarray(plant(deck.poses))
    return deck


def assert_matches_oracle(got, want32, want64=None):
    """Same NaN positions as the FP32 oracle; parity on the rest."""
    assert np.array_equal(np.isnan(got), np.isnan(want32)), (np.flatnonzero(np.isnan(got) != np.isnan(want32))[:10])
    fin = np.isfinite(want32)
    assert np.all(np.isfinite(got[fin]))
    max_diff, failed = validate(got[fin], want32[fin])
    assert not failed and max_diff < 0.025, (max_diff, failed[:5])
    if want64 is not None:
        both = fin & np.isfinite(want64)
        err = np.abs(got[both].astype(np.float64) - want64[both]) / np.maximum(np.abs(want64[both]), 1.0)
        assert err.max(initial=0.0) < F64_TOL, err.max()


@pytest.fixture(scope="module")
def ctx(built_library):
    c = GpuContext(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def deck_and_refs():
    d = irregular_deck()
    return d, oracle.fasten_f32(d), oracle.fasten_f64(d)


def test_oracle_pins_the_planted_cases(deck_and_refs):
    # The planted cases mean what the file says they mean.
    _, e32, _ = deck_and_refs
    nan_at = {1, 2, 3, 4, 5, 6, 7, 8, 31, 32, 63, 64, 999}
    assert set(np.flatnonzero(np.isnan(e32))) == nan_at
    assert e32[9] == 0 and e32[10] == 0 and e32[12] == 0 and e32[13] == 0
    assert np.isfinite(e32[11]) and e32[11] != 0


@pytest.mark.parametrize("ppwi,wgsize,split,tile,unroll,cluster", [
    (8, 128, 1, 64, 2, 1), (16, 256, 4, 64, 1, 0), (4, 64, 3, 32, 4, 1), (1, 32, 1, 8, 1, 1), (2, 96, 7, 64, 2, 0)])
def test_plain_path(ctx, deck_and_refs, ppwi, wgsize, split, tile, unroll, cluster):
    deck, e32, e64 = deck_and_refs
    ctx.upload(deck)
    ctx.run(launch_cfg(ppwi, wgsize, split, tile, unroll, cluster=cluster))
    assert_matches_oracle(ctx.download(), e32, e64)


def test_host_and_streamed_paths(ctx, deck_and_refs):
    deck, e32, e64 = deck_and_refs
    ctx.upload(deck)
    cfg = launch_cfg(8, 128, 2, 64, 2)
    out = np.full(deck.nposes, 7.0, np.float32)
    ctx.score_host(cfg, deck.poses, out)
    assert_matches_oracle(out, e32, e64)
    for chunk in (33, 320, 5000):
        out = np.full(deck.nposes, 7.0, np.float32)
        ctx.score_stream(cfg, deck.poses, out, chunk=chunk)
        assert_matches_oracle(out, e32, e64)


def test_regular_poses_keep_their_bits(ctx, deck_and_refs):
    # Rescoring the irregular poses leaves every other energy exactly as the exact kernel wrote it.
    deck, _, _ = deck_and_refs
    clean = synthetic_deck(SMALL, 11, deck.nposes)
    cfg = launch_cfg(8, 128, 2, 64, 2)
    ctx.upload(clean)
    ctx.run(cfg)
    a = ctx.download()
    ctx.upload(deck)
    ctx.run(cfg)
    b = ctx.download()
    planted = sorted({i for i, _, _ in PLANTED} | {deck.nposes - 1})
    keep = np.setdiff1d(np.arange(deck.nposes), planted)
    assert np.array_equal(a[keep], b[keep])


def ff_variant(kind):
    """A deck whose forcefield or atoms leave the range of the saturating restatement."""
    deck = synthetic_deck(SMALL, 5, 300)
    ff = deck.forcefield.copy()
    lig = deck.ligand.copy()
    prot = deck.protein.copy()
    lt, pt = int(lig["type"][0]), int(prot["type"][0])
    if kind == "zero_radius_sum":   # radius_L + radius_P == 0 for one pair type: NaN everywhere
        ff["radius"][lt] = 0.0
        ff["radius"][pt] = 0.0
    elif kind == "negative_radius":  # radius sum < 0: the steric term is 0, not 76
        ff["radius"][lt] = -4.0
    elif kind == "nan_hphb":
        ff["hphb"][pt] = np.nan
    elif kind == "inf_elsc":
        ff["elsc"][lt] = np.inf
    elif kind == "far_ligand_atom":  # one ligand atom 1e11 A out: finite energies, outside the bound
        lig["x"][0] = 1e11
    elif kind == "nan_protein_atom":
        prot["y"][3] = np.nan
    elif kind == "overflowing_ligand_atom":
        lig["z"][1] = 3e19
    return dataclasses.replace(deck, forcefield=ff, ligand=lig, protein=prot)


@pytest.mark.parametrize("kind", ["zero_radius_sum", "negative_radius", "nan_hphb", "inf_elsc", "far_ligand_atom",
                                  "nan_protein_atom", "overflowing_ligand_atom"])
def test_irregular_decks(ctx, kind):
    deck = ff_variant(kind)
    e32, e64 = oracle.fasten_f32(deck), oracle.fasten_f64(deck)
    ctx.upload(deck)
    for cfg in (launch_cfg(8, 128, 1, 64, 2), launch_cfg(4, 64, 3, 32, 1, cluster=0)):
        ctx.run(cfg)
        assert_matches_oracle(ctx.download(), e32, e64)


def irregular_batch(seed=0):
    deck, _, _ = load_golden("bm2_head")
    b = synthetic_batch(BatchSpec("irr", 7, 12, 40, 40, 700), deck.protein, deck.forcefield, seed)
    poses = [p.copy() for p in b.poses]
    ligands = [l.copy() for l in b.ligands]
    poses[1] = plant(poses[1])                 # irregular poses in a regular ligand
    ligands[3]["x"][0] = np.nan                # every pose of ligand 3 is NaN
    ligands[5]["y"][2] = 1e11                  # ligand 5 is outside the bound, its energies finite
    poses[6][4, :5] = np.inf                   # the last ligand's first poses
    return dataclasses.replace(b, poses=poses, ligands=ligands)


def oracle_batch(b):
    e32 = np.concatenate([oracle.fasten_f32(b.deck(l)) for l in range(b.nligands)])
    e64 = np.concatenate([oracle.fasten_f64(b.deck(l)) for l in range(b.nligands)])
    return e32, e64


@pytest.fixture(scope="module")
def batch_and_refs():
    b = irregular_batch()
    return b, oracle_batch(b)


@pytest.mark.parametrize("cfg,per_ligand", [(launch_cfg(8, 128, 1, 64, 2, cluster=0), False),
                                            (launch_cfg(16, 64, 3, 64, 1, cluster=0), False),
                                            (launch_cfg(8, 128, 1, 64, 2), True)])
def test_batch_paths(ctx, batch_and_refs, cfg, per_ligand):
    b, (e32, e64) = batch_and_refs
    ctx.upload_batch(b)
    ctx.run_batch(cfg, per_ligand=per_ligand)
    got = ctx.download_batch()
    assert_matches_oracle(got, e32, e64)
    off = np.cumsum([0] + [p.shape[1] for p in b.poses])
    assert np.all(np.isnan(got[off[3]:off[4]]))


def test_same_shape_reupload_updates_the_captured_graph(ctx):
    # A batch of the same shape keeps its captured graph; the irregular-ligand flags it reads live on
    # the device, so a re-upload that makes a ligand irregular (or regular again) is honoured.
    b = irregular_batch(seed=2)
    clean = dataclasses.replace(b, ligands=[l.copy() for l in b.ligands], poses=[p.copy() for p in b.poses])
    clean.ligands[3]["x"][0] = 0.5
    clean.ligands[5]["y"][2] = 0.5
    clean.poses[1] = synthetic_batch(BatchSpec("irr", 7, 12, 40, 40, 700), b.protein, b.forcefield, 2).poses[1]
    clean.poses[6][4, :5] = 0.0
    cfg = launch_cfg(8, 128, 1, 64, 2, cluster=0)
    for batch in (clean, b, clean):
        ctx.upload_batch(batch)
        ctx.run_batch(cfg)
        e32, e64 = oracle_batch(batch)
        assert_matches_oracle(ctx.download_batch(), e32, e64)


def test_screen_reports_irregular_poses_exactly(ctx, batch_and_refs):
    b, (e32, _) = batch_and_refs
    ctx.upload_batch(b)
    ctx.surrogate_init(b.protein, b.forcefield, seed=1)
    ctx.screen(launch_cfg(8, 64, 2, 64, 2, cluster=0), top_frac=0.05, audit_frac=0.05, audit_tol=1e9, seed=3)
    final, rescored, _ = ctx.screen_download(b.nligands)
    nan = np.isnan(e32)
    assert np.all(np.isnan(final[nan])) and np.all(rescored[nan])
    # every energy the screen marks as rescored is an exact one
    r = rescored.astype(bool) & ~nan
    max_diff, failed = validate(final[r], e32[r])
    assert not failed and max_diff < 0.025


def test_training_skips_irregular_poses(ctx, batch_and_refs):
    b, _ = batch_and_refs
    ctx.upload_batch(b)
    ctx.surrogate_init(b.protein, b.forcefield, seed=1)
    loss, _ = ctx.surrogate_train(epochs=2, batch_poses=512, seed=4)
    assert np.isfinite(loss)
    assert np.all(np.isfinite(ctx.surrogate_params()))


def test_golden_nonfinite_fixture(ctx):
    # The committed fixture whose energies come from the reference's own serial model.
    deck, refs, f64 = load_golden("nonfinite")
    ctx.upload(deck)
    for cfg in (launch_cfg(8, 128, 1, 64, 2), launch_cfg(16, 32, 4, 64, 1, cluster=0)):
        ctx.run(cfg)
        assert_matches_oracle(ctx.download(), refs, f64)
