"""Parity of the exact kernel (through the C-ABI) with the oracle and the reference's golden
energies.  Tolerance: the reference driver's own check, max_diff_% < 0.025 (src/bude.h:11), plus
|e - e_fp64| <= 2e-4 * max(|e_fp64|, 1) against the FP64 rerun (the bound the FP32 oracle itself
meets on every fixture)."""
import itertools

import numpy as np
import pytest

import oracle
from conftest import GOLDEN_DECKS, load_golden
from minibude_gb300 import LARGE, SMALL, synthetic_deck, validate
from minibude_gb300.capi import BUDE_ERR_ARG, BUDE_ERR_STATE, BUDE_ERR_TYPE, BudeError
from minibude_gb300.deck import ATOM_DTYPE
from minibude_gb300.model import GpuContext, launch_cfg

pytestmark = pytest.mark.gpu

F64_TOL = 2e-4


def assert_parity(got, refs, f64=None):
    assert np.all(np.isfinite(got))
    max_diff, failed = validate(got, refs)
    assert not failed and max_diff < 0.025, (max_diff, failed[:5])
    if f64 is not None:
        err = np.abs(got.astype(np.float64) - f64) / np.maximum(np.abs(f64), 1.0)
        assert err.max() < F64_TOL, err.max()


@pytest.fixture(scope="module")
def ctx(built_library):
    c = GpuContext(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", GOLDEN_DECKS)
def test_golden_default_shape(ctx, name):
    deck, refs, f64 = load_golden(name)
    ctx.upload(deck)
    ctx.run(ctx.default_cfg(8, 128))
    assert_parity(ctx.download(), refs, f64)


SHAPES = list(itertools.product([1, 2, 4, 8, 16], [32, 128, 512], [1, 2, 8], [8, 64, 256], [1, 2, 4]))


@pytest.mark.parametrize("ppwi,wgsize,split,tile,unroll", SHAPES)
def test_small_all_shapes(ctx, ppwi, wgsize, split, tile, unroll):
    deck, refs, f64 = load_golden("small_head")
    ctx.upload(deck)
    ctx.run(launch_cfg(ppwi, wgsize, split, tile, unroll))
    assert_parity(ctx.download(), refs, f64)


@pytest.mark.parametrize("ppwi,wgsize,split,unroll", [(8, 128, 3, 2), (16, 256, 16, 1), (4, 64, 64, 4),
                                                      (2, 32, 5, 2), (1, 96, 7, 1)])
def test_global_reduce_split_matches_cluster(ctx, ppwi, wgsize, split, unroll):
    # Slices summed through the global buffer give the same bits as the in-cluster sum (same
    # slice order), and both meet the parity bar.
    deck, refs, f64 = load_golden("small_head")
    ctx.upload(deck)
    ctx.run(launch_cfg(ppwi, wgsize, split, 64, unroll, cluster=0))
    a = ctx.download()
    assert_parity(a, refs, f64)
    if split <= 8:
        ctx.run(launch_cfg(ppwi, wgsize, split, 64, unroll, cluster=1))
        assert np.array_equal(a, ctx.download())


@pytest.mark.parametrize("name", ["small_head", "bm2_head", "large_head"])
def test_autotune_pick_is_correct(ctx, name):
    deck, refs, f64 = load_golden(name)
    ctx.upload(deck)
    cfg, ms = ctx.autotune(max_ms=200)
    assert ms > 0
    ctx.run(cfg)
    assert_parity(ctx.download(), refs, f64)
    # cached for the same deck shape
    cfg2, _ = ctx.autotune(max_ms=200)
    assert cfg2.as_dict() == cfg.as_dict()


@pytest.mark.parametrize("n", [1, 7, 31, 33, 129, 1000])
def test_ragged_pose_counts(ctx, n):
    deck, refs, f64 = load_golden("small_head")
    ctx.upload(deck.head(n))
    ctx.run(launch_cfg(8, 128, 2, 64))
    assert_parity(ctx.download(), refs[:n], f64[:n])


@pytest.mark.parametrize("split", [20, 24, 29, 64])
def test_thin_protein_slices(ctx, split):
    # The autotuner's second pass tries slices down to 32 atoms (938 atoms: 20 slices of 48, 24 of
    # 40); 29 and 64 slices leave trailing blocks with no atoms, which must add nothing.
    deck, refs, f64 = load_golden("small_head")
    ctx.upload(deck)
    ctx.run(launch_cfg(8, 128, split, 64, 2, cluster=0))
    assert_parity(ctx.download(), refs, f64)


def test_bm2_all_splits(ctx):
    deck, refs, f64 = load_golden("bm2_head")
    ctx.upload(deck)
    for split in (1, 3, 8):
        ctx.run(launch_cfg(4, 32, split, 128))
        assert_parity(ctx.download(), refs, f64)


def test_deterministic_and_position_independent(ctx):
    # Each pose's sum order depends only on the launch shape, not on where the pose sits: a
    # permutation of the poses permutes the energies bit for bit.
    deck = synthetic_deck(SMALL, 3, 4096)
    cfg = launch_cfg(8, 128, 4, 64)
    ctx.upload(deck)
    ctx.run(cfg)
    a = ctx.download()
    ctx.run(cfg)
    assert np.array_equal(a, ctx.download())
    perm = np.random.default_rng(0).permutation(deck.nposes)
    d2 = deck.head(deck.nposes)
    d2.poses = np.ascontiguousarray(deck.poses[:, perm])
    ctx.upload(d2)
    ctx.run(cfg)
    assert np.array_equal(a[perm], ctx.download())


def test_large_deck_full_size_properties(ctx):
    # Full 1,048,576-pose deck: a sampled subset matches the oracle, the energies of the first
    # 256 poses match the reference's golden values, and a pose's energy does not depend on the
    # other poses in the launch.
    deck = synthetic_deck(LARGE, 0)
    ctx.upload(deck)
    cfg = ctx.default_cfg(8, 128)
    ctx.run(cfg)
    e = ctx.download()
    assert np.all(np.isfinite(e))
    _, refs, f64 = load_golden("large_head")
    assert_parity(e[:256], refs, f64)
    idx = np.random.default_rng(1).choice(deck.nposes, 512, replace=False)
    sub = deck.head(deck.nposes)
    sub.poses = np.ascontiguousarray(deck.poses[:, idx])
    assert_parity(e[idx], oracle.fasten_f32(sub), oracle.fasten_f64(sub))
    ctx.upload(sub)
    ctx.run(cfg)
    assert np.array_equal(ctx.download(), e[idx])


def test_empty_and_degenerate(ctx):
    deck = synthetic_deck(SMALL, 0, 64)
    empty_lig = deck.head(64)
    empty_lig.ligand = np.zeros(0, ATOM_DTYPE)
    ctx.upload(empty_lig)
    ctx.run(launch_cfg(8, 64, 1, 64))
    assert np.array_equal(ctx.download(), np.zeros(64, np.float32))
    empty_pro = deck.head(64)
    empty_pro.protein = np.zeros(0, ATOM_DTYPE)
    ctx.upload(empty_pro)
    ctx.run(launch_cfg(8, 64, 2, 64))
    assert np.array_equal(ctx.download(), np.zeros(64, np.float32))
    no_poses = deck.head(0)
    ctx.upload(no_poses)
    ctx.run(launch_cfg(8, 64, 1, 64))
    assert ctx.download().size == 0


def test_errors(ctx):
    deck = synthetic_deck(SMALL, 0, 64)
    bad = deck.head(64)
    bad.protein = bad.protein.copy()
    bad.protein["type"][5] = -1
    with pytest.raises(BudeError) as ei:
        ctx.upload(bad)
    assert ei.value.code == BUDE_ERR_TYPE
    with pytest.raises(BudeError) as ei:
        ctx.run(launch_cfg(8, 128, 1, 64))  # the failed upload left no deck
    assert ei.value.code == BUDE_ERR_STATE
    with pytest.raises(BudeError) as ei:
        ctx.download()  # nor energies to read back
    assert ei.value.code == BUDE_ERR_STATE
    ctx.upload(deck)
    for cfg in (launch_cfg(3, 128, 1, 64), launch_cfg(8, 100, 1, 64), launch_cfg(8, 128, 9, 64),
                launch_cfg(8, 128, 1, 12), launch_cfg(8, 1024, 1, 64), launch_cfg(8, 128, 1, 64, 3),
                launch_cfg(8, 128, 65, 64, 2, 0), launch_cfg(8, 128, 2, 64, 2, 2)):
        with pytest.raises(BudeError) as ei:
            ctx.run(cfg)
        assert ei.value.code == BUDE_ERR_ARG


def test_fasten_one_shot_and_model(built_library):
    from minibude_gb300.model import Gb300Bude
    deck, refs, f64 = load_golden("bm1_head")
    m = Gb300Bude(4)
    assert m.name() == "gb300"
    devs = m.enumerate_devices()
    assert devs and "sm_103" in devs[0][1]
    assert m.compatible(deck, 64, 0)
    s = m.fasten(deck, 64, 0, iterations=3, warmup=2)
    assert len(s.kernel_times) == 5 and len(s.kernel_ms) == 5
    assert_parity(s.energies, refs, f64)


def test_score_host_round_trip(ctx):
    from minibude_gb300.model import PinnedBuffer
    deck, refs, f64 = load_golden("small_head")
    ctx.upload(deck)
    cfg = launch_cfg(8, 128, 2, 64)
    pin_p = PinnedBuffer((6, deck.nposes))
    pin_p.array[...] = deck.poses
    pin_e = PinnedBuffer((deck.nposes,))
    ctx.score_host(cfg, pin_p.array, pin_e.array, ligand=deck.ligand)
    assert_parity(pin_e.array.copy(), refs, f64)
    pin_p.free()
    pin_e.free()


def test_bounded_wait_runs_out_and_the_context_stays_usable(built_library):
    # A device wait that can never finish (an mbarrier nothing arrives on) gives up at its limit,
    # the host reads BUDE_ERR_TIMEOUT with the error text of a real timeout, and the context goes
    # on working: the next evaluation matches one from before.
    from minibude_gb300 import capi
    from minibude_gb300.capi import BUDE_ERR_TIMEOUT
    deck, _, _ = load_golden("bm1_head")
    with GpuContext(0) as ctx:
        ctx.upload(deck)
        ctx.run(launch_cfg(8, 128))
        before = ctx.download()
        for limit_us in (200, 2000):
            rc, ms = ctx.selftest_wait(limit_us)
            assert rc == BUDE_ERR_TIMEOUT
            assert "bounded device wait ran out" in capi.last_error()
            assert limit_us * 1e-3 <= ms < limit_us * 1e-3 + 50.0, (limit_us, ms)
        ctx.run(launch_cfg(8, 128))
        assert np.array_equal(ctx.download(), before)
        rc, _ = ctx.selftest_wait(0)
        assert rc != 0 and rc != BUDE_ERR_TIMEOUT


@pytest.mark.parametrize("chunk", [1, 7, 333, 4096])
def test_stream_in_small_chunks_equals_one_shot(ctx, chunk):
    # Host-resident poses streamed in chunks (bude_gpu_score_stream), from a row-strided array:
    # every chunk size gives the one-shot energies bit for bit.
    deck, _, _ = load_golden("bm1_head")
    ctx.upload(deck)
    cfg = launch_cfg(4, 64, 2, 32, 2, cluster=0)
    ctx.run(cfg)
    want = ctx.download()
    wide = np.zeros((6, deck.nposes + 5), np.float32)
    wide[:, :deck.nposes] = deck.poses
    e = np.full(deck.nposes, np.nan, np.float32)
    ctx.score_stream(cfg, wide[:, :deck.nposes], e, chunk=chunk)
    assert np.array_equal(e, want)


@pytest.mark.parametrize("ntypes,natpro,natlig", [(1, 50, 3), (150, 700, 40), (64, 1, 1)])
def test_forcefield_and_deck_sizes(ctx, ntypes, natpro, natlig):
    # A one-type and a 150-type forcefield (the slab holds a row per type), a one-atom protein and
    # ligand: the reference's check passes with and without a protein split.  Against FP64 the
    # unsplit launch stays within the bound of test_zy_fp64_error (4x the reference's own FP32
    # error, at least 2e-4); a split adds the slices' partial sums in another order, which on the
    # 28,000-term energies of the 150-type deck moves a near-zero energy by up to ~5e-4.
    from minibude_gb300.deck import DeckSpec
    spec = DeckSpec(f"t{ntypes}", natpro, 15.0, natlig, ntypes, 777)
    deck = synthetic_deck(spec, seed=ntypes)
    want = oracle.fasten_f32(deck)
    f64 = oracle.fasten_f64(deck)
    ref_err = (np.abs(want.astype(np.float64) - f64) / np.maximum(np.abs(f64), 1.0)).max()
    ctx.upload(deck)
    for cfg, bound in ((launch_cfg(8, 64, 1, 32, 2), max(2e-4, 4 * ref_err)),
                       (launch_cfg(8, 64, 2, 32, 2, cluster=0), 1e-3)):
        ctx.run(cfg)
        got = ctx.download()
        max_diff, failed = validate(got, want)
        assert not failed and max_diff < 0.025, (cfg.split, max_diff, failed[:5])
        err = np.abs(got.astype(np.float64) - f64) / np.maximum(np.abs(f64), 1.0)
        assert err.max() < bound, (cfg.split, err.max(), bound)
