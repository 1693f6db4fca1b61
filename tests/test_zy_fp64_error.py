"""Error of the GPU energies against an FP64 evaluation of the reference kernel, per workload.

The FP64 restatement (oracle/bude_oracle.c, serial/fasten.hpp:18-132 in double) is run on a
sample of each workload's poses: bm1 and bm2 (the reference's decks, first 4096 poses of the
committed heads), the 938-atom deck of 65,536 poses, the 4096 x 64 deck of 1,048,576 poses and the
256-ligand batch.  The test prints one line per workload (max and 99.9th percentile of
|E_gpu - E_f64| / max(|E_f64|, 1), and the same for the reference's own FP32 fast-math path,
oracle.fasten_f32) and bounds the GPU error by the FP32 reference's error plus a small margin."""
import numpy as np
import pytest

import oracle
from conftest import load_golden
from minibude_gb300 import BATCH, LARGE, SMALL, synthetic_batch, synthetic_deck
from minibude_gb300.model import GpuContext

pytestmark = pytest.mark.gpu


def rel(got, f64):
    e = np.abs(got.astype(np.float64) - f64) / np.maximum(np.abs(f64), 1.0)
    return float(e.max()), float(np.quantile(e, 0.999))


def report(name, gpu, f32, f64):
    g, f = rel(gpu, f64), rel(f32, f64)
    print(f"\nFP64 error {name}: gpu max {g[0]:.3e} p99.9 {g[1]:.3e} | reference-fp32 max {f[0]:.3e} "
          f"p99.9 {f[1]:.3e} | poses {len(f64)}")
    assert g[0] < max(2e-4, 4 * f[0])


@pytest.fixture(scope="module")
def ctx(built_library):
    c = GpuContext(0)
    yield c
    c.close()


def score(ctx, deck):
    ctx.upload(deck)
    cfg, _ = ctx.autotune(max_ms=300)
    ctx.run(cfg)
    return ctx.download()


@pytest.mark.parametrize("name", ["bm1_head", "bm2_head"])
def test_reference_decks(ctx, name):
    deck, _, _ = load_golden(name)
    report(name, score(ctx, deck), oracle.fasten_f32(deck), oracle.fasten_f64(deck))


@pytest.mark.parametrize("spec,n", [(SMALL, 65536), (LARGE, 4096)])
def test_synthetic_decks(ctx, spec, n):
    deck = synthetic_deck(spec, seed=0)
    gpu = score(ctx, deck)[:n]
    sub = deck.head(n)
    report(f"{spec.name} (first {n} poses)", gpu, oracle.fasten_f32(sub), oracle.fasten_f64(sub))


def test_batch(ctx):
    bm2, _, _ = load_golden("bm2_head")
    b = synthetic_batch(BATCH, bm2.protein, bm2.forcefield, 0)
    ctx.upload_batch(b)
    cfg, _ = ctx.autotune_batch()
    ctx.run_batch(cfg)
    e = ctx.download_batch()
    off = b.pose_offsets()
    # 8 ligands spread over the atom-count range, first 2048 poses of each
    pick = np.argsort([len(l) for l in b.ligands])[np.linspace(0, b.nligands - 1, 8).astype(int)]
    gpu, f32, f64 = [], [], []
    for l in pick:
        d = b.deck(int(l)).head(2048)
        gpu.append(e[off[l]:off[l] + d.nposes])
        f32.append(oracle.fasten_f32(d))
        f64.append(oracle.fasten_f64(d))
    report(f"{BATCH.name} (8 ligands x 2048 poses)", np.concatenate(gpu), np.concatenate(f32), np.concatenate(f64))
