"""Validation and throughput statistics of the reference driver (src/main.cpp:96-110, 329-396).

`validate` keeps the reference's rule exactly, quirks included:
  * poses where both |ref| < 1 and |energy| < 1 are skipped (src/main.cpp:336);
  * difference(a, b) = |a - b| / a with the SIGNED reference a in the denominator
    (src/main.cpp:329), so a pose with a negative reference can never fail;
  * the run is valid when 100 * max difference < DIFF_TOLERANCE_PCT = 0.025 (src/bude.h:11,
    src/main.cpp:371).
`validate_abs` is the corrected check (|ref| in the denominator) reported beside it.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Sequence, Tuple

import numpy as np

DIFF_TOLERANCE_PCT = 0.025  # src/bude.h:11 (a float there: 0.025f)


def difference(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """src/main.cpp:329: fabs(double(a) - b) / a, elementwise, a = reference."""
    a64 = np.asarray(a, np.float32).astype(np.float64)
    b64 = np.asarray(b, np.float32).astype(np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.abs(a64 - b64) / a64


def _checked(refs: np.ndarray, energies: np.ndarray) -> np.ndarray:
    refs = np.asarray(refs, np.float32)
    energies = np.asarray(energies, np.float32)
    return ~((np.abs(refs) < 1.0) & (np.abs(energies) < 1.0))


def validate(energies: np.ndarray, refs: np.ndarray) -> Tuple[float, List[int]]:
    """(max_diff_% , failed indices) exactly as src/main.cpp:331-342."""
    energies = np.asarray(energies, np.float32)
    refs = np.asarray(refs, np.float32)[: energies.size]
    mask = _checked(refs, energies)
    diff = difference(refs, energies)
    diff = np.where(mask, diff, 0.0)
    # `if (diff > maxdiff)` never takes a NaN; 0.0 is the start value.
    finite = np.where(np.isnan(diff), 0.0, diff)
    maxdiff = float(max(0.0, finite.max())) if finite.size else 0.0
    failed = np.nonzero(mask & (100.0 * diff > DIFF_TOLERANCE_PCT))[0].tolist()
    return 100.0 * maxdiff, failed


def validate_abs(energies: np.ndarray, refs: np.ndarray) -> float:
    """Max |e - ref| / |ref| in percent over the poses the reference checks (its sign quirk fixed)."""
    energies = np.asarray(energies, np.float32)
    refs = np.asarray(refs, np.float32)[: energies.size]
    mask = _checked(refs, energies)
    if not mask.any():
        return 0.0
    a = refs[mask].astype(np.float64)
    b = energies[mask].astype(np.float64)
    return float(100.0 * np.max(np.abs(a - b) / np.abs(a)))


def is_valid(max_diff_pct: float) -> bool:
    return max_diff_pct < DIFF_TOLERANCE_PCT


@dataclasses.dataclass
class SummaryStats:
    """src/main.cpp:96-110 (population variance)."""
    min: float
    max: float
    sum: float
    mean: float
    variance: float
    std_dev: float

    @classmethod
    def of(cls, ys: Sequence[float]) -> "SummaryStats":
        ys = [float(y) for y in ys]
        s = sum(ys)
        mean = s / len(ys)
        var = sum((y - mean) ** 2 for y in ys) / len(ys)
        return cls(min(ys), max(ys), s, mean, var, math.sqrt(var))


def ops_per_wg(ppwi: int, natlig: int, natpro: int) -> int:
    """The reference's FLOP count per work group (src/main.cpp:359)."""
    return ppwi * 27 + natlig * (2 + ppwi * 18 + natpro * (10 + ppwi * 30)) + ppwi


def algorithmic_flops(nposes: int, natlig: int, natpro: int) -> float:
    """PPWI-independent part of the reference's count: 30 per interaction, 18 per (pose, ligand
    atom) and 28 per pose."""
    return 30.0 * nposes * natlig * natpro + 18.0 * nposes * natlig + 28.0 * nposes


def reference_formula_flops(nposes: int, natlig: int, natpro: int, ppwi: int) -> float:
    """The reference's own FLOP count for a launch with `ppwi` poses per work-item (src/main.cpp:359:
    ops_per_wg = 27 P + natlig (2 + 18 P + natpro (10 + 30 P)) + P, times nposes / P groups).  It
    counts the per-pair setup once per PPWI group, so it depends on PPWI; the PPWI-independent
    part is `algorithmic_flops`."""
    p = float(ppwi)
    ops_per_wg = 27.0 * p + natlig * (2.0 + 18.0 * p + natpro * (10.0 + 30.0 * p)) + p
    return ops_per_wg * (nposes / p)


@dataclasses.dataclass
class Result:
    valid: bool
    max_diff_pct: float
    ms: SummaryStats
    gflops: float
    ginsts: float
    interactions_per_sec: float


def evaluate(kernel_ms: Sequence[float], warmup: int, ppwi: int, nposes: int, natlig: int, natpro: int,
             energies: np.ndarray, refs: np.ndarray) -> Result:
    """src/main.cpp:344-396: drop the warm-up iterations, average, derive the rates."""
    if len(kernel_ms) == 0:
        raise RuntimeError("Sample size is 0, this implementation did not measure kernel runtime!")
    timed = list(kernel_ms)[warmup:]
    ms = sum(timed) / len(timed)
    runtime = ms * 1e-3
    total_ops = float(ops_per_wg(ppwi, natlig, natpro)) * (float(nposes) / float(ppwi))
    gflops = total_ops / runtime / 1e9
    ginsts = 25.0 * natpro * natlig * nposes / runtime / 1e9
    ips = float(nposes) * natlig * natpro / runtime
    max_diff, _ = validate(energies, refs)
    valid = is_valid(max_diff)
    if not valid:
        return Result(False, max_diff, SummaryStats.of([float(np.finfo(np.float64).max)]), 0.0, 0.0, 0.0)
    return Result(True, max_diff, SummaryStats.of(timed), gflops, ginsts, ips)
