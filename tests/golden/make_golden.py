"""Generate the golden fixtures under tests/golden/.  Runs only where the reference tree exists.

Each fixture is a deck directory in the reference's file layout plus:
  ref_energies.out   text energies (the reference's golden format)
  ref_energies.f32   the same values as little-endian float32 (no text rounding)
  f64_energies.f64   the oracle's FP64 rerun of the same poses (for the per-deck error statement)
  source.txt         where the decks and the energies came from

Fixtures:
  bm1_head/   the first 1024 poses of the reference's data/bm1 deck with the first 1024 lines of
              its ref_energies.out (the reference's own published golden vectors)
  bm2_head/   the first 32 poses of data/bm2 with its golden energies
  small_head/ the first 2048 poses of the seeded synthetic bm1-sized deck (938 x 26, seed 0);
              energies from the reference's OmpBude<16>::fasten compiled from its sources
              (oracle/_ref/libref.so)
  large_head/ the first 256 poses of the seeded 4096 x 64 deck (seed 0); energies from OmpBude<16>
  edge/       a hand-made deck (2 protein atoms, 3 ligand atoms, 4 types covering '-', 'D', 'E',
              'F', hphb of both signs and zero) with poses at overlap, contact, each cut-off and
              far away; energies from the reference's SerialBude<1>::fasten
  nonfinite/  the first 80 poses of the seeded synthetic bm1-sized deck (seed 11) with NaN and
              infinite angles and translations, translations whose squared distance overflows
              FP32, far but finite translations and a huge finite angle planted at fixed poses;
              energies from the reference's SerialBude<1>::fasten (NaN where it gives NaN)

Usage (from the repository root):  python tests/golden/make_golden.py [--reference DIR]  (default: oracle/Makefile's BUDE_REFERENCE)
"""
from __future__ import annotations

import argparse
import math
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from minibude_gb300.deck import (ATOM_DTYPE, FF_DTYPE, LARGE, SMALL, Deck, read_deck, synthetic_deck,  # noqa: E402
                                 write_deck)


def save(name: str, deck: Deck, refs: np.ndarray, source: str, fmt: str = "%.6f") -> None:
    d = os.path.join(HERE, name)
    if os.path.isdir(d):
        shutil.rmtree(d)
    write_deck(d, deck, refs, fmt=fmt)
    np.asarray(refs, "<f4").tofile(os.path.join(d, "ref_energies.f32"))
    oracle.fasten_f64(deck).astype("<f8").tofile(os.path.join(d, "f64_energies.f64"))
    with open(os.path.join(d, "source.txt"), "w") as f:
        f.write(source.strip() + "\n")
    print(f"{name}: {deck.natpro} x {deck.natlig} x {deck.nposes}")


def edge_deck() -> Deck:
    ff = np.zeros(4, FF_DTYPE)
    ff[0] = (ord("-"), 1.5, -1.2, 0.0)
    ff[1] = (ord("D"), 1.8, 0.7, 0.4)
    ff[2] = (ord("E"), 1.3, 0.0, -0.6)
    ff[3] = (ord("F"), 2.0, -0.3, 0.9)
    protein = np.zeros(2, ATOM_DTYPE)
    protein[0] = (0.0, 0.0, 0.0, 3)
    protein[1] = (6.0, 1.0, -2.0, 1)
    ligand = np.zeros(3, ATOM_DTYPE)
    ligand[0] = (0.0, 0.0, 0.0, 3)
    ligand[1] = (1.0, 0.0, 0.0, 0)
    ligand[2] = (0.0, -1.5, 0.5, 2)
    # Identity rotations with translations along x hitting overlap, contact and each cut-off,
    # plus a few rotated poses and a far-away pose.
    xs = [0.0, 0.5, 1.0, 2.0, 3.0, 3.5, 4.0, 5.0, 6.0, 7.5, 8.0, 9.5, 11.0, 40.0]
    cols = [[0.0, 0.0, 0.0, x, 0.0, 0.0] for x in xs]
    cols += [[0.3, 1.1, 2.9, 1.0, -2.0, 0.5], [math.pi, 0.0, 0.5 * math.pi, 0.0, 0.0, 0.0],
             [6.0, 5.5, 0.1, -3.0, 3.0, 3.0], [1.0, 2.0, 3.0, 2.5, 2.5, -2.5]]
    poses = np.ascontiguousarray(np.asarray(cols, np.float32).T)
    return Deck(protein, ligand, ff, poses, None, poses.shape[1], "<edge>")


# (pose, field, value) planted into the nonfinite fixture; fields 0-2 are angles, 3-5 translations.
NONFINITE_PLANTED = [
    (1, 0, math.nan), (2, 1, math.inf), (3, 2, -math.inf), (4, 3, math.inf), (5, 4, -math.inf), (6, 5, math.nan),
    (7, 3, 1e30), (8, 4, 2e19), (9, 5, 1e19), (10, 3, 1e12), (11, 0, 1e30), (12, 3, 3e11), (13, 4, 2.7e11),
    (31, 3, math.nan), (32, 4, math.nan), (63, 5, 1e25), (64, 0, -math.inf), (79, 3, math.nan),
]


def nonfinite_deck() -> Deck:
    deck = synthetic_deck(SMALL, seed=11, nposes=80)
    poses = deck.poses.copy()
    for i, f, v in NONFINITE_PLANTED:
        poses[f, i] = v
    deck.poses = np.ascontiguousarray(poses)
    return deck


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=oracle.reference_root())
    ap.add_argument("--only", default="", help="comma-separated fixture names to regenerate (default: all)")
    args = ap.parse_args()
    only = set(filter(None, args.only.split(",")))
    want = lambda name: not only or name in only
    ref = args.reference
    if not os.path.isdir(os.path.join(ref, "data")):
        sys.exit(f"reference tree not found at {ref}")
    oracle.build(ref=True)

    if want("bm1_head"):
        bm1 = read_deck(os.path.join(ref, "data", "bm1"), 1024)
        save("bm1_head", bm1, bm1.ref_energies[:1024],
             "data/bm1 of the reference (first 1024 poses of poses.in; first 1024 lines of ref_energies.out)")
    if want("bm2_head"):
        bm2 = read_deck(os.path.join(ref, "data", "bm2"), 32)
        save("bm2_head", bm2, bm2.ref_energies[:32],
             "data/bm2 of the reference (first 32 poses of poses.in; first 32 lines of ref_energies.out)")
    if want("small_head"):
        small = synthetic_deck(SMALL, seed=0, nposes=2048)
        save("small_head", small, oracle.ref_omp_fasten(small, 16),
             "minibude_gb300.deck.synthetic_deck(SMALL, seed=0, nposes=2048); energies: reference "
             "OmpBude<16>::fasten (src/omp/fasten.hpp) built by oracle/Makefile")
    if want("large_head"):
        large = synthetic_deck(LARGE, seed=0, nposes=256)
        save("large_head", large, oracle.ref_omp_fasten(large, 16),
             "minibude_gb300.deck.synthetic_deck(LARGE, seed=0, nposes=256); energies: reference "
             "OmpBude<16>::fasten (src/omp/fasten.hpp) built by oracle/Makefile")
    if want("edge"):
        edge = edge_deck()
        save("edge", edge, oracle.ref_serial_fasten(edge),
             "tests/golden/make_golden.py:edge_deck(); energies: reference SerialBude<1>::fasten "
             "(src/serial/fasten.hpp) built by oracle/Makefile")
    if want("nonfinite"):
        nf = nonfinite_deck()
        omp = oracle.ref_omp_fasten(nf, 16)
        serial = oracle.ref_serial_fasten(nf)
        nan = np.isnan(serial)
        save("nonfinite", nf, serial,
             "tests/golden/make_golden.py:nonfinite_deck(); energies: reference SerialBude<1>::fasten "
             "(src/serial/fasten.hpp) built by oracle/Makefile, NaN at poses "
             + " ".join(str(i) for i in np.flatnonzero(nan)) + ".  The reference's OmpBude<16> built with its "
             "release flags (-ffast-math, which lets the compiler assume no NaN) gives "
             + " ".join("%.6g" % v for v in omp[nan][:4]) + " ... at those poses and matches elsewhere: "
             "max_diff_%% %.6f." % (100.0 * float(np.max(np.abs(omp[~nan] - serial[~nan]) /
                                                          np.maximum(np.abs(serial[~nan]), 1.0)))))


if __name__ == "__main__":
    main()
