"""Generate the deck-generator fixtures under tests/golden/makedeck/.  Runs only where the reference
tree exists (it builds and runs the reference's own makedeck, oracle/Makefile `make makedeck`).

Inputs copied (gzip-compressed) from the reference's makedeck/raw:
  by_atom.bhff.gz        bhffs/2_heavy_by-atom_2016-v1.bhff (one residue: atoms matched by type)
  by_residue.bhff.gz     bhffs/4_heavy_by-residue_2016-v1.bhff (31 residues: matched by residue)
  bm2_protein.mol2.gz    mol2s/1212_bude_1gcz_proA.mol2, the protein and ligand of data/bm2
  conf_ligand.mol2.gz    mol2s/1186_EXPERIMENTAL.mol2 (9 columns, two @<BUDE>CONF blocks)
  chain_a.mol2.gz        mol2s/1184_2ZTA_chainA_syb.mol2 (10 columns; its ACE cap is missing from
                         by_residue.bhff: the reference fails with "Cannot match key ACE.C")
  bm2_syb.mol2.gz        mol2s/1213_bude_1gcz_proA_syb.mol2 (the same protein, 10 columns)

Expected outputs:
  bm2.sha256             sha256 of data/bm2/{forcefield,protein,ligand,poses}.in: the reference's
                         committed deck, made by makedeck from by_atom + bm2_protein (data/bm2/
                         params.txt), 65,536 poses, seed 42
  by_residue/, by_atom/  the deck the reference's makedeck (built here with GCC on x86-64) writes
                         for (by_residue, bm2_syb, bm2_syb) and (by_atom, conf_ligand,
                         conf_ligand) with -n 256 -s 7: forcefield.in, protein.in, ligand.in,
                         poses.in and its CPU ref_energies.out
  conformations.f32      the two conformations of conf_ligand.mol2 as x, y, z floats, parsed here

Usage (from the repository root):  python tests/golden/make_golden_makedeck.py [--reference DIR]  (default: oracle/Makefile's BUDE_REFERENCE)
"""
from __future__ import annotations

import argparse
import gzip
import hashlib
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "makedeck")
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

INPUTS = {
    "by_atom.bhff": "bhffs/2_heavy_by-atom_2016-v1.bhff",
    "by_residue.bhff": "bhffs/4_heavy_by-residue_2016-v1.bhff",
    "bm2_protein.mol2": "mol2s/1212_bude_1gcz_proA.mol2",
    "conf_ligand.mol2": "mol2s/1186_EXPERIMENTAL.mol2",
    "chain_a.mol2": "mol2s/1184_2ZTA_chainA_syb.mol2",
    "bm2_syb.mol2": "mol2s/1213_bude_1gcz_proA_syb.mol2",
}
CASES = {
    "by_residue": ("by_residue.bhff", "bm2_syb.mol2", "bm2_syb.mol2"),
    "by_atom": ("by_atom.bhff", "conf_ligand.mol2", "conf_ligand.mol2"),
}
DECK_FILES = ["forcefield.in", "protein.in", "ligand.in", "poses.in"]


def conformations(mol2_path):
    """x, y, z of every @<BUDE>CONF block, in file order: the first (number of heavy atoms) lines of
    each block, the lines the reference reads (makedeck/input-utils.cpp:185-200)."""
    lines = [l.strip() for l in open(mol2_path)]
    start = lines.index("@<TRIPOS>ATOM") + 1
    heavy = 0
    for l in lines[start:]:
        if l.startswith("@<TRIPOS>"):
            break
        if l and l[0] not in "#%" and l.split()[5] not in ("H", "h"):
            heavy += 1
    out = []
    for i, l in enumerate(lines):
        f = l.split()
        if len(f) == 2 and f[0] == "@<BUDE>CONF":
            out += [[float(v) for v in lines[i + 1 + a].split()] for a in range(heavy)]
    return np.asarray(out, np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=oracle.reference_root())
    args = ap.parse_args()
    raw = os.path.join(args.reference, "makedeck", "raw")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "makedeck", f"REF={args.reference}"], check=True)
    refmk = os.path.join(ROOT, "oracle", "_ref", "makedeck")
    os.makedirs(OUT, exist_ok=True)
    tmp = os.path.join(OUT, "_tmp")
    shutil.rmtree(tmp, ignore_errors=True)
    os.makedirs(tmp)
    for name, src in INPUTS.items():
        data = open(os.path.join(raw, src), "rb").read()
        open(os.path.join(tmp, name), "wb").write(data)
        with gzip.GzipFile(os.path.join(OUT, name + ".gz"), "wb", mtime=0) as g:
            g.write(data)
    with open(os.path.join(OUT, "bm2.sha256"), "w") as f:
        for name in DECK_FILES:
            h = hashlib.sha256(open(os.path.join(args.reference, "data", "bm2", name), "rb").read()).hexdigest()
            f.write(f"{h}  {name}\n")
    for case, (ff, p, l) in CASES.items():
        deck = os.path.join(tmp, case)
        subprocess.run([refmk, "-f", os.path.join(tmp, ff), "-p", os.path.join(tmp, p), "-l", os.path.join(tmp, l),
                        "-n", "256", "-s", "7", "-o", deck, "--force"], check=True, stdout=subprocess.DEVNULL)
        dst = os.path.join(OUT, case)
        os.makedirs(dst, exist_ok=True)
        for name in DECK_FILES + ["ref_energies.out"]:
            shutil.copy(os.path.join(deck, name), os.path.join(dst, name))
    conformations(os.path.join(tmp, "conf_ligand.mol2")).tofile(os.path.join(OUT, "conformations.f32"))
    shutil.rmtree(tmp)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
