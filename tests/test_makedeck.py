"""gb300-makedeck against the reference's deck generator (makedeck/): byte-identical decks, the
reference's pose KAT (makedeck/test-bude.cpp:94-111), conformations, and the error cases.  The
fixtures come from tests/golden/make_golden_makedeck.py."""
import gzip
import hashlib
import os
import shutil
import subprocess

import numpy as np
import pytest

from minibude_gb300 import build, read_deck, validate

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "makedeck")
DECK_FILES = ["forcefield.in", "protein.in", "ligand.in", "poses.in"]


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    """The built tool and the fixture inputs, decompressed into a scratch directory."""
    build.build_library()
    exe = build.build_makedeck()
    d = tmp_path_factory.mktemp("inputs")
    for f in os.listdir(FIX):
        if f.endswith(".gz"):
            with gzip.open(os.path.join(FIX, f), "rb") as g:
                (d / f[:-3]).write_bytes(g.read())
    return exe, d


def run(exe, *args):
    return subprocess.run([exe, *map(str, args)], capture_output=True, text=True)


def make(tool, out, ff, p, l, *extra):
    exe, d = tool
    r = run(exe, "-f", d / ff, "-p", d / p, "-l", d / l, "-o", out, "--force", *extra)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def test_regenerates_the_reference_bm2_deck(tool, tmp_path):
    # data/bm2 was made by the reference's makedeck from these inputs (its params.txt): 65,536 poses,
    # seed 42.  Every deck file must come out byte for byte.
    out = make(tool, tmp_path / "bm2", "by_atom.bhff", "bm2_protein.mol2", "bm2_protein.mol2", "--no-energies")
    want = dict(reversed(l.split()) for l in open(os.path.join(FIX, "bm2.sha256")))
    for name in DECK_FILES:
        assert hashlib.sha256((out / name).read_bytes()).hexdigest() == want[name], name
    head = read_deck(os.path.join(HERE, "golden", "bm2_head"))
    deck = read_deck(str(out), need_refs=False)
    assert np.array_equal(deck.poses[:, :head.nposes], head.poses)


@pytest.mark.parametrize("case,ff,mol", [("by_atom", "by_atom.bhff", "conf_ligand.mol2"),
                                         ("by_residue", "by_residue.bhff", "bm2_syb.mol2")])
def test_matches_the_reference_generator_built_for_x86(tool, tmp_path, case, ff, mol):
    # The reference generator compiled with GCC on x86-64 draws the grid indices z first.
    out = make(tool, tmp_path / case, ff, mol, mol, "-n", 256, "-s", 7, "--draw-order", "z-first", "--no-energies")
    for name in DECK_FILES:
        assert (out / name).read_bytes() == open(os.path.join(FIX, case, name), "rb").read(), name
    # tilt first (the default) draws the same grid in another order: same count, other poses
    out2 = make(tool, tmp_path / (case + "_t"), ff, mol, mol, "-n", 256, "-s", 7, "--no-energies")
    a = np.fromfile(out / "poses.in", "<f4").reshape(6, -1)
    b = np.fromfile(out2 / "poses.in", "<f4").reshape(6, -1)
    assert a.shape == b.shape and not np.array_equal(a, b)


def test_pose_grid_kat(tmp_path):
    # makedeck/test-bude.cpp:94-111: one pose from one-element ranges (180/pi degrees, 1 A) is all ones.
    src = tmp_path / "kat.cpp"
    src.write_text(r'''
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include "deck_builder.h"
int main() {
  const std::vector<float> rad{(float)(180.0 / M_PI)}, one{1.f};
  for (auto order : {bude_deck::DrawOrder::TiltFirst, bude_deck::DrawOrder::ZFirst}) {
    auto p = bude_deck::generate_poses(1, 42, {rad, rad, rad, one, one, one}, order);
    for (auto &f : p) { if (f.size() != 1 || f[0] != 1.f) { std::printf("bad %g\n", f.empty() ? -1.0 : f[0]); return 1; } }
  }
  try { bude_deck::generate_poses(2, 42, {rad, rad, rad, one, one, one}); return 2; }
  catch (const std::invalid_argument &) {}
  std::printf("ok\n");
  return 0;
}
''')
    d = os.path.join(build.PKG, "makedeck")
    exe = tmp_path / "kat"
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{build.INCLUDE}", f"-I{d}", str(src),
                    os.path.join(d, "deck_builder.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout


def test_conformations_and_params(tool, tmp_path):
    out = make(tool, tmp_path / "conf", "by_atom.bhff", "conf_ligand.mol2", "conf_ligand.mol2", "-n", 512,
               "--conformations", "--no-energies")
    lig = np.fromfile(out / "ligand.in", [("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("t", "<i4")])
    confs = np.fromfile(out / "ligand_conformations.in", lig.dtype)
    want = np.fromfile(os.path.join(FIX, "conformations.f32"), "<f4").reshape(-1, 3)
    assert len(confs) == len(want) and len(confs) % len(lig) == 0 and len(confs) // len(lig) == 2
    assert np.array_equal(np.stack([confs["x"], confs["y"], confs["z"]], 1), want)
    assert np.array_equal(confs["t"], np.tile(lig["t"], 2))
    params = (out / "params.txt").read_text()
    assert params.startswith("-f ") and params.endswith("--no-energies \n")


def test_errors(tool, tmp_path):
    exe, d = tool
    base = ["-f", d / "by_atom.bhff", "-p", d / "conf_ligand.mol2", "-l", d / "conf_ligand.mol2"]
    r = run(exe, *base, "-o", tmp_path / "a", "-n", 100, "--no-energies")
    assert r.returncode != 0 and "cannot be divided by WGSIZE(256)" in r.stderr
    r = run(exe, *base, "--no-energies")
    assert r.returncode != 0 and "--out is a required parameter" in r.stderr
    (tmp_path / "exists").mkdir()
    r = run(exe, *base, "-o", tmp_path / "exists", "--no-energies")
    assert r.returncode != 0 and "pass --force" in r.stderr
    # 10-column mol2 whose ACE cap is not in the forcefield: the reference's message
    r = run(exe, "-f", d / "by_residue.bhff", "-p", d / "chain_a.mol2", "-l", d / "chain_a.mol2",
            "-o", tmp_path / "b", "--no-energies")
    assert r.returncode != 0 and "Cannot match key ACE.C in forcefield." in r.stderr and "chain_a.mol2:18" in r.stderr
    # 9-column mol2 against a multi-residue forcefield
    r = run(exe, "-f", d / "by_residue.bhff", "-p", d / "conf_ligand.mol2", "-l", d / "conf_ligand.mol2",
            "-o", tmp_path / "c", "--no-energies")
    assert r.returncode != 0 and "doesn't have 10 columns" in r.stderr
    # no atom section
    bad = tmp_path / "bad.mol2"
    bad.write_text("@<TRIPOS>MOLECULE\nx\n")
    r = run(exe, "-f", d / "by_atom.bhff", "-p", bad, "-l", bad, "-o", tmp_path / "d", "--no-energies")
    assert r.returncode != 0 and "Begin atom marker" in r.stderr
    r = run(exe, "--bogus")
    assert r.returncode != 0 and "Unrecognized argument" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("case,ff,mol", [("by_atom", "by_atom.bhff", "conf_ligand.mol2"),
                                         ("by_residue", "by_residue.bhff", "bm2_syb.mol2")])
def test_gpu_energies_match_the_reference_generator(tool, tmp_path, case, ff, mol):
    out = make(tool, tmp_path / case, ff, mol, mol, "-n", 256, "-s", 7, "--draw-order", "z-first")
    got = np.loadtxt(out / "ref_energies.out", dtype=np.float64)
    want = np.loadtxt(os.path.join(FIX, case, "ref_energies.out"), dtype=np.float64)
    max_diff, failed = validate(got.astype(np.float32), want)
    assert not failed and max_diff < 0.025, (max_diff, failed[:5])
    text = (out / "ref_energies.out").read_text().splitlines()
    assert len(text) == 256 and all(len(t.split(".")[1]) == 5 for t in text)


def test_conformation_batch(tool, tmp_path):
    from minibude_gb300 import conformation_batch, read_conformations
    out = make(tool, tmp_path / "conf", "by_atom.bhff", "conf_ligand.mol2", "conf_ligand.mol2", "-n", 256,
               "--conformations", "--no-energies")
    deck = read_deck(str(out), need_refs=False)
    confs = read_conformations(str(out), len(deck.ligand))
    assert len(confs) == 2
    b = conformation_batch(deck, confs)
    assert b.nligands == 3 and b.total_poses == 3 * deck.nposes
    assert np.array_equal(b.ligands[0], deck.ligand) and np.array_equal(b.ligands[2], confs[1])
    with pytest.raises(ValueError):
        conformation_batch(deck, [confs[0][:-1]])


@pytest.mark.gpu
def test_conformations_times_poses_on_gpu(tool, tmp_path):
    # One batched launch over (conformation, pose) equals one exact launch per conformation, bit
    # for bit, and matches the oracle.
    import oracle
    from minibude_gb300 import conformation_batch, read_conformations
    from minibude_gb300.model import GpuContext, launch_cfg
    out = make(tool, tmp_path / "conf", "by_atom.bhff", "conf_ligand.mol2", "conf_ligand.mol2", "-n", 1024,
               "--conformations", "--no-energies")
    deck = read_deck(str(out), need_refs=False)
    b = conformation_batch(deck, read_conformations(str(out), len(deck.ligand)))
    with GpuContext(0) as ctx:
        ctx.upload_batch(b)
        ctx.run_batch(launch_cfg(8, 128, 1, 64, 2))
        e = ctx.download_batch().reshape(b.nligands, deck.nposes)
        for l in range(b.nligands):
            ctx.upload(b.deck(l))
            ctx.run(launch_cfg(8, 128, 1, 64, 2))
            assert np.array_equal(e[l], ctx.download())
            max_diff, failed = validate(e[l], oracle.fasten_f32(b.deck(l)))
            assert not failed and max_diff < 0.025
    # the conformations are different molecules: their energy landscapes differ
    assert not np.array_equal(e[1], e[2])
