"""Deck files and seeded synthetic decks.

A deck is the reference's input directory (src/bude.h:15-20): ``protein.in`` and ``ligand.in``
(packed 16-byte ``Atom`` records, src/bude.h:39-42), ``forcefield.in`` (packed 16-byte
``FFParams``, src/bude.h:44-49), ``poses.in`` (six consecutive blocks of N float32: tilt, roll,
pan in radians, then x, y, z translation; src/main.cpp:296-311) and ``ref_energies.out`` (one
decimal energy per line, makedeck/main.cpp:199-202).

`read_deck` follows the reference loader (src/main.cpp:283-322) including its error behaviour;
`write_deck` writes the same layout; `synthetic_deck` builds the seeded decks of the benchmark
configurations.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Optional, Sequence

import numpy as np

ATOM_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("type", "<i4")])
FF_DTYPE = np.dtype([("hbtype", "<i4"), ("radius", "<f4"), ("hphb", "<f4"), ("elsc", "<f4")])

FILE_LIGAND = "ligand.in"
FILE_PROTEIN = "protein.in"
FILE_FORCEFIELD = "forcefield.in"
FILE_POSES = "poses.in"
FILE_REF_ENERGIES = "ref_energies.out"

# bhff electrostatic type codes (ASCII of column 2, makedeck/input-utils.cpp:84).  The kernel only
# tells 'F' and 'E' apart from the rest (src/serial/fasten.hpp:83-85).
HBTYPE_PLAIN = ord("-")  # 45
HBTYPE_DIPOLE = ord("D")  # 68, same kernel behaviour as '-'
HBTYPE_E = ord("E")  # 69: donor-or-acceptor, charge term forced attractive
HBTYPE_F = ord("F")  # 70: formal charge, longer charge cut-off when both atoms are 'F'
# The synthetic decks draw "plain / donor / acceptor" from the three behaviours the kernel has.
SYNTHETIC_HBTYPES = (HBTYPE_PLAIN, HBTYPE_E, HBTYPE_F)


@dataclasses.dataclass
class Deck:
    protein: np.ndarray  # ATOM_DTYPE [natpro]
    ligand: np.ndarray  # ATOM_DTYPE [natlig]
    forcefield: np.ndarray  # FF_DTYPE [ntypes]
    poses: np.ndarray  # float32 [6, nposes], C-contiguous
    ref_energies: Optional[np.ndarray] = None  # float32 [>= nposes]
    max_poses: int = 0
    path: str = ""

    @property
    def natpro(self) -> int:
        return int(self.protein.shape[0])

    @property
    def natlig(self) -> int:
        return int(self.ligand.shape[0])

    @property
    def ntypes(self) -> int:
        return int(self.forcefield.shape[0])

    @property
    def nposes(self) -> int:
        return int(self.poses.shape[1])

    @property
    def interactions(self) -> int:
        """nposes * natlig * natpro (src/main.cpp:368)."""
        return self.nposes * self.natlig * self.natpro

    def head(self, n: int) -> "Deck":
        """The first n poses (and reference energies) of this deck."""
        refs = None if self.ref_energies is None else self.ref_energies[:n].copy()
        return dataclasses.replace(self, poses=np.ascontiguousarray(self.poses[:, :n]), ref_energies=refs)


def _read_n_struct(path: str, dtype: np.dtype) -> np.ndarray:
    """src/main.cpp:138-151: the whole file as records; a trailing partial record is dropped."""
    if not os.path.isfile(path):
        raise ValueError(f"Bad file: {path}")
    raw = np.fromfile(path, dtype=np.uint8)
    n = raw.size // dtype.itemsize
    return raw[: n * dtype.itemsize].view(dtype).copy()


def read_ref_energies(path: str) -> np.ndarray:
    """One float per line, parsed like std::stof (src/main.cpp:314-318)."""
    out = []
    with open(path) as f:
        for line in f:
            s = line.strip()
            if s:
                out.append(float(s))
    return np.asarray(out, dtype=np.float32)


def read_deck(deck_dir: str, nposes: int = 0, need_refs: bool = True) -> Deck:
    """Load a deck directory the way src/main.cpp:290-322 does.

    ``nposes`` = 0 takes every pose.  Raises ValueError for a pose file whose size is not a
    multiple of 6 floats, for more poses than the deck has, and (when ``need_refs``) for fewer
    reference energies than poses -- the reference's std::invalid_argument cases.
    """
    ligand = _read_n_struct(os.path.join(deck_dir, FILE_LIGAND), ATOM_DTYPE)
    protein = _read_n_struct(os.path.join(deck_dir, FILE_PROTEIN), ATOM_DTYPE)
    ff = _read_n_struct(os.path.join(deck_dir, FILE_FORCEFIELD), FF_DTYPE)
    flat = _read_n_struct(os.path.join(deck_dir, FILE_POSES), np.dtype("<f4"))
    if flat.size % 6 != 0:
        raise ValueError(f"Pose size ({flat.size}) not divisible my 6!")
    max_poses = flat.size // 6
    n = max_poses if nposes == 0 else nposes
    if n > max_poses:
        raise ValueError(f"Requested poses ({n}) exceeded max poses ({max_poses}) for deck")
    poses = np.ascontiguousarray(flat.reshape(6, max_poses)[:, :n])
    refs = None
    ref_path = os.path.join(deck_dir, FILE_REF_ENERGIES)
    if need_refs:
        refs = read_ref_energies(ref_path) if os.path.isfile(ref_path) else np.zeros(0, np.float32)
        if n > refs.size:
            raise ValueError(f"Size of reference energies ({refs.size}) is less than poses ({n})")
    elif os.path.isfile(ref_path):
        refs = read_ref_energies(ref_path)
    return Deck(protein, ligand, ff, poses, refs, max_poses, deck_dir)


def write_deck(deck_dir: str, deck: Deck, ref_energies: Optional[np.ndarray] = None, fmt: str = "%.6f") -> None:
    """Write the five deck files (refs only when given or already on the deck)."""
    os.makedirs(deck_dir, exist_ok=True)
    deck.protein.astype(ATOM_DTYPE).tofile(os.path.join(deck_dir, FILE_PROTEIN))
    deck.ligand.astype(ATOM_DTYPE).tofile(os.path.join(deck_dir, FILE_LIGAND))
    deck.forcefield.astype(FF_DTYPE).tofile(os.path.join(deck_dir, FILE_FORCEFIELD))
    np.ascontiguousarray(deck.poses, dtype=np.float32).tofile(os.path.join(deck_dir, FILE_POSES))
    refs = ref_energies if ref_energies is not None else deck.ref_energies
    if refs is not None:
        with open(os.path.join(deck_dir, FILE_REF_ENERGIES), "w") as f:
            for e in np.asarray(refs, dtype=np.float32):
                f.write((fmt % float(e)) + "\n")


# ----------------------------------------------------------------------------------------------
# Seeded synthetic decks

def synthetic_forcefield(rng: np.random.Generator, ntypes: int) -> np.ndarray:
    """Types with radius U[1.0, 2.5] A, hphb U[-3, 3], elsc U[-1, 1], hbtype uniform over
    '-' / 'E' / 'F'."""
    ff = np.zeros(ntypes, FF_DTYPE)
    ff["radius"] = rng.uniform(1.0, 2.5, ntypes)
    ff["hphb"] = rng.uniform(-3.0, 3.0, ntypes)
    ff["elsc"] = rng.uniform(-1.0, 1.0, ntypes)
    ff["hbtype"] = np.asarray(SYNTHETIC_HBTYPES, np.int32)[rng.integers(0, len(SYNTHETIC_HBTYPES), ntypes)]
    return ff


def synthetic_protein(rng: np.random.Generator, natpro: int, half_box: float, ntypes: int) -> np.ndarray:
    """Atoms uniform in a [-half_box, half_box]^3 box with uniform types."""
    p = np.zeros(natpro, ATOM_DTYPE)
    xyz = rng.uniform(-half_box, half_box, (natpro, 3))
    p["x"], p["y"], p["z"] = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    p["type"] = rng.integers(0, ntypes, natpro)
    return p


def synthetic_ligand(rng: np.random.Generator, natlig: int, radius: float, ntypes: int) -> np.ndarray:
    """Atoms uniform within a ball of `radius` around the origin with uniform types."""
    d = rng.normal(size=(natlig, 3))
    d /= np.maximum(np.linalg.norm(d, axis=1, keepdims=True), 1e-12)
    r = radius * rng.uniform(0.0, 1.0, natlig) ** (1.0 / 3.0)
    xyz = d * r[:, None]
    lig = np.zeros(natlig, ATOM_DTYPE)
    lig["x"], lig["y"], lig["z"] = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    lig["type"] = rng.integers(0, ntypes, natlig)
    return lig


def synthetic_poses(rng: np.random.Generator, nposes: int, max_trans: float = 3.0) -> np.ndarray:
    """Euler angles U[0, 2pi), translations U[-max_trans, max_trans]: float32 [6, nposes]."""
    poses = np.empty((6, nposes), np.float32)
    poses[0:3] = rng.uniform(0.0, 2.0 * math.pi, (3, nposes))
    poses[3:6] = rng.uniform(-max_trans, max_trans, (3, nposes))
    return poses


@dataclasses.dataclass(frozen=True)
class DeckSpec:
    """Shape of a synthetic plain-kernel deck."""
    name: str
    natpro: int
    half_box: float
    natlig: int
    ntypes: int
    nposes: int
    ligand_radius: float = 5.0
    max_trans: float = 3.0


# The two plain-kernel workloads: a bm1-sized deck (938 x 26 x 65,536) and the scaled-up deck
# (4,096 atoms in a +-30 A box, 64 ligand atoms, 1,048,576 poses).
SMALL = DeckSpec("synthetic-938x26x65536", 938, 20.0, 26, 34, 65536)
LARGE = DeckSpec("synthetic-4096x64x1048576", 4096, 30.0, 64, 34, 1048576)
SPECS = {"small": SMALL, "large": LARGE}


def synthetic_deck(spec: DeckSpec, seed: int = 0, nposes: Optional[int] = None) -> Deck:
    """Seeded deck of the given shape.  The first k poses of a deck do not depend on `nposes`,
    so `synthetic_deck(spec, seed, k)` is the head of the full deck."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ff = synthetic_forcefield(rng, spec.ntypes)
    protein = synthetic_protein(rng, spec.natpro, spec.half_box, spec.ntypes)
    ligand = synthetic_ligand(rng, spec.natlig, spec.ligand_radius, spec.ntypes)
    n = spec.nposes if nposes is None else int(nposes)
    prng = np.random.Generator(np.random.PCG64([seed, 1]))
    # Draw poses in fixed-size chunks so every prefix is independent of the total count.
    chunk = 4096
    parts = []
    left = n
    while left > 0:
        parts.append(synthetic_poses(prng, chunk, spec.max_trans))
        left -= chunk
    poses = np.ascontiguousarray(np.concatenate(parts, axis=1)[:, :n]) if parts else np.zeros((6, 0), np.float32)
    return Deck(protein, ligand, ff, poses, None, n, f"<{spec.name} seed={seed}>")


@dataclasses.dataclass
class BatchDeck:
    """Many ligands, each with its own atoms and poses, against one protein."""
    protein: np.ndarray  # ATOM_DTYPE [natpro]
    forcefield: np.ndarray  # FF_DTYPE [ntypes]
    ligands: list  # of ATOM_DTYPE arrays
    poses: list  # of float32 [6, n_l] arrays
    name: str = ""

    @property
    def nligands(self) -> int:
        return len(self.ligands)

    @property
    def natpro(self) -> int:
        return int(self.protein.shape[0])

    @property
    def ntypes(self) -> int:
        return int(self.forcefield.shape[0])

    def ligand_offsets(self) -> np.ndarray:
        return np.concatenate([[0], np.cumsum([len(l) for l in self.ligands])]).astype(np.int32)

    def pose_offsets(self) -> np.ndarray:
        return np.concatenate([[0], np.cumsum([p.shape[1] for p in self.poses])]).astype(np.int64)

    @property
    def total_poses(self) -> int:
        return int(sum(p.shape[1] for p in self.poses))

    @property
    def interactions(self) -> int:
        return int(sum(len(l) * p.shape[1] for l, p in zip(self.ligands, self.poses))) * self.natpro

    def atoms(self) -> np.ndarray:
        return concat_atoms(self.ligands)

    def pose_block(self) -> np.ndarray:
        if not self.poses:
            return np.zeros((6, 0), np.float32)
        return np.ascontiguousarray(np.concatenate(self.poses, axis=1), dtype=np.float32)

    def deck(self, l: int) -> Deck:
        """Ligand l as a plain deck."""
        return Deck(self.protein, self.ligands[l], self.forcefield, np.ascontiguousarray(self.poses[l]), None,
                    self.poses[l].shape[1], f"{self.name}[{l}]")

    def subset(self, ligands, max_poses=None) -> "BatchDeck":
        """Some of the ligands, optionally with only their first max_poses poses."""
        return BatchDeck(self.protein, self.forcefield, [self.ligands[l] for l in ligands],
                         [np.ascontiguousarray(self.poses[l][:, :max_poses]) for l in ligands], self.name)


FILE_CONFORMATIONS = "ligand_conformations.in"


def read_conformations(deck_dir: str, natlig: int) -> list:
    """The ligand conformations gb300-makedeck writes with --conformations (ligand_conformations.in:
    natlig packed atom records per conformation, conformation after conformation); [] if absent."""
    path = os.path.join(deck_dir, FILE_CONFORMATIONS)
    if not os.path.isfile(path):
        return []
    recs = _read_n_struct(path, ATOM_DTYPE)
    if natlig <= 0 or recs.size % natlig:
        raise ValueError(f"{path}: {recs.size} atom records is not a whole number of {natlig}-atom conformations")
    return [np.ascontiguousarray(recs[i:i + natlig]) for i in range(0, recs.size, natlig)]


def conformation_batch(deck: Deck, conformations: list, include_deck_ligand: bool = True) -> "BatchDeck":
    """Every conformation of the deck's ligand against every pose of the deck, as a batch: ligand l
    of the batch is conformation l (the deck's own ligand first when include_deck_ligand), each with
    the deck's poses, so one batched launch scores conformations x poses.  The reference's deck
    generator parses the @<BUDE>CONF conformations of a mol2 and drops them
    (makedeck/input-utils.cpp:185-200)."""
    ligs = ([deck.ligand] if include_deck_ligand else []) + list(conformations)
    for c in ligs:
        if len(c) != len(deck.ligand) or not np.array_equal(c["type"], deck.ligand["type"]):
            raise ValueError("a conformation must have the ligand's atoms (same count and types)")
    poses = np.ascontiguousarray(deck.poses, np.float32)
    return BatchDeck(deck.protein, deck.forcefield, [np.ascontiguousarray(c, ATOM_DTYPE) for c in ligs],
                     [poses] * len(ligs), f"{deck.path} conformations")


@dataclasses.dataclass(frozen=True)
class BatchSpec:
    """Shape of a synthetic batch: ligand atom counts uniform in [atoms_lo, atoms_hi], pose counts
    log-uniform in [poses_lo, poses_hi] (or all equal to poses_lo when poses_hi == poses_lo)."""
    name: str
    nligands: int
    atoms_lo: int
    atoms_hi: int
    poses_lo: int
    poses_hi: int
    ligand_radius: float = 5.0
    max_trans: float = 3.0


# 256 ligands of 12-96 atoms with 4,096-65,536 poses each (log-uniform) against one protein.
BATCH = BatchSpec("batch-256-ligands-12to96-atoms-4096to65536-poses", 256, 12, 96, 4096, 65536)


def synthetic_batch(spec: BatchSpec, protein: np.ndarray, forcefield: np.ndarray, seed: int = 0) -> BatchDeck:
    """Seeded ligands (atoms uniform within ligand_radius of the origin, types uniform over the
    forcefield) and poses (angles U[0, 2pi), translations U[-max_trans, max_trans])."""
    rng = np.random.Generator(np.random.PCG64([seed, 2]))
    ntypes = forcefield.shape[0]
    ligands, poses = [], []
    for _ in range(spec.nligands):
        natlig = int(rng.integers(spec.atoms_lo, spec.atoms_hi + 1))
        if spec.poses_hi > spec.poses_lo:
            n = int(round(math.exp(rng.uniform(math.log(spec.poses_lo), math.log(spec.poses_hi)))))
        else:
            n = spec.poses_lo
        ligands.append(synthetic_ligand(rng, natlig, spec.ligand_radius, ntypes))
        poses.append(synthetic_poses(rng, n, spec.max_trans))
    return BatchDeck(np.ascontiguousarray(protein, ATOM_DTYPE), np.ascontiguousarray(forcefield, FF_DTYPE), ligands,
                     poses, spec.name)


def shard_range(n: int, rank: int, world: int):
    """[start, stop) of rank's contiguous share of n independent items (poses or ligands); shares
    differ by at most one item and cover 0..n exactly once."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard_deck(deck: Deck, rank: int, world: int) -> Deck:
    """The rank's contiguous slice of the deck's poses (and reference energies)."""
    a, b = shard_range(deck.nposes, rank, world)
    refs = None if deck.ref_energies is None else deck.ref_energies[a:b].copy()
    return dataclasses.replace(deck, poses=np.ascontiguousarray(deck.poses[:, a:b]), ref_energies=refs)


def pose_block(poses: np.ndarray) -> np.ndarray:
    """Poses as one C-contiguous float32 [6, n] block (what the C-ABI expects)."""
    return np.ascontiguousarray(poses, dtype=np.float32)


def concat_atoms(parts: Sequence[np.ndarray]) -> np.ndarray:
    return np.concatenate([np.asarray(p, ATOM_DTYPE) for p in parts]) if parts else np.zeros(0, ATOM_DTYPE)
