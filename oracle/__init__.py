"""The oracle: CPU checkers for the exact kernel.  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may import this package.
It wraps
  * liboracle.so / liboracle_fast.so -- bude_oracle.c, a C restatement of the reference's
    fasten_main (src/serial/fasten.hpp:18-132, parallelised like src/omp/fasten.hpp:235-254),
    in FP32 and in FP64;
  * _ref/libref.so (when built) -- the reference's own OmpBude / SerialBude models compiled from
    the reference sources by oracle/Makefile; present only where the reference tree is.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
_libs = {}


def reference_root() -> str:
    """Where the reference tree is: oracle/Makefile's BUDE_REFERENCE setting (the environment
    variable of that name overrides it).  The tree exists only on the machine that makes fixtures."""
    r = subprocess.run(["make", "-s", "-C", HERE, "print-reference"], stdout=subprocess.PIPE,
                       stderr=subprocess.DEVNULL, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


def reference_tree_present() -> bool:
    root = reference_root()
    return bool(root) and os.path.isfile(os.path.join(root, "src", "main.cpp"))


def build(ref: bool = False) -> None:
    """make the restatement (and, with ref=True, the reference itself from REF)."""
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE, *targets], check=True, stdout=subprocess.DEVNULL)


def _load(name: str) -> ctypes.CDLL:
    if name not in _libs:
        path = os.path.join(HERE, name)
        if not os.path.exists(path):
            build(ref=name.startswith("_ref"))
        l = ctypes.CDLL(path)
        if name.startswith("_ref"):
            l.ref_omp_fasten.restype = ctypes.c_int
            l.ref_omp_fasten.argtypes = [ctypes.c_int] + [ctypes.c_void_p, ctypes.c_int] * 2 + [
                ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_long, ctypes.c_long, ctypes.c_void_p]
            l.ref_serial_fasten.restype = ctypes.c_int
            l.ref_serial_fasten.argtypes = [ctypes.c_void_p, ctypes.c_int] * 2 + [
                ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_long, ctypes.c_long, ctypes.c_void_p]
        else:
            for fn in ("oracle_fasten_f32", "oracle_fasten_f64"):
                f = getattr(l, fn)
                f.restype = ctypes.c_int
                f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                              ctypes.c_int]
            l.oracle_max_threads.restype = ctypes.c_int
        _libs[name] = l
    return _libs[name]


def _arrays(deck):
    from minibude_gb300.deck import ATOM_DTYPE, FF_DTYPE
    protein = np.ascontiguousarray(deck.protein, ATOM_DTYPE)
    ligand = np.ascontiguousarray(deck.ligand, ATOM_DTYPE)
    ff = np.ascontiguousarray(deck.forcefield, FF_DTYPE)
    poses = np.ascontiguousarray(deck.poses, np.float32)
    return protein, ligand, ff, poses


def fasten_f32(deck, nthreads: int = 0, fast: bool = False) -> np.ndarray:
    """FP32 energies of every pose (strict-FP build unless fast=True: the reference's -ffast-math
    release flags, used for timing)."""
    l = _load("liboracle_fast.so" if fast else "liboracle.so")
    protein, ligand, ff, poses = _arrays(deck)
    n = poses.shape[1]
    out = np.zeros(n, np.float32)
    rc = l.oracle_fasten_f32(ligand.size, protein.size, ff.size, n, protein.ctypes.data, ligand.ctypes.data,
                             ff.ctypes.data, poses.ctypes.data, n, out.ctypes.data, nthreads)
    if rc:
        raise ValueError(f"oracle_fasten_f32 failed: {rc}")
    return out


def fasten_f64(deck, nthreads: int = 0) -> np.ndarray:
    """The same kernel in double (the FP64 rerun)."""
    l = _load("liboracle.so")
    protein, ligand, ff, poses = _arrays(deck)
    n = poses.shape[1]
    out = np.zeros(n, np.float64)
    rc = l.oracle_fasten_f64(ligand.size, protein.size, ff.size, n, protein.ctypes.data, ligand.ctypes.data,
                             ff.ctypes.data, poses.ctypes.data, n, out.ctypes.data, nthreads)
    if rc:
        raise ValueError(f"oracle_fasten_f64 failed: {rc}")
    return out


def max_threads() -> int:
    return _load("liboracle.so").oracle_max_threads()


def reference_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libref.so"))


def ref_omp_fasten(deck, ppwi: int = 16) -> np.ndarray:
    """Energies from the reference's own OmpBude<ppwi>::fasten (needs _ref/libref.so)."""
    l = _load("_ref/libref.so")
    protein, ligand, ff, poses = _arrays(deck)
    n = poses.shape[1]
    out = np.zeros(n, np.float32)
    rc = l.ref_omp_fasten(ppwi, protein.ctypes.data, protein.size, ligand.ctypes.data, ligand.size, ff.ctypes.data,
                          ff.size, poses.ctypes.data, n, n, out.ctypes.data)
    if rc:
        raise ValueError(f"ref_omp_fasten failed: {rc}")
    return out


def ref_serial_fasten(deck) -> np.ndarray:
    """Energies from the reference's own SerialBude<1>::fasten (needs _ref/libref.so)."""
    l = _load("_ref/libref.so")
    protein, ligand, ff, poses = _arrays(deck)
    n = poses.shape[1]
    out = np.zeros(n, np.float32)
    rc = l.ref_serial_fasten(protein.ctypes.data, protein.size, ligand.ctypes.data, ligand.size, ff.ctypes.data,
                             ff.size, poses.ctypes.data, n, n, out.ctypes.data)
    if rc:
        raise ValueError(f"ref_serial_fasten failed: {rc}")
    return out
