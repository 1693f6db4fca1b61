"""bude_gpu_fasten_noalloc: the evaluation entry point for callers that may not allocate device
memory (code inside a framework whose allocator owns the device heap, plugin hosts that hand over
buffers, loops where cudaMalloc/cudaFree are not allowed).

The test plays such a caller: its device buffers come from its own allocator (PyTorch's), it calls
the entry point through the C-ABI twice in a row with different decks, and each result is checked
against the existing entry point (bude_gpu_fasten, host buffers) with the tolerance of the other
parity tests: the reference's max_diff_% < 0.025 and |e - e_fp64| <= 2e-4 * max(|e_fp64|, 1).
Collected last so a run that stops at the first failure has run everything else first."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden
from minibude_gb300 import validate

pytestmark = pytest.mark.gpu

F64_TOL = 2e-4


def existing_entry_point(lib, deck):
    """Energies from bude_gpu_fasten (host buffers, library-owned device memory)."""
    from minibude_gb300.capi import check
    from minibude_gb300.deck import ATOM_DTYPE, FF_DTYPE
    protein = np.ascontiguousarray(deck.protein, ATOM_DTYPE)
    ligand = np.ascontiguousarray(deck.ligand, ATOM_DTYPE)
    ff = np.ascontiguousarray(deck.forcefield, FF_DTYPE)
    poses = np.ascontiguousarray(deck.poses, np.float32)
    out = np.zeros(deck.nposes, np.float32)
    check(lib.bude_gpu_fasten(0, 8, 128, protein.ctypes.data, protein.size, ligand.ctypes.data, ligand.size,
                              ff.ctypes.data, ff.size, poses.ctypes.data, deck.nposes, deck.nposes, 1,
                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), None, None))
    return out


def test_noalloc_matches_existing_entry_point_on_two_calls(built_library):
    torch = pytest.importorskip("torch")
    from minibude_gb300.capi import check
    lib = built_library
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    for name in ("small_head", "bm1_head"):
        deck, refs, f64 = load_golden(name)
        want = existing_entry_point(lib, deck)
        # The caller's own device buffers.
        t_protein = torch.from_numpy(deck.protein.view(np.uint8).copy()).to(dev)
        t_ligand = torch.from_numpy(deck.ligand.view(np.uint8).copy()).to(dev)
        t_ff = torch.from_numpy(deck.forcefield.view(np.uint8).copy()).to(dev)
        t_poses = torch.from_numpy(np.ascontiguousarray(deck.poses, np.float32)).to(dev)
        t_energies = torch.full((deck.nposes,), float("nan"), dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        check(lib.bude_gpu_fasten_noalloc(t_protein.data_ptr(), deck.natpro, t_ligand.data_ptr(), deck.natlig,
                                          t_ff.data_ptr(), deck.ntypes, t_poses.data_ptr(), deck.nposes, deck.nposes,
                                          t_energies.data_ptr(), None))
        got = t_energies.cpu().numpy()
        assert np.all(np.isfinite(got))
        max_diff, failed = validate(got, want)
        assert not failed and max_diff < 0.025, (name, max_diff, failed[:5])
        max_diff, failed = validate(got, refs)
        assert not failed and max_diff < 0.025, (name, max_diff, failed[:5])
        err = np.abs(got.astype(np.float64) - f64) / np.maximum(np.abs(f64), 1.0)
        assert err.max() < F64_TOL, (name, err.max())
