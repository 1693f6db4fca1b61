"""bude_gpu_fasten_noalloc: the evaluation entry point for callers that may not allocate device
memory (code inside a framework whose allocator owns the device heap, plugin hosts that hand over
buffers, loops where cudaMalloc/cudaFree are not allowed).

The tests play such a caller: its device buffers come from its own allocator (PyTorch's), it calls
the entry point through the C-ABI, and each result is checked against the existing entry point
(bude_gpu_fasten, host buffers) and the oracle with the tolerance of the other parity tests: the
reference's max_diff_% < 0.025 and |e - e_fp64| <= 2e-4 * max(|e_fp64|, 1).  They also cover the
refusals (sizes beyond the fixed working array, host or misaligned buffers, atom types outside the
forcefield), the unsplit launch, empty ligands and proteins, non-finite poses, and that a call
allocates no device memory.  Collected last so a run that stops at the first failure has run
everything else first."""
import ctypes

import numpy as np
import pytest

import oracle
from conftest import load_golden
from minibude_gb300 import SMALL, synthetic_deck, validate
from minibude_gb300.capi import BUDE_ERR_ARG, BUDE_ERR_TYPE, check

pytestmark = pytest.mark.gpu

F64_TOL = 2e-4
MAX_POSES = 65536          # BUDE_NOALLOC_MAX_POSES
MAX_SLAB_RECORDS = 131072  # BUDE_NOALLOC_MAX_SLAB_RECORDS


def existing_entry_point(lib, deck):
    """Energies from bude_gpu_fasten (host buffers, library-owned device memory)."""
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


class Caller:
    """A deck in the caller's own device buffers (allocated by PyTorch, not by the library)."""

    def __init__(self, torch, deck):
        dev = torch.device("cuda:0")
        as_bytes = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).to(dev)
        self.deck = deck
        self.protein = as_bytes(deck.protein) if deck.natpro else torch.zeros(16, dtype=torch.uint8, device=dev)
        self.ligand = as_bytes(deck.ligand) if deck.natlig else torch.zeros(16, dtype=torch.uint8, device=dev)
        self.ff = as_bytes(deck.forcefield)
        self.poses = torch.from_numpy(np.ascontiguousarray(deck.poses, np.float32)).to(dev)
        self.energies = torch.full((max(deck.nposes, 1),), 7.0, dtype=torch.float32, device=dev)
        torch.cuda.synchronize()

    def call(self, lib, **over):
        d = self.deck
        a = dict(protein=self.protein.data_ptr(), natpro=d.natpro, ligand=self.ligand.data_ptr(), natlig=d.natlig,
                 ff=self.ff.data_ptr(), ntypes=d.ntypes, poses=self.poses.data_ptr(), stride=d.nposes,
                 nposes=d.nposes, energies=self.energies.data_ptr())
        a.update(over)
        return lib.bude_gpu_fasten_noalloc(a["protein"], a["natpro"], a["ligand"], a["natlig"], a["ff"], a["ntypes"],
                                           a["poses"], a["stride"], a["nposes"], a["energies"], None)

    def result(self):
        return self.energies[:self.deck.nposes].cpu().numpy()


def assert_parity(got, want, f64=None):
    assert np.all(np.isfinite(got))
    max_diff, failed = validate(got, want)
    assert not failed and max_diff < 0.025, (max_diff, failed[:5])
    if f64 is not None:
        err = np.abs(got.astype(np.float64) - f64) / np.maximum(np.abs(f64), 1.0)
        assert err.max() < F64_TOL, err.max()


@pytest.fixture(scope="module")
def torch_cuda(built_library):
    torch = pytest.importorskip("torch")
    torch.cuda.set_device(0)
    return torch


def test_noalloc_matches_existing_entry_point_on_two_calls(built_library, torch_cuda):
    lib = built_library
    for name in ("small_head", "bm1_head"):
        deck, refs, f64 = load_golden(name)
        want = existing_entry_point(lib, deck)
        c = Caller(torch_cuda, deck)
        check(c.call(lib))
        got = c.result()
        assert_parity(got, want)
        assert_parity(got, refs, f64)


def test_noalloc_allocates_nothing(built_library, torch_cuda):
    # Free device memory is the same before and after a call (the first call on the device has
    # loaded the module and looked up the working array already).
    lib = built_library
    deck, refs, f64 = load_golden("bm2_head")
    c = Caller(torch_cuda, deck)
    check(c.call(lib))
    first = c.result()
    free0, _ = torch_cuda.cuda.mem_get_info()
    check(c.call(lib))
    free1, _ = torch_cuda.cuda.mem_get_info()
    assert free1 == free0
    assert np.array_equal(first, c.result())
    assert_parity(first, refs, f64)


def test_noalloc_unsplit_at_the_pose_limit(built_library, torch_cuda):
    # MAX_POSES poses against a 64-atom protein: enough pose blocks that the protein is not split.
    lib = built_library
    base = synthetic_deck(SMALL, 21, MAX_POSES)
    deck = base.__class__(base.protein[:64].copy(), base.ligand, base.forcefield, base.poses, None, MAX_POSES, "cut")
    c = Caller(torch_cuda, deck)
    check(c.call(lib))
    got = c.result()
    assert_parity(got, existing_entry_point(lib, deck))
    sample = np.arange(0, MAX_POSES, 97)
    sub = deck.head(MAX_POSES)
    sub.poses = np.ascontiguousarray(deck.poses[:, sample])
    assert_parity(got[sample], oracle.fasten_f32(sub), oracle.fasten_f64(sub))


@pytest.mark.parametrize("which", ["ligand", "protein"])
def test_noalloc_empty_side_gives_zero(built_library, torch_cuda, which):
    lib = built_library
    deck = synthetic_deck(SMALL, 3, 500)
    if which == "ligand":
        deck.ligand = deck.ligand[:0].copy()
    else:
        deck.protein = deck.protein[:0].copy()
    c = Caller(torch_cuda, deck)
    check(c.call(lib))
    assert np.array_equal(c.result(), np.zeros(500, np.float32))


def test_noalloc_irregular_poses_match_the_oracle(built_library, torch_cuda):
    from test_irregular_gpu import assert_matches_oracle, irregular_deck
    lib = built_library
    deck = irregular_deck(2000, seed=7)
    c = Caller(torch_cuda, deck)
    check(c.call(lib))
    assert_matches_oracle(c.result(), oracle.fasten_f32(deck), oracle.fasten_f64(deck))


def test_noalloc_refusals_leave_energies_and_the_next_call_intact(built_library, torch_cuda):
    lib = built_library
    deck = synthetic_deck(SMALL, 9, 300)
    c = Caller(torch_cuda, deck)
    cases = []
    # more poses than the working array holds (rejected before any buffer is read)
    cases.append((BUDE_ERR_ARG, dict(nposes=MAX_POSES + 1, stride=MAX_POSES + 1)))
    # more slab records than it holds: ntypes x padded protein atoms
    cases.append((BUDE_ERR_ARG, dict(ntypes=MAX_SLAB_RECORDS // 8 + 1)))
    # host memory
    host_poses = np.ascontiguousarray(deck.poses, np.float32)
    cases.append((BUDE_ERR_ARG, dict(poses=host_poses.ctypes.data)))
    host_out = np.zeros(deck.nposes, np.float32)
    cases.append((BUDE_ERR_ARG, dict(energies=host_out.ctypes.data)))
    # a ligand that is not 16-byte aligned
    cases.append((BUDE_ERR_ARG, dict(ligand=c.ligand.data_ptr() + 4)))
    # negative sizes, a stride shorter than the pose count
    cases.append((BUDE_ERR_ARG, dict(natpro=-1)))
    cases.append((BUDE_ERR_ARG, dict(stride=deck.nposes - 1)))
    for code, over in cases:
        assert c.call(lib, **over) == code, over
        assert np.all(c.result() == 7.0), over
    assert np.all(host_out == 0.0)
    # atom types outside the forcefield: BUDE_ERR_TYPE, energies unwritten
    for side in ("ligand", "protein"):
        bad = deck.head(deck.nposes)
        arr = (bad.ligand if side == "ligand" else bad.protein).copy()
        arr["type"][1] = deck.ntypes + 3
        if side == "ligand":
            bad.ligand = arr
        else:
            bad.protein = arr
        cb = Caller(torch_cuda, bad)
        assert cb.call(lib) == BUDE_ERR_TYPE, side
        assert np.all(cb.result() == 7.0), side
    # the shared working array still serves a good call
    check(c.call(lib))
    assert_parity(c.result(), oracle.fasten_f32(deck), oracle.fasten_f64(deck))


def test_noalloc_refuses_another_gpus_memory(built_library, torch_cuda):
    if torch_cuda.cuda.device_count() < 2:
        pytest.skip("one GPU: no other device's memory to pass")
    lib = built_library
    deck = synthetic_deck(SMALL, 9, 100)
    c = Caller(torch_cuda, deck)
    other = torch_cuda.zeros(deck.nposes, dtype=torch_cuda.float32, device="cuda:1")
    assert c.call(lib, energies=other.data_ptr()) == BUDE_ERR_ARG
