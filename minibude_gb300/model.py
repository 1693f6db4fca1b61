"""Python host mirror of the reference's model interface, over the C-ABI.

`Gb300Bude` has the shape of `Bude<PPWI>` (src/bude.h:95-101): `name`, `enumerate_devices`,
`compatible` and `fasten`, with the reference's semantics -- `fasten` owns every device
allocation of the call, runs `iterations + warmup` evaluations and returns a `Sample` whose
energies are in pose order and whose kernel times include the warm-ups (src/main.cpp:344-351).
`GpuContext` is the lower-level handle used by the benchmark and the tests.
"""
from __future__ import annotations

import ctypes
import dataclasses
import time
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import capi
from .capi import SURROGATE_NPARAMS, BudeLaunchCfg, BudeScreenCfg, BudeScreenStats, check, fptr, ptr
from .deck import ATOM_DTYPE, FF_DTYPE, Deck


def _atoms(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=ATOM_DTYPE)


def _ff(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=FF_DTYPE)


def _poses(p) -> np.ndarray:
    p = np.ascontiguousarray(p, dtype=np.float32)
    if p.ndim != 2 or p.shape[0] != 6:
        raise ValueError("poses must be a float32 [6, nposes] block")
    return p


def launch_cfg(ppwi: int, wgsize: int, split: int = 1, tile: int = 64, unroll: int = 0,
               cluster: int = 1) -> BudeLaunchCfg:
    """A launch shape; unroll 0 picks the usual unroll for ppwi."""
    if unroll == 0:
        unroll = 1 if ppwi >= 16 else 2
    return BudeLaunchCfg(ppwi, wgsize, split, tile, unroll, cluster)


class GpuContext:
    """One bude_gpu_ctx: a device, a stream and an uploaded deck."""

    def __init__(self, device: int = 0):
        self._lib = capi.lib()
        h = ctypes.c_void_p()
        check(self._lib.bude_gpu_create(device, ctypes.byref(h)))
        self.handle = h
        self.device = device
        self.nposes = 0
        self._keep = []

    def close(self) -> None:
        if self.handle:
            self._lib.bude_gpu_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, deck: Deck) -> None:
        protein, ligand, ff = _atoms(deck.protein), _atoms(deck.ligand), _ff(deck.forcefield)
        poses = _poses(deck.poses)
        check(self._lib.bude_gpu_upload(self.handle, ptr(protein), protein.size, ptr(ligand), ligand.size, ptr(ff),
                                        ff.size, ptr(poses), poses.shape[1], poses.shape[1]))
        self.nposes = poses.shape[1]

    def set_poses(self, poses: np.ndarray, ligand: Optional[np.ndarray] = None) -> None:
        poses = _poses(poses)
        lig = None if ligand is None else _atoms(ligand)
        check(self._lib.bude_gpu_set_poses(self.handle, ptr(lig), 0 if lig is None else lig.size, ptr(poses),
                                           poses.shape[1], poses.shape[1]))
        self.nposes = poses.shape[1]

    def default_cfg(self, ppwi: int, wgsize: int) -> BudeLaunchCfg:
        cfg = BudeLaunchCfg()
        check(self._lib.bude_gpu_default_cfg(self.handle, ppwi, wgsize, ctypes.byref(cfg)))
        return cfg

    def autotune(self, max_ms: int = 400):
        """(launch shape, predicted ms per evaluation) picked by the library's autotuner."""
        cfg = BudeLaunchCfg()
        ms = ctypes.c_float()
        check(self._lib.bude_gpu_autotune(self.handle, max_ms, ctypes.byref(cfg), ctypes.byref(ms)))
        return cfg, ms.value

    def run(self, cfg: BudeLaunchCfg) -> float:
        ms = ctypes.c_float()
        check(self._lib.bude_gpu_run(self.handle, ctypes.byref(cfg), ctypes.byref(ms)))
        return ms.value

    def run_many(self, cfg: BudeLaunchCfg, iterations: int, flush_l2: bool = True):
        """(per-evaluation ms, exact-kernel-only ms) for `iterations` timed evaluations."""
        out = np.zeros(max(iterations, 1), np.float32)
        exact = np.zeros(max(iterations, 1), np.float32)
        check(self._lib.bude_gpu_run_many(self.handle, ctypes.byref(cfg), iterations, int(flush_l2), fptr(out),
                                          fptr(exact)))
        return out[:iterations], exact[:iterations]

    def download(self) -> np.ndarray:
        out = np.zeros(self.nposes, np.float32)
        check(self._lib.bude_gpu_download(self.handle, fptr(out), self.nposes))
        return out

    def score_host(self, cfg: BudeLaunchCfg, poses: np.ndarray, energies: np.ndarray,
                   ligand: Optional[np.ndarray] = None) -> np.ndarray:
        """End to end from host buffers: poses (and ligand) in, energies out."""
        poses = _poses(poses)
        lig = None if ligand is None else _atoms(ligand)
        check(self._lib.bude_gpu_score_host(self.handle, ctypes.byref(cfg), ptr(lig),
                                            0 if lig is None else lig.size, ptr(poses), poses.shape[1],
                                            poses.shape[1], fptr(energies)))
        self.nposes = poses.shape[1]
        return energies

    def score_stream(self, cfg: BudeLaunchCfg, poses: np.ndarray, energies: np.ndarray, chunk: int = 65536) -> float:
        """Evaluate host-resident poses (six fields, [6][n] or any array with a row stride) against
        the uploaded deck's protein and ligand, `chunk` poses at a time with copies overlapped;
        returns the CUDA-event time in ms.  Energies land in `energies` (n floats)."""
        if poses.ndim != 2 or poses.shape[0] != 6 or poses.dtype != np.float32 or poses.strides[1] != 4:
            raise ValueError("poses must be a float32 [6][n] array with contiguous rows")
        n, stride = poses.shape[1], poses.strides[0] // 4
        if energies.dtype != np.float32 or energies.size < n or not energies.flags.c_contiguous:
            raise ValueError("energies must be a contiguous float32 array of at least n values")
        ms = ctypes.c_float()
        check(self._lib.bude_gpu_score_stream(self.handle, ctypes.byref(cfg), ctypes.c_void_p(poses.ctypes.data),
                                              stride, n, chunk, fptr(energies), ctypes.byref(ms)))
        return ms.value

    # -- batches of ligands -------------------------------------------------------------------
    def upload_batch(self, batch) -> None:
        protein, ff = _atoms(batch.protein), _ff(batch.forcefield)
        atoms = _atoms(batch.atoms())
        lig_off = np.ascontiguousarray(batch.ligand_offsets(), np.int32)
        pose_off = np.ascontiguousarray(batch.pose_offsets(), np.int64)
        poses = _poses(batch.pose_block())
        check(self._lib.bude_gpu_upload_batch(self.handle, ptr(protein), protein.size, ptr(ff), ff.size,
                                              batch.nligands, ptr(atoms), ptr(lig_off), ptr(poses), poses.shape[1],
                                              ptr(pose_off)))
        self.batch_poses = poses.shape[1]

    def autotune_batch(self, max_ms: int = 2000):
        cfg = BudeLaunchCfg()
        ms = ctypes.c_float()
        check(self._lib.bude_gpu_autotune_batch(self.handle, max_ms, ctypes.byref(cfg), ctypes.byref(ms)))
        return cfg, ms.value

    def run_batch(self, cfg: BudeLaunchCfg, per_ligand: bool = False) -> float:
        ms = ctypes.c_float()
        check(self._lib.bude_gpu_run_batch(self.handle, ctypes.byref(cfg), int(per_ligand), ctypes.byref(ms)))
        return ms.value

    def upload_batch_arrays(self, protein, forcefield, atoms, lig_off, poses, pose_off) -> None:
        """bude_gpu_upload_batch from prepared arrays: the ligands' atoms concatenated, int32 atom
        offsets and int64 pose offsets (nligands + 1 each), and poses as a float32 [6][total]
        array with contiguous rows and any row stride (a PinnedBuffer view, for example)."""
        protein, ff, atoms = _atoms(protein), _ff(forcefield), _atoms(atoms)
        lig_off = np.ascontiguousarray(lig_off, np.int32)
        pose_off = np.ascontiguousarray(pose_off, np.int64)
        if poses.ndim != 2 or poses.shape[0] != 6 or poses.dtype != np.float32 or poses.strides[1] != 4:
            raise ValueError("poses must be a float32 [6][n] array with contiguous rows")
        if len(pose_off) < 1 or pose_off[-1] != poses.shape[1]:
            raise ValueError("the pose offsets must end at the number of poses")
        check(self._lib.bude_gpu_upload_batch(self.handle, ptr(protein), protein.size, ptr(ff), ff.size,
                                              len(lig_off) - 1, ptr(atoms), ptr(lig_off),
                                              ctypes.c_void_p(poses.ctypes.data), poses.strides[0] // 4,
                                              ptr(pose_off)))
        self.batch_poses = poses.shape[1]

    def download_batch(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Energies of the last batch evaluation, into `out` (a float32 array of the batch's pose
        count, e.g. a PinnedBuffer's) or a new array."""
        if out is None:
            out = np.zeros(self.batch_poses, np.float32)
        elif out.dtype != np.float32 or out.size < self.batch_poses or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous float32 array of the batch's pose count")
        check(self._lib.bude_gpu_download_batch(self.handle, fptr(out), self.batch_poses))
        return out

    # -- learned pre-screen --------------------------------------------------------------------
    def surrogate_init(self, protein, forcefield, extent: float = 11.0, spacing: float = 1.25, seed: int = 0):
        protein, ff = _atoms(protein), _ff(forcefield)
        check(self._lib.bude_surrogate_init(self.handle, ptr(protein), protein.size, ptr(ff), ff.size, extent, spacing,
                                            seed))

    def surrogate_train(self, epochs: int, batch_poses: int = 8192, lr: float = 1e-3, labels=None, seed: int = 0):
        """Train on the uploaded batch; returns (last-epoch mean loss, GPU ms)."""
        lab = None if labels is None else np.ascontiguousarray(labels, np.float32)
        loss, ms = ctypes.c_float(), ctypes.c_float()
        check(self._lib.bude_surrogate_train(self.handle, epochs, batch_poses, lr, ptr(lab), seed, ctypes.byref(loss),
                                             ctypes.byref(ms)))
        return loss.value, ms.value

    def surrogate_score(self) -> float:
        ms = ctypes.c_float()
        check(self._lib.bude_surrogate_score(self.handle, ctypes.byref(ms)))
        return ms.value

    def surrogate_set_scorer(self, scorer: str) -> None:
        """Select the scoring kernel: "tcgen05" (default) or "mma_sync"."""
        kinds = {"tcgen05": capi.SCORER_TCGEN05, "mma_sync": capi.SCORER_MMA_SYNC}
        if scorer not in kinds:
            raise ValueError(f"unknown scorer {scorer!r}; expected one of {sorted(kinds)}")
        check(self._lib.bude_surrogate_set_scorer(self.handle, kinds[scorer]))

    def surrogate_download(self) -> np.ndarray:
        out = np.zeros(self.batch_poses, np.float32)
        check(self._lib.bude_surrogate_download(self.handle, fptr(out), self.batch_poses))
        return out

    def surrogate_gradient(self, poses, labels):
        poses = np.ascontiguousarray(poses, np.int32)
        labels = np.ascontiguousarray(labels, np.float32)
        grads = np.zeros(SURROGATE_NPARAMS, np.float32)
        pred = np.zeros(poses.size, np.float32)
        check(self._lib.bude_surrogate_gradient(self.handle, ptr(poses), poses.size, ptr(labels), fptr(grads),
                                                fptr(pred)))
        return grads, pred

    def surrogate_features(self, poses, rows: int):
        poses = np.ascontiguousarray(poses, np.int32)
        X = np.zeros((rows, 32), np.float32)
        types = np.zeros(rows, np.int32)
        check(self._lib.bude_surrogate_features(self.handle, ptr(poses), poses.size, fptr(X), ptr(types)))
        return X, types

    def surrogate_params(self, new=None) -> np.ndarray:
        out = np.zeros(SURROGATE_NPARAMS, np.float32)
        src = None if new is None else np.ascontiguousarray(new, np.float32)
        check(self._lib.bude_surrogate_params(self.handle, fptr(out), fptr(src), SURROGATE_NPARAMS))
        return out

    def surrogate_save(self, path: str):
        check(self._lib.bude_surrogate_save(self.handle, path.encode()))

    def surrogate_load(self, path: str):
        check(self._lib.bude_surrogate_load(self.handle, path.encode()))

    # -- screening -------------------------------------------------------------------------------
    def screen(self, exact_cfg: BudeLaunchCfg, top_frac: float = 0.02, audit_frac: float = 0.005,
               audit_tol: float = 0.05, seed: int = 1, chunks: int = 0,
               rescore_cfg: Optional[BudeLaunchCfg] = None) -> dict:
        """Surrogate-screened scoring of the uploaded batch (bude_screen_run); chunks = ligand
        chunks of the surrogate / exact-rescoring pipeline (0: automatic); rescore_cfg = pose shape
        (ppwi, wgsize, unroll) of the exact rescoring (None: chosen by the library)."""
        cfg = BudeScreenCfg(top_frac, audit_frac, audit_tol, seed, exact_cfg, chunks,
                            rescore_cfg if rescore_cfg is not None else BudeLaunchCfg())
        st = BudeScreenStats()
        check(self._lib.bude_screen_run(self.handle, ctypes.byref(cfg), ctypes.byref(st)))
        return st.as_dict()

    def screen_download(self, nligands: int):
        final = np.zeros(self.batch_poses, np.float32)
        rescored = np.zeros(self.batch_poses, np.uint8)
        err = np.zeros(max(nligands, 1), np.float32)
        check(self._lib.bude_screen_download(self.handle, fptr(final), ptr(rescored), fptr(err), self.batch_poses))
        return final, rescored.astype(bool), err[:nligands]

    def selftest_wait(self, limit_us: int) -> Tuple[int, float]:
        """Run the bounded-wait self-test kernel (bude_gpu_selftest_wait): (status, kernel ms)."""
        ms = ctypes.c_float()
        return self._lib.bude_gpu_selftest_wait(self.handle, int(limit_us), ctypes.byref(ms)), ms.value

    def launch_count(self) -> int:
        n = ctypes.c_int64()
        check(self._lib.bude_gpu_launch_count(self.handle, ctypes.byref(n)))
        return n.value

    def energies(self, deck: Deck, cfg: Optional[BudeLaunchCfg] = None) -> np.ndarray:
        """Upload, evaluate once and download: the energies of every pose of `deck`."""
        self.upload(deck)
        if cfg is None:
            cfg = self.default_cfg(8, 128)
        self.run(cfg)
        return self.download()


class PinnedBuffer:
    """Page-locked host memory viewed as a numpy array."""

    def __init__(self, shape, dtype=np.float32):
        self._lib = capi.lib()
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        p = ctypes.c_void_p()
        check(self._lib.bude_host_alloc(nbytes, ctypes.byref(p)))
        self._p = p
        buf = (ctypes.c_byte * max(nbytes, 1)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if self._p:
            self.array = None
            self._lib.bude_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


@dataclasses.dataclass
class Sample:
    """src/bude.h:84-91: per-call results of `fasten`."""
    ppwi: int
    wgsize: int
    energies: np.ndarray
    kernel_times: List[Tuple[float, float]]  # host clock (start, end) per iteration, seconds
    kernel_ms: List[float]  # CUDA-event time per iteration
    context_time: Optional[Tuple[float, float]] = None


def device_count() -> int:
    n = ctypes.c_int()
    check(capi.lib().bude_gpu_device_count(ctypes.byref(n)))
    return n.value


def sm_count(device: int) -> int:
    n = ctypes.c_int()
    check(capi.lib().bude_gpu_sm_count(device, ctypes.byref(n)))
    return n.value


def device_name(device: int) -> str:
    buf = ctypes.create_string_buffer(256)
    check(capi.lib().bude_gpu_device_name(device, buf, len(buf)))
    return buf.value.decode()


class Gb300Bude:
    """The GB300 model behind the reference's `Bude<PPWI>` interface."""

    def __init__(self, ppwi: int = 1):
        self.ppwi = int(ppwi)

    def name(self) -> str:
        return "gb300"

    def enumerate_devices(self) -> List[Tuple[int, str]]:
        """src/cuda/fasten.hpp:181-196."""
        return [(i, device_name(i)) for i in range(device_count())]

    def compatible(self, deck: Deck, wgsize: int, device: int) -> bool:
        """src/cuda/fasten.hpp:218-248: kernel and device compute capabilities agree."""
        k, d, ok = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(capi.lib().bude_gpu_compatible(device, ctypes.byref(k), ctypes.byref(d), ctypes.byref(ok)))
        return bool(ok.value)

    def fasten(self, deck: Deck, wgsize: int, device: int, iterations: int = 8, warmup: int = 2) -> Sample:
        """src/cuda/fasten.hpp:250-305: allocate + copy (context), run iterations + warm-ups
        with a synchronise after each, copy the energies back, free."""
        t0 = time.perf_counter()
        ctx = GpuContext(device)
        try:
            ctx.upload(deck)
            t1 = time.perf_counter()
            cfg = ctx.default_cfg(self.ppwi, wgsize)
            times, ms = [], []
            for _ in range(iterations + warmup):
                s = time.perf_counter()
                ms.append(ctx.run(cfg))
                times.append((s, time.perf_counter()))
            energies = ctx.download()
        finally:
            ctx.close()
        return Sample(self.ppwi, wgsize, energies, times, ms, (t0, t1))
