"""ctypes binding of libbude_gb300.so (declarations in include/minibude_gb300.h).

This module only describes the C-ABI; `minibude_gb300.model` builds the reference-shaped
interface on top of it.  Loading fails loudly when the library is missing: there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

from . import build as _build

c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_float_p = ctypes.POINTER(ctypes.c_float)
c_void_p = ctypes.c_void_p

BUDE_OK = 0
BUDE_ERR_ARG = -1
BUDE_ERR_CUDA = -2
BUDE_ERR_STATE = -3
BUDE_ERR_TIMEOUT = -4
BUDE_ERR_TYPE = -5

SCORER_TCGEN05 = 0
SCORER_MMA_SYNC = 1

STATUS_NAMES = {
    BUDE_OK: "BUDE_OK", BUDE_ERR_ARG: "BUDE_ERR_ARG", BUDE_ERR_CUDA: "BUDE_ERR_CUDA",
    BUDE_ERR_STATE: "BUDE_ERR_STATE", BUDE_ERR_TIMEOUT: "BUDE_ERR_TIMEOUT", BUDE_ERR_TYPE: "BUDE_ERR_TYPE",
}


class BudeLaunchCfg(ctypes.Structure):
    _fields_ = [("ppwi", c_int32), ("wgsize", c_int32), ("split", c_int32), ("tile", c_int32), ("unroll", c_int32),
                ("cluster", c_int32)]

    def as_dict(self):
        return {"ppwi": self.ppwi, "wgsize": self.wgsize, "split": self.split, "tile": self.tile,
                "unroll": self.unroll, "cluster": self.cluster}

    def __repr__(self):
        return "BudeLaunchCfg(%s)" % ", ".join(f"{k}={v}" for k, v in self.as_dict().items())


class BudeScreenCfg(ctypes.Structure):
    _fields_ = [("top_frac", ctypes.c_float), ("audit_frac", ctypes.c_float), ("audit_tol", ctypes.c_float),
                ("seed", ctypes.c_uint32), ("exact", BudeLaunchCfg), ("chunks", c_int32),
                ("rescore", BudeLaunchCfg)]


class BudeScreenStats(ctypes.Structure):
    _fields_ = [("total_ms", ctypes.c_float), ("surrogate_ms", ctypes.c_float), ("rescore_ms", ctypes.c_float),
                ("fallback_ms", ctypes.c_float), ("rescored_poses", c_int64), ("fallback_ligands", c_int32),
                ("fallback_poses", c_int64), ("max_audit_error", ctypes.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


SURROGATE_NPARAMS = 38404


class BudeError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


# (name, restype, argtypes) of every exported symbol.
_P = c_void_p
SIGNATURES = [
    ("bude_gpu_last_error", ctypes.c_char_p, []),
    ("bude_gpu_version", ctypes.c_char_p, []),
    ("bude_gpu_device_count", ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
    ("bude_gpu_device_name", ctypes.c_int, [ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t]),
    ("bude_gpu_sm_count", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    ("bude_gpu_compatible", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_int)]),
    ("bude_gpu_create", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(c_void_p)]),
    ("bude_gpu_destroy", ctypes.c_int, [_P]),
    ("bude_gpu_upload", ctypes.c_int, [_P, _P, c_int32, _P, c_int32, _P, c_int32, _P, c_int64, c_int64]),
    ("bude_gpu_set_poses", ctypes.c_int, [_P, _P, c_int32, _P, c_int64, c_int64]),
    ("bude_gpu_default_cfg", ctypes.c_int, [_P, c_int32, c_int32, ctypes.POINTER(BudeLaunchCfg)]),
    ("bude_gpu_autotune", ctypes.c_int, [_P, c_int32, ctypes.POINTER(BudeLaunchCfg), c_float_p]),
    ("bude_gpu_run", ctypes.c_int, [_P, ctypes.POINTER(BudeLaunchCfg), c_float_p]),
    ("bude_gpu_run_many", ctypes.c_int, [_P, ctypes.POINTER(BudeLaunchCfg), c_int32, c_int32, c_float_p,
                                         c_float_p]),
    ("bude_gpu_download", ctypes.c_int, [_P, c_float_p, c_int64]),
    ("bude_gpu_score_host", ctypes.c_int, [_P, ctypes.POINTER(BudeLaunchCfg), _P, c_int32, _P, c_int64, c_int64,
                                           c_float_p]),
    ("bude_gpu_score_stream", ctypes.c_int, [_P, ctypes.POINTER(BudeLaunchCfg), _P, c_int64, c_int64, c_int64,
                                             c_float_p, c_float_p]),
    ("bude_gpu_fasten", ctypes.c_int, [ctypes.c_int, c_int32, c_int32, _P, c_int32, _P, c_int32, _P, c_int32, _P,
                                       c_int64, c_int64, c_int32, c_float_p, c_float_p, c_float_p]),
    ("bude_gpu_upload_batch", ctypes.c_int, [_P, _P, c_int32, _P, c_int32, c_int32, _P, _P, _P, c_int64, _P]),
    ("bude_gpu_autotune_batch", ctypes.c_int, [_P, c_int32, ctypes.POINTER(BudeLaunchCfg), c_float_p]),
    ("bude_gpu_run_batch", ctypes.c_int, [_P, ctypes.POINTER(BudeLaunchCfg), c_int32, c_float_p]),
    ("bude_gpu_download_batch", ctypes.c_int, [_P, c_float_p, c_int64]),
    ("bude_surrogate_init", ctypes.c_int, [_P, _P, c_int32, _P, c_int32, ctypes.c_float, ctypes.c_float,
                                           ctypes.c_uint64]),
    ("bude_surrogate_train", ctypes.c_int, [_P, c_int32, c_int32, ctypes.c_float, _P, ctypes.c_uint64, c_float_p,
                                            c_float_p]),
    ("bude_surrogate_score", ctypes.c_int, [_P, c_float_p]),
    ("bude_surrogate_download", ctypes.c_int, [_P, c_float_p, c_int64]),
    ("bude_surrogate_set_scorer", ctypes.c_int, [_P, ctypes.c_int32]),
    ("bude_surrogate_gradient", ctypes.c_int, [_P, _P, c_int32, _P, c_float_p, c_float_p]),
    ("bude_surrogate_features", ctypes.c_int, [_P, _P, c_int32, c_float_p, _P]),
    ("bude_surrogate_params", ctypes.c_int, [_P, c_float_p, c_float_p, c_int64]),
    ("bude_surrogate_save", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("bude_surrogate_load", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("bude_screen_run", ctypes.c_int, [_P, ctypes.POINTER(BudeScreenCfg), ctypes.POINTER(BudeScreenStats)]),
    ("bude_screen_download", ctypes.c_int, [_P, c_float_p, _P, c_float_p, c_int64]),
    ("bude_gpu_launch_count", ctypes.c_int, [_P, ctypes.POINTER(c_int64)]),
    ("bude_gpu_selftest_wait", ctypes.c_int, [_P, c_int32, ctypes.POINTER(ctypes.c_float)]),
    ("bude_gpu_fasten_noalloc", ctypes.c_int, [_P, c_int32, _P, c_int32, _P, c_int32, _P, c_int64, c_int64, _P, _P]),
    ("bude_host_alloc", ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(c_void_p)]),
    ("bude_host_free", ctypes.c_int, [c_void_p]),
]

_lib: Optional[ctypes.CDLL] = None


def library_path() -> str:
    return _build.LIB


def lib() -> ctypes.CDLL:
    """The loaded library (built on first use if the sources are newer)."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(f"libbude_gb300.so is missing ({path}); build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'` -- there is no CPU fallback")
        l = ctypes.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def last_error() -> str:
    return lib().bude_gpu_last_error().decode()


def check(code: int) -> None:
    if code != BUDE_OK:
        raise BudeError(code, last_error())


def ptr(a) -> c_void_p:
    """Data pointer of a numpy array (None stays NULL)."""
    if a is None:
        return None
    return c_void_p(a.ctypes.data)


def fptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(c_float_p)
