"""The C-ABI library on CPU: it loads, exports every function include/minibude_gb300.h declares,
and its host-only paths (argument checks, error text) work without a GPU."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(bude_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_functions():
    names = declared_functions()
    assert "bude_gpu_upload" in names and "bude_gpu_run" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(built_library):
    for name in declared_functions():
        assert hasattr(built_library, name), name


def test_binding_covers_header(built_library):
    from minibude_gb300.capi import SIGNATURES
    bound = {n for n, _, _ in SIGNATURES}
    assert set(declared_functions()) <= bound


def test_version_and_error_text(built_library):
    from minibude_gb300 import capi
    assert b"sm_103a" in built_library.bude_gpu_version()
    rc = built_library.bude_gpu_create(0, None)
    assert rc == capi.BUDE_ERR_ARG
    assert "NULL" in capi.last_error()
    cfg = capi.BudeLaunchCfg(8, 128, 1, 64, 1, 1)
    assert built_library.bude_gpu_run(None, ctypes.byref(cfg), None) == capi.BUDE_ERR_ARG


def test_library_has_no_oracle_dependency():
    # The product library never links the oracle.
    from minibude_gb300 import build
    data = open(build.LIB, "rb").read() if os.path.exists(build.LIB) else b""
    assert b"oracle_fasten" not in data
