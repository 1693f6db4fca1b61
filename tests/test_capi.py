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


def test_ctypes_structs_match_the_header(tmp_path):
    # The ctypes mirrors of the header's structs have the C compiler's sizes and field offsets.
    import subprocess
    from minibude_gb300 import capi
    structs = {"bude_launch_cfg": capi.BudeLaunchCfg, "bude_screen_cfg": capi.BudeScreenCfg,
               "bude_screen_stats": capi.BudeScreenStats}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "minibude_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    for cname, names in (("bude_atom", ("x", "y", "z", "type")), ("bude_ffparams", ("hbtype", "radius", "hphb", "elsc"))):
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field in names:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{os.path.join(ROOT, 'include')}", str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        cname, key, value = line.split()
        got[(cname, key)] = int(value)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)
    # the numpy record types of the deck files
    from minibude_gb300.deck import ATOM_DTYPE, FF_DTYPE
    for cname, dt in (("bude_atom", ATOM_DTYPE), ("bude_ffparams", FF_DTYPE)):
        assert got[(cname, "size")] == dt.itemsize, cname
        for field in dt.names:
            assert got[(cname, field)] == dt.fields[field][1], (cname, field)
