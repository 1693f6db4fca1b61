"""The GB300 model header drops into the reference's own driver unchanged.

The reference's src/main.cpp (unmodified) is compiled against the reference's src/bude.h with
gb300/fasten.hpp standing in the model slot: a scratch tree mirrors the reference's src/ through
symlinks, with `cuda/fasten.hpp` -> our gb300/fasten.hpp so that `-DCUDA` selects it without
editing main.cpp.  Runs only where the reference tree is present (the test-fixture machine)."""
import os
import subprocess

import pytest

import oracle
from conftest import ROOT

REF = oracle.reference_root()


@pytest.mark.skipif(not oracle.reference_tree_present(), reason="reference tree not present")
def test_reference_driver_compiles_with_gb300_model(tmp_path):
    from minibude_gb300 import build
    build.build_library()
    src = tmp_path / "src"
    src.mkdir()
    os.symlink(os.path.join(REF, "src", "bude.h"), src / "bude.h")
    os.symlink(os.path.join(REF, "src", "main.cpp"), src / "main.cpp")
    (src / "cuda").mkdir()
    os.symlink(os.path.join(ROOT, "minibude_gb300", "model", "gb300", "fasten.hpp"), src / "cuda" / "fasten.hpp")
    exe = tmp_path / "gb300-bude-ref"
    cmd = ["g++", "-std=c++17", "-O2", "-DCUDA", f"-I{ROOT}/include", str(src / "main.cpp"), "-o", str(exe),
           f"-L{os.path.dirname(build.LIB)}", "-lbude_gb300", f"-Wl,-rpath,{os.path.dirname(build.LIB)}"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    # The reference driver's own CLI runs on top of the GB300 model.
    h = subprocess.run([str(exe), "--help"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=60)
    assert h.returncode == 0 and "--ppwi" in h.stdout
