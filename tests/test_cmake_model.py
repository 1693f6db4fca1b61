"""The GB300 model registered with the reference's own CMake model registry, as a maintainer would.

A copy of the reference's build files and sources gets the three edits of the integration steps:
the model directory under src/gb300/, `register_model(gb300 GB300 fasten.hpp)` beside the other
models (CMakeLists.txt:158-171) and the `GB300` branch of main.cpp's model selection
(main.cpp:55-89).  `cmake -DMODEL=gb300` then loads src/gb300/model.cmake through
cmake/register_models.cmake:115-147, which compiles the CUDA sources into libbude_gb300 for sm_103a
and links it to the driver, `gb300-bude`, whose main.cpp the C++ compiler builds.  The build runs here (nvcc cross-compiles;
no GPU is needed), and the reference driver's own command line comes up on top of the model.
Runs only where the reference tree and cmake are present."""
import os
import re
import shutil
import subprocess

import pytest

import oracle
from conftest import ROOT

REF = oracle.reference_root()
needs = pytest.mark.skipif(not oracle.reference_tree_present() or shutil.which("cmake") is None
                           or shutil.which("nvcc") is None, reason="reference tree, cmake or nvcc not present")


def integrate(tree):
    """Apply the integration steps to a copy of the reference tree."""
    shutil.copytree(os.path.join(ROOT, "minibude_gb300", "model", "gb300"), os.path.join(tree, "src", "gb300"))
    cml = os.path.join(tree, "CMakeLists.txt")
    text = open(cml).read()
    last = list(re.finditer(r"^register_model\(.*\)[^\n]*$", text, re.M))[-1]
    text = text[:last.end()] + "\nregister_model(gb300 GB300 fasten.hpp)" + text[last.end():]
    open(cml, "w").write(text)
    main = os.path.join(tree, "src", "main.cpp")
    text = open(main).read()
    chain_end = text.index('#else\n  #error "No model defined"')
    text = text[:chain_end] + '#elif defined(GB300)\n  #include "gb300/fasten.hpp"\n' + text[chain_end:]
    open(main, "w").write(text)


@needs
def test_cmake_registers_builds_and_runs_the_gb300_model(tmp_path):
    tree = str(tmp_path / "miniBUDE")
    os.makedirs(tree)
    shutil.copy(os.path.join(REF, "CMakeLists.txt"), tree)
    shutil.copytree(os.path.join(REF, "cmake"), os.path.join(tree, "cmake"))
    shutil.copytree(os.path.join(REF, "src"), os.path.join(tree, "src"))
    integrate(tree)
    build = str(tmp_path / "build")
    cfg = subprocess.run(["cmake", "-S", tree, "-B", build, "-DMODEL=gb300", f"-DGB300_ROOT={ROOT}",
                          "-DGB300_NVCC=" + shutil.which("nvcc"), "-DUSAGE=OFF"],
                         stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    assert cfg.returncode == 0, cfg.stdout[-4000:]
    assert "Selected model  :  gb300" in cfg.stdout
    jobs = str(max(2, min(8, os.cpu_count() or 2)))
    b = subprocess.run(["cmake", "--build", build, "-j", jobs], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=900)
    assert b.returncode == 0, b.stdout[-4000:]
    exe = os.path.join(build, "gb300-bude")
    assert os.path.exists(exe)
    h = subprocess.run([exe, "--help"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=60)
    assert h.returncode == 0, h.stdout
    assert "--ppwi" in h.stdout and "--deck" in h.stdout


def test_cmake_model_lists_every_translation_unit():
    # model.cmake and minibude_gb300/build.py compile the same .cu files.
    from minibude_gb300 import build
    text = open(os.path.join(ROOT, "minibude_gb300", "model", "gb300", "model.cmake")).read()
    listed = re.search(r"set\(GB300_CU_SOURCES ([^)]*)\)", text).group(1).split()
    assert sorted(t + ".cu" for t in listed) == sorted(build.CU_SOURCES)
