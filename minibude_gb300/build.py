"""Build the native parts in-tree: libbude_gb300.so (nvcc, sm_103a) and the C++ driver.

Used by ``__graft_entry__.build()`` and by ``python -m minibude_gb300.build``.  Outputs land next
to the sources (git-ignored) so the library that runs is always the in-tree one.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libbude_gb300.so")
DRIVER_BIN = os.path.join(PKG, "bin", "gb300-bude")
MAKEDECK_BIN = os.path.join(PKG, "bin", "gb300-makedeck")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]

# Translation units of libbude_gb300.so; each compiles in parallel.
CU_SOURCES = ["bude_gb300.cu", "autotune.cu", "batch.cu", "surrogate.cu", "screen.cu", "noalloc.cu", "stream.cu",
              "arch_probe.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _csrc_deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def build_library(force: bool = False, verbose: bool = False) -> str:
    """Compile every .cu file for sm_103a and link libbude_gb300.so."""
    os.makedirs(BUILD, exist_ok=True)
    deps = _csrc_deps()
    if not force and not _stale(LIB, deps):
        return LIB
    jobs, link = library_commands()
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    _run(link)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def _c_string(s: str) -> str:
    return '"' + s.replace("\\", "\\\\").replace('"', '\\"').replace("\n", " ") + '"'


def _git(*args) -> str:
    r = subprocess.run(["git", "-C", ROOT, *args], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    if r.returncode != 0:
        raise RuntimeError("git " + " ".join(args))
    return r.stdout.strip()


def library_commands():
    """The command lines that build libbude_gb300.so (one per translation unit, then the link)."""
    nv = nvcc()
    objs = [os.path.join(BUILD, os.path.splitext(src)[0] + ".o") for src in CU_SOURCES]
    cmds = [[nv, *ARCH, *NVCC_FLAGS, "-Xptxas", "-v", "-c", os.path.join(CSRC, src), "-o", obj]
            for src, obj in zip(CU_SOURCES, objs)]
    return cmds, [nv, *ARCH, "-shared", "-o", LIB + ".tmp", *objs]


def write_meta_header(driver_cmd) -> str:
    """_build/meta_build.h: the build's provenance for the driver's YAML header (the reference's
    meta_build.h / meta_vcs.h, src/main.cpp:16-21, 570-584): version, compile commands and the
    state of the git checkout when there is one.  Rewritten only when its content changes."""
    os.makedirs(BUILD, exist_ok=True)
    comp, link = library_commands()
    cmds = [" ".join(c) for c in comp + [link, driver_cmd]]
    lines = ["#pragma once", '#define GB300_BUDE_VERSION "0.1"',
             "#define GB300_BUDE_COMPILE_COMMANDS { " + ", ".join(_c_string(c) for c in cmds) + " }"]
    try:
        sha = _git("rev-parse", "HEAD")
        dirty = 1 if _git("status", "--porcelain", "--untracked-files=no") else 0
        name, email, date, subject = (_git("log", "-1", f"--format=%{f}") for f in ("an", "ae", "cI", "s"))
        lines += ["#define GB300_BUDE_VCS_RETRIEVED_STATE 1", f"#define GB300_BUDE_VCS_HEAD_SHA1 {_c_string(sha)}",
                  f"#define GB300_BUDE_VCS_IS_DIRTY {dirty}",
                  f"#define GB300_BUDE_VCS_AUTHOR_NAME {_c_string(name)}",
                  f"#define GB300_BUDE_VCS_AUTHOR_EMAIL {_c_string(email)}",
                  f"#define GB300_BUDE_VCS_COMMIT_DATE_ISO8601 {_c_string(date)}",
                  f"#define GB300_BUDE_VCS_COMMIT_SUBJECT {_c_string(subject)}"]
    except (OSError, RuntimeError):
        lines += ["#define GB300_BUDE_VCS_RETRIEVED_STATE 0"]
    text = "\n".join(lines) + "\n"
    path = os.path.join(BUILD, "meta_build.h")
    if not os.path.exists(path) or open(path).read() != text:
        with open(path, "w") as f:
            f.write(text)
    return path


def build_driver(force: bool = False) -> str:
    """The C++ driver binary (gb300-bude): the reference's CLI/YAML contract over the C-ABI."""
    src = os.path.join(PKG, "driver", "main.cpp")
    if not os.path.exists(src):
        return ""
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", f"-I{INCLUDE}", f"-I{os.path.join(PKG, 'driver')}",
           f"-I{os.path.join(PKG, 'model')}", f"-I{BUILD}", "-DGB300", src, "-o", DRIVER_BIN, f"-L{PKG}",
           "-lbude_gb300", f"-Wl,-rpath,{PKG}"]
    meta = write_meta_header(cmd)
    deps = [src, LIB, meta] + [os.path.join(PKG, "driver", f) for f in os.listdir(os.path.join(PKG, "driver"))]
    deps += [os.path.join(PKG, "model", "gb300", f) for f in os.listdir(os.path.join(PKG, "model", "gb300"))]
    if not force and not _stale(DRIVER_BIN, deps):
        return DRIVER_BIN
    os.makedirs(os.path.dirname(DRIVER_BIN), exist_ok=True)
    _run(cmd)
    return DRIVER_BIN


def build_makedeck(force: bool = False) -> str:
    """The deck generator binary (gb300-makedeck): makedeck's command line over the C-ABI."""
    d = os.path.join(PKG, "makedeck")
    srcs = [os.path.join(d, "main.cpp"), os.path.join(d, "deck_builder.cpp")]
    deps = srcs + [os.path.join(d, "deck_builder.h"), LIB]
    if not force and not _stale(MAKEDECK_BIN, deps):
        return MAKEDECK_BIN
    os.makedirs(os.path.dirname(MAKEDECK_BIN), exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    _run([cxx, "-std=c++17", "-O2", "-Wall", f"-I{INCLUDE}", f"-I{d}"] + srcs +
         ["-o", MAKEDECK_BIN, f"-L{PKG}", "-lbude_gb300", f"-Wl,-rpath,{PKG}"])
    return MAKEDECK_BIN


def build_all(force: bool = False, verbose: bool = False) -> None:
    build_library(force=force, verbose=verbose)
    build_driver(force=force)
    build_makedeck(force=force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose=True)
    print(LIB)
