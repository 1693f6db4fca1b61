"""The host rule that cuts a ligand's poses into batch-kernel items (`for_each_item`,
minibude_gb300/csrc/internal.h), compiled with g++ against the library's own header and run on
the CPU: items cover the poses exactly once, in order, none larger than a block, and a remainder
in (ppb/2, 3ppb/4] is cut into ppb/2 + the rest from 8 poses per thread up (the cut the batch
kernel runs with half and a quarter of the poses per thread)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

HARNESS = r"""
#include <cstdio>
#include <cstdlib>
#include "internal.h"
int main(int argc, char **argv) {
  const int ppwi = std::atoi(argv[1]), ppb = std::atoi(argv[2]);
  for (int i = 3; i < argc; ++i) {
    const long long n = std::atoll(argv[i]);
    std::printf("%lld:", n);
    bude::for_each_item(n, ppwi, ppb, [&](long long p, int k) { std::printf(" %lld+%d", p, k); });
    std::printf("\n");
  }
  return 0;
}
"""


def _cuda_include():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.isfile(os.path.join(cand, "include", "cuda_runtime.h")):
            return os.path.join(cand, "include")
    nvcc = shutil.which("nvcc")
    if nvcc:
        inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
        if os.path.isfile(os.path.join(inc, "cuda_runtime.h")):
            return inc
    return None


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    inc = _cuda_include()
    if inc is None or shutil.which("g++") is None:
        pytest.skip("g++ or the CUDA headers are missing")
    d = tmp_path_factory.mktemp("items")
    src, exe = d / "items.cpp", d / "items"
    src.write_text(HARNESS)
    r = subprocess.run(["g++", "-std=c++17", "-O1", f"-I{inc}", f"-I{os.path.join(ROOT, 'minibude_gb300', 'csrc')}",
                        str(src), "-o", str(exe)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    return str(exe)


def cut(exe, ppwi, ppb, ns):
    out = subprocess.run([exe, str(ppwi), str(ppb), *map(str, ns)], stdout=subprocess.PIPE, text=True, check=True)
    res = {}
    for line in out.stdout.splitlines():
        n, items = line.split(":")
        res[int(n)] = [tuple(int(x) for x in it.split("+")) for it in items.split()]
    return res


def expected(n, ppwi, ppb):
    items, p = [], 0
    while n - p >= ppb:
        items.append((p, ppb))
        p += ppb
    r = n - p
    if ppwi >= 8 and 2 * r > ppb and 4 * r <= 3 * ppb:
        items += [(p, ppb // 2), (p + ppb // 2, r - ppb // 2)]
    elif r > 0:
        items.append((p, r))
    return items


@pytest.mark.parametrize("ppwi,wgsize", [(2, 128), (4, 64), (8, 32), (8, 128), (16, 64), (16, 256)])
def test_items_cover_the_poses_once(harness, ppwi, wgsize):
    ppb = ppwi * wgsize
    ns = sorted({0, 1, 2, ppb // 4, ppb // 2, ppb // 2 + 1, 3 * ppb // 4, 3 * ppb // 4 + 1, ppb - 1, ppb, ppb + 1,
                 2 * ppb + ppb // 2 + 1, 5 * ppb + 3 * ppb // 4, 410, 16384, 65536 + 7})
    got = cut(harness, ppwi, ppb, ns)
    for n in ns:
        items = got[n]
        assert items == expected(n, ppwi, ppb), n
        pos = 0
        for first, count in items:  # contiguous, in order, non-empty, at most one block
            assert first == pos and 0 < count <= ppb
            pos += count
        assert pos == n


def test_screen_picks_cut(harness):
    # 410 picks per ligand (2% + 0.5% of 16,384 poses) in one-warp blocks of 8 poses per thread:
    # one full 256-pose item, then 128 + 26 (run with 4 and 2 poses per thread).
    assert cut(harness, 8, 256, [410])[410] == [(0, 256), (256, 128), (384, 26)]
