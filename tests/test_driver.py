"""The gb300-bude driver binary: the reference driver's CLI / deck / YAML / validation contract."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


@pytest.fixture(scope="module")
def driver():
    from minibude_gb300 import build
    build.build_library()
    path = build.build_driver()
    assert os.path.exists(path)
    return path


def run(driver, *args):
    return subprocess.run([driver, *args], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=600)


def test_help(driver):
    r = run(driver, "--help")
    assert r.returncode == 0
    for opt in ("--device", "--iter", "--poses", "--ppwi", "--wgsize", "--deck", "--out", "--rows", "--csv", "--list"):
        assert opt in r.stdout


def test_unknown_argument(driver):
    r = run(driver, "--bogus")
    assert r.returncode != 0 and "Unrecognized argument" in r.stdout


def test_bad_ppwi_and_ints(driver):
    r = run(driver, "-p", "3", "--deck", os.path.join(GOLDEN, "bm1_head"))
    assert r.returncode != 0 and "not a supported value" in r.stderr
    r = run(driver, "-i", "abc")
    assert r.returncode != 0 and "integer required" in r.stderr
    r = run(driver, "-i")
    assert r.returncode != 0 and "no value was given" in r.stderr


def test_yaml_header_provenance(driver):
    # The header the reference prints before any device work (src/main.cpp:570-636): version,
    # every compile command of this build, the git state it was built from, the host CPU.
    # `--list` needs a device afterwards, so only the header is checked here.
    out = run(driver, "--list").stdout
    head = out[:out.index("time: {")]
    assert head.startswith("miniBUDE:  gb300 ")
    cmds = re.findall(r'^   - "(.*)"$', head, re.M)
    assert len(cmds) >= 10 and sum("arch=compute_103a,code=sm_103a" in c for c in cmds) >= 9
    vcs = head[head.index("vcs:"):head.index("host_cpu:")]
    assert re.search(r"commit:  [0-9a-f]{40}\*?\n", vcs) or "# not built from a git checkout" in vcs
    cpu = head[head.index("host_cpu:"):]
    assert re.search(r'arch: +"(x86 \(|aarch64)', cpu) or cpu.strip().endswith("~")


def test_deck_errors(driver, tmp_path):
    r = run(driver, "--deck", os.path.join(GOLDEN, "bm1_head"), "-n", "5000")
    assert r.returncode != 0 and "exceeded max poses" in r.stderr
    bad = tmp_path / "deck"
    shutil.copytree(os.path.join(GOLDEN, "bm1_head"), bad)
    with open(bad / "poses.in", "ab") as f:
        f.write(b"\0\0\0\0")
    r = run(driver, "--deck", str(bad))
    assert r.returncode != 0 and "not divisible" in r.stderr
    r = run(driver, "--deck", str(tmp_path / "missing"))
    assert r.returncode != 0 and "Bad file" in r.stderr


@pytest.mark.gpu
def test_bm1_head_yaml(driver, tmp_path):
    out = tmp_path / "e.txt"
    r = run(driver, "--deck", os.path.join(GOLDEN, "bm1_head"), "-p", "1,8,128", "-w", "1,64,256", "-i", "3",
            "-o", str(out))
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("outcome:") == 9
    assert "valid: false" not in r.stdout
    for key in ("max_diff_%", "raw_iterations", "context_ms", "giga_interactions/s", "gflop/s", "fp32_peak_%", "best:"):
        assert key in r.stdout
    raws = re.findall(r"raw_iterations:\s+\[([^\]]*)\]", r.stdout)
    assert all(len(x.split(",")) == 5 for x in raws)  # 3 iterations + 2 warm-ups
    assert len(open(out).read().split()) == 1024


@pytest.mark.gpu
def test_csv_and_list(driver):
    r = run(driver, "--list")
    assert r.returncode == 0 and "GB300" in r.stdout
    r = run(driver, "--deck", os.path.join(GOLDEN, "small_head"), "-p", "4,8", "-w", "64,128", "--csv")
    assert r.returncode == 0
    rows = [l for l in r.stdout.splitlines() if not l.startswith("#")]
    assert rows[0].startswith("ppwi,wgsize,sum_ms") and rows[1].startswith("4,64,")
    # The reference's heatmap.py reads this output as pandas.read_csv(comment="#", skiprows=1)
    # and pivots sum_ms over (ppwi, wgsize): the same read, without pandas.
    lines = [l.split("#")[0] for l in r.stdout.splitlines()[1:]]
    lines = [l for l in lines if l.strip()]
    head = lines[0].split(",")
    table = np.array([[float(x) for x in l.split(",")] for l in lines[1:]])
    cols = {k: table[:, head.index(k)] for k in ("ppwi", "wgsize", "sum_ms")}
    assert sorted(set(cols["ppwi"])) == [4, 8] and sorted(set(cols["wgsize"])) == [64, 128]
    assert len(table) == 4 and np.all(cols["sum_ms"] > 0)


@pytest.mark.gpu
def test_failed_validation_exit_status(driver, tmp_path):
    bad = tmp_path / "deck"
    shutil.copytree(os.path.join(GOLDEN, "bm1_head"), bad)
    refs = np.fromfile(os.path.join(GOLDEN, "bm1_head", "ref_energies.f32"), "<f4") * 1.01
    with open(bad / "ref_energies.out", "w") as f:
        f.write("".join("%.6f\n" % x for x in refs))
    r = run(driver, "--deck", str(bad), "-i", "1")
    assert r.returncode != 0
    assert "Verification failed" in r.stderr and "valid: false" in r.stdout
