"""Layout arithmetic of the training kernels, checked on the host (tests/layouts_check.cu built
with nvcc and run on the CPU: no GPU call)."""
import os
import subprocess

from minibude_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))


def test_operand_tile_layouts(tmp_path):
    exe = str(tmp_path / "layouts_check")
    r = subprocess.run([B.nvcc(), *B.ARCH, "-std=c++17", "--expt-relaxed-constexpr", "-I", B.CSRC,
                        os.path.join(HERE, "layouts_check.cu"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", (out.stdout, out.stderr)
