"""Host-side invariants of the plain path's two-threads-per-cell split (pn_device.cuh), checked by
a small program compiled with nvcc and run on the host (no GPU): for every compiled order and
class the lower half starts at moment 0, the split sits at a degree boundary, and the halves'
degree masks partition the class's mask; the series coefficients 1/n! are the doubles nearest
to them."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else shutil.which("nvcc")


def test_split_invariants(tmp_path):
    nvcc = _nvcc()
    if not nvcc:
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "split_check")
    src = os.path.join(ROOT, "tests", "native", "split_check.cu")
    r = subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-O1",
                        "-I", os.path.join(ROOT, "pnepma_gb300", "csrc"), src, "-o", exe],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
