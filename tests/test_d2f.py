"""The integer-pipe double-to-float conversions of the FP32 copy kernels
(d2f_rn, d2f_split in persiansph_gb300/csrc/psph_common.cuh) give the bits of
the compiler's own conversion: hi = (float)x and lo = (float)(x - (double)hi)
over 8M doubles (random bit patterns, FP32's range, ties, carries, range
edges). Compiled for the host with nvcc, so it runs without a GPU."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_d2f_matches_the_conversion_instruction(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "d2f_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                    "-I", os.path.join(REPO, "persiansph_gb300", "csrc"),
                    os.path.join(REPO, "tests", "cxx", "d2f_check.cu"), "-o", exe],
                   check=True, capture_output=True, text=True)
    res = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "mismatches 0" in res.stdout
