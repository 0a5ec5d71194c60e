"""quotient() (luma_gb300/csrc/quotient.cuh): the FP64 divisions of the
banded LU's forward solve and of the moving markers' kernel evaluations are
formed from the divisor's reciprocal with two Markstein corrections.  This
checks that the result is CUDA's division bit for bit: ~80 M pseudo-random
operand pairs over exponent spans up to 2^+-420 (beyond the +-400 bound
where quotient() takes the division itself) and every pair of a set of
special values (signed zeros, subnormals, infinities, NaN, operands at the
bound)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "luma_gb300", "csrc")


def test_quotient_matches_division(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "quotient_check")
    subprocess.run([nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-fmad=false",
                    "-I", CSRC, os.path.join(HERE, "gpu_src", "quotient_check.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mismatches 0" in out.stdout, out.stdout
