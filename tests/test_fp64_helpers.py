"""The FP64 helpers of csrc/mf_fp64.cuh on the GPU: the reciprocal and
logarithm (used by the FP64 charge-exchange rates of the mixed-precision and
FP64-fast paths) against the CUDA library's correctly rounded 1/x and its
log, and the integer FP32 <-> FP64 conversions against the conversion
instructions, bit for bit."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "ms-flukss-multifluid_gb300", "csrc")


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    return None


def test_fp64_helpers_compile(tmp_path):
    """Cross-compiles the check for sm_103a (no GPU needed)."""
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    out = tmp_path / "fp64_check.o"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I", CSRC, "-c", os.path.join(HERE, "cuda", "fp64_check.cu"), "-o", str(out)],
                   check=True, capture_output=True)


@pytest.mark.gpu
def test_fp64_helpers_accuracy(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = tmp_path / "fp64_check"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I", CSRC, os.path.join(HERE, "cuda", "fp64_check.cu"), "-o", str(exe)],
                   check=True, capture_output=True)
    r = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120)
    vals = dict(line.split(maxsplit=1) for line in r.stdout.strip().splitlines())
    assert vals["status"] == "no error"
    # 1/x: within 1 ulp of the correctly rounded quotient
    assert float(vals["rcp64_ulp"]) <= 1.0
    # log: a few units of 2^-53 absolute (relative to max(1, |log x|))
    assert float(vals["log64_ulp"]) <= 4.0
    # zero, negatives, subnormals, inf and NaN fall back to the library
    assert int(vals["special_mismatch"]) == 0
    # the integer FP32 -> FP64 and FP64 -> FP32 conversions equal the
    # conversion instructions bit for bit (ties included)
    assert int(vals["f2d_mismatch"]) == 0
    assert int(vals["d2f_mismatch"]) == 0
