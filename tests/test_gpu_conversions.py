"""The integer-pipe FP64/FP32 conversions of csrc/df.cuh (used by the
streaming kernels, where FP64 conversions on GB300's FP64 pipe set the time,
and by the double-float staging of the element passes) against the hardware
conversions: tests/cuda/conv_check.cu, built with nvcc for sm_103a and run on
the GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.gpu
def test_integer_pipe_conversions_match_hardware(gpu, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "conv_check")
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                        "-I", os.path.join(ROOT, "topopt_in_petsc_transient_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "cuda", "conv_check.cu"), "-o", exe],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "conversions OK" in r.stdout, r.stdout + r.stderr
