"""The integer-pipe FP64 -> double-float split (csrc/df.cuh, f64_to_df) and
the double-float arithmetic on the host: the split also builds the
double-float element constants, and on the GPU it replaces an FP64
subtraction per staged value.  tests/cuda/df_host_check.cu is compiled for the
host with nvcc; it checks the split for exactness on 3 M values and the error
bounds of operator+, add_lazy (the element math's unrenormalised sums),
operator* and an 8-point butterfly of lazy sums against long double (the
device split is checked against the hardware conversions by
tests/test_gpu_conversions.py)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_f64_to_df_split_is_exact_on_the_host(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "df_host_check")
    r = subprocess.run([nvcc, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "topopt_in_petsc_transient_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "cuda", "df_host_check.cu"), "-o", exe],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "split OK" in r.stdout, r.stdout + r.stderr
