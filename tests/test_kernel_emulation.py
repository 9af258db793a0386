"""CPU execution of the device source of the alternative kernel forms: the
z-marching slab operator kernel (slab.cuh) against the brick kernel
(tile.cuh) for FP32, FP64 and double-float with one and two staged inputs
and through the grid reduction of a policy with dot products, the solver's
own policies (the FP32 Krylov product, the double-float replacement product
with its early exit, the double-float K-only product) through both forms, and the
line-segment Kronecker passes against the staged ones (kron.cuh), compiled as
host C++ (tests/kernel_emu/cuda_runtime.h) and run with one host thread per
CUDA thread; outputs must agree bitwise, every node be written once, and the
reduced sums match the host's."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "topopt_in_petsc_transient_gb300", "csrc")
EMU = os.path.join(HERE, "kernel_emu")


@pytest.mark.parametrize("src,ok", [("slab_emu.cpp", "slab emulation OK"), ("kron_emu.cpp", "kron emulation OK"),
                                    ("policy_emu.cpp", "policy emulation OK")])
def test_kernel_forms_agree_bitwise_on_host_threads(tmp_path, src, ok):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / src.replace(".cpp", ""))
    r = subprocess.run([gxx, "-std=c++20", "-O1", "-w", "-I", EMU, "-I", CSRC, os.path.join(EMU, src), "-o", exe,
                        "-pthread"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and ok in r.stdout, r.stdout + r.stderr
