"""The C ABI from C++: tests/cabi/main_loop.cc (main.cc's design loop through
include/topopt_gb300.h alone) is compiled with g++ and linked with
libtopopt_gb300.so.  Without a GPU it must refuse loudly; on the GPU its
objectives, constraint values and design changes equal the Python mirror's
design loop (the same kernels behind host-pointer instead of device-pointer
entry points), and its SOMMG object reports the reduced matrices of the
Python object."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LINE = re.compile(r"It\.: (\d+), True fx: (\S+), Scaled fx: (\S+), gx\[0\]: (\S+), ch: (\S+), mnd: (\S+)")


def _driver(tmp_path):
    from topopt_in_petsc_transient_gb300 import build
    lib = build.build()
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "main_loop")
    libdir = os.path.dirname(lib)
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cabi", "main_loop.cc"), "-o", exe, "-L", libdir,
                        "-ltopopt_gb300", "-Wl,-rpath," + libdir], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _run(exe, args):
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=1200)
    return r


def test_driver_builds_and_refuses_without_a_gpu(tmp_path):
    import torch
    exe = _driver(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = _run(exe, [])
    assert r.returncode == 1 and "no CPU fallback" in r.stderr


ARGS = dict(nelx=16, nely=8, nelz=8, nlvls=3, ncp=2, tsc=5, t1=0.05, maxItr=3, objective=3, loadsignal=1, mixed=1,
            rtol=1e-10, volfrac=0.12, rmin=2.0)


def _python_loop(**kw):
    from topopt_in_petsc_transient_gb300 import TopOpt, design_iteration
    o = TopOpt(nelx=kw["nelx"], nely=kw["nely"], nelz=kw["nelz"], nlvls=kw["nlvls"], ncp=kw["ncp"], tsc=kw["tsc"],
               t1=kw["t1"], objective=kw["objective"], loadsignal=kw["loadsignal"], mixed=bool(kw["mixed"]),
               rtol=kw["rtol"], volfrac=kw["volfrac"], rmin=kw["rmin"], Emax=1.0, Ef=1e-9, Rmax=1.0, Rf=1e-3,
               dalpha=0.0, dbeta=1e-3, filter=2, projectionFilter=False, reduction=bool(kw.get("reduction", 0)),
               basis=kw.get("basis", 4), omega0=kw.get("omega0", 0.01)).setup()
    rows = [design_iteration(o) for _ in range(kw["maxItr"])]
    return o, rows


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [1, 0])
def test_cpp_driver_equals_python_design_loop(gpu, tmp_path, mixed):
    exe = _driver(tmp_path)
    kw = dict(ARGS, mixed=mixed)
    r = _run(exe, sum([["-" + k, v] for k, v in kw.items()], []))
    assert r.returncode == 0, r.stderr[-2000:]
    got = [tuple(float(v) for v in m.groups()[1:]) + (int(m.group(1)),) for m in LINE.finditer(r.stdout)]
    assert len(got) == kw["maxItr"] and "# Optimization has terminated" in r.stdout
    _, rows = _python_loop(**kw)
    for (fx, fxs, gx, ch, mnd, itr), (pfx, pfxs, pgx, pch, pmnd) in zip(got, rows):
        assert abs(fx - pfx) <= 1e-12 * abs(pfx), (itr, fx, pfx)
        assert abs(fxs - pfxs) <= 1e-12 * abs(pfxs)
        assert abs(gx - pgx) <= 1e-13 and abs(mnd - pmnd) <= 1e-13
        # main.cc prints ch before "if (gx[0] > 0) ch = 1" (main.cc:133-145);
        # design_iteration returns it after
        if pgx > 0:
            assert pch == 1.0
        else:
            assert abs(ch - pch) <= 1e-12 * max(abs(pch), 1e-30)
    assert got[-1][0] != got[0][0]  # the design moved


@pytest.mark.gpu
def test_cpp_driver_sommg_members(gpu, tmp_path):
    exe = _driver(tmp_path)
    # omega0 below the first eigenfrequency of the 0.12-density beam (about
    # 0.0076), where P0 = K - om^2 M is positive definite
    kw = dict(ARGS, nelx=8, nely=4, nelz=4, nlvls=2, maxItr=2, mixed=0, rtol=1e-13, reduction=1, basis=4,
              omega0=0.004)
    r = _run(exe, sum([["-" + k, v] for k, v in kw.items()], []))
    assert r.returncode == 0, r.stderr[-2000:]
    diag = [tuple(float(v) for v in m.groups()) for m in
            re.finditer(r"Kr\[\d+\]\[\d+\]: (\S+) Mr: (\S+) Cr: (\S+) Pr\[\d+\]: (\S+)", r.stdout)]
    assert len(diag) == 4
    o, _ = _python_loop(**kw)
    Q, Kr, Mr, Pr = o.physics.reduced_system()
    Cr = o.dalpha * Mr + o.dbeta * Kr
    for i, (k, m, c, p) in enumerate(diag):
        assert abs(k - Kr[i, i]) <= 1e-12 * abs(Kr[i, i])
        assert abs(m - Mr[i, i]) <= 1e-12 * abs(Mr[i, i])
        assert abs(c - Cr[i, i]) <= 1e-12 * abs(Cr[i, i])
        assert abs(p - Pr[i]) <= 1e-12 * np.abs(Pr).max()
    assert np.allclose(Q @ Q.T, np.eye(4), atol=1e-10)  # an orthonormal basis (SOMMG.cc:195-210)
