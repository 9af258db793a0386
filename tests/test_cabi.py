"""CPU checks of the C ABI: the library loads, exports exactly what
include/topopt_gb300.h declares, refuses to run without a GPU, and its
element algebra equals the oracle's Gauss quadrature (LinearElasticity.cc:3089-3333)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from topopt_in_petsc_transient_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def _declared():
    src = open(os.path.join(ROOT, "include", "topopt_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return set(re.findall(r"\b(topo_[a-z0-9_]+)\s*\(", src))


def test_header_and_exports_agree(lib):
    declared = _declared()
    assert declared == set(_lib.EXPORTS)
    for name in declared:
        assert hasattr(lib, name), name


def test_status_strings(lib):
    assert lib.topo_status_str(0) == b"ok"
    assert lib.topo_status_str(4) == b"linear solve did not converge"


def test_no_gpu_is_a_loud_error(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = _lib.LEParams()
    lib.topo_le_default_params(C.byref(p), 8, 4, 4)
    h = C.c_void_p()
    assert lib.topo_le_create(C.byref(h), C.byref(p)) == 2
    assert b"no CPU fallback" in lib.topo_last_error()
    from topopt_in_petsc_transient_gb300 import LinearElasticity, TopoError
    with pytest.raises(TopoError):
        LinearElasticity(8, 4, 4)


@pytest.mark.parametrize("h", [(1.0, 1.0, 1.0), (0.5, 1.5, 2.0), (2.0, 2.0, 2.0)])
def test_mode_basis_element_matrices_equal_gauss_quadrature(lib, h):
    KE = np.zeros((24, 24))
    ME = np.zeros((24, 24))
    lib.topo_box_element_matrices(h[0], h[1], h[2], 0.3, KE.ctypes.data, ME.ctypes.data)
    K2, M2 = O.hex8_ke_me(*h)
    assert np.abs(KE - K2).max() <= 2e-15 * np.abs(K2).max()
    assert np.abs(ME - M2).max() <= 2e-15 * np.abs(M2).max()


def test_default_params_match_reference_defaults(lib):
    p = _lib.LEParams()
    lib.topo_le_default_params(C.byref(p), 64, 32, 32)
    # TopOpt.cc:75-159 defaults for the cantilever
    assert (p.nx, p.ny, p.nz) == (65, 33, 33)
    assert p.nu == 0.3 and p.nlvls == 4 and p.ncp == 2 and p.tsc == 25 and p.t1 == 50.0
    assert p.dalpha == 1e-4 and p.dbeta == 1e-4 and p.ti == 1 and p.sInt == 1 and p.mInt == 0


def test_petsc_binary_vector_records(lib, tmp_path):
    # VecView / VecLoad binary format: big-endian int32 class id 1211214 and
    # length, then big-endian doubles; records appended in one file
    from topopt_in_petsc_transient_gb300 import TopoError, read_petsc_vecs, write_petsc_vecs
    rng = np.random.default_rng(2)
    a, b = rng.standard_normal(7), rng.standard_normal(3)
    p = str(tmp_path / "Restart00.dat")
    write_petsc_vecs(p, [a, b])
    raw = open(p, "rb").read()
    assert len(raw) == 2 * 8 + 8 * (7 + 3)
    assert raw[:8] == (1211214).to_bytes(4, "big") + (7).to_bytes(4, "big")
    assert np.array_equal(np.frombuffer(raw[8:64], dtype=">f8"), a)
    assert raw[64:72] == (1211214).to_bytes(4, "big") + (3).to_bytes(4, "big")
    assert np.array_equal(np.frombuffer(raw[72:], dtype=">f8"), b)
    a2, b2 = np.zeros(7), np.zeros(3)
    read_petsc_vecs(p, [a2, b2])
    assert np.array_equal(a2, a) and np.array_equal(b2, b)
    b3 = np.zeros(3)
    read_petsc_vecs(p, [b3], first=1)
    assert np.array_equal(b3, b)
    with pytest.raises(TopoError):
        read_petsc_vecs(p, [np.zeros(5)])  # length mismatch is an error, not a silent read
    with pytest.raises(TopoError):
        read_petsc_vecs(p, [np.zeros(3)], first=2)  # no third record
