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


def test_mpiio_result_file_layout(lib, tmp_path):
    # MPIIO layout read back the way bin2vtu.py reads it: banner, header,
    # names, float32 DMDA coordinates, hex8 cells in DMDAGetElements_3D order,
    # then datasets of uint64 itr + field-major float32 point and cell fields
    from mpiio_reader import point_fields_of, read_result_file

    from topopt_in_petsc_transient_gb300 import MPIIO, TopoError
    nelx, nely, nelz = 3, 2, 4
    nx, ny, nz = nelx + 1, nely + 1, nelz + 1
    nn, nel = nx * ny * nz, nelx * nely * nelz
    xc = (-1.0, 2.0, 0.0, 0.7, 5.0, 6.3)
    rng = np.random.default_rng(7)
    p = str(tmp_path / "outputPhysics0_00000.dat")
    io = MPIIO((nelx, nely, nelz), 3, "ux, uy, uz", 1, "xPhys", p, xc=xc)
    U = [rng.standard_normal(3 * nn) for _ in range(3)]
    xp = rng.random(nel)
    for t in range(3):
        io.WriteVTK(U[t], xp, 10 * t)
    with pytest.raises(TopoError):
        io.WriteVTK(U[0], U[1], U[2], xp, xp, xp, 9)  # 9 point fields on a 3-field file
    io.Flush()
    r = read_result_file(p)
    assert r["banner"] == "TopOpt result version 1.1\n"
    assert (r["nPointsT"], r["nCellsT"], r["nPFields"], r["nCFields"], r["nodesPerElement"]) == (nn, nel, 3, 1, 8)
    assert r["pointFieldNames"] == ["ux", "uy", "uz"] and r["cellFieldNames"] == ["xPhys"]
    # DMDASetUniformCoordinates: xmin + i (xmax - xmin) / (n - 1), natural node order
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ref = np.stack([xc[0] + i * ((xc[1] - xc[0]) / (nx - 1)), xc[2] + j * ((xc[3] - xc[2]) / (ny - 1)),
                    xc[4] + k * ((xc[5] - xc[4]) / (nz - 1))], axis=-1).reshape(-1, 3).astype(np.float32)
    assert np.array_equal(r["points"], ref)
    # hex8 cells: n0, n0+x, n0+x+y, n0+y, then the same four one node layer up
    ek, ej, ei = np.meshgrid(np.arange(nelz), np.arange(nely), np.arange(nelx), indexing="ij")
    n0 = (ei + nx * (ej + ny * ek)).reshape(-1)
    quad = np.stack([n0, n0 + 1, n0 + 1 + nx, n0 + nx], axis=1)
    assert np.array_equal(r["cells"], np.concatenate([quad, quad + nx * ny], axis=1).astype(np.uint64))
    assert np.array_equal(r["offsets"], 8 * np.arange(1, nel + 1, dtype=np.uint64))
    assert np.all(r["types"] == 12)
    assert [d[0] for d in r["datasets"]] == [0, 10, 20]
    for t, (_, pf, cf) in enumerate(r["datasets"]):
        assert np.array_equal(pf, point_fields_of(U[t]))
        assert np.array_equal(cf[0], xp.astype(np.float32))
    del io

    # design file (main.cc:42): no point fields, x / xTilde / xPhys per iteration
    p = str(tmp_path / "outputDesign_00000.dat")
    io = MPIIO((nelx, nely, nelz), 0, "", 3, "x, xTilde, xPhys", p)
    X = [rng.random(nel) for _ in range(3)]
    io.WriteVTK(X[0], X[1], X[2], 1)
    with pytest.raises(TopoError):
        io.WriteVTK(U[0], xp, 2)  # displacement on a design-only file
    io.WriteVTK(X[2], X[0], X[1], 2)
    del io
    r = read_result_file(p)
    assert r["nPFields"] == 0 and r["pointFieldNames"] == [""]
    assert r["cellFieldNames"] == ["x", "xTilde", "xPhys"]
    assert np.array_equal(r["points"][-1], np.array([nelx, nely, nelz], dtype=np.float32))  # default box
    assert [d[0] for d in r["datasets"]] == [1, 2]
    assert np.array_equal(r["datasets"][0][2], np.stack(X).astype(np.float32))
    assert np.array_equal(r["datasets"][1][2], np.stack([X[2], X[0], X[1]]).astype(np.float32))

    # all-fields overload (U, DU, DDU, x, xTilde, xPhys), then the design-only
    # overload, which repeats the previous point fields (zeros before any)
    p = str(tmp_path / "outputAll_00000.dat")
    io = MPIIO((nelx, nely, nelz), 9, "ux, uy, uz, vx, vy, vz, ax, ay, az", 3, "x, xTilde, xPhys", p, slots=2)
    io.WriteVTK(X[0], X[1], X[2], 0)
    io.WriteVTK(U[0], U[1], U[2], X[0], X[1], X[2], 1)
    io.WriteVTK(X[1], X[2], X[0], 2)
    io.WriteVTK(X[2], X[1], X[0], 3)
    io.Flush()
    r = read_result_file(p)
    assert len(r["pointFieldNames"]) == 9 and r["pointFieldNames"][3] == "vx"
    pf = [d[1] for d in r["datasets"]]
    assert np.array_equal(pf[0], np.zeros((9, nn), np.float32))
    assert np.array_equal(pf[1], point_fields_of(*U))
    assert np.array_equal(pf[2], pf[1]) and np.array_equal(pf[3], pf[1])
    assert np.array_equal(r["datasets"][2][2], np.stack([X[1], X[2], X[0]]).astype(np.float32))


def test_mpiio_rejects_bad_arguments(lib, tmp_path):
    # argument errors are statuses (TopoError), never partial files or crashes
    import ctypes as C

    from topopt_in_petsc_transient_gb300 import MPIIO, TopoError
    with pytest.raises(TopoError):
        MPIIO((0, 2, 2), 3, "ux, uy, uz", 1, "xPhys", str(tmp_path / "a.dat"))  # no elements along x
    with pytest.raises(TopoError):
        MPIIO((2, 2, 2), 3, "ux, uy, uz", 1, "xPhys", str(tmp_path / "missing" / "a.dat"))  # no such folder
    with pytest.raises(TopoError):
        MPIIO((2, 2, 2), 3, "ux, uy, uz", 1, "xPhys", str(tmp_path / "a.dat"), slots=1)  # a ring needs two
    io = MPIIO((2, 2, 2), 3, "ux, uy, uz", 1, "xPhys", str(tmp_path / "a.dat"))
    with pytest.raises(TypeError):
        io.WriteVTK(np.zeros(81), 0)  # no overload takes one array
    with pytest.raises(ValueError):
        io.WriteVTK(np.zeros(80), np.zeros(8), 0)  # 27 nodes x 3 values required
    with pytest.raises(TypeError):
        io.WriteVTK(np.zeros(81, dtype=np.float32), np.zeros(8), 0)  # float64 only
    box = (C.c_double * 6)(0, 1, 0, 1, 0, 1)
    h = C.c_void_p()
    assert lib.topo_mpiio_create(C.byref(h), 3, 3, 3, box, -1, b"", 0, b"", str(tmp_path / "b.dat").encode(), 0) != 0
    assert lib.topo_mpiio_create(C.byref(h), 3, 3, 3, None, 0, b"", 0, b"", str(tmp_path / "b.dat").encode(), 0) != 0
    assert lib.topo_mpiio_flush(None) != 0
    lib.topo_mpiio_destroy(None)  # a null writer is ignored
    io.Flush()
    del io
