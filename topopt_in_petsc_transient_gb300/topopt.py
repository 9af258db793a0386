"""Host-side mirror of the reference classes on the transient hot path.

Same class names, method names, argument meaning and call order as
TopOpt_in_PETSc_Transient's C++ (LinearElasticity.h, PDEFilter.h, Filter.h,
MMA.h, TopOpt.h); a non-zero status raises TopoError instead of returning a
PetscErrorCode.  Arrays are either host numpy float64 arrays (VecGetArray
semantics: DMDA natural order) or CUDA float64 torch tensors (device
pointers, no copies).  All arithmetic happens in libtopopt_gb300.so.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import LEParams, LEStats, TopoError, check


def _is_dev(a):
    return hasattr(a, "is_cuda") and a.is_cuda


def _addr(a, n=None, name="array"):
    """(is_device, address) of a float64 contiguous buffer."""
    if _is_dev(a):
        import torch
        if a.dtype != torch.float64 or not a.is_contiguous():
            raise TypeError("%s must be a contiguous float64 CUDA tensor" % name)
        if n is not None and a.numel() < n:
            raise ValueError("%s has %d values, %d required" % (name, a.numel(), n))
        return True, a.data_ptr()
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("%s must be a C-contiguous float64 numpy array or CUDA tensor" % name)
    if n is not None and a.size < n:
        raise ValueError("%s has %d values, %d required" % (name, a.size, n))
    return False, a.ctypes.data


def write_petsc_vecs(path, vectors, append=False):
    """The vectors as consecutive PETSc binary records (VecView with a binary
    viewer; big-endian class id 1211214, length, values), host arrays or CUDA
    tensors."""
    import os
    lib = _lib.load()
    for k, v in enumerate(vectors):
        n = v.numel() if _is_dev(v) else np.asarray(v).size
        dev, a = _addr(v, n, "vector %d" % k)
        check(lib.topo_petsc_vec_write(os.fsencode(path), int(append or k > 0), a, n, int(dev)), "PETSc vector write")


def read_petsc_vecs(path, outs, first=0):
    """Records first, first + 1, ... of a PETSc binary file into outs (VecLoad);
    each record must hold as many values as its output."""
    import os
    lib = _lib.load()
    for k, v in enumerate(outs):
        n = v.numel() if _is_dev(v) else np.asarray(v).size
        dev, a = _addr(v, n, "vector %d" % k)
        check(lib.topo_petsc_vec_read(os.fsencode(path), first + k, a, n, int(dev)), "PETSc vector read")


def VecScale(v, alpha):
    """PETSc's VecScale as main.cc uses it on dfdx (main.cc:121, :127):
    v <- alpha v in place, for a CUDA float64 tensor (one library kernel) or a
    host float64 array."""
    if _is_dev(v):
        _, a = _addr(v, None, "vector")
        check(_lib.load().topo_vec_scale_dev(a, v.numel(), float(alpha)), "VecScale")
    else:
        np.multiply(v, alpha, out=v)
    return 0


class LinearElasticity:
    """LinearElasticity (LinearElasticity.h:23-240) on the GPU.

    Constructor arguments follow LinearElasticity::LinearElasticity
    (LinearElasticity.h:29) with the DMDA replaced by its node counts and
    element size; `mixed`, `rtol`, `maxit`, `smooth`, `cheb_ratio`,
    `use_graphs` control the GB300 solver.
    """

    def __init__(self, nelx, nely, nelz, nu=0.3, nlvls=4, ncp=2, tsc=25, t1=50.0, ti=1, objective=0,
                 stiffnessInterpolation=1, massInterpolation=0, t0=0.0, boundaries=1, loadloc=1, reduction=False,
                 basis=5, dalpha=1e-4, dbeta=1e-4, omega0=1.0, optimizationRegion=2, V0=None, h=(1.0, 1.0, 1.0),
                 loadsignal=0, mixed=True, rtol=1e-10, maxit=500, smooth=3, cheb_ratio=30.0, use_graphs=True,
                 coarse_dense_max=None, coarse_smooth=None, sens_fp32=None, inner_tol=None, inner_maxit=None,
                 adaptive_kappa=None, extrapolate=None, mass_precond=None, mass_precond_share=None,
                 mass_precond_smooth=None, load2_node=-1, load2_phase=0.0, out_dof=-1):
        L = _lib.load()
        p = LEParams()
        L.topo_le_default_params(C.byref(p), nelx, nely, nelz)
        p.hx, p.hy, p.hz = h
        p.nu = nu
        p.nlvls, p.ncp, p.tsc, p.t1, p.ti = nlvls, ncp, tsc, t1, ti
        p.objective, p.sInt, p.mInt = objective, stiffnessInterpolation, massInterpolation
        p.boundaries, p.loadloc, p.optregion, p.loadsignal = boundaries, loadloc, optimizationRegion, loadsignal
        p.dalpha, p.dbeta = dalpha, dbeta
        p.reduction, p.basis, p.omega0 = int(bool(reduction)), int(basis), float(omega0)
        p.load2_node, p.load2_phase, p.out_dof = int(load2_node), float(load2_phase), int(out_dof)
        p.mixed, p.rtol, p.maxit, p.smooth = int(bool(mixed)), rtol, maxit, smooth
        p.cheb_ratio, p.use_graphs = cheb_ratio, int(bool(use_graphs))
        if coarse_dense_max is not None:
            p.coarse_dense_max = coarse_dense_max
        if coarse_smooth is not None:
            p.coarse_smooth = coarse_smooth
        if sens_fp32 is not None:
            p.sens_fp32 = int(bool(sens_fp32))
        if inner_tol is not None:
            p.inner_tol = inner_tol
        if inner_maxit is not None:
            p.inner_maxit = inner_maxit
        if adaptive_kappa is not None:
            p.adaptive_kappa = adaptive_kappa
        if extrapolate is not None:
            p.extrapolate = int(extrapolate)
        if mass_precond is not None:
            p.mass_precond = int(mass_precond)
        if mass_precond_share is not None:
            p.mass_precond_share = mass_precond_share
        if mass_precond_smooth is not None:
            p.mass_precond_smooth = mass_precond_smooth
        self.params = p
        self.nelx, self.nely, self.nelz = nelx, nely, nelz
        self.nel = nelx * nely * nelz
        self.nn = (nelx + 1) * (nely + 1) * (nelz + 1)
        self.ndof = 3 * self.nn
        self.Ts = ncp * tsc + 1
        self.dt = t1 / (self.Ts - 1)
        h_ = C.c_void_p()
        check(L.topo_le_create(C.byref(h_), C.byref(p)), "LinearElasticity")
        self._h = h_

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().topo_le_destroy(h)
            self._h = None

    def _attach(self, write, output):
        """Attach `output` (an MPIIO writer) for one call when `write` is set."""
        io = output._h if (write and output is not None) else None
        check(_lib.load().topo_le_set_output(self._h, io), "physics output")
        return io is not None

    def _detach(self, attached):
        if attached:
            _lib.load().topo_le_set_output(self._h, None)

    def CompleteInitialState(self, xPhys, Emin, Emax, Rmin, Rmax, penalK, penalM, dalpha=None, dbeta=None,
                             write=False, output=None):
        """LinearElasticity::CompleteInitialState (LinearElasticity.cc:956-1206).
        With write and an MPIIO output the initial displacement is written as
        dataset 0 with xPhys (LinearElasticity.cc:1087-1114)."""
        L = _lib.load()
        dev, a = _addr(xPhys, self.nel, "xPhys")
        f = L.topo_le_complete_initial_state_dev if dev else L.topo_le_complete_initial_state
        att = self._attach(write, output)
        try:
            check(f(self._h, a, Emin, Emax, Rmin, Rmax, penalK, penalM), "CompleteInitialState")
        finally:
            self._detach(att)
        return 0

    def GenerateCheckPoints(self, write=False, xPhys=None, output=None):
        """LinearElasticity::GenerateCheckPoints (LinearElasticity.cc:1208-1280).
        With write and an MPIIO output (and ncp > 1) every time step
        tsc*c + j + 1 is written with the xPhys of CompleteInitialState."""
        att = self._attach(write, output)
        try:
            check(_lib.load().topo_le_generate_checkpoints(self._h), "GenerateCheckPoints")
        finally:
            self._detach(att)
        return 0

    def ComputeObjectiveSensitivities(self, dfdx, *args, write=False, output=None):
        """LinearElasticity::ComputeObjectiveSensitivities (LinearElasticity.cc:1625-1908).

        Overwrites dfdx and returns fx (the reference writes *fx).  The
        reference's (xPhys, Emin, Emax, Rmin, Rmax, penalK, penalM, dalpha,
        dbeta, write, output) may follow dfdx; the material data are those of
        CompleteInitialState.  With write and an MPIIO output and ncp == 1,
        every time step is written (LinearElasticity.cc:1736-1742)."""
        if len(args) > 9:
            write = args[9]
        if len(args) > 10:
            output = args[10]
        L = _lib.load()
        dev, a = _addr(dfdx, self.nel, "dfdx")
        fx = C.c_double()
        f = L.topo_le_compute_objective_sensitivities_dev if dev else L.topo_le_compute_objective_sensitivities
        att = self._attach(write, output)
        try:
            check(f(self._h, C.byref(fx), a), "ComputeObjectiveSensitivities")
        finally:
            self._detach(att)
        return fx.value

    def VolumeConstraint(self, dgdx, xPhys, volfrac):
        """LinearElasticity::VolumeConstraint (LinearElasticity.cc:1283-1296); returns gx[0]."""
        L = _lib.load()
        dev1, a = _addr(dgdx, self.nel, "dgdx")
        dev2, b = _addr(xPhys, self.nel, "xPhys")
        if dev1 != dev2:
            raise TypeError("dgdx and xPhys must both be host or both be device arrays")
        gx = C.c_double()
        f = L.topo_le_volume_constraint_dev if dev1 else L.topo_le_volume_constraint
        check(f(self._h, C.byref(gx), a, b, volfrac), "VolumeConstraint")
        return gx.value

    def reduced_system(self):
        """SOMMG's QQ, Kr, Mr, Pr (SOMMG.h:21-22) of the current design, as numpy arrays."""
        L = _lib.load()
        kb, nd = self.params.basis, self.ndof
        Q = np.zeros((kb, nd))
        Kr = np.zeros((kb, kb))
        Mr = np.zeros((kb, kb))
        Pr = np.zeros(kb)
        check(L.topo_le_reduced_system(self._h, Q.ctypes.data, Kr.ctypes.data, Mr.ctypes.data, Pr.ctypes.data),
              "reduced_system")
        return Q, Kr, Mr, Pr

    # -- inspection --------------------------------------------------------
    def state(self, which, j):
        out = np.zeros(self.ndof)
        check(_lib.load().topo_le_get_state(self._h, which, j, out.ctypes.data), "get_state")
        return out

    def checkpoint(self, c):
        """Checkpoint c (U, DU, DDU: the state at the start of block c)."""
        U, DU, DDU = np.zeros(self.ndof), np.zeros(self.ndof), np.zeros(self.ndof)
        check(_lib.load().topo_le_get_checkpoint(self._h, int(c), U.ctypes.data, DU.ctypes.data, DDU.ctypes.data),
              "checkpoint")
        return U, DU, DDU

    def WriteCheckPoints(self, directory):
        """cp%04d.dat of every block in the reference's format (three PETSc
        binary records U, DU, DDU each, LinearElasticity.cc:1134-1136, :1260-1270),
        written from the HBM checkpoints."""
        import os
        for c in range(self.params.ncp):
            write_petsc_vecs(os.path.join(directory, "cp%04d.dat" % c), list(self.checkpoint(c)))
        return 0

    def restart_state(self):
        """(DDU0, LT, DDL0): the initial acceleration, the terminal adjoint of
        the last reverse sweep and the adjoint acceleration at t = 0."""
        out = [np.zeros(self.ndof) for _ in range(3)]
        check(_lib.load().topo_le_get_restart_state(self._h, *[a.ctypes.data for a in out]), "restart state")
        return tuple(out)

    def WriteRestartFiles(self, directory):
        """LinearElasticity::WriteRestartFiles (LinearElasticity.cc:2457-2496):
        DDU0, LT, DDL0 into RestartSol00.dat / RestartSol01.dat, the two sets
        alternating (flip starts true, LinearElasticity.cc:2685); returns the
        file written."""
        import os
        self._flip = not getattr(self, "_flip", True)
        path = os.path.join(directory, "RestartSol%s.dat" % ("01" if self._flip else "00"))
        write_petsc_vecs(path, list(self.restart_state()))
        return path

    def set_initial_displacement(self, U0):
        """Initial displacement for the next CompleteInitialState (None: rest)."""
        if U0 is None:
            check(_lib.load().topo_le_set_initial_displacement(self._h, None, 0), "initial displacement")
            return
        dev, a = _addr(U0, self.ndof, "U0")
        check(_lib.load().topo_le_set_initial_displacement(self._h, a, int(dev)), "initial displacement")

    def LoadSolutionAsU0(self, path):
        """LinearElasticity::LoadSolutionAsU0 with -onlyLoadDesign -solutionAsU0
        (LinearElasticity.cc:2621-2677): the first record of the PETSc vector
        file `path` (-restartFileVecSol) becomes the initial displacement."""
        U0 = np.zeros(self.ndof)
        read_petsc_vecs(path, [U0])
        self.set_initial_displacement(U0)
        return U0

    def LoadRestartSol(self, path):
        """The -restartFileVecSol read of SetUpSolver1/2
        (LinearElasticity.cc:2716-2738): DDU0, LT, DDL0 from a RestartSol file,
        checked against this mesh.  The reference uses them only as starting
        guesses of three Krylov solves; the GPU solves start from their own
        predictors, which gives the same solutions to the solve tolerance, so
        the vectors are returned, not installed."""
        out = [np.zeros(self.ndof) for _ in range(3)]
        read_petsc_vecs(path, out)
        return tuple(out)

    def apply_km(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        K = np.zeros(self.ndof)
        M = np.zeros(self.ndof)
        check(_lib.load().topo_le_apply_km(self._h, x.ctypes.data, K.ctypes.data, M.ctypes.data), "apply_km")
        return K, M

    def stats(self):
        s = LEStats()
        check(_lib.load().topo_le_get_stats(self._h, C.byref(s)), "get_stats")
        return {"cg_iterations": s.cg_iterations, "solves": s.solves, "device_bytes": s.device_bytes,
                "last_fx": s.last_fx, "graph_body_launches": s.graph_body_launches, "mg_solves": s.mg_solves,
                "step_precond": s.step_precond, "replacements": s.replacements}


class SOMMG:
    """SOMMG (SOMMG.h:14-34): the second-order moment-matching reduction of a
    LinearElasticity object created with reduction=True.  SOMMG(physics,
    order) stands for SOMMG(Vec x, order) (SOMMG.cc:11-24); order must equal
    the object's basis.  ConstructBasis(om) is SOMMG::ConstructBasis on the
    object's operators of its current design (SOMMG.cc:40-265); QQ (order x
    3 nn), Kr, Mr, Cr (order x order) and Pr (order) are its public members
    (SOMMG.h:21-22), read back as numpy arrays."""

    def __init__(self, physics, order):
        h_ = C.c_void_p()
        check(_lib.load().topo_sommg_create(C.byref(h_), physics._h, int(order)), "SOMMG")
        self._h = h_
        self.physics = physics
        self.order = int(order)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().topo_sommg_destroy(h)
            self._h = None

    def ConstructBasis(self, om):
        check(_lib.load().topo_sommg_construct_basis(self._h, float(om)), "ConstructBasis")
        return 0

    def _members(self):
        k = self.order
        Q = np.zeros((k, self.physics.ndof))
        Kr, Mr, Cr, Pr = np.zeros((k, k)), np.zeros((k, k)), np.zeros((k, k)), np.zeros(k)
        check(_lib.load().topo_sommg_get(self._h, Q.ctypes.data, Kr.ctypes.data, Mr.ctypes.data, Cr.ctypes.data,
                                         Pr.ctypes.data), "SOMMG members")
        return Q, Kr, Mr, Cr, Pr

    @property
    def QQ(self):
        return self._members()[0]

    @property
    def Kr(self):
        return self._members()[1]

    @property
    def Mr(self):
        return self._members()[2]

    @property
    def Cr(self):
        return self._members()[3]

    @property
    def Pr(self):
        return self._members()[4]


class MPIIO:
    """MPIIO (MPIIO.h:27-100): result files for bin2vtu.py.

    MPIIO(mesh, nPf, pnames, nCf, cnames, filename) follows
    MPIIO::MPIIO(da_nodes, nPf, pnames, nCf, cnames, filename)
    (MPIIO.cc:32-150) with the DMDA replaced by `mesh`: an object with
    nelx/nely/nelz (TopOpt, LinearElasticity) or a tuple (nelx, nely, nelz).
    `xc` = (xmin, xmax, ymin, ymax, zmin, zmax) of the node box (default:
    origin to the element counts times the mesh's element size h); `workdir`
    puts the file at ./workdir/filename like the reference's -workdir option
    (MPIIO.cc:430-443).  Datasets are converted on the device and appended
    by a writer thread; Flush() (or deleting the object) waits for the file.
    """

    def __init__(self, mesh, nPf, pnames, nCf, cnames, filename="output_00000.dat", xc=None, workdir=None,
                 slots=4):
        import os
        if isinstance(mesh, (tuple, list)):
            nelx, nely, nelz = (int(v) for v in mesh[:3])
            h = (1.0, 1.0, 1.0)
        else:
            nelx, nely, nelz = int(mesh.nelx), int(mesh.nely), int(mesh.nelz)
            h = getattr(mesh, "h", None)
            if h is None and hasattr(mesh, "params"):
                h = (mesh.params.hx, mesh.params.hy, mesh.params.hz)
            h = tuple(h) if h is not None else (1.0, 1.0, 1.0)
        if xc is None:
            xc = (0.0, nelx * h[0], 0.0, nely * h[1], 0.0, nelz * h[2])
        self.filename = os.path.join(".", workdir, filename) if workdir else filename
        self.nelx, self.nely, self.nelz = nelx, nely, nelz
        self.nel = nelx * nely * nelz
        self.nn = (nelx + 1) * (nely + 1) * (nelz + 1)
        self.nPf, self.nCf = int(nPf), int(nCf)
        lib = _lib.load()
        box = (C.c_double * 6)(*[float(v) for v in xc])
        h_ = C.c_void_p()
        check(lib.topo_mpiio_create(C.byref(h_), nelx + 1, nely + 1, nelz + 1, box, self.nPf, pnames.encode(),
                                    self.nCf, cnames.encode(), os.fsencode(self.filename), int(slots)), "MPIIO")
        self._h = h_

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().topo_mpiio_destroy(h)
            self._h = None

    def WriteVTK(self, *args):
        """MPIIO::WriteVTK (MPIIO.cc:152-406), the overload chosen by the
        argument count like the reference's C++ overloads:
          (U, xPhys, itr)                         3 point fields, 1 cell field
          (x, xTilde, xPhys, itr)                 the previous point fields, 3 cell fields
          (U, x, xTilde, xPhys, itr)              3 point fields, 3 cell fields
          (U, DU, DDU, x, xTilde, xPhys, itr)     9 point fields, 3 cell fields
        Nodal vectors hold 3*nn DOF-interleaved values, cell fields nel; all
        host numpy float64 or all CUDA float64 tensors (read on torch's
        current stream)."""
        split = {3: 1, 4: 0, 5: 1, 7: 3}
        if len(args) not in split:
            raise TypeError("WriteVTK takes (U, xPhys, itr), (x, xTilde, xPhys, itr), (U, x, xTilde, xPhys, itr) "
                            "or (U, DU, DDU, x, xTilde, xPhys, itr)")
        *arrays, itr = args
        k = split[len(args)]
        kinds = set()
        nodal, cells = [], []
        for i, a in enumerate(arrays):
            dev, p = _addr(a, 3 * self.nn if i < k else self.nel, "WriteVTK argument %d" % i)
            kinds.add(dev)
            (nodal if i < k else cells).append(p)
        if len(kinds) > 1:
            raise TypeError("WriteVTK arrays must all be host arrays or all CUDA tensors")
        dev = kinds.pop()
        stream = None
        if dev:
            import torch
            stream = torch.cuda.current_stream().cuda_stream
        P = C.c_void_p
        nv = (P * max(k, 1))(*nodal)
        cv = (P * max(len(cells), 1))(*cells)
        check(_lib.load().topo_mpiio_write(self._h, int(itr), nv, k, cv, len(cells), int(dev), stream), "WriteVTK")
        return 0

    def Flush(self):
        """Waits until every dataset written so far is in the file."""
        check(_lib.load().topo_mpiio_flush(self._h), "MPIIO flush")


class PDEFilt:
    """PDEFilt (PDEFilter.h:29-74): Helmholtz filter on the nodal grid."""

    def __init__(self, nelx, nely, nelz, rmin, h=(1.0, 1.0, 1.0), rtol=1e-10, maxit=5000):
        L = _lib.load()
        h_ = C.c_void_p()
        check(L.topo_pdefilt_create(C.byref(h_), nelx + 1, nely + 1, nelz + 1, h[0], h[1], h[2], rmin, rtol, maxit),
              "PDEFilt")
        self._h = h_
        self.nel = nelx * nely * nelz

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().topo_pdefilt_destroy(h)
            self._h = None

    def FilterProject(self, OX, FX):
        """PDEFilt::FilterProject (PDEFilter.cc:193-222)."""
        L = _lib.load()
        d1, a = _addr(OX, self.nel, "OX")
        d2, b = _addr(FX, self.nel, "FX")
        if d1 != d2:
            raise TypeError("OX and FX must both be host or both be device arrays")
        f = L.topo_pdefilt_filter_project_dev if d1 else L.topo_pdefilt_filter_project
        check(f(self._h, a, b), "PDEFilt::FilterProject")
        return 0

    def Gradients(self, OS, FS):
        """PDEFilt::Gradients (PDEFilter.cc:224): the same symmetric operator."""
        return self.FilterProject(OS, FS)


class Filter:
    """Filter (Filter.h:34-92) with the smoothed Heaviside projection:
    filterType 0 (sensitivity filter), 1 (density filter) and 2 (PDE filter)."""

    def __init__(self, nelx, nely, nelz, filterT, Rin, h=(1.0, 1.0, 1.0), rtol=1e-10, maxit=5000):
        if filterT not in (0, 1, 2):
            raise TopoError(1, "Filter", "filterType must be 0, 1 or 2")
        self.filterT = filterT
        self.dens = None
        self.pdef = None
        self.nel = nelx * nely * nelz
        if filterT == 2:
            self.pdef = PDEFilt(nelx, nely, nelz, Rin, h=h, rtol=rtol, maxit=maxit)
        else:
            hh = C.c_void_p()
            check(_lib.load().topo_densfilt_create(C.byref(hh), nelx, nely, nelz, h[0], h[1], h[2], filterT, Rin),
                  "Filter")
            self.dens = hh

    def __del__(self):
        h = getattr(self, "dens", None)
        if h is not None and h.value:
            _lib.load().topo_densfilt_destroy(h)
            self.dens = None

    def FilterProject(self, x, xTilde, xPhys, projectionFilter, beta, eta):
        """Filter::FilterProject (Filter.cc:60-119)."""
        L = _lib.load()
        d = [_addr(v, self.nel, n) for v, n in ((x, "x"), (xTilde, "xTilde"), (xPhys, "xPhys"))]
        if len({t[0] for t in d}) != 1:
            raise TypeError("x, xTilde, xPhys must all be host or all be device arrays")
        if self.dens is not None:
            f = L.topo_densfilt_filter_project_dev if d[0][0] else L.topo_densfilt_filter_project
            h = self.dens
        else:
            f = L.topo_filter_project_dev if d[0][0] else L.topo_filter_project
            h = self.pdef._h
        check(f(h, d[0][1], d[1][1], d[2][1], int(bool(projectionFilter)), beta, eta), "Filter::FilterProject")
        return 0

    def Gradients(self, x, xTilde, dfdx, m, dgdx, projectionFilter, beta, eta):
        """Filter::Gradients (Filter.cc:122-206); dfdx and dgdx (m x nel) in place."""
        L = _lib.load()
        d = [_addr(v, n_, nm) for v, n_, nm in ((x, self.nel, "x"), (xTilde, self.nel, "xTilde"),
                                                 (dfdx, self.nel, "dfdx"), (dgdx, self.nel * m, "dgdx"))]
        if len({t[0] for t in d}) != 1:
            raise TypeError("x, xTilde, dfdx, dgdx must all be host or all be device arrays")
        if self.dens is not None:
            f = L.topo_densfilt_gradients_dev if d[0][0] else L.topo_densfilt_gradients
            check(f(self.dens, d[0][1], d[1][1], d[2][1], m, d[3][1], int(bool(projectionFilter)), beta, eta),
                  "Filter::Gradients")
        else:
            f = L.topo_filter_gradients_dev if d[0][0] else L.topo_filter_gradients
            check(f(self.pdef._h, d[1][1], d[2][1], m, d[3][1], int(bool(projectionFilter)), beta, eta),
                  "Filter::Gradients")
        return 0

    def GetMND(self, x):
        """Filter::GetMND (Filter.cc:208-227)."""
        L = _lib.load()
        dev, a = _addr(x, self.nel, "x")
        out = C.c_double()
        if self.dens is not None:
            f = L.topo_densfilt_mnd_dev if dev else L.topo_densfilt_mnd
            check(f(self.dens, a, C.byref(out)), "Filter::GetMND")
        else:
            f = L.topo_filter_mnd_dev if dev else L.topo_filter_mnd
            check(f(self.pdef._h, a, C.byref(out)), "Filter::GetMND")
        return out.value

    @staticmethod
    def IncreaseBeta(beta, betaFinal, gx, itr, ch):
        """Filter::IncreaseBeta (Filter.cc:274-300): scalar continuation logic;
        returns (changeBeta, beta)."""
        change = False
        if (ch < 0.01 or itr % 10 == 0) and beta < betaFinal and gx <= 0.0:
            change = True
            beta = beta + 1 if beta < 7 else beta * 1.2
            if beta > betaFinal:
                beta = betaFinal
                change = False
        return change, beta


class MMA:
    """MMA (MMA.h:9-120) with design vectors on the device.  The four
    reference constructors: MMA(n, m, x[, a, c, d]) and the restart forms
    MMA(n, m, itr=..., xo1=..., xo2=..., U=..., L=...[, a, c, d]) (MMA.h:12-19)."""

    def __init__(self, n, m, x=None, a=None, c=None, d=None, itr=None, xo1=None, xo2=None, U=None, L=None):
        lib = _lib.load()
        a = np.zeros(m) if a is None else np.ascontiguousarray(a, dtype=np.float64)
        c = np.full(m, 1000.0) if c is None else np.ascontiguousarray(c, dtype=np.float64)
        d = np.zeros(m) if d is None else np.ascontiguousarray(d, dtype=np.float64)
        h_ = C.c_void_p()
        if itr is None:
            check(lib.topo_mma_create(C.byref(h_), n, m, a.ctypes.data, c.ctypes.data, d.ctypes.data), "MMA")
        else:
            v = [_addr(t, n, nm) for t, nm in ((xo1, "xo1"), (xo2, "xo2"), (U, "U"), (L, "L"))]
            if len({t[0] for t in v}) != 1:
                raise TypeError("xo1, xo2, U, L must all be host or all be device arrays")
            f = lib.topo_mma_create_restart_dev if v[0][0] else lib.topo_mma_create_restart
            check(f(C.byref(h_), n, m, int(itr), v[0][1], v[1][1], v[2][1], v[3][1], a.ctypes.data, c.ctypes.data,
                    d.ctypes.data), "MMA")
        self._h = h_
        self.n, self.m = n, m

    def Restart(self, xo1, xo2, U, L):
        """MMA::Restart (MMA.cc:307-350): fills xo1, xo2, U, L for a later restart."""
        v = [_addr(t, self.n, nm) for t, nm in ((xo1, "xo1"), (xo2, "xo2"), (U, "U"), (L, "L"))]
        if len({t[0] for t in v}) != 1:
            raise TypeError("xo1, xo2, U, L must all be host or all be device arrays")
        lib = _lib.load()
        f = lib.topo_mma_restart_dev if v[0][0] else lib.topo_mma_restart
        check(f(self._h, v[0][1], v[1][1], v[2][1], v[3][1]), "MMA::Restart")
        return 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().topo_mma_destroy(h)
            self._h = None

    def SetAsymptotes(self, init, decrease, increase):
        check(_lib.load().topo_mma_set_asymptotes(self._h, init, decrease, increase), "MMA::SetAsymptotes")
        return 0

    def SetOuterMovelimit(self, Xmin, Xmax, movlim, x, xmin, xmax):
        """MMA::SetOuterMovelimit (MMA.cc:374-393); device arrays."""
        d = [_addr(v, self.n, n) for v, n in ((x, "x"), (xmin, "xmin"), (xmax, "xmax"))]
        if len({t[0] for t in d}) != 1:
            raise TypeError("x, xmin, xmax must all be host or all be device arrays")
        L = _lib.load()
        f = L.topo_mma_set_outer_movelimit_dev if d[0][0] else L.topo_mma_set_outer_movelimit
        check(f(self._h, Xmin, Xmax, movlim, d[0][1], d[1][1], d[2][1]), "MMA::SetOuterMovelimit")
        return 0

    def Update(self, xval, dfdx, gx, dgdx, xmin, xmax):
        """MMA::Update (MMA.cc:487-507): xval updated in place."""
        L = _lib.load()
        g = np.ascontiguousarray(np.atleast_1d(np.asarray(gx, dtype=np.float64)))
        d = [_addr(v, n_, nm) for v, n_, nm in ((xval, self.n, "xval"), (dfdx, self.n, "dfdx"),
                                                 (dgdx, self.n * self.m, "dgdx"), (xmin, self.n, "xmin"),
                                                 (xmax, self.n, "xmax"))]
        if len({t[0] for t in d}) != 1:
            raise TypeError("MMA::Update arrays must all be host or all be device arrays")
        f = L.topo_mma_update_dev if d[0][0] else L.topo_mma_update
        check(f(self._h, d[0][1], d[1][1], g.ctypes.data, d[2][1], d[3][1], d[4][1]), "MMA::Update")
        return 0

    def DesignChange(self, x, xold):
        """MMA::DesignChange (MMA.cc:395-414): returns the inf-norm change, xold <- x."""
        d = [_addr(v, self.n, n) for v, n in ((x, "x"), (xold, "xold"))]
        if len({t[0] for t in d}) != 1:
            raise TypeError("x and xold must both be host or both be device arrays")
        L = _lib.load()
        f = L.topo_mma_design_change_dev if d[0][0] else L.topo_mma_design_change
        ch = C.c_double()
        check(f(self._h, d[0][1], d[1][1], C.byref(ch)), "MMA::DesignChange")
        return ch.value

    def KKTresidual(self, x, dfdx, fx, dgdx, xmin, xmax):
        """MMA::KKTresidual (MMA.cc:416-484); device arrays; returns (norm2, normInf)."""
        fxa = np.ascontiguousarray(np.atleast_1d(np.asarray(fx, dtype=np.float64)))
        d = [_addr(v, n_, nm) for v, n_, nm in ((x, self.n, "x"), (dfdx, self.n, "dfdx"),
                                                 (dgdx, self.n * self.m, "dgdx"), (xmin, self.n, "xmin"),
                                                 (xmax, self.n, "xmax"))]
        if not all(t[0] for t in d):
            raise TypeError("KKTresidual takes device arrays")
        n2, ni = C.c_double(), C.c_double()
        check(_lib.load().topo_mma_kkt_residual_dev(self._h, d[0][1], d[1][1], fxa.ctypes.data, d[2][1], d[3][1],
                                                     d[4][1], C.byref(n2), C.byref(ni)), "MMA::KKTresidual")
        return n2.value, ni.value
