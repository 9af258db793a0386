"""ctypes binding of the C oracle (test infrastructure only; see topo_oracle.h)."""
import ctypes as C
import numpy as np

from . import build as _build

_lib = None


class Params(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("hx", C.c_double), ("hy", C.c_double), ("hz", C.c_double),
        ("nu", C.c_double),
        ("ncp", C.c_int), ("tsc", C.c_int),
        ("t1", C.c_double),
        ("ti", C.c_int), ("objective", C.c_int), ("sInt", C.c_int), ("mInt", C.c_int),
        ("boundaries", C.c_int), ("loadloc", C.c_int), ("optregion", C.c_int), ("loadsignal", C.c_int),
        ("Emin", C.c_double), ("Emax", C.c_double), ("Rmin", C.c_double), ("Rmax", C.c_double),
        ("penalK", C.c_double), ("penalM", C.c_double), ("dalpha", C.c_double), ("dbeta", C.c_double),
        ("rtol", C.c_double), ("maxit", C.c_int),
        ("load2_node", C.c_int), ("load2_phase", C.c_double), ("out_dof", C.c_int),
    ]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        L.oracle_le_create.restype = C.c_void_p
        L.oracle_le_create.argtypes = [C.POINTER(Params)]
        L.oracle_le_destroy.argtypes = [C.c_void_p]
        for f in ("oracle_le_complete_initial_state",):
            getattr(L, f).argtypes = [C.c_void_p, dp]
        L.oracle_le_generate_checkpoints.argtypes = [C.c_void_p]
        L.oracle_le_compute_objective_sensitivities.argtypes = [C.c_void_p, dp, dp, dp]
        L.oracle_le_sizes.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.oracle_le_set_u0.argtypes = [C.c_void_p, dp]
        L.oracle_le_get_vectors.argtypes = [C.c_void_p, dp, dp, dp]
        L.oracle_le_get_newmark.argtypes = [C.c_void_p, dp, dp]
        L.oracle_le_get_initial_state.argtypes = [C.c_void_p, dp, dp, dp]
        L.oracle_le_get_last_block.argtypes = [C.c_void_p, C.c_int, dp, dp, dp]
        L.oracle_le_get_adjoint0.argtypes = [C.c_void_p, dp, dp]
        L.oracle_le_get_restart_state.argtypes = [C.c_void_p, dp, dp, dp]
        L.oracle_le_total_cg_iterations.argtypes = [C.c_void_p]
        L.oracle_le_total_cg_iterations.restype = C.c_long
        L.oracle_le_apply_KM.argtypes = [C.c_void_p, dp, dp, dp]
        L.oracle_le_reduced_objective_sensitivities.argtypes = [C.c_void_p, dp, C.c_int, C.c_double, dp, dp, dp, dp,
                                                                dp]
        L.oracle_load_signal.argtypes = [C.c_int, C.c_double]
        L.oracle_load_signal.restype = C.c_double
        L.oracle_hex8_ke_me.argtypes = [C.c_double] * 4 + [dp, dp]
        L.oracle_le_volume_constraint.argtypes = [C.c_int, dp, C.c_double, dp, dp]
        L.oracle_pde_filter.argtypes = [C.c_int] * 3 + [C.c_double] * 4 + [dp, dp, C.c_double]
        L.oracle_pde_filter_matrix.argtypes = [C.c_double] * 4 + [dp]
        L.oracle_filter_project.argtypes = ([C.c_int] * 3 + [C.c_double] * 4 + [dp, dp, dp, C.c_int, C.c_double,
                                            C.c_double, C.c_double])
        L.oracle_filter_gradients.argtypes = ([C.c_int] * 3 + [C.c_double] * 4 + [dp, dp, C.c_int, dp, C.c_int,
                                              C.c_double, C.c_double, C.c_double])
        L.oracle_dens_filter_apply.argtypes = [C.c_int] * 3 + [C.c_double] * 4 + [dp, dp]
        L.oracle_dens_filter_project.argtypes = ([C.c_int] * 3 + [C.c_double] * 3 + [C.c_int, C.c_double] +
                                                 [dp, dp, dp, C.c_int, C.c_double, C.c_double])
        L.oracle_dens_filter_gradients.argtypes = ([C.c_int] * 3 + [C.c_double] * 3 + [C.c_int, C.c_double] +
                                                   [dp, dp, dp, C.c_int, dp, C.c_int, C.c_double, C.c_double])
        L.oracle_filter_mnd.argtypes = [C.c_int, dp]
        L.oracle_filter_mnd.restype = C.c_double
        L.oracle_increase_beta.argtypes = [dp, C.c_double, C.c_double, C.c_int, C.c_double]
        L.oracle_mma_create.restype = C.c_void_p
        L.oracle_mma_create.argtypes = [C.c_int, C.c_int, dp, dp, dp, dp]
        L.oracle_mma_destroy.argtypes = [C.c_void_p]
        L.oracle_mma_set_asymptotes.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
        L.oracle_mma_set_outer_movelimit.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, dp, dp, dp]
        L.oracle_mma_update.argtypes = [C.c_void_p, dp, dp, dp, dp, dp, dp]
        L.oracle_mma_design_change.argtypes = [C.c_int, dp, dp]
        L.oracle_mma_design_change.restype = C.c_double
        L.oracle_mma_kkt_residual.argtypes = [C.c_void_p, dp, dp, dp, dp, dp, dp, dp, dp]
        L.oracle_mma_get_state.argtypes = [C.c_void_p, dp, dp, dp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def hex8_ke_me(hx=1.0, hy=1.0, hz=1.0, nu=0.3):
    KE = np.zeros((24, 24)); ME = np.zeros((24, 24))
    lib().oracle_hex8_ke_me(hx, hy, hz, nu, _p(KE), _p(ME))
    return KE, ME


def load_signal(which, t):
    return lib().oracle_load_signal(int(which), float(t))


DEFAULTS = dict(hx=1.0, hy=1.0, hz=1.0, nu=0.3, ncp=1, tsc=10, t1=0.1, ti=1, objective=3, sInt=1, mInt=0,
                boundaries=1, loadloc=1, optregion=2, loadsignal=0, Emin=1e-9, Emax=1.0, Rmin=1e-3, Rmax=1.0,
                penalK=3.0, penalM=1.0, dalpha=0.0, dbeta=1e-3, rtol=1e-13, maxit=100000, load2_node=-1,
                load2_phase=0.0, out_dof=-1)


class LinearElasticity:
    """Oracle mirror of the reference LinearElasticity class (LinearElasticity.h:23-240)."""

    def __init__(self, nelx, nely, nelz, **kw):
        d = dict(DEFAULTS)
        d.update(kw)
        self.params = d
        p = Params(nx=nelx + 1, ny=nely + 1, nz=nelz + 1, **d)
        self._p = p
        self._h = lib().oracle_le_create(C.byref(p))
        nd, ne, ts = C.c_int(), C.c_int(), C.c_int()
        lib().oracle_le_sizes(self._h, C.byref(nd), C.byref(ne), C.byref(ts))
        self.ndof, self.nel, self.Ts = nd.value, ne.value, ts.value
        self.nelx, self.nely, self.nelz = nelx, nely, nelz

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_le_destroy(self._h)
            self._h = None

    def CompleteInitialState(self, xPhys):
        x = _f64(xPhys)
        return lib().oracle_le_complete_initial_state(self._h, _p(x))

    def GenerateCheckPoints(self):
        return lib().oracle_le_generate_checkpoints(self._h)

    def ComputeObjectiveSensitivities(self, xPhys):
        x = _f64(xPhys)
        fx = np.zeros(1)
        df = np.zeros(self.nel)
        rc = lib().oracle_le_compute_objective_sensitivities(self._h, _p(x), _p(fx), _p(df))
        return rc, float(fx[0]), df

    def objective_sensitivities(self, xPhys):
        """CompleteInitialState + GenerateCheckPoints + ComputeObjectiveSensitivities (main.cc:82-90)."""
        rc = self.CompleteInitialState(xPhys)
        rc |= self.GenerateCheckPoints()
        rc2, fx, df = self.ComputeObjectiveSensitivities(xPhys)
        return rc | rc2, fx, df

    def reduced_objective_sensitivities(self, xPhys, basis, omega0):
        """SOMMG reduced path (SOMMG.cc:40-265 + the reduction branches of
        LinearElasticity.cc): returns rc, fx, dfdx, Q (basis x ndof), Kr, Mr."""
        x = _f64(xPhys)
        fx = np.zeros(1)
        df = np.zeros(self.nel)
        Q = np.zeros((basis, self.ndof))
        Kr = np.zeros((basis, basis))
        Mr = np.zeros((basis, basis))
        rc = lib().oracle_le_reduced_objective_sensitivities(self._h, _p(x), int(basis), float(omega0), _p(fx), _p(df),
                                                             _p(Q), _p(Kr), _p(Mr))
        return rc, float(fx[0]), df, Q, Kr, Mr

    def vectors(self):
        N = np.zeros(self.ndof); P = np.zeros(self.nel); R = np.zeros(self.ndof)
        lib().oracle_le_get_vectors(self._h, _p(N), _p(P), _p(R))
        return N, P, R

    def newmark(self):
        a = np.zeros(6); dt = np.zeros(1)
        lib().oracle_le_get_newmark(self._h, _p(a), _p(dt))
        return a, float(dt[0])

    def initial_state(self):
        U = np.zeros(self.ndof); DU = np.zeros(self.ndof); DDU = np.zeros(self.ndof)
        lib().oracle_le_get_initial_state(self._h, _p(U), _p(DU), _p(DDU))
        return U, DU, DDU

    def set_u0(self, U0):
        """LoadSolutionAsU0: initial displacement of the next CompleteInitialState (None: rest)."""
        lib().oracle_le_set_u0(self._h, None if U0 is None else _p(_f64(U0)))

    def last_block_state(self, j):
        U = np.zeros(self.ndof); DU = np.zeros(self.ndof); DDU = np.zeros(self.ndof)
        lib().oracle_le_get_last_block(self._h, int(j), _p(U), _p(DU), _p(DDU))
        return U, DU, DDU

    def adjoint0(self):
        L1 = np.zeros(self.ndof); DDL0 = np.zeros(self.ndof)
        lib().oracle_le_get_adjoint0(self._h, _p(L1), _p(DDL0))
        return L1, DDL0

    def restart_state(self):
        """(DDU0, LT, DDL0) of WriteRestartFiles (LinearElasticity.cc:2457-2496)."""
        out = [np.zeros(self.ndof) for _ in range(3)]
        lib().oracle_le_get_restart_state(self._h, *[_p(v) for v in out])
        return tuple(out)

    def apply_KM(self, x):
        x = _f64(x)
        K = np.zeros(self.ndof); M = np.zeros(self.ndof)
        lib().oracle_le_apply_KM(self._h, _p(x), _p(K), _p(M))
        return K, M

    def cg_iterations(self):
        return lib().oracle_le_total_cg_iterations(self._h)


def volume_constraint(xPhys, volfrac):
    x = _f64(xPhys)
    gx = np.zeros(1); dg = np.zeros(x.size)
    lib().oracle_le_volume_constraint(x.size, _p(x), volfrac, _p(gx), _p(dg))
    return float(gx[0]), dg


def pde_filter_matrix(hx, hy, hz, R):
    KF = np.zeros((8, 8))
    lib().oracle_pde_filter_matrix(hx, hy, hz, R, _p(KF))
    return KF


def pde_filter(nelx, nely, nelz, x, rmin, h=(1.0, 1.0, 1.0), rtol=1e-14):
    x = _f64(x)
    out = np.zeros_like(x)
    lib().oracle_pde_filter(nelx + 1, nely + 1, nelz + 1, h[0], h[1], h[2], rmin, _p(x), _p(out), rtol)
    return out


def filter_project(nelx, nely, nelz, x, rmin, projection, beta, eta, h=(1.0, 1.0, 1.0), rtol=1e-14):
    x = _f64(x)
    xt = np.zeros_like(x); xp = np.zeros_like(x)
    lib().oracle_filter_project(nelx + 1, nely + 1, nelz + 1, h[0], h[1], h[2], rmin, _p(x), _p(xt), _p(xp),
                                int(projection), beta, eta, rtol)
    return xt, xp


def filter_gradients(nelx, nely, nelz, xTilde, dfdx, dgdx, rmin, projection, beta, eta, h=(1.0, 1.0, 1.0),
                     rtol=1e-14):
    xt = _f64(xTilde)
    df = _f64(dfdx).copy()
    dg = _f64(dgdx).copy()
    m = dg.size // xt.size
    lib().oracle_filter_gradients(nelx + 1, nely + 1, nelz + 1, h[0], h[1], h[2], rmin, _p(xt), _p(df), m, _p(dg),
                                  int(projection), beta, eta, rtol)
    return df, dg


def dens_filter_apply(nelx, nely, nelz, v, R, h=(1.0, 1.0, 1.0)):
    """H v of the filterType 0/1 filter (Filter.cc:302-531)."""
    v = _f64(v)
    out = np.zeros_like(v)
    lib().oracle_dens_filter_apply(nelx, nely, nelz, h[0], h[1], h[2], R, _p(v), _p(out))
    return out


def dens_filter_project(nelx, nely, nelz, ftype, x, R, projection, beta, eta, h=(1.0, 1.0, 1.0)):
    """Filter::FilterProject for filterType 0/1 (Filter.cc:60-119)."""
    x = _f64(x)
    xt = np.zeros_like(x)
    xp = np.zeros_like(x)
    lib().oracle_dens_filter_project(nelx, nely, nelz, h[0], h[1], h[2], ftype, R, _p(x), _p(xt), _p(xp),
                                     int(projection), beta, eta)
    return xt, xp


def dens_filter_gradients(nelx, nely, nelz, ftype, x, xTilde, dfdx, dgdx, R, projection, beta, eta,
                          h=(1.0, 1.0, 1.0)):
    """Filter::Gradients for filterType 0/1 (Filter.cc:122-206)."""
    x = _f64(x)
    xt = _f64(xTilde)
    df = _f64(dfdx).copy()
    dg = _f64(dgdx).copy()
    m = dg.size // xt.size
    lib().oracle_dens_filter_gradients(nelx, nely, nelz, h[0], h[1], h[2], ftype, R, _p(x), _p(xt), _p(df), m,
                                       _p(dg), int(projection), beta, eta)
    return df, dg


def filter_mnd(x):
    x = _f64(x)
    return lib().oracle_filter_mnd(x.size, _p(x))


def increase_beta(beta, betaFinal, gx, itr, ch):
    b = np.array([beta], dtype=np.float64)
    ch_ = lib().oracle_increase_beta(_p(b), betaFinal, gx, itr, ch)
    return bool(ch_), float(b[0])


class MMA:
    """Oracle mirror of MMA (MMA.h:9-120), m constraints."""

    def __init__(self, n, m, x, a=None, c=None, d=None):
        a = _f64(np.zeros(m) if a is None else a)
        c = _f64(np.full(m, 1000.0) if c is None else c)
        d = _f64(np.zeros(m) if d is None else d)
        x = _f64(x)
        self.n, self.m = n, m
        self._h = lib().oracle_mma_create(n, m, _p(x), _p(a), _p(c), _p(d))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_mma_destroy(self._h)
            self._h = None

    def SetAsymptotes(self, init, dec, inc):
        lib().oracle_mma_set_asymptotes(self._h, init, dec, inc)

    @staticmethod
    def SetOuterMovelimit(Xmin, Xmax, movlim, x):
        x = _f64(x)
        xmin = np.zeros_like(x); xmax = np.zeros_like(x)
        lib().oracle_mma_set_outer_movelimit(x.size, Xmin, Xmax, movlim, _p(x), _p(xmin), _p(xmax))
        return xmin, xmax

    def Update(self, x, dfdx, gx, dgdx, xmin, xmax):
        """Updates x in place (MMA::Update, MMA.cc:487)."""
        assert x.dtype == np.float64 and x.flags.c_contiguous
        df = _f64(dfdx); g = _f64(np.atleast_1d(gx)); dg = _f64(dgdx); lo = _f64(xmin); hi = _f64(xmax)
        lib().oracle_mma_update(self._h, _p(x), _p(df), _p(g), _p(dg), _p(lo), _p(hi))

    @staticmethod
    def DesignChange(x, xold):
        x = _f64(x)
        assert xold.dtype == np.float64
        return lib().oracle_mma_design_change(x.size, _p(x), _p(xold))

    def KKTresidual(self, x, dfdx, fx, dgdx, xmin, xmax):
        n2 = np.zeros(1); ni = np.zeros(1)
        lib().oracle_mma_kkt_residual(self._h, _p(_f64(x)), _p(_f64(dfdx)), _p(_f64(np.atleast_1d(fx))),
                                      _p(_f64(dgdx)), _p(_f64(xmin)), _p(_f64(xmax)), _p(n2), _p(ni))
        return float(n2[0]), float(ni[0])

    def state(self):
        L = np.zeros(self.n); U = np.zeros(self.n); lam = np.zeros(self.m)
        lib().oracle_mma_get_state(self._h, _p(L), _p(U), _p(lam))
        return L, U, lam
