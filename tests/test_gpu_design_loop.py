"""GPU parity beyond the small meshes: the full design iteration of the
48x24x24 cantilever (100 Newmark steps, 4 multigrid levels, PDE filter r = 2,
MMA) against the oracle, the multigrid V-cycle inside the mixed path, the
physics restart files and the torch.autograd binding of the forward/adjoint
pair.

Tolerances: plain FP64 path at rtol 1e-12 (1e-13 over the 100-step
horizon): objective 1e-10 relative,
sensitivities 1e-9 of max|dfdx|; mixed path at the default rtol 1e-10 with FP32
sensitivity element math: objective 1e-6 relative, sensitivities 1e-5 of
max|dfdx|.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

MAT = dict(Emin=1e-9, Emax=1.0, Rmin=1e-3, Rmax=1.0)
M6 = (1e-9, 1.0, 1e-3, 1.0, 3.0, 1.0)
N48 = (48, 24, 24)


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def _cantilever_case(loadsignal):
    # loadsignal 1: sin(2 pi t) for t < 0.5 over 100 steps of dt = 0.01;
    # loadsignal 0: the reference's pulse (LinearElasticity.cc:597-606, centred at t = 8) over 100 steps of dt = 0.16
    t1 = 1.0 if loadsignal == 1 else 16.0
    return dict(ncp=1, tsc=100, t1=t1, objective=3, loadsignal=loadsignal, dalpha=0.0, dbeta=1e-3)


_ORACLE = {}


def _oracle_design_iteration(loadsignal, x):
    """The oracle's main.cc iteration on the 48x24x24 cantilever: filter,
    physics, volume constraint, filter chain rule, objective scaling, MMA."""
    if loadsignal in _ORACLE:
        return _ORACLE[loadsignal]
    n = int(np.prod(N48))
    xt, xp = O.filter_project(*N48, x, 2.0, False, 0.1, 0.15, rtol=1e-14)
    le = O.LinearElasticity(*N48, rtol=1e-13, **_cantilever_case(loadsignal), **MAT)
    rc, fx, df = le.objective_sensitivities(xp)
    assert rc == 0
    gx, dg = O.volume_constraint(xp, 0.12)
    dff, dgf = O.filter_gradients(*N48, xt, df, dg, 2.0, False, 0.1, 0.15, rtol=1e-14)
    dff = dff / fx  # fscale = 1 / fx of the first iteration (main.cc:113-121)
    mma = O.MMA(n, 1, x)
    mma.SetAsymptotes(0.1, 0.6, 1.05)
    lo, hi = O.MMA.SetOuterMovelimit(0.0, 1.0, 0.2, x)
    xn = x.copy()
    mma.Update(xn, dff, np.array([gx]), dgf, lo, hi)
    _ORACLE[loadsignal] = dict(xp=xp, fx=fx, df=df, gx=gx, dff=dff, xn=xn)
    return _ORACLE[loadsignal]


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("loadsignal", [1, 0])
def test_cantilever_48x24x24_design_iteration_matches_oracle(gpu, loadsignal, mixed):
    from topopt_in_petsc_transient_gb300 import MMA, Filter, LinearElasticity, VecScale
    n = int(np.prod(N48))
    rng = np.random.default_rng(0x7A11)
    x = 0.12 + rng.uniform(-0.02, 0.02, n)
    ref = _oracle_design_iteration(loadsignal, x)
    dev = dict(dtype=torch.float64, device="cuda")
    xd = torch.tensor(x, **dev)
    xt, xp = torch.zeros_like(xd), torch.zeros_like(xd)
    F = Filter(*N48, 2, 2.0, rtol=1e-14)
    F.FilterProject(xd, xt, xp, False, 0.1, 0.15)
    assert _rel(xp.cpu().numpy(), ref["xp"]) < 1e-10
    rtol = 1e-10 if mixed else 1e-13
    le = LinearElasticity(*N48, nlvls=4, mixed=mixed, rtol=rtol, **_cantilever_case(loadsignal))
    le.CompleteInitialState(xp, *M6)
    le.GenerateCheckPoints()
    df = torch.zeros_like(xd)
    fx = le.ComputeObjectiveSensitivities(df)
    tol_f, tol_d = (1e-6, 1e-5) if mixed else (1e-10, 1e-9)
    assert abs(fx - ref["fx"]) <= tol_f * abs(ref["fx"]), (fx, ref["fx"])
    assert _rel(df.cpu().numpy(), ref["df"]) < tol_d
    dg = torch.zeros_like(xd)
    gx = le.VolumeConstraint(dg, xp, 0.12)
    assert abs(gx - ref["gx"]) < 1e-11
    F.Gradients(xd, xt, df, 1, dg, False, 0.1, 0.15)
    VecScale(df, 1.0 / fx)
    assert _rel(df.cpu().numpy(), ref["dff"]) < tol_d
    mma = MMA(n, 1)
    mma.SetAsymptotes(0.1, 0.6, 1.05)
    lo, hi = torch.zeros_like(xd), torch.zeros_like(xd)
    mma.SetOuterMovelimit(0.0, 1.0, 0.2, xd, lo, hi)
    mma.Update(xd, df, [gx], dg, lo, hi)
    # the design update follows the sensitivities continuously
    dx_ref = ref["xn"] - x
    assert np.abs(xd.cpu().numpy() - ref["xn"]).max() <= (1e-3 if mixed else 1e-7) * np.abs(dx_ref).max()


def test_mixed_multigrid_in_the_reference_regime(gpu):
    # the reference's default material (Emax 1e3, Rmax 4.1667e-4) and pulse
    # with dt = 0.4: the Newmark operator is stiffness-dominated, the solver
    # picks the multigrid V-cycle, and the mixed path runs its FP32 V-cycle
    # (Chebyshev-Jacobi smoothing, dense coarsest inverse) inside FCG.  Its
    # FP64-accurate residuals are double-float products, good to about 2^-48
    # of the summed element terms; with this operator's cancellation that
    # floors the reachable tolerance between 1e-11 and 1e-12 (the plain path
    # reaches 1e-12), so the tight case runs at rtol 1e-11
    from topopt_in_petsc_transient_gb300 import LinearElasticity
    n = (16, 8, 8)
    kw = dict(ncp=4, tsc=10, t1=16.0, objective=3, loadsignal=0, dalpha=1e-4, dbeta=1e-4)
    mat = (1e-6, 1e3, 4.1667e-7, 4.1667e-4, 3.0, 1.0)
    rng = np.random.default_rng(12)
    x = 0.3 + 0.2 * rng.random(np.prod(n))
    ref = O.LinearElasticity(*n, Emin=mat[0], Emax=mat[1], Rmin=mat[2], Rmax=mat[3], **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert rc == 0
    for rtol, sens32, tf, td in ((1e-11, False, 1e-10, 1e-9), (1e-10, True, 1e-6, 1e-5)):
        le = LinearElasticity(*n, nlvls=3, mixed=True, rtol=rtol, sens_fp32=sens32, **kw)
        xd = torch.tensor(x, dtype=torch.float64, device="cuda")
        df = torch.zeros_like(xd)
        le.CompleteInitialState(xd, *mat)
        le.GenerateCheckPoints()
        fx = le.ComputeObjectiveSensitivities(df)
        st = le.stats()
        assert st["step_precond"] == 0 and st["mg_solves"] >= 4 * 10 * 2
        assert abs(fx - fx_r) <= tf * abs(fx_r), (rtol, fx, fx_r)
        assert _rel(df.cpu().numpy(), df_r) < td


def test_physics_restart_files(gpu, tmp_path):
    # LinearElasticity::WriteRestartFiles (RestartSol0x.dat: DDU0, LT, DDL0,
    # LinearElasticity.cc:2457-2496) against the oracle's vectors, the two
    # alternating file names, and -onlyLoadDesign -solutionAsU0
    # (LoadSolutionAsU0, :2621-2677): a displacement file becomes the initial
    # state, and the objective and sensitivities follow the oracle's with U0
    from topopt_in_petsc_transient_gb300 import LinearElasticity, read_petsc_vecs, write_petsc_vecs
    n = (16, 8, 8)
    kw = dict(ncp=2, tsc=5, t1=0.1, objective=5, loadsignal=1, dalpha=1e-3, dbeta=1e-3)
    rng = np.random.default_rng(23)
    x = 0.2 + 0.3 * rng.random(np.prod(n))
    le = LinearElasticity(*n, nlvls=3, mixed=False, rtol=1e-13, **kw)
    le.CompleteInitialState(x, *M6)
    le.GenerateCheckPoints()
    le.ComputeObjectiveSensitivities(np.zeros(x.size))
    ref = O.LinearElasticity(*n, rtol=1e-14, **kw)
    assert ref.objective_sensitivities(x)[0] == 0
    p0 = le.WriteRestartFiles(str(tmp_path))
    p1 = le.WriteRestartFiles(str(tmp_path))
    assert p0.endswith("RestartSol00.dat") and p1.endswith("RestartSol01.dat")
    got = [np.zeros(le.ndof) for _ in range(3)]
    read_petsc_vecs(p1, got)
    mine = le.restart_state()
    for a, b, r in zip(got, mine, ref.restart_state()):
        assert np.array_equal(a, b)
        assert _rel(a, r) < 1e-10
    assert np.abs(got[1]).max() > 0.0 and np.abs(got[2]).max() > 0.0
    # initial displacement from a vector file (the first record)
    N, _, _ = ref.vectors()
    u0 = N * 1e-3 * np.sin(np.arange(le.ndof) * 0.37)
    path = str(tmp_path / "u0.dat")
    write_petsc_vecs(path, [u0, np.zeros(le.ndof)])
    le2 = LinearElasticity(*n, nlvls=3, mixed=False, rtol=1e-13, **kw)
    assert np.array_equal(le2.LoadSolutionAsU0(path), u0)
    le2.CompleteInitialState(x, *M6)
    le2.GenerateCheckPoints()
    df = np.zeros(x.size)
    fx = le2.ComputeObjectiveSensitivities(df)
    assert np.array_equal(le2.checkpoint(0)[0], u0)
    ref2 = O.LinearElasticity(*n, rtol=1e-14, **kw)
    ref2.set_u0(u0)
    rc, fx_r, df_r = ref2.objective_sensitivities(x)
    assert rc == 0
    assert abs(fx - fx_r) <= 1e-10 * abs(fx_r)
    assert _rel(df, df_r) < 1e-9
    assert _rel(le2.restart_state()[0], ref2.restart_state()[0]) < 1e-10
    # the warm-start read checks its mesh and hands the vectors back
    assert all(np.array_equal(a, b) for a, b in zip(le.LoadRestartSol(p1), mine))


@pytest.mark.parametrize("mixed", [False, True])
def test_autograd_binding_matches_finite_differences(gpu, mixed):
    # the forward/adjoint pair behind torch.autograd.Function: gradients
    # through a composed loss equal the chain rule of the adjoint
    # sensitivities, which equal central differences (h = 1e-4) of the
    # forward objective and the oracle's sensitivities
    from autograd_binding import objective

    from topopt_in_petsc_transient_gb300 import LinearElasticity
    n = (12, 6, 6)
    kw = dict(ncp=2, tsc=6, t1=0.12, objective=3, loadsignal=1, dalpha=0.0, dbeta=1e-3)
    rng = np.random.default_rng(31)
    x = 0.12 + 0.02 * (2 * rng.random(np.prod(n)) - 1)
    le = LinearElasticity(*n, nlvls=2, mixed=mixed, rtol=1e-13, sens_fp32=False, **kw)
    xd = torch.tensor(x, dtype=torch.float64, device="cuda", requires_grad=True)
    f = objective(xd, le, M6)
    loss = 3.0 * f * f + f  # d loss / dx = (6 f + 1) df/dx
    loss.backward()
    g = xd.grad.cpu().numpy()
    fv = float(f.detach())
    ref = O.LinearElasticity(*n, **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert abs(fv - fx_r) <= 1e-10 * abs(fx_r)
    assert _rel(g, (6 * fv + 1) * df_r) < 1e-9
    h = 1e-4
    for e in rng.choice(x.size, 6, replace=False):
        xp, xm = x.copy(), x.copy()
        xp[e] += h
        xm[e] -= h
        with torch.no_grad():
            fp = float(objective(torch.tensor(xp, device="cuda"), le, M6))
            fm = float(objective(torch.tensor(xm, device="cuda"), le, M6))
        fd = (fp - fm) / (2 * h)
        assert abs((6 * fv + 1) * fd - g[e]) <= 1e-6 * np.abs(g).max(), (e, fd, g[e])


def test_sommg_object_construct_basis(gpu):
    # the SOMMG object of a reduced LinearElasticity: ConstructBasis with a
    # new expansion frequency rebuilds QQ, Kr, Mr, Cr, Pr on the current
    # design (SOMMG.cc:40-265) and the reduced sweeps that follow use them
    from topopt_in_petsc_transient_gb300 import SOMMG, LinearElasticity
    n = (8, 4, 4)
    kw = dict(ncp=2, tsc=6, t1=0.24, objective=3, loadsignal=1, dalpha=1e-3, dbeta=1e-3)
    rng = np.random.default_rng(8)
    x = 0.3 + 0.1 * (2 * rng.random(np.prod(n)) - 1)
    # both frequencies below the first eigenfrequency of this beam (about
    # 0.019), where P0 = K - om^2 M is positive definite
    le = LinearElasticity(*n, nlvls=2, mixed=False, rtol=1e-13, reduction=True, basis=4, omega0=0.01, **kw)
    le.CompleteInitialState(x, *M6)
    red = SOMMG(le, 4)
    Q1 = red.QQ
    red.ConstructBasis(0.005)
    Q, Kr, Mr, Cr, Pr = red._members()
    assert np.abs(Q - Q1).max() > 1e-6  # the basis depends on om
    df = np.zeros(x.size)
    fx = le.ComputeObjectiveSensitivities(df)
    ref = O.LinearElasticity(*n, rtol=1e-13, **kw)
    rc, fx_r, df_r, Q_r, Kr_r, Mr_r = ref.reduced_objective_sensitivities(x, 4, 0.005)
    assert rc == 0
    assert _rel(Q, Q_r) < 1e-8 and _rel(Kr, Kr_r) < 1e-8 and _rel(Mr, Mr_r) < 1e-8
    assert np.allclose(Cr, 1e-3 * Mr + 1e-3 * Kr, rtol=1e-14, atol=0.0)
    assert abs(fx - fx_r) <= 1e-8 * abs(fx_r)
    assert _rel(df, df_r) < 1e-7
    with pytest.raises(Exception):
        SOMMG(le, 3)  # order must equal the object's basis
