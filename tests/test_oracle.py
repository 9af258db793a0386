"""CPU checks of the oracle (the FP64 restatement used as checker).

Parity status of the oracle: unpinned against the reference binary (PETSc/MPI
absent); these tests pin it to known answers derived from the reference source
and to finite differences.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O

MAT = dict(Emin=1e-9, Emax=1.0, Rmin=1e-3, Rmax=1.0, penalK=3.0, penalM=1.0)


def test_element_matrices_known_answers():
    # Hex8IsoparametricKE/ME, LinearElasticity.cc:3089-3333
    for h in [(1.0, 1.0, 1.0), (0.5, 1.5, 2.0)]:
        KE, ME = O.hex8_ke_me(*h)
        V = h[0] * h[1] * h[2]
        assert np.abs(KE - KE.T).max() < 1e-15
        assert np.abs(ME - ME.T).max() < 1e-16
        # rigid-body modes are in the null space of KE
        X = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]]) * h
        modes = []
        for c in range(3):
            t = np.zeros(24)
            t[c::3] = 1.0
            modes.append(t)
        for (a, b) in [(0, 1), (1, 2), (0, 2)]:
            r = np.zeros(24)
            r[a::3] = -X[:, b]
            r[b::3] = X[:, a]
            modes.append(r)
        for m in modes:
            assert np.abs(KE @ m).max() < 1e-13 * np.abs(KE).max()
        assert np.linalg.matrix_rank(KE, tol=1e-10) == 18
        # consistent mass: total = 3 V (one per component), diagonal V/27
        assert abs(ME.sum() - 3 * V) < 1e-14
        assert np.allclose(np.diag(ME), V / 27.0)
    KE, _ = O.hex8_ke_me()
    assert len(np.unique(np.round(np.abs(KE), 12))) == 10


def test_newmark_constants():
    # SetUpTimeIntegration, LinearElasticity.cc:185-219 (values printed at :212-217)
    le = O.LinearElasticity(2, 2, 2, ncp=2, tsc=5, t1=1.0, ti=1)
    a, dt = le.newmark()
    assert dt == pytest.approx(0.1)
    np.testing.assert_allclose(a, [-1.0, 0.0, 2 / dt, 4 / dt, 1.0, 4 / dt ** 2], rtol=1e-15)
    le = O.LinearElasticity(2, 2, 2, ncp=2, tsc=5, t1=1.0, ti=0)
    a, dt = le.newmark()
    np.testing.assert_allclose(a, [0.0, 0.0, 1 / dt, 1 / dt, 0.0, 1 / dt ** 2], rtol=1e-15)


def _closed_form_kf(dx, dy, dz, RR):
    """The closed-form 8x8 PDE filter matrix written out in
    PDEFilt::PDEFilterMatrix (PDEFilter.cc:485-578), restated."""
    t3 = 1.0 / dx / dy
    t4 = 1 / dz
    t5 = RR * RR
    t7 = t5 * dx * dx
    t9 = t7 * dy * dy
    t10 = 3.0 * t9
    t12 = t7 * dz * dz
    t13 = 3.0 * t12
    t15 = t5 * dy * dy * dz * dz
    t16 = 3.0 * t15
    t18 = dx * dx * dy * dy * dz * dz
    t22 = t3 * t4 * (t10 + t13 + t16 + t18) / 27.0
    t23 = 6.0 * t15
    t27 = t3 * t4 * (t10 + t13 - t23 + t18) / 54.0
    t28 = 6.0 * t12
    t32 = t3 * t4 * (t10 - t28 - t23 + t18) / 108.0
    t36 = t3 * t4 * (t10 - t28 + t16 + t18) / 54.0
    t37 = 6.0 * t9
    t41 = t3 * t4 * (t37 - t13 - t16 - t18) / 54.0
    t45 = t3 * t4 * (t37 - t13 + t23 - t18) / 108.0
    t49 = t3 * t4 * (t37 + t28 + t23 - t18) / 216.0
    t53 = t3 * t4 * (t37 + t28 - t16 - t18) / 108.0
    rows = [[t22, t27, t32, t36, -t41, -t45, -t49, -t53], [t27, t22, t36, t32, -t45, -t41, -t53, -t49],
            [t32, t36, t22, t27, -t49, -t53, -t41, -t45], [t36, t32, t27, t22, -t53, -t49, -t45, -t41],
            [-t41, -t45, -t49, -t53, t22, t27, t32, t36], [-t45, -t41, -t53, -t49, t27, t22, t36, t32],
            [-t49, -t53, -t41, -t45, t32, t36, t22, t27], [-t53, -t49, -t45, -t41, t36, t32, t27, t22]]
    return np.array(rows)


@pytest.mark.parametrize("h", [(1.0, 1.0, 1.0), (0.7, 1.1, 1.9)])
def test_pde_filter_matrix_matches_reference_closed_form(h):
    R = 2.0 / 2.0 / math.sqrt(3.0)
    KF = O.pde_filter_matrix(h[0], h[1], h[2], R)
    np.testing.assert_allclose(KF, _closed_form_kf(h[0], h[1], h[2], R), rtol=1e-13, atol=1e-15)


def test_pde_filter_preserves_constants_and_is_symmetric():
    n = (6, 4, 4)
    x = np.full(96, 0.37)
    np.testing.assert_allclose(O.pde_filter(*n, x, 2.0), x, rtol=1e-12)
    rng = np.random.default_rng(0)
    a, b = rng.random(96), rng.random(96)
    assert abs(a @ O.pde_filter(*n, b, 2.0) - b @ O.pde_filter(*n, a, 2.0)) < 1e-12


def test_projection_and_chain_rule():
    n = (4, 2, 2)
    rng = np.random.default_rng(1)
    x = rng.random(16)
    xt, xp = O.filter_project(*n, x, 1.5, True, 1e-6, 0.3)
    assert np.abs(xp - xt).max() < 1e-5  # beta -> 0: the projection is the identity
    beta, eta, hh = 8.0, 0.3, 1e-6
    xt, xp = O.filter_project(*n, x, 1.5, True, beta, eta)
    df, dg = O.filter_gradients(*n, xt, np.ones(16), np.ones(16), 1.5, True, beta, eta)
    # the gradient chain equals the transpose (= the filter itself) of d xPhys / d x
    for e in (0, 7):
        xp_p = O.filter_project(*n, x + hh * np.eye(16)[e], 1.5, True, beta, eta)[1]
        xp_m = O.filter_project(*n, x - hh * np.eye(16)[e], 1.5, True, beta, eta)[1]
        assert abs((xp_p - xp_m).sum() / (2 * hh) - df[e]) < 1e-6 * max(1.0, abs(df[e]))


def test_mma_converges_on_separable_problem():
    # min sum (x_i - c_i)^2 s.t. mean(x) <= 0.4, 0 <= x <= 1
    n = 50
    rng = np.random.default_rng(2)
    c = rng.random(n)
    x = np.full(n, 0.5)
    mma = O.MMA(n, 1, x)
    mma.SetAsymptotes(0.1, 0.6, 1.05)
    xold = x.copy()
    for _ in range(60):
        df = 2 * (x - c)
        g = np.array([x.mean() - 0.4])
        dg = np.full(n, 1.0 / n)
        lo, hi = O.MMA.SetOuterMovelimit(0.0, 1.0, 0.2, x)
        mma.Update(x, df, g, dg, lo, hi)
        ch = O.MMA.DesignChange(x, xold)
    assert ch < 1e-4
    # KKT: x = clip(c - lam/(2n)), mean(x) = 0.4
    assert abs(x.mean() - 0.4) < 1e-4
    lam = 2 * n * np.median((c - x)[(x > 1e-3) & (x < 1 - 1e-3)])
    np.testing.assert_allclose(x, np.clip(c - lam / (2 * n), 0, 1), atol=2e-3)


@pytest.mark.parametrize("objective", range(8))
def test_adjoint_sensitivities_match_finite_differences(objective):
    # objective 7 (output-DOF displacement) and the second point load are the
    # extended workloads' additions; the second load rides along on objective 7
    kw = dict(ncp=2, tsc=4, t1=0.8, objective=objective, loadsignal=1, dalpha=0.01, dbeta=0.01,
              mInt=1 if objective == 4 else 0)
    if objective == 7:
        kw.update(load2_node=7, load2_phase=0.7)
    le = O.LinearElasticity(4, 2, 2, **kw)
    rng = np.random.default_rng(objective)
    x = 0.3 + 0.4 * rng.random(le.nel)
    rc, fx, df = le.objective_sensitivities(x)
    assert rc == 0 and np.isfinite(fx)
    h = 1e-5
    for e in (0, 6, 13):
        xp, xm = x.copy(), x.copy()
        xp[e] += h
        xm[e] -= h
        fd = (le.objective_sensitivities(xp)[1] - le.objective_sensitivities(xm)[1]) / (2 * h)
        assert abs(fd - df[e]) <= 5e-7 * np.abs(df).max(), (objective, e, fd, df[e])


@pytest.mark.parametrize("region,objective", [(0, 0), (1, 3), (3, 5)])
def test_region_weighted_sensitivities_match_finite_differences(region, objective):
    # SetUpOptimizationRegion (LinearElasticity.cc:222-335): the objective sums
    # over the region's elements only; region 0 with the boundaries 0 supports
    # and the load of loadloc 0 on its top edge, region 1 on hz = 0.75 elements
    # (centres inside the mid-height slab)
    kw = dict(ncp=2, tsc=4, t1=0.8, objective=objective, loadsignal=1, dalpha=0.01, dbeta=0.01, optregion=region)
    if region == 0:
        kw.update(boundaries=0, loadloc=0, loadsignal=0, t1=8.0)
    if region == 1:
        kw.update(hz=0.75)
    le = O.LinearElasticity(4, 2, 2, **kw)
    rng = np.random.default_rng(20 + region)
    x = 0.3 + 0.4 * rng.random(le.nel)
    rc, fx, df = le.objective_sensitivities(x)
    assert rc == 0 and fx > 0.0
    full = O.LinearElasticity(4, 2, 2, **dict(kw, optregion=2)).objective_sensitivities(x)[1]
    assert fx < full  # a strict part of the domain
    h = 1e-5
    for e in (0, 5, 10, 15):
        xp, xm = x.copy(), x.copy()
        xp[e] += h
        xm[e] -= h
        fd = (le.objective_sensitivities(xp)[1] - le.objective_sensitivities(xm)[1]) / (2 * h)
        assert abs(fd - df[e]) <= 5e-7 * np.abs(df).max(), (region, e, fd, df[e])


@pytest.mark.parametrize("objective", [0, 3, 5])
def test_initial_displacement_sensitivities_match_finite_differences(objective):
    # LoadSolutionAsU0 (-solutionAsU0, LinearElasticity.cc:2621-2677): the
    # transient starts from a loaded displacement instead of rest; u0 enters
    # the initial acceleration (K u0, LinearElasticity.cc:1049-1066) and the
    # t = 0 sensitivities through dK u0
    kw = dict(ncp=2, tsc=4, t1=0.8, objective=objective, loadsignal=1, dalpha=0.01, dbeta=0.01)
    le = O.LinearElasticity(4, 2, 2, **kw)
    rng = np.random.default_rng(30 + objective)
    x = 0.3 + 0.4 * rng.random(le.nel)
    N, _, _ = le.vectors()
    u0 = N * 1e-2 * np.sin(np.arange(le.ndof) * 0.37)  # zero on clamped DOFs
    rest = le.objective_sensitivities(x)[1]
    le.set_u0(u0)
    rc, fx, df = le.objective_sensitivities(x)
    assert rc == 0 and np.isfinite(fx) and abs(fx - rest) > 1e-3 * abs(rest)
    U0, DU0, DDU0 = le.initial_state()
    assert np.array_equal(U0, u0) and not np.any(DU0)
    h = 1e-5
    for e in (0, 6, 13):
        xp, xm = x.copy(), x.copy()
        xp[e] += h
        xm[e] -= h
        fd = (le.objective_sensitivities(xp)[1] - le.objective_sensitivities(xm)[1]) / (2 * h)
        assert abs(fd - df[e]) <= 5e-7 * np.abs(df).max(), (objective, e, fd, df[e])
    le.set_u0(None)  # back to rest (the solves start warm: equal to their tolerance)
    assert abs(le.objective_sensitivities(x)[1] - rest) <= 1e-10 * abs(rest)


def test_reference_pulse_objective_fd():
    # reference load signal (Gaussian-modulated cosines, LinearElasticity.cc:597-606), t in [0, 16]
    kw = dict(ncp=4, tsc=10, t1=16.0, objective=0, loadsignal=0, Emax=1e3, Rmax=4.1667e-4, Rmin=4.1667e-7,
              Emin=1e-6, dalpha=1e-4, dbeta=1e-4)
    le = O.LinearElasticity(4, 2, 2, **kw)
    x = np.full(le.nel, 0.3)
    x[3] = 0.5
    rc, fx, df = le.objective_sensitivities(x)
    h = 1e-5
    xp, xm = x.copy(), x.copy()
    xp[5] += h
    xm[5] -= h
    fd = (le.objective_sensitivities(xp)[1] - le.objective_sensitivities(xm)[1]) / (2 * h)
    assert abs(fd - df[5]) <= 1e-6 * np.abs(df).max()


def test_checkpoint_blocking_does_not_change_results():
    # GenerateCheckPoints + reverse block recomputation (LinearElasticity.cc:1208-1280, 1625-1908)
    rng = np.random.default_rng(5)
    x = 0.2 + 0.5 * rng.random(16)
    res = []
    for ncp, tsc in [(1, 12), (2, 6), (3, 4), (12, 1)]:
        le = O.LinearElasticity(4, 2, 2, ncp=ncp, tsc=tsc, t1=1.2, objective=5, loadsignal=1)
        res.append(le.objective_sensitivities(x)[1:])
    for fx, df in res[1:]:
        assert abs(fx - res[0][0]) < 1e-12 * abs(res[0][0])
        np.testing.assert_allclose(df, res[0][1], rtol=1e-9, atol=1e-12 * np.abs(res[0][1]).max())


def test_load_location_and_dirichlet_mask():
    le = O.LinearElasticity(4, 2, 2, boundaries=1, loadloc=1)
    N, P, R = le.vectors()
    nx, ny, nz = 5, 3, 3
    node = lambda i, j, k: i + nx * (j + ny * k)
    for j in range(ny):
        for k in range(nz):
            assert all(N[3 * node(0, j, k) + c] == 0 for c in range(3))
    assert N.sum() == 3 * (nx * ny * nz - ny * nz)
    # cantilever line load: z-DOF at x = xmax, z = zmax/2, ends halved (LinearElasticity.cc:650-662)
    zl = [R[3 * node(4, j, 1) + 2] for j in range(ny)]
    assert zl == [0.5, 1.0, 0.5] and R.sum() == 2.0
    assert P.sum() == 16


def test_golden_fixtures_reproduce():
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz")
    g = np.load(path)
    x = g["x"]
    for obj in range(7):
        le = O.LinearElasticity(4, 2, 2, ncp=2, tsc=3, t1=0.6, objective=obj, loadsignal=1, dalpha=0.01,
                                dbeta=0.01)
        rc, fx, df = le.objective_sensitivities(x)
        assert abs(fx - g["fx%d" % obj]) <= 1e-12 * abs(g["fx%d" % obj])
        np.testing.assert_allclose(df, g["df%d" % obj], rtol=1e-10, atol=1e-13 * np.abs(g["df%d" % obj]).max())
    KE, ME = O.hex8_ke_me()
    np.testing.assert_allclose(KE, g["KE"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(O.pde_filter(4, 2, 2, x, 2.0), g["xfilt"], rtol=1e-11)


def test_sommg_basis_and_reduced_matrices():
    # SOMMG.cc:40-252: orthonormal basis from P0 = K - om^2 M solves, reduced
    # matrices Kr = Q'KQ, Mr = Q'MQ symmetric; Kr matches Q'(K Q) formed here
    n = (8, 4, 4)
    kw = dict(ncp=1, tsc=6, t1=0.12, objective=3, loadsignal=1, dalpha=1e-3, dbeta=1e-3, rtol=1e-13)
    rng = np.random.default_rng(3)
    x = 0.3 + 0.1 * (2 * rng.random(np.prod(n)) - 1)
    le = O.LinearElasticity(*n, **kw)
    rc, fx, df, Q, Kr, Mr = le.reduced_objective_sensitivities(x, 4, 0.01)
    assert rc == 0 and np.isfinite(fx) and np.all(np.isfinite(df))
    assert np.abs(Q @ Q.T - np.eye(4)).max() < 1e-12
    assert np.abs(Kr - Kr.T).max() < 1e-12 * np.abs(Kr).max()
    assert np.abs(Mr - Mr.T).max() < 1e-12 * np.abs(Mr).max()
    N, P, R = le.vectors()
    assert np.abs(Q[:, N == 0.0]).max() == 0.0  # the basis vanishes on clamped DOFs
    KQ = np.stack([le.apply_KM(q)[0] for q in Q])
    assert np.abs(Q @ KQ.T - Kr).max() < 1e-12 * np.abs(Kr).max()


def test_density_and_sensitivity_filter_restatement():
    # Filter.cc:302-531: stencil ElemConn = max_a(ceil(R/h_a) - 1) >= 1, identity
    # when ElemConn == 1, weights R - dist between element centres
    n = (6, 5, 4)
    nel = int(np.prod(n))
    rng = np.random.default_rng(12)
    x = 0.2 + 0.6 * rng.random(nel)
    assert np.array_equal(O.dens_filter_apply(*n, x, 2.0), x)  # R = 2 on unit elements: identity
    H = np.stack([O.dens_filter_apply(*n, np.eye(nel)[k], 3.0) for k in range(nel)], 1)
    assert np.abs(H - H.T).max() == 0.0  # cubic elements: symmetric
    assert H[0, 0] == 3.0 and H[0, 1] == 2.0 and H[0, 2] == 1.0  # face neighbours at 1 and 2
    assert abs(H[0, 1 + 6] - (3.0 - np.sqrt(2.0))) < 1e-15  # edge neighbour
    hs = H.sum(1)
    xt, xp = O.dens_filter_project(*n, 1, x, 3.0, False, 1.0, 0.5)
    assert np.abs(xt - H @ x / hs).max() < 1e-14 and np.array_equal(xt, xp)
    xt0, _ = O.dens_filter_project(*n, 0, x, 3.0, False, 1.0, 0.5)
    assert np.array_equal(xt0, x)
    df = rng.standard_normal(nel)
    dg = rng.standard_normal(nel)
    d1, g1 = O.dens_filter_gradients(*n, 1, x, xt, df, dg, 3.0, False, 1.0, 0.5)
    assert np.abs(d1 - H @ (df / hs)).max() < 1e-13 and np.abs(g1 - H @ (dg / hs)).max() < 1e-13
    d0, g0 = O.dens_filter_gradients(*n, 0, x, x, df, dg, 3.0, False, 1.0, 0.5)
    assert np.abs(d0 - (H @ (df * x)) / hs / x).max() < 1e-12 and np.array_equal(g0, dg)
    # anisotropic elements: ElemConn from the smallest size, per-axis upper limits
    Ha = np.stack([O.dens_filter_apply(*n, np.eye(nel)[k], 2.5, h=(1.0, 2.0, 1.0)) for k in range(nel)], 1)
    assert Ha[0, 0] == 2.5 and Ha[0, 6] == 0.5 and Ha[6, 0] == 0.5


def test_increase_beta_host_logic_matches_oracle():
    # Filter::IncreaseBeta (Filter.cc:273-300): the host mirror and the oracle
    # on every branch (change by +1 below 7, by 20% above, capped at betaFinal
    # with the change revoked, blocked by gx > 0 or by ch >= 0.01 off the
    # every-10th iteration)
    from topopt_in_petsc_transient_gb300.topopt import Filter
    for beta in (0.1, 1.0, 6.5, 7.0, 20.0, 47.0, 48.0):
        for gx in (-0.1, 0.0, 1e-9):
            for itr in (9, 10, 11):
                for ch in (0.005, 0.01, 0.2):
                    got = Filter.IncreaseBeta(beta, 48.0, gx, itr, ch)
                    ref = O.increase_beta(beta, 48.0, gx, itr, ch)
                    assert got == ref, (beta, gx, itr, ch, got, ref)


def test_volume_constraint_and_load_signals():
    # VolumeConstraint (LinearElasticity.cc:1283-1296) and the two load
    # signals: the reference pulse (LinearElasticity.cc:597-606) peaks at
    # t = 8 with value 1, the workload's sin(2 pi t) stops at t = 0.5
    x = np.linspace(0.0, 1.0, 11)
    gx, dg = O.volume_constraint(x, 0.3)
    assert abs(gx - (x.mean() - 0.3)) < 1e-15 and np.all(dg == 1.0 / x.size)
    assert O.load_signal(0, 8.0) == 1.0
    assert abs(O.load_signal(0, 8.0 + 1e-3)) < 1.0
    assert abs(O.load_signal(1, 0.25) - 1.0) < 1e-15 and abs(O.load_signal(1, 0.125) - 0.5 ** 0.5) < 1e-15
    assert O.load_signal(1, 0.0) == 0.0 and O.load_signal(1, 0.75) == 0.0
