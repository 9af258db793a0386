"""GPU parity: the sm_103a library, called through the C ABI, against the
FP64 oracle on the same seeded inputs.

Tolerances: plain FP64 path (FP64 preconditioner inside FP64 flexible CG,
solves to rtol 1e-12): objective 1e-10 relative, sensitivities 1e-9 of
max|dfdx|.  Mixed path (FP32 flexible-CG recurrence with an FP32 Kronecker or
multigrid preconditioner, convergence decided on FP64-accurate residuals):
the same bounds at the same solve tolerance; FP32 sensitivity element math
and the default tolerance rtol 1e-10 are tested at the looser bounds each
test states.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

MAT = dict(Emin=1e-9, Emax=1.0, Rmin=1e-3, Rmax=1.0, penalK=3.0, penalM=1.0)
M6 = (MAT["Emin"], MAT["Emax"], MAT["Rmin"], MAT["Rmax"], MAT["penalK"], MAT["penalM"])


def _le(n, **kw):
    from topopt_in_petsc_transient_gb300 import LinearElasticity
    return LinearElasticity(*n, **kw)


def _run_gpu(le, x):
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    df = torch.zeros_like(xd)
    le.CompleteInitialState(xd, *M6)
    le.GenerateCheckPoints()
    fx = le.ComputeObjectiveSensitivities(df)
    return fx, df.cpu().numpy()


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


@pytest.mark.parametrize("mixed", [False, True])
def test_operator_apply_matches_assembled_matrices(gpu, mixed):
    # mixed: the FP64-accurate passes run in double-float (FP32 pairs)
    n = (16, 8, 8)
    rng = np.random.default_rng(0)
    x = 0.1 + 0.8 * rng.random(np.prod(n))
    le = _le(n, nlvls=3, ncp=1, tsc=2, t1=0.02, mixed=mixed)
    le.CompleteInitialState(x, *M6)
    ref = O.LinearElasticity(*n, ncp=1, tsc=2, t1=0.02)
    ref.CompleteInitialState(x)
    v = rng.standard_normal(le.ndof)
    K, M = le.apply_km(v)
    K2, M2 = ref.apply_KM(v)
    tol = 1e-12 if mixed else 1e-13
    assert _rel(K, K2) < tol
    assert _rel(M, M2) < tol


@pytest.mark.parametrize("objective", range(7))
@pytest.mark.parametrize("mixed", [False, True])
def test_objective_and_sensitivities_match_oracle(gpu, objective, mixed):
    n = (8, 4, 4)
    kw = dict(ncp=2, tsc=5, t1=0.5, objective=objective, loadsignal=1, dalpha=0.01, dbeta=0.01,
              mInt=1 if objective == 4 else 0)
    rng = np.random.default_rng(10 + objective)
    x = 0.1 + 0.5 * rng.random(np.prod(n))
    le = _le(n, nlvls=2, mixed=mixed, rtol=1e-12, sens_fp32=False, **{k: v for k, v in kw.items() if k != "mInt"},
             massInterpolation=kw["mInt"])
    fx, df = _run_gpu(le, x)
    ref = O.LinearElasticity(*n, **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert rc == 0
    assert abs(fx - fx_r) <= 1e-10 * abs(fx_r), (fx, fx_r)
    assert _rel(df, df_r) < 1e-9


@pytest.mark.parametrize("region,objective,mixed", [(0, 0, False), (1, 3, True), (3, 5, False), (3, 1, True)])
def test_optimisation_regions_match_oracle(gpu, region, objective, mixed):
    # SetUpOptimizationRegion (LinearElasticity.cc:222-335) weights every
    # objective per element: 0 the top column at x = 0 (here under the load of
    # loadloc 0, with the boundaries 0 supports: roller face x = 0 and the
    # bottom edge at x = xmax), 1 the mid-height slab |z - zmax/2| < 0.5
    # (hz = 0.75 puts element centres inside it), 3 the box of half-width 2.5
    # around (0.75 xmax, ymax/2, zmax/2); region 2 (everything) is every other test
    n = (16, 8, 8)
    kw = dict(ncp=2, tsc=4, t1=0.4, objective=objective, loadsignal=1, dalpha=0.01, dbeta=0.01)
    h = (1.0, 1.0, 0.75 if region == 1 else 1.0)
    if region == 0:
        kw.update(t1=8.0, loadsignal=0, boundaries=0, loadloc=0)
    rng = np.random.default_rng(40 + region)
    x = 0.1 + 0.5 * rng.random(np.prod(n))
    le = _le(n, nlvls=2, mixed=mixed, rtol=1e-12, sens_fp32=False, optimizationRegion=region, h=h, **kw)
    fx, df = _run_gpu(le, x)
    ref = O.LinearElasticity(*n, optregion=region, hx=h[0], hy=h[1], hz=h[2], **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert rc == 0 and fx_r > 0.0
    assert abs(fx - fx_r) <= 1e-10 * abs(fx_r), (fx, fx_r)
    assert _rel(df, df_r) < 1e-9


@pytest.mark.parametrize("ncp,tsc,graphs", [(1, 12, True), (3, 4, True), (4, 3, False)])
def test_states_and_checkpointing(gpu, ncp, tsc, graphs):
    n = (16, 8, 8)
    rng = np.random.default_rng(3)
    x = 0.12 + 0.04 * rng.random(np.prod(n))
    kw = dict(ncp=ncp, tsc=tsc, t1=0.12, objective=3, loadsignal=1, dalpha=0.0, dbeta=1e-3)
    le = _le(n, nlvls=3, mixed=True, rtol=1e-12, use_graphs=graphs, sens_fp32=False, **kw)
    fx, df = _run_gpu(le, x)
    ref = O.LinearElasticity(*n, **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert abs(fx - fx_r) <= 1e-10 * abs(fx_r)
    assert _rel(df, df_r) < 1e-9
    # after the reverse sweep block 0 is resident: compare its last state
    U, DU, DDU = ref.last_block_state(tsc - 1)
    assert _rel(le.state(0, tsc - 1), U) < 1e-10
    assert _rel(le.state(1, tsc - 1), DU) < 1e-9
    assert _rel(le.state(2, tsc - 1), DDU) < 1e-8


@pytest.mark.parametrize("nlvls,coarse_smooth", [(1, 10), (2, 8), (3, 6)])
def test_mixed_default_fp32_sensitivities(gpu, nlvls, coarse_smooth):
    # the mixed-path default: FP32 element math in the sensitivity kernel
    # (state combinations formed in FP64); stated tolerance 1e-6 on the
    # objective and 1e-5 of max|dfdx| on the sensitivities.  The multigrid
    # preconditioner is forced (mass_precond 0: this mass-dominated operator
    # would otherwise take the Kronecker one) at full depth (adaptive_kappa 0)
    # with an iterative coarsest level, so the FP32 V-cycle of nlvls levels
    # and its coarse Chebyshev solve of degree coarse_smooth run
    n = (16, 8, 8)
    kw = dict(ncp=2, tsc=6, t1=0.06, objective=3, loadsignal=1, dalpha=0.0, dbeta=1e-3)
    rng = np.random.default_rng(21)
    x = 0.12 + 0.02 * (2 * rng.random(np.prod(n)) - 1)
    le = _le(n, nlvls=nlvls, coarse_smooth=coarse_smooth, mixed=True, rtol=1e-10, mass_precond=0,
             coarse_dense_max=0, adaptive_kappa=0.0, **kw)
    fx, df = _run_gpu(le, x)
    st = le.stats()
    assert st["step_precond"] == 0 and st["mg_solves"] == st["solves"]
    # convergence of a mixed solve is decided on an FP64-accurate replacement
    # residual: a few per solve at most
    assert 1 <= st["replacements"] <= 4 * st["solves"]
    ref = O.LinearElasticity(*n, **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert abs(fx - fx_r) <= 1e-6 * abs(fx_r)
    assert _rel(df, df_r) < 1e-5


@pytest.mark.parametrize("ncp,tsc,uniform", [(1, 200, True), (2, 100, True), (2, 100, False)])
def test_long_horizon_tracked_products(gpu, ncp, tsc, uniform):
    # 200 steps, the load pulse ending at step 100: the mixed forward sweep
    # forms its right-hand sides from tracked products A u, A du, A ddu
    # (re-formed at block starts and every 32 steps); smooth free vibration
    # lets the predictor reach the solve tolerance, so solves that stop at
    # their initial guess are exercised too.  Default tolerance rtol 1e-10:
    # objective within 1e-7 of the oracle, displacement and velocity of the
    # resident block within 1e-6 (the acceleration carries the alternating
    # high-frequency part of the solve error and is not compared).
    n = (16, 8, 8)
    kw = dict(ncp=ncp, tsc=tsc, t1=0.005 * ncp * tsc, objective=3, loadsignal=1, dalpha=0.0, dbeta=1e-3)
    rng = np.random.default_rng(5)
    x = np.full(np.prod(n), 0.12) if uniform else 0.1 + 0.2 * rng.random(np.prod(n))
    le = _le(n, nlvls=3, mixed=True, rtol=1e-10, sens_fp32=False, **kw)
    fx, df = _run_gpu(le, x)
    ref = O.LinearElasticity(*n, **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert abs(fx - fx_r) <= 1e-7 * abs(fx_r)
    assert _rel(df, df_r) < 1e-6
    U, DU, DDU = ref.last_block_state(tsc - 1)
    assert _rel(le.state(0, tsc - 1), U) < 1e-6
    assert _rel(le.state(1, tsc - 1), DU) < 1e-6


@pytest.mark.parametrize("objective,mixed", [(3, False), (3, True), (0, True), (4, False)])
def test_backward_euler_integrator(gpu, objective, mixed):
    # ti = 0: the reference's backward-Euler constants (LinearElasticity.cc:189-196)
    # through the same forward/adjoint kernels
    n = (8, 4, 4)
    kw = dict(ncp=2, tsc=5, t1=0.5, ti=0, objective=objective, loadsignal=1, dalpha=0.01, dbeta=0.01)
    rng = np.random.default_rng(30 + objective)
    x = 0.1 + 0.5 * rng.random(np.prod(n))
    le = _le(n, nlvls=2, mixed=mixed, rtol=1e-12, sens_fp32=False, **kw)
    fx, df = _run_gpu(le, x)
    ref = O.LinearElasticity(*n, **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert rc == 0
    assert abs(fx - fx_r) <= 1e-10 * abs(fx_r), (fx, fx_r)
    assert _rel(df, df_r) < 1e-9


@pytest.mark.parametrize("objective", range(7))
def test_fp32_sensitivities_every_objective(gpu, objective):
    # FP32 element math of the sensitivity kernel for every objective, on the
    # per-node FP64 combinations and FP32 copies of lambda and the states
    n = (12, 6, 6)
    kw = dict(ncp=2, tsc=4, t1=0.08, objective=objective, loadsignal=1, dalpha=1e-3, dbeta=1e-3)
    rng = np.random.default_rng(5 + objective)
    x = 0.3 + 0.1 * (2 * rng.random(np.prod(n)) - 1)
    le = _le(n, nlvls=2, mixed=True, rtol=1e-12, sens_fp32=True, **kw)
    fx, df = _run_gpu(le, x)
    ref = O.LinearElasticity(*n, **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert abs(fx - fx_r) <= 1e-6 * abs(fx_r)
    assert _rel(df, df_r) < 1e-5


@pytest.mark.parametrize("objective,mixed", [(3, False), (0, False), (4, True), (6, True), (5, False)])
def test_sommg_reduced_path_matches_oracle(gpu, objective, mixed):
    # SOMMG basis (SOMMG.cc:40-252) from FCG solves with P0 = K - om^2 M,
    # reduced Newmark forward/adjoint, sensitivities from the accumulated
    # reduced outer products; the oracle lifts every step to the full grid
    # as the reference does (LinearElasticity.cc:1683-1868)
    n = (8, 4, 4)
    kw = dict(ncp=2, tsc=6, t1=0.24, objective=objective, loadsignal=1, dalpha=1e-3, dbeta=1e-3)
    rng = np.random.default_rng(3)
    x = 0.3 + 0.1 * (2 * rng.random(np.prod(n)) - 1)
    # plain path: FP64 basis, FP64 dot products (measured 1e-13); mixed path:
    # the basis stored in FP32, whose rounding Gram-Schmidt amplifies into the
    # later rows (measured 1.6e-6), the reduced matrices from the tensor-core
    # Gram product (2.8e-7), FP32 Phi rows in the sensitivity pass (objective
    # 1.3e-6, sensitivities 3e-6 of max on GB300)
    le = _le(n, nlvls=2, mixed=mixed, rtol=1e-13, reduction=True, basis=4, omega0=0.01, **kw)
    fx, df = _run_gpu(le, x)
    Q, Kr, Mr, Pr = le.reduced_system()
    ref = O.LinearElasticity(*n, rtol=1e-13, **kw)
    rc, fx_r, df_r, Q_r, Kr_r, Mr_r = ref.reduced_objective_sensitivities(x, 4, 0.01)
    assert rc == 0
    tq, tm, tf, td = (5e-6, 1e-6, 5e-6, 1e-5) if mixed else (1e-8, 1e-8, 1e-8, 1e-7)
    assert _rel(Q, Q_r) < tq
    assert _rel(Kr, Kr_r) < tm and _rel(Mr, Mr_r) < tm
    assert abs(fx - fx_r) <= tf * abs(fx_r), (fx, fx_r)
    assert _rel(df, df_r) < td
    assert np.abs(Q @ Q.T - np.eye(4)).max() < (1e-6 if mixed else 1e-12)
    assert np.all(np.isfinite(le.state(0, kw["tsc"] - 1)))


@pytest.mark.parametrize("objective,mixed", [(7, False), (7, True), (3, True)])
def test_extended_workload_load_and_output_objective(gpu, objective, mixed):
    # the extended workloads: a second point load at a seeded node with a
    # seeded phase, and objective 7 (dt/2 u^2 of the tip-centre z DOF)
    n = (12, 6, 6)
    rng = np.random.default_rng(0x7A11)
    node = int(rng.integers(0, 13 * 7 * 7))
    phase = float(rng.uniform(0.0, 2.0 * np.pi))
    kw = dict(ncp=2, tsc=5, t1=0.2, objective=objective, loadsignal=1, dalpha=1e-3, dbeta=1e-3, load2_node=node,
              load2_phase=phase)
    x = 0.3 + 0.02 * (2 * rng.random(np.prod(n)) - 1)
    le = _le(n, nlvls=2, mixed=mixed, rtol=1e-12, sens_fp32=False, **kw)
    fx, df = _run_gpu(le, x)
    ref = O.LinearElasticity(*n, **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert rc == 0
    assert abs(fx - fx_r) <= 1e-9 * abs(fx_r)
    assert _rel(df, df_r) < 1e-8


def test_reference_pulse_and_defaults(gpu):
    # reference defaults: Emax 1e3, Rmax 4.1667e-4, reference load pulse, dt = 0.4
    n = (8, 4, 4)
    kw = dict(ncp=4, tsc=10, t1=16.0, objective=0, loadsignal=0, dalpha=1e-4, dbeta=1e-4)
    mat = (1e-6, 1e3, 4.1667e-7, 4.1667e-4, 3.0, 1.0)
    rng = np.random.default_rng(4)
    x = 0.3 + 0.2 * rng.random(np.prod(n))
    le = _le(n, nlvls=2, mixed=False, rtol=1e-12, **kw)
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    df = torch.zeros_like(xd)
    le.CompleteInitialState(xd, *mat)
    le.GenerateCheckPoints()
    fx = le.ComputeObjectiveSensitivities(df)
    ref = O.LinearElasticity(*n, Emin=mat[0], Emax=mat[1], Rmin=mat[2], Rmax=mat[3], **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert abs(fx - fx_r) <= 1e-10 * abs(fx_r)
    assert _rel(df.cpu().numpy(), df_r) < 1e-9


def test_golden_fixture(gpu):
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz"))
    for obj in (0, 3, 6):
        le = _le((4, 2, 2), nlvls=2, ncp=2, tsc=3, t1=0.6, objective=obj, loadsignal=1, dalpha=0.01, dbeta=0.01,
                 mixed=False, rtol=1e-13)
        fx, df = _run_gpu(le, g["x"])
        assert abs(fx - g["fx%d" % obj]) <= 1e-10 * abs(g["fx%d" % obj])
        assert _rel(df, g["df%d" % obj]) < 1e-9


def test_host_and_device_entry_points_agree(gpu):
    n = (8, 4, 4)
    rng = np.random.default_rng(6)
    x = 0.2 + 0.3 * rng.random(np.prod(n))
    kw = dict(nlvls=2, ncp=2, tsc=4, t1=0.4, objective=3, loadsignal=1, dbeta=1e-3, dalpha=0.0)
    a = _le(n, **kw)
    fx1, df1 = _run_gpu(a, x)
    b = _le(n, **kw)
    b.CompleteInitialState(x, *M6)
    b.GenerateCheckPoints()
    df2 = np.zeros(np.prod(n))
    fx2 = b.ComputeObjectiveSensitivities(df2)
    assert fx1 == fx2 and np.array_equal(df1, df2)  # deterministic kernels: bitwise
    dg = np.zeros(np.prod(n))
    gx = b.VolumeConstraint(dg, x, 0.3)
    assert abs(gx - (x.mean() - 0.3)) < 1e-14 and np.allclose(dg, 1.0 / x.size)


def test_pde_filter_and_projection(gpu):
    from topopt_in_petsc_transient_gb300 import Filter, PDEFilt
    n = (16, 8, 8)
    rng = np.random.default_rng(8)
    x = rng.random(np.prod(n))
    f = PDEFilt(*n, 2.0, rtol=1e-13)
    out = np.zeros_like(x)
    f.FilterProject(x, out)
    assert _rel(out, O.pde_filter(*n, x, 2.0)) < 1e-10
    F = Filter(*n, 2, 2.0, rtol=1e-13)
    xt, xp = np.zeros_like(x), np.zeros_like(x)
    F.FilterProject(x, xt, xp, True, 4.0, 0.3)
    xt_r, xp_r = O.filter_project(*n, x, 2.0, True, 4.0, 0.3)
    assert _rel(xt, xt_r) < 1e-10 and _rel(xp, xp_r) < 1e-10
    df = rng.standard_normal(x.size)
    dg = np.full(x.size, 1.0 / x.size)
    df_r, dg_r = O.filter_gradients(*n, xt_r, df, dg, 2.0, True, 4.0, 0.3)
    F.Gradients(x, xt, df, 1, dg, True, 4.0, 0.3)
    assert _rel(df, df_r) < 1e-9 and _rel(dg, dg_r) < 1e-9
    assert abs(F.GetMND(xp) - O.filter_mnd(xp)) < 1e-13


def test_mma_matches_oracle(gpu):
    from topopt_in_petsc_transient_gb300 import MMA
    n = 2000
    rng = np.random.default_rng(9)
    c = rng.random(n)
    x = np.full(n, 0.5)
    xo = x.copy()
    mo = O.MMA(n, 1, x)
    mo.SetAsymptotes(0.1, 0.6, 1.05)
    mg = MMA(n, 1)
    mg.SetAsymptotes(0.1, 0.6, 1.05)
    xg = torch.tensor(x, dtype=torch.float64, device="cuda")
    lo = torch.zeros_like(xg)
    hi = torch.zeros_like(xg)
    for it in range(5):
        df = 2 * (xo - c) * (1 + 0.1 * it)
        g = np.array([xo.mean() - 0.4])
        dg = np.full(n, 1.0 / n)
        lo_r, hi_r = O.MMA.SetOuterMovelimit(0.0, 1.0, 0.2, xo)
        mo.Update(xo, df, g, dg, lo_r, hi_r)
        mg.SetOuterMovelimit(0.0, 1.0, 0.2, xg, lo, hi)
        mg.Update(xg, torch.tensor(df, device="cuda"), g, torch.tensor(dg, device="cuda"), lo, hi)
        assert _rel(xg.cpu().numpy(), xo) < 1e-10, it


def test_mma_restart_continues_bitwise(gpu):
    # MMA::Restart and the restart constructor MMA(n, m, itr, xo1, xo2, U, L)
    # (MMA.h:16-27): three updates, restart, a fourth update equals four
    # uninterrupted updates bit for bit (host and device restart arrays)
    from topopt_in_petsc_transient_gb300 import MMA
    n = 1500
    rng = np.random.default_rng(19)
    c = rng.random(n)

    def step(mg, xg, it):
        lo, hi = torch.zeros_like(xg), torch.zeros_like(xg)
        xh = xg.cpu().numpy()
        df = torch.tensor(2 * (xh - c) * (1 + 0.1 * it), device="cuda")
        g = np.array([xh.mean() - 0.4])
        mg.SetOuterMovelimit(0.0, 1.0, 0.2, xg, lo, hi)
        mg.Update(xg, df, g, torch.full_like(xg, 1.0 / n), lo, hi)

    ref = MMA(n, 1)
    ref.SetAsymptotes(0.1, 0.6, 1.05)
    xr = torch.full((n,), 0.5, dtype=torch.float64, device="cuda")
    for it in range(4):
        step(ref, xr, it)
    for device in (True, False):
        a = MMA(n, 1)
        a.SetAsymptotes(0.1, 0.6, 1.05)
        xa = torch.full((n,), 0.5, dtype=torch.float64, device="cuda")
        for it in range(3):
            step(a, xa, it)
        st = [torch.zeros_like(xa) for _ in range(4)] if device else [np.zeros(n) for _ in range(4)]
        a.Restart(*st)
        b = MMA(n, 1, itr=3, xo1=st[0], xo2=st[1], U=st[2], L=st[3])
        b.SetAsymptotes(0.1, 0.6, 1.05)
        step(b, xa, 3)
        assert torch.equal(xa, xr)


def test_restart_files_continue_the_design_loop(gpu, tmp_path):
    # TopOpt::WriteRestartFiles and the -restartFileVec branch of
    # AllocateMMAwithRestart (TopOpt.cc:600-735): three design iterations,
    # restart files, a fresh TopOpt continued from them: the restored design
    # is bitwise the written one and the next objective agrees to the solve
    # tolerance (the uninterrupted objects start their iterative solves warm);
    # the HBM checkpoints export as cp%04d.dat
    from topopt_in_petsc_transient_gb300 import (TopOpt, design_iteration, load_restart, read_petsc_vecs,
                                                 write_restart_files)
    kw = dict(nelx=16, nely=8, nelz=8, nlvls=2, ncp=2, tsc=3, t1=0.03, objective=3, loadsignal=1, dalpha=0.0,
              dbeta=1e-3)
    a = TopOpt(**kw).setup()
    for _ in range(3):
        design_iteration(a)
    vec = write_restart_files(a, str(tmp_path))
    assert vec.endswith("Restart00.dat")
    x3, xp3 = a.x.clone(), a.xPhys.clone()
    fa = design_iteration(a)[0]
    b = TopOpt(**kw).setup()
    load_restart(b, vec, str(tmp_path / "Restart00_itr_f0.dat"))
    assert b.itr == 3 and b.fscale == a.fscale
    assert torch.equal(b.x, x3) and torch.equal(b.xPhys, xp3) and torch.equal(b.xold, x3)
    fb = design_iteration(b)[0]
    assert abs(fb - fa) <= 1e-8 * abs(fa)
    assert _rel(b.x.cpu().numpy(), a.x.cpu().numpy()) < 1e-2
    a.physics.WriteCheckPoints(str(tmp_path))
    U, DU, DDU = a.physics.checkpoint(1)
    got = [np.zeros(U.size) for _ in range(3)]
    read_petsc_vecs(str(tmp_path / "cp0001.dat"), got)
    assert np.array_equal(got[0], U) and np.array_equal(got[1], DU) and np.array_equal(got[2], DDU)


@pytest.mark.parametrize("ncp,tsc,reduction", [(2, 3, False), (1, 4, False), (2, 3, True)])
def test_physics_output_files(gpu, tmp_path, ncp, tsc, reduction):
    # the `write, output` arguments of CompleteInitialState (dataset 0),
    # GenerateCheckPoints (every step when ncp > 1) and
    # ComputeObjectiveSensitivities (every step when ncp == 1): each dataset is
    # the float32 displacement of one step and xPhys, bitwise the device states
    from mpiio_reader import point_fields_of, read_result_file

    from topopt_in_petsc_transient_gb300 import MPIIO, TopoError
    n = (8, 4, 4)
    rng = np.random.default_rng(11)
    x = 0.3 + 0.1 * (2 * rng.random(np.prod(n)) - 1)
    kw = dict(ncp=ncp, tsc=tsc, t1=0.02 * ncp * tsc, objective=3, loadsignal=1, dalpha=1e-3, dbeta=1e-3)
    red = dict(reduction=True, basis=4, omega0=0.01, rtol=1e-13) if reduction else {}
    le = _le(n, nlvls=2, **kw, **red)
    p = str(tmp_path / "outputPhysics0_00000.dat")
    io = MPIIO(le, 3, "ux, uy, uz", 1, "xPhys", p)
    with pytest.raises(TopoError):  # a design-only writer cannot take the physics output
        le.CompleteInitialState(x, *M6, write=True, output=MPIIO(le, 0, "", 3, "x, xTilde, xPhys",
                                                                  str(tmp_path / "d.dat")))
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    df = torch.zeros_like(xd)
    le.CompleteInitialState(xd, *M6, write=True, output=io)
    le.GenerateCheckPoints(True, xd, io)
    io.Flush()
    r = read_result_file(p)
    T = ncp * tsc
    expect = T + 1 if ncp > 1 else 1
    assert [d[0] for d in r["datasets"]] == list(range(expect))
    if ncp > 1:  # the last block is resident after GenerateCheckPoints
        for j in range(tsc):
            assert np.array_equal(r["datasets"][T - tsc + j + 1][1], point_fields_of(le.state(0, j)))
        if not reduction:
            assert np.array_equal(r["datasets"][0][1], point_fields_of(le.checkpoint(0)[0]))
            assert np.array_equal(r["datasets"][tsc][1], point_fields_of(le.checkpoint(1)[0]))
    le.ComputeObjectiveSensitivities(df, write=True, output=io)
    io.Flush()
    r = read_result_file(p)
    assert [d[0] for d in r["datasets"]] == list(range(T + 1))  # ncp == 1: the steps come from here
    if ncp == 1:
        for j in range(tsc):
            assert np.array_equal(r["datasets"][j + 1][1], point_fields_of(le.state(0, j)))
    for _, pf, cf in r["datasets"]:
        assert np.array_equal(cf[0], x.astype(np.float32))
        assert np.all(np.isfinite(pf))
    assert np.abs(r["datasets"][-1][1]).max() > 0.0
    # without write nothing is added
    le.CompleteInitialState(xd, *M6, write=False, output=io)
    io.Flush()
    assert len(read_result_file(p)["datasets"]) == T + 1


def test_result_file_overloads_from_device_tensors(gpu, tmp_path):
    # MPIIO::WriteVTK overloads with CUDA tensors: the float32 conversion and
    # the DOF-interleaved to field-major scatter run on the device, straight
    # into the pinned records; a ring of two records wraps several times
    from mpiio_reader import point_fields_of, read_result_file

    from topopt_in_petsc_transient_gb300 import MPIIO
    n = (5, 3, 2)
    nn, nel = 6 * 4 * 3, 30
    g = torch.Generator(device="cuda").manual_seed(5)
    dev = dict(dtype=torch.float64, device="cuda", generator=g)
    p = str(tmp_path / "outputAll_00000.dat")
    io = MPIIO(n, 9, "ux, uy, uz, vx, vy, vz, ax, ay, az", 3, "x, xTilde, xPhys", p, slots=2)
    hist = []
    for t in range(7):
        U = [torch.randn(3 * nn, **dev) for _ in range(3)]
        X = [torch.rand(nel, **dev) for _ in range(3)]
        if t % 3 == 2:
            io.WriteVTK(*X, t)  # design-only overload: previous point fields again
            hist.append((hist[-1][0], X))
        else:
            io.WriteVTK(*U, *X, t)
            hist.append((U, X))
    del io
    r = read_result_file(p)
    assert [d[0] for d in r["datasets"]] == list(range(7))
    for (U, X), (_, pf, cf) in zip(hist, r["datasets"]):
        assert np.array_equal(pf, point_fields_of(*[u.cpu().numpy() for u in U]))
        assert np.array_equal(cf, np.stack([v.cpu().numpy() for v in X]).astype(np.float32))


def test_design_loop_result_files(gpu, tmp_path):
    # main.cc:38-49, :102-105, :163-176: the design fields every iteration,
    # the physics of the first iteration, the physics of the final design
    from mpiio_reader import read_result_file

    from topopt_in_petsc_transient_gb300 import TopOpt, design_iteration, final_physics_output
    opt = TopOpt(nelx=8, nely=4, nelz=4, nlvls=2, ncp=2, tsc=3, t1=0.06, objective=3, loadsignal=1, dalpha=1e-3,
                 dbeta=1e-3, outputDesign=True, outputPhysics0=True, outputPhysics1=True,
                 workdir=str(tmp_path)).setup()
    xp0 = opt.xPhys.cpu().numpy().astype(np.float32)
    for _ in range(2):
        design_iteration(opt)
    final_physics_output(opt)
    d = read_result_file(str(tmp_path / "outputDesign_00000.dat"))
    assert d["cellFieldNames"] == ["x", "xTilde", "xPhys"] and d["nPFields"] == 0
    assert [t[0] for t in d["datasets"]] == [1, 2]
    assert np.array_equal(d["datasets"][0][2][2], xp0)
    p0 = read_result_file(str(tmp_path / "outputPhysics0_00000.dat"))
    assert [t[0] for t in p0["datasets"]] == list(range(7))  # first iteration only
    assert all(np.array_equal(t[2][0], xp0) for t in p0["datasets"])
    p1 = read_result_file(str(tmp_path / "outputPhysics1_00000.dat"))
    assert [t[0] for t in p1["datasets"]] == list(range(7))
    xpf = opt.xPhys.cpu().numpy().astype(np.float32)
    assert all(np.array_equal(t[2][0], xpf) for t in p1["datasets"])
    assert not np.array_equal(xpf, xp0)


def test_sommg_basis_solves_descend_the_multigrid_hierarchy(gpu):
    # the shifted operator K - om^2 M has negative element-wise lower bounds;
    # they must not make the V-cycle stop at the fine level (a one-level
    # Chebyshev solve took 86 FCG iterations per basis solve on this mesh,
    # the full V-cycle about 12)
    n = (48, 24, 24)
    le = _le(n, nlvls=4, ncp=1, tsc=10, t1=0.05, objective=3, loadsignal=1, dalpha=0.0, dbeta=1e-3, mixed=False,
             rtol=1e-10, reduction=1, basis=4, omega0=1e-4)
    s0 = le.stats()
    le.CompleteInitialState(np.full(np.prod(n), 0.12), *M6)
    s1 = le.stats()
    its = (s1["cg_iterations"] - s0["cg_iterations"]) / (s1["solves"] - s0["solves"])
    assert its < 25
    assert s1["replacements"] == 0  # the plain FP64 path has no replacement residuals


@pytest.mark.parametrize("ftype,R,h", [(1, 3.0, (1.0, 1.0, 1.0)), (0, 3.0, (1.0, 1.0, 1.0)), (1, 2.0, (1.0, 1.0, 1.0)),
                                       (1, 2.5, (1.0, 2.0, 1.0)), (0, 2.0, (1.0, 1.0, 1.0))])
def test_density_and_sensitivity_filters(gpu, ftype, R, h):
    # Filter for filterType 0 / 1 (Filter.cc:60-206, :302-531) against the
    # oracle, with and without the smoothed Heaviside projection; host and
    # device entry points agree bitwise
    from topopt_in_petsc_transient_gb300 import Filter
    n = (10, 6, 5)
    nel = int(np.prod(n))
    rng = np.random.default_rng(17)
    x = 0.05 + 0.9 * rng.random(nel)
    f = Filter(*n, ftype, R, h=h)
    for proj in (False, True):
        xt, xp = np.zeros(nel), np.zeros(nel)
        f.FilterProject(x, xt, xp, proj, 4.0, 0.5)
        xt_r, xp_r = O.dens_filter_project(*n, ftype, x, R, proj, 4.0, 0.5, h=h)
        assert _rel(xt, xt_r) < 1e-13 and _rel(xp, xp_r) < 1e-13
        df, dg = rng.standard_normal(nel), rng.standard_normal(nel)
        df1, dg1 = df.copy(), dg.copy()
        f.Gradients(x, xt, df1, 1, dg1, proj, 4.0, 0.5)
        df_r, dg_r = O.dens_filter_gradients(*n, ftype, x, xt_r, df, dg, R, proj, 4.0, 0.5, h=h)
        assert _rel(df1, df_r) < 1e-12 and _rel(dg1, dg_r) < 1e-12
        xd = torch.tensor(x, device="cuda")
        xtd, xpd = torch.zeros_like(xd), torch.zeros_like(xd)
        f.FilterProject(xd, xtd, xpd, proj, 4.0, 0.5)
        assert np.array_equal(xtd.cpu().numpy(), xt) and np.array_equal(xpd.cpu().numpy(), xp)
    assert abs(f.GetMND(x) - O.filter_mnd(x)) < 1e-14


def test_design_iteration_with_density_filter(gpu):
    # main.cc loop with -filter 1 (standard density filter, rmin 3)
    from topopt_in_petsc_transient_gb300 import TopOpt, design_iteration
    opt = TopOpt(nelx=16, nely=8, nelz=8, nlvls=2, ncp=1, tsc=4, t1=0.02, objective=3, loadsignal=1, filter=1,
                 rmin=3.0, dalpha=0.0, dbeta=1e-3).setup()
    fx, fxs, gx, ch, mnd = design_iteration(opt)
    assert np.isfinite(fx) and np.isfinite(fxs) and np.isfinite(gx) and 0.0 <= mnd <= 1.0
    # the design moves by at most movlim; ch reads 1 while the volume
    # constraint is violated (main.cc:146-150)
    assert (0.0 < ch <= 0.2 + 1e-12) or (gx > 0.0 and ch == 1.0)
    xp = opt.xPhys.cpu().numpy()
    assert np.all(np.isfinite(xp)) and xp.min() >= 0.0 and xp.max() <= 1.0


def test_solver_failures_are_reported(gpu):
    from topopt_in_petsc_transient_gb300 import TopoError
    with pytest.raises(TopoError) as e:
        _le((8, 4, 4), nlvls=4)  # 4 elements cannot be halved 3 times (TopOpt.cc:200-219)
    assert e.value.status == 1
    le = _le((8, 4, 4), nlvls=2, ncp=2, tsc=2, t1=0.2, loadsignal=1)
    with pytest.raises(TopoError) as e:
        le.GenerateCheckPoints()  # before CompleteInitialState
    assert e.value.status == 7
    # with ncp > 1 the reverse sweep restarts from checkpoints of this design:
    # sensitivities without GenerateCheckPoints are refused, not computed from
    # stale checkpoints (main.cc:84-90 calls it between the two)
    le.CompleteInitialState(np.full(128, 0.3), *M6)
    with pytest.raises(TopoError) as e:
        le.ComputeObjectiveSensitivities(np.zeros(128))
    assert e.value.status == 7
    le.GenerateCheckPoints()
    le.ComputeObjectiveSensitivities(np.zeros(128))
    # an iteration cap of 1 must surface as "not converged", not as a wrong answer
    le = _le((8, 4, 4), nlvls=2, ncp=2, tsc=2, t1=0.2, loadsignal=1, maxit=1, rtol=1e-14)
    x = np.full(128, 0.3)
    with pytest.raises(TopoError) as e:
        le.CompleteInitialState(x, *M6)
        le.GenerateCheckPoints()
    assert e.value.status == 4


def test_finite_difference_check_on_gpu(gpu):
    # central differences h = 1e-4 on seeded elements (the check of the
    # 192x96x96 workload, here on a small mesh)
    n = (8, 4, 4)
    kw = dict(nlvls=2, ncp=2, tsc=5, t1=0.5, objective=3, loadsignal=1, dalpha=0.0, dbeta=1e-3, mixed=True,
              rtol=1e-13, sens_fp32=False)
    rng = np.random.default_rng(11)
    x = 0.12 + 0.02 * (2 * rng.random(np.prod(n)) - 1)
    le = _le(n, **kw)
    fx, df = _run_gpu(le, x)
    h = 1e-4
    for e in rng.choice(x.size, 6, replace=False):
        xp, xm = x.copy(), x.copy()
        xp[e] += h
        xm[e] -= h
        fd = (_run_gpu(le, xp)[0] - _run_gpu(le, xm)[0]) / (2 * h)
        assert abs(fd - df[e]) <= 1e-6 * np.abs(df).max(), (e, fd, df[e])


def test_mixed_path_is_scale_invariant(gpu):
    # a 4-step horizon of the sine pulse leaves states ~1e-12 and adjoints far
    # smaller: the FP32 recurrence must not underflow (it runs on residuals
    # scaled to unit RMS)
    n = (16, 8, 8)
    kw = dict(ncp=1, tsc=4, t1=0.02, objective=3, loadsignal=1, dalpha=0.0, dbeta=1e-3)
    x = np.full(np.prod(n), 0.12)
    le = _le(n, nlvls=1, coarse_smooth=10, mixed=True, rtol=1e-10, sens_fp32=False, **kw)
    fx, df = _run_gpu(le, x)
    ref = O.LinearElasticity(*n, **kw)
    rc, fx_r, df_r = ref.objective_sensitivities(x)
    assert fx_r < 1e-10
    assert abs(fx - fx_r) <= 1e-8 * abs(fx_r)
    assert _rel(df, df_r) < 1e-7
