"""Throughput of the transient forward + adjoint design iteration on GB300.

Workload (the cantilever the headline metric is quoted on): 96x48x48 unit hex8
elements (698,691 DOFs), E0 = 1, Emin = 1e-9, nu = 0.3, mass density 1, SIMP
p = 3, Rayleigh alpha = 0, beta = 1e-3, clamped face x = 0, line load at the
mid line of face x = nelx with f(t) = sin(2 pi t) for t < 0.5, 200 Newmark
steps of dt = 0.005, uniform density 0.12, PDE filter radius 2, MMA, 5
multigrid levels.  Objective: reference objective 3 (potential energy, the
reference-expressible form of time-integrated compliance).  Synthetic inputs
(no dataset is involved).

A "step" is one design iteration of main.cc's loop: CompleteInitialState,
ComputeObjectiveSensitivities (forward + adjoint + sensitivities),
VolumeConstraint, Filter::Gradients, MMA::Update, Filter::FilterProject.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "forward+adjoint design iters/s on 1 GB300: mixed vs plain FP64 at equal obj. error"

# DRAM bytes (read + write) per launch of the roofline kernel classes, keyed by
# (mesh, kernel class), from one `ncu --set full` capture of each pass on the
# named mesh summarised under profiles/ (mean over the three Kronecker passes);
# below the algorithmic bytes where vectors stay in L2; absent pairs report null
TRAFFIC = {
    ("96x48x48", "k_kron_pass<float>"): (5.624e6 + 2.819e6 + 11.22e6) / 3.0,
    ("96x48x48", "k_tile<float,PolPQ32>"): 7.627e6,
    ("192x96x96", "k_kron_pass<float>"): (43.62e6 + 0.437e6 + 21.82e6 + 87.26e6 + 5.977e6) / 3.0,
    ("192x96x96", "k_tile<float,PolPQ32>"): 59.60e6 + 6.723e6,
}
UNIT = "design_iter/s"


def workload(args):
    nel = tuple(int(v) for v in args.mesh.split("x"))
    return dict(nelx=nel[0], nely=nel[1], nelz=nel[2], nlvls=args.nlvls, volfrac=0.12, V0=0.12, rmin=2.0,
                penalK=3.0, penalM=1.0, Emax=1.0, Ef=1e-9, Rmax=1.0, Rf=1e-3, filter=2, sInt=1, mInt=0, ti=1,
                t1=args.dt * args.nsteps, ncp=args.ncp, tsc=args.nsteps // args.ncp, dalpha=0.0, dbeta=1e-3,
                objective=args.objective, boundaries=1, loadloc=1, optimizationRegion=2, projectionFilter=False,
                loadsignal=1, movlim=0.2, smooth=args.smooth, cheb_ratio=args.cheb_ratio, rtol=args.rtol,
                coarse_dense_max=args.coarse_dense_max, coarse_smooth=args.coarse_smooth, sens_fp32=args.sens_fp32,
                inner_tol=args.inner_tol, inner_maxit=args.inner_maxit, use_graphs=not args.no_graphs,
                reduction=args.reduction, basis=args.basis, omega0=args.omega0,
                noise=args.noise, tile_form=args.tile_form, kron_form=args.kron_form, **load2(args))


def load2(args):
    """Second point load of the extended workload: a seeded free node in the
    outer half of the beam and a seeded phase (generator seed 0x7A11)."""
    if not args.load2:
        return {}
    import numpy as np
    nel = [int(v) for v in args.mesh.split("x")]
    rng = np.random.default_rng(0x7A11)
    i = int(rng.integers(nel[0] // 2, nel[0] + 1))
    j = int(rng.integers(0, nel[1] + 1))
    k = int(rng.integers(0, nel[2] + 1))
    node = i + (nel[0] + 1) * (j + (nel[1] + 1) * k)
    return {"load2_node": node, "load2_phase": float(rng.uniform(0.0, 2.0 * np.pi))}


def workload_name(args):
    red = (", SOMMG reduction: %d basis vectors at omega0=%g" % (args.basis, args.omega0)) if args.reduction else ""
    ext = ""
    if args.noise > 0:
        ext += ", density noise U(-%g,%g) seed 0x7A11" % (args.noise, args.noise)
    if args.load2:
        ext += ", second point load (node %(load2_node)d, phase %(load2_phase).4f)" % load2(args)
    return ("cantilever %s hex8, %d Newmark steps dt=%g, %d-level GMG, PDE filter r=2, MMA; objective %d%s%s"
            % (args.mesh, args.nsteps, args.dt, args.nlvls, args.objective, red, ext))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.idx = device_index
        self.proc = None
        self.out = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [v.strip() for v in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_time(t_local, ws, device):
    """Job time of N independent replicas: the maximum over the ranks of
    each rank's timed-region time (an all-reduce MAX on the process group)."""
    if ws <= 1:
        return t_local
    import torch
    import torch.distributed as dist
    tt = torch.tensor([t_local], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def replica_value(steps, ws, t_job):
    """Whole-job throughput: every replica ran `steps` design iterations."""
    return ws * steps / t_job


def run_gb300(args):
    import numpy as np
    import torch

    from topopt_in_petsc_transient_gb300 import TopOpt, design_iteration, _lib
    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    L = _lib.load()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def flush_l2():
        flush.zero_()
        torch.cuda.synchronize()

    # ---- headline: mixed-precision path, design vectors resident in HBM ----
    wl = workload(args)
    opt = TopOpt(mixed=True, **wl).setup()
    for _ in range(args.warmup):
        design_iteration(opt)
    le_stats0 = opt.physics.stats()
    launches0 = L.topo_kernel_launches()
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    times = []
    fxs = []
    for _ in range(args.steps):
        flush_l2()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push("timed_design_iteration")  # lets a profiler select the timed region
        e0.record()
        fx, fxs_, gx, ch, mnd = design_iteration(opt)  # every library call returns synchronised
        e1.record()
        e1.synchronize()
        torch.cuda.nvtx.range_pop()
        times.append(e0.elapsed_time(e1) / 1e3)
        fxs.append(fx)
    barrier()
    clocks = sampler.stop()
    le_stats1 = opt.physics.stats()
    launches = (L.topo_kernel_launches() - launches0) + (le_stats1["graph_body_launches"] -
                                                          le_stats0["graph_body_launches"])
    t_total = replica_time(sum(times), ws, "cuda")
    value = replica_value(args.steps, ws, t_total)
    iters_per_solve = ((le_stats1["cg_iterations"] - le_stats0["cg_iterations"]) /
                       max(1, le_stats1["solves"] - le_stats0["solves"]))

    # ---- plain FP64 path and objective agreement on the same initial design ----
    plain = None
    if args.plain_steps > 0:
        # both paths from the same uniform design: objective and sensitivity
        # agreement on the first iteration; the plain path is then timed on
        # the same iterations as the headline (after the warm-up iterations)
        a = TopOpt(mixed=True, **wl).setup()
        b = TopOpt(mixed=False, **wl).setup()
        fa = design_iteration(a)[0]
        dfa = a.dfdx.clone()
        fb = design_iteration(b)[0]
        dfb = b.dfdx.clone()
        del a
        for _ in range(max(0, args.warmup - 1)):
            design_iteration(b)
        torch.cuda.synchronize()
        tp = []
        for k in range(args.plain_steps):
            flush_l2()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            design_iteration(b)
            e1.record()
            e1.synchronize()
            tp.append(e0.elapsed_time(e1) / 1e3)
        plain = {"value": len(tp) / sum(tp), "unit": UNIT, "steps": len(tp), "warmup": args.warmup,
                 "objective_rel_diff_mixed_vs_plain": abs(fa - fb) / abs(fb),
                 "dfdx_maxrel_diff_mixed_vs_plain": float((dfa - dfb).abs().max() / dfb.abs().max()),
                 "speedup_mixed_over_plain": value / ws / (len(tp) / sum(tp))}
        del b

    # ---- end to end through the C ABI with host buffers ----
    e2e = None
    if args.e2e_steps > 0:
        e2e = run_e2e(args, wl, flush_l2)

    # ---- roofline of the dominant kernels, timed in the solve ----
    # One extra design iteration per kernel class (outside the timed region,
    # the same kernels launched directly instead of from CUDA graphs)
    # brackets each launch of that class with CUDA events on the library
    # stream; achieved = algorithmic bytes per launch / mean launch time.
    import ctypes as C
    nel = opt.nel
    nn = (wl["nelx"] + 1) * (wl["nely"] + 1) * (wl["nelz"] + 1)
    probe = TopOpt(mixed=True, **dict(wl, use_graphs=False)).setup()
    for _ in range(args.warmup):
        design_iteration(probe)
    peaks = load_peaks()
    # algorithmic bytes per launch (FP32 vectors of 3 nn values, 1-byte
    # clamp mask per node, FP32 element factors kf, mf):
    #   PQ32: stage z and p_prev, write p and q (4 x 12 B/node), mask, kf/mf
    #   Kronecker pass: x pass reads r and the per-DOF masked scale and writes
    #     its output (36 B/node); y pass reads and writes one vector (24 B/node);
    #     z pass reads its input, r, the masked scale and q and writes z
    #     (60 B/node)
    #   smoothing step: x, b, 1/diag, d read, d and x written (72 B/node), mask, kf/mf
    classes = [(1, "k_tile<float,PolPQ32> (FCG operator product q = A p with p = z + beta p_prev, FP32)",
                49.0 * nn + 8.0 * nel),
               (2, "k_kron_pass<float> (one axis pass of the Kronecker mass inverse, 17-tap stencil, FP32)",
                (36.0 + 24.0 + 60.0) / 3.0 * nn),
               (0, "k_tile<float,PolCheb> (FP32 Chebyshev-Jacobi smoothing step)", 73.0 * nn + 8.0 * nel)]
    kern = []
    for cls, name, nbytes in classes:
        _lib.check(L.topo_le_kernel_timing(probe.physics._h, cls, 1, None, None), "kernel_timing")
        design_iteration(probe)
        tot_ms, nlaunch = C.c_double(), C.c_longlong()
        _lib.check(L.topo_le_kernel_timing(probe.physics._h, cls, 0, C.byref(tot_ms), C.byref(nlaunch)),
                   "kernel_timing")
        if nlaunch.value == 0:
            continue
        ms_launch = tot_ms.value / nlaunch.value
        ach = nbytes / (ms_launch * 1e-3) / 1e9
        kern.append({"kernel": name, "bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / peaks["hbm_gbs"], "ms_per_launch": ms_launch, "launches_timed": nlaunch.value,
                     "ms_per_design_iter": tot_ms.value, "algorithmic_bytes": nbytes,
                     "traffic": TRAFFIC.get((args.mesh, name.split(" ")[0]))})
    ms_fp64 = C.c_double()
    _lib.check(L.topo_le_time_apply(probe.physics._h, 0, 5, 50, C.byref(ms_fp64)), "time_apply")
    del probe
    kern.sort(key=lambda k: -k["ms_per_design_iter"])
    roof = dict(kern[0]) if kern else {"kernel": None}
    roof.update({"peak_source": peaks["source"],
                 "timing": "CUDA events around every launch of the class in one design iteration, library stream",
                 "other_kernels": kern[1:],
                 "fp64_apply": {"kernel": "k_tile<double,PolResid>", "ms_per_launch": ms_fp64.value,
                                "achieved_gbs": (3 * nn * 3 * 8 + 2 * nel * 8 + nn) / (ms_fp64.value * 1e-3) / 1e9}})

    cpu = None
    if rank == 0 and args.cpu_sample and ws == 1:
        cpu = cpu_baseline(args, wl)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seedless uniform density 0.12, analytic load pulse)",
        "config": {"workload": workload_name(args), "mode": "mixed: FP32 flexible-CG recurrence, Kronecker mass preconditioner (multigrid when the stiffness share is large), FP64-accurate residual replacements",
                   "dofs": 3 * nn, "elements": nel, "steps_per_design_iter": args.nsteps, "ncp": args.ncp,
                   "rtol": args.rtol, "smooth": args.smooth, "nlvls": args.nlvls,
                   "operator_kernels": "z-marching slabs" if args.tile_form == 1 else "bricks",
                   "kronecker_passes": "register line segments" if args.kron_form == 1 else "staged lines",
                   "l2": "state history %.1f GB > 129 MB L2; 256 MB L2 flush between timed iterations"
                         % (3 * args.nsteps / args.ncp * 3 * nn * 8 / 1e9),
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "objective": fxs[-1] if fxs else None, "krylov_iters_per_solve": iters_per_solve,
        "plain_fp64": plain, "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clocks,
        "gpu_launches": int(launches),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_e2e(args, wl, flush_l2):
    """The same design iteration through the host-pointer C ABI (VecGetArray
    semantics): design vectors live in host memory; every call copies its
    inputs host->device and results device->host inside the timed region."""
    import numpy as np

    from topopt_in_petsc_transient_gb300 import MMA, Filter, LinearElasticity, TopOpt
    o = TopOpt(mixed=True, **wl)
    n = o.nel
    ph = LinearElasticity(o.nelx, o.nely, o.nelz, nlvls=o.nlvls, ncp=o.ncp, tsc=o.tsc, t1=o.t1, objective=o.objective,
                          dalpha=o.dalpha, dbeta=o.dbeta, loadsignal=o.loadsignal, mixed=True, rtol=o.rtol,
                          smooth=o.smooth, cheb_ratio=o.cheb_ratio, use_graphs=o.use_graphs,
                          coarse_dense_max=o.coarse_dense_max, coarse_smooth=o.coarse_smooth, sens_fp32=o.sens_fp32,
                          inner_tol=o.inner_tol, inner_maxit=o.inner_maxit, reduction=o.reduction, basis=o.basis,
                          omega0=o.omega0, load2_node=o.load2_node, load2_phase=o.load2_phase, out_dof=o.out_dof)
    filt = Filter(o.nelx, o.nely, o.nelz, 2, o.rmin)
    mma = MMA(n, 1)
    mma.SetAsymptotes(0.1, 0.6, 1.05)
    x = np.full(n, o.V0)
    if o.noise > 0.0:
        x += np.random.default_rng(o.seed).uniform(-o.noise, o.noise, n)
    xT = np.zeros(n)
    xP = np.zeros(n)
    xold = x.copy()
    df = np.zeros(n)
    dg = np.zeros(n)
    lo = np.zeros(n)
    hi = np.zeros(n)
    filt.FilterProject(x, xT, xP, False, o.beta, o.eta)
    fscale = None
    h2d = d2h = 0
    times = []
    nwarm = max(1, args.warmup)  # the first pass also captures the CUDA graphs
    for k in range(nwarm + args.e2e_steps):
        flush_l2()
        t0 = time.perf_counter()
        ph.CompleteInitialState(xP, o.Emin, o.Emax, o.Rmin, o.Rmax, o.penalK, o.penalM)
        if o.ncp > 1:  # main.cc:84-86
            ph.GenerateCheckPoints()
        fx = ph.ComputeObjectiveSensitivities(df)
        gx = ph.VolumeConstraint(dg, xP, o.volfrac)
        filt.Gradients(x, xT, df, 1, dg, False, o.beta, o.eta)
        filt.GetMND(xP)
        if fscale is None:
            fscale = 1.0 / fx
        df *= fscale
        mma.SetOuterMovelimit(o.Xmin, o.Xmax, o.movlim, x, lo, hi)
        mma.Update(x, df, [gx], dg, lo, hi)
        mma.DesignChange(x, xold)
        filt.FilterProject(x, xT, xP, False, o.beta, o.eta)
        t1 = time.perf_counter()
        if k >= nwarm:  # the same design iterations as the headline
            times.append(t1 - t0)
    b = 8 * n
    h2d = b * (1 + 0 + 1 + 3 + 1 + 1 + 5 + 2 + 1)
    d2h = b * (0 + 1 + 1 + 2 + 0 + 2 + 1 + 1 + 2)
    return {"value": len(times) / sum(times), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": len(times), "timer": "host wall clock around the synchronous C-ABI calls"}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            hbm = d.get("hbm_gbs") or d.get("hbm_GBps") or d.get("hbm")
            if isinstance(hbm, dict):
                hbm = hbm.get("value")
            if hbm:
                return {"hbm_gbs": float(hbm), "source": "measured (MEASURED_PEAKS.json)"}
        except (ValueError, OSError):
            pass
    return {"hbm_gbs": 6800.0, "source": "fallback 6.8 TB/s"}


def cpu_baseline(args, wl, steps_small=(2, 4)):
    """The oracle (CPU FP64 restatement of the reference path: assembled
    27-point block operators, Jacobi-PCG, the reference's dense 24x24 element
    loops) on the host cores, on a bounded sample of the same workload: the
    design iteration at horizons of 2 and 4 steps, extrapolated linearly to the
    full horizon (the per-step cost is the same for every step)."""
    import numpy as np

    from oracle import oracle as O
    ncores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(ncores))
    t = []
    for s in steps_small:
        le = O.LinearElasticity(wl["nelx"], wl["nely"], wl["nelz"], ncp=1, tsc=s, t1=args.dt * s,
                                objective=wl["objective"], loadsignal=1, dalpha=0.0, dbeta=1e-3, rtol=1e-10,
                                Emin=1e-9, Emax=1.0, Rmin=1e-3, Rmax=1.0)
        x = np.full(le.nel, 0.12)
        t0 = time.perf_counter()
        le.objective_sensitivities(x)
        t.append(time.perf_counter() - t0)
        del le
    per_step = (t[1] - t[0]) / (steps_small[1] - steps_small[0])
    fixed = t[0] - steps_small[0] * per_step
    # filter + gradients + MMA of one design iteration
    n = wl["nelx"] * wl["nely"] * wl["nelz"]
    x = np.full(n, 0.12)
    t0 = time.perf_counter()
    xt, xp = O.filter_project(wl["nelx"], wl["nely"], wl["nelz"], x, wl["rmin"], False, 0.1, 0.15, rtol=1e-8)
    O.filter_gradients(wl["nelx"], wl["nely"], wl["nelz"], xt, np.ones(n), np.full(n, 1.0 / n), wl["rmin"], False,
                       0.1, 0.15, rtol=1e-8)
    mma = O.MMA(n, 1, x)
    lo, hi = O.MMA.SetOuterMovelimit(0.0, 1.0, 0.2, x)
    mma.Update(x, np.ones(n) * 1e-3, np.array([0.0]), np.full(n, 1.0 / n), lo, hi)
    t_design = time.perf_counter() - t0
    t_iter = fixed + args.nsteps * per_step + t_design
    return {"value": 1.0 / t_iter, "unit": UNIT, "cores": int(os.environ.get("OMP_NUM_THREADS", ncores)),
            "kind": "port",
            "sample": "oracle (C, OpenMP) design iteration at horizons %s steps on the full %s mesh, per-step cost "
                      "extrapolated to %d steps, + filter/MMA at full size (%.1f s total)"
                      % (list(steps_small), args.mesh, args.nsteps, sum(t) + t_design),
            "seconds_per_design_iter": t_iter}


def run_reference(args):
    """Reference arm: the reference's algorithm restated on the CPU (the
    reference itself needs PETSc + MPI, absent here), timed on the host cores;
    each step is a bounded sample of the design iteration extrapolated to the
    full horizon."""
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    wl = workload(args)
    for _ in range(args.warmup):
        cpu_baseline(args, wl, steps_small=(1, 2))
    vals = []
    t0 = time.perf_counter()
    last = None
    for _ in range(args.steps):
        last = cpu_baseline(args, wl, steps_small=(1, 2))
        vals.append(last["value"])
    wall = time.perf_counter() - t0
    value = statistics.mean(vals)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic (uniform density 0.12, analytic load pulse)",
            "config": {"workload": workload_name(args), "mode": "CPU FP64 restatement of the reference",
                       "parallelism": "OpenMP host threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": last["cores"], "kind": "port",
                             "sample": last["sample"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mesh", default="96x48x48")
    ap.add_argument("--nsteps", type=int, default=200)
    ap.add_argument("--dt", type=float, default=0.005)
    ap.add_argument("--ncp", type=int, default=1)
    ap.add_argument("--nlvls", type=int, default=5)
    ap.add_argument("--smooth", type=int, default=3)
    ap.add_argument("--cheb-ratio", dest="cheb_ratio", type=float, default=30.0)
    ap.add_argument("--rtol", type=float, default=1e-10)
    ap.add_argument("--coarse-dense-max", dest="coarse_dense_max", type=int, default=4096)
    ap.add_argument("--coarse-smooth", dest="coarse_smooth", type=int, default=12)
    ap.add_argument("--sens-fp64", dest="sens_fp32", action="store_false",
                    help="FP64 element math in the sensitivity kernel of the mixed path (default FP32)")
    ap.add_argument("--inner-tol", dest="inner_tol", type=float, default=1e-5)
    ap.add_argument("--inner-maxit", dest="inner_maxit", type=int, default=40)
    ap.add_argument("--objective", type=int, default=3, help="0..6 reference objectives, 7 output-DOF displacement")
    ap.add_argument("--noise", type=float, default=0.0, help="seeded U(-a, a) noise on the initial design")
    ap.add_argument("--load2", action="store_true", help="seeded second point load with a seeded phase")
    ap.add_argument("--reduction", action="store_true", help="SOMMG reduced-order path")
    ap.add_argument("--basis", type=int, default=8, help="SOMMG basis vectors (with --reduction)")
    ap.add_argument("--omega0", type=float, default=1e-4,
                    help="SOMMG expansion frequency; below the first eigenfrequency for an SPD P0")
    ap.add_argument("--no-graphs", dest="no_graphs", action="store_true",
                    help="launch every kernel directly (profilers see each launch); same kernels")
    ap.add_argument("--plain-steps", dest="plain_steps", type=int, default=1)
    ap.add_argument("--e2e-steps", dest="e2e_steps", type=int, default=2)
    ap.add_argument("--no-cpu", dest="cpu_sample", action="store_false")
    ap.add_argument("--tile-form", dest="tile_form", type=int, default=0,
                    help="operator kernels: 0 bricks of 7x7x7 output nodes, 1 z-marching slabs")
    ap.add_argument("--kron-form", dest="kron_form", type=int, default=0,
                    help="Kronecker y/z passes: 0 lines staged in shared memory, 1 register line segments")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
