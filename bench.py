"""Throughput of the transient forward + adjoint design iteration on GB300.

Workload (the cantilever the headline metric is quoted on): 192x96x96 unit
hex8 elements (5,447,811 DOFs), E0 = 1, Emin = 1e-9, nu = 0.3, mass density 1,
SIMP p = 3, Rayleigh alpha = 0, beta = 1e-3, clamped face x = 0, line load at
the mid line of face x = nelx with f(t) = sin(2 pi t) for t < 0.5 plus a second
point load at a seeded node with a seeded phase, 400 Newmark steps of
dt = 0.0025 in 20 checkpoint blocks of 20 steps, initial density 0.12 plus
seeded U(-0.02, 0.02) noise, PDE filter radius 2, MMA, 6 multigrid levels.
Objective: reference objective 3 (potential energy, the reference-expressible
form of time-integrated compliance).  Synthetic inputs (no dataset is
involved).

A "step" is one design iteration of main.cc's loop: CompleteInitialState,
GenerateCheckPoints, ComputeObjectiveSensitivities (forward + adjoint +
sensitivities), VolumeConstraint, Filter::Gradients, MMA::Update,
Filter::FilterProject.

Besides the timed legs the line carries the accuracy of the mixed and plain
paths against the FP64 oracle on one full design evaluation of the
96x48x48 cantilever (200 steps, not extrapolated), and a central
finite-difference check of the adjoint sensitivities on seeded elements of
the headline workload.

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
    ("192x96x96", "k_tile<df,PolProduct>"): 57.80e6 + 7.868e6,
}
# warp instructions per launch of the instruction-issue-bound classes (ncu,
# smsp__inst_executed.sum of one launch; profiles/): the double-float tile
# kernels are bound by issue, not by HBM, and this is their roofline
ISSUE = {
    ("192x96x96", "k_tile<df,PolProduct>"): 208.4e6,
}
SMSP_PER_SM = 4  # warp schedulers per SM: one warp instruction each per clock
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
                noise=args.noise, **load2(args))


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


MAT6 = ("Emin", "Emax", "Rmin", "Rmax", "penalK", "penalM")


def make_physics(o, **over):
    """A LinearElasticity object for the TopOpt options `o` (the constructor
    call of main.cc:33), with solver options overridden by `over`."""
    from topopt_in_petsc_transient_gb300 import LinearElasticity
    kw = dict(nlvls=o.nlvls, ncp=o.ncp, tsc=o.tsc, t1=o.t1, objective=o.objective, dalpha=o.dalpha,
              dbeta=o.dbeta, loadsignal=o.loadsignal, mixed=o.mixed, rtol=o.rtol, smooth=o.smooth,
              cheb_ratio=o.cheb_ratio, use_graphs=o.use_graphs, coarse_dense_max=o.coarse_dense_max,
              coarse_smooth=o.coarse_smooth, sens_fp32=o.sens_fp32, inner_tol=o.inner_tol,
              inner_maxit=o.inner_maxit, reduction=o.reduction, basis=o.basis, omega0=o.omega0,
              load2_node=o.load2_node, load2_phase=o.load2_phase, out_dof=o.out_dof)
    kw.update(over)
    return LinearElasticity(o.nelx, o.nely, o.nelz, **kw)


def evaluate(ph, o, xPhys):
    """CompleteInitialState + GenerateCheckPoints + ComputeObjectiveSensitivities
    (main.cc:82-90) on device xPhys; returns (fx, dfdx tensor)."""
    import torch
    ph.CompleteInitialState(xPhys, *[getattr(o, k) for k in MAT6])
    ph.GenerateCheckPoints()
    df = torch.zeros_like(xPhys)
    fx = ph.ComputeObjectiveSensitivities(df)
    return fx, df


def timed_iterations(opt, k, flush_l2, events=True):
    """k design iterations, each bracketed by CUDA events after an L2 flush;
    returns the per-iteration seconds and objectives."""
    import torch

    from topopt_in_petsc_transient_gb300 import design_iteration
    times, fxs = [], []
    for _ in range(k):
        flush_l2()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push("timed_design_iteration")  # lets a profiler select the timed region
        e0.record()
        fx = design_iteration(opt)[0]  # every library call returns synchronised
        e1.record()
        e1.synchronize()
        torch.cuda.nvtx.range_pop()
        times.append(e0.elapsed_time(e1) / 1e3)
        fxs.append(fx)
    return times, fxs


def spread(times):
    return {"min_s": min(times), "median_s": statistics.median(times), "max_s": max(times)}


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
    xphys0 = opt.xPhys.clone()  # the filtered initial design (finite-difference check)
    raw = {}
    for w in range(args.warmup):
        if w == 0:  # the unscaled, unfiltered sensitivities of iteration 1 (mixed vs plain)
            raw["mixed"] = evaluate(opt.physics, opt, opt.xPhys)
        design_iteration(opt)
    le_stats0 = opt.physics.stats()
    launches0 = L.topo_kernel_launches()
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    times, fxs = timed_iterations(opt, args.steps, flush_l2)
    barrier()
    clocks = sampler.stop()
    le_stats1 = opt.physics.stats()
    launches = (L.topo_kernel_launches() - launches0) + (le_stats1["graph_body_launches"] -
                                                          le_stats0["graph_body_launches"])
    t_total = replica_time(sum(times), ws, "cuda")
    value = replica_value(args.steps, ws, t_total)
    iters_per_solve = ((le_stats1["cg_iterations"] - le_stats0["cg_iterations"]) /
                       max(1, le_stats1["solves"] - le_stats0["solves"]))
    replacements_per_solve = ((le_stats1["replacements"] - le_stats0["replacements"]) /
                              max(1, le_stats1["solves"] - le_stats0["solves"]))

    # ---- plain FP64 path: the same design iterations (after the same
    # number of warm-up iterations), and iteration 1's objective and
    # sensitivities against the mixed path's on the same initial design ----
    plain = None
    if args.plain_steps > 0:
        b = TopOpt(mixed=False, **wl).setup()
        for w in range(args.warmup):
            if w == 0:
                raw["plain"] = evaluate(b.physics, b, b.xPhys)
            design_iteration(b)
        tp, _ = timed_iterations(b, args.plain_steps, flush_l2)
        (fa, dfa), (fb, dfb) = raw["mixed"], raw["plain"]
        same = min(args.steps, args.plain_steps)
        plain = {"value": len(tp) / sum(tp), "unit": UNIT, "steps": len(tp), "warmup": args.warmup,
                 "iterations": "design iterations %d..%d, as the headline" % (args.warmup + 1,
                                                                             args.warmup + len(tp)),
                 "seconds": spread(tp), "mixed_seconds": spread(times),
                 "objective_rel_diff_mixed_vs_plain": abs(fa - fb) / abs(fb),
                 "dfdx_maxrel_diff_mixed_vs_plain": float((dfa - dfb).abs().max() / dfb.abs().max()),
                 "speedup_mixed_over_plain": value / ws / (len(tp) / sum(tp)),
                 "speedup_same_iterations": sum(tp[:same]) / sum(times[:same])}
        del b
    raw.clear()

    # ---- end to end through the C ABI with host buffers ----
    e2e = None
    if args.e2e_steps > 0:
        e2e = run_e2e(args, wl, flush_l2)

    # ---- roofline of the dominant kernels, timed in the solve ----
    roof = roofline(args, wl, opt) if args.roofline else None

    # ---- central finite differences of the adjoint sensitivities ----
    fd = None
    if args.fd_check > 0:
        fd = fd_check(args, opt, xphys0)
    del opt

    # ---- CPU legs: the bounded baseline sample, then the accuracy of both
    # GPU paths against one full (not extrapolated) oracle evaluation ----
    cpu = acc = None
    if rank == 0 and ws == 1:
        if args.cpu_sample:
            cpu = cpu_baseline(args, wl)
        if args.oracle_check:
            acc = oracle_accuracy(args)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded density noise and second load, analytic load pulse)" if args.noise > 0 else
                "synthetic (uniform density, analytic load pulse)",
        "config": {"workload": workload_name(args), "mode": "mixed: FP32 flexible-CG recurrence, Kronecker mass preconditioner (multigrid when the stiffness share is large), FP64-accurate residual replacements",
                   "dofs": 3 * (wl["nelx"] + 1) * (wl["nely"] + 1) * (wl["nelz"] + 1), "elements": opt_nel(wl),
                   "steps_per_design_iter": args.nsteps, "ncp": args.ncp,
                   "rtol": args.rtol, "smooth": args.smooth, "nlvls": args.nlvls,
                   "l2": "state history %.1f GB > 129 MB L2; 256 MB L2 flush between timed iterations"
                         % (3 * args.nsteps / args.ncp * 3 * (wl["nelx"] + 1) * (wl["nely"] + 1) * (wl["nelz"] + 1)
                            * 8 / 1e9),
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "objective": fxs[-1] if fxs else None, "seconds": spread(times), "krylov_iters_per_solve": iters_per_solve,
        "fp64_replacements_per_solve": replacements_per_solve,
        "dof_updates_per_s": 2.0 * 3 * (wl["nelx"] + 1) * (wl["nely"] + 1) * (wl["nelz"] + 1) * args.nsteps
                             * value / ws,
        "plain_fp64": plain, "accuracy_vs_oracle": acc, "fd_check": fd, "e2e": e2e, "roofline": roof,
        "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": int(launches),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def opt_nel(wl):
    return wl["nelx"] * wl["nely"] * wl["nelz"]


def roofline(args, wl, opt):
    """One extra design iteration per kernel class (outside the timed region,
    the same kernels launched directly instead of from CUDA graphs) brackets
    each launch of that class with CUDA events on the library stream;
    achieved = algorithmic bytes per launch / mean launch time."""
    import ctypes as C

    from topopt_in_petsc_transient_gb300 import TopOpt, design_iteration, _lib
    L = _lib.load()
    nel = opt_nel(wl)
    nn = (wl["nelx"] + 1) * (wl["nely"] + 1) * (wl["nelz"] + 1)
    import torch
    nsm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
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
    #   double-float products: FP64 x staged, FP64 y written (48 B/node);
    #     the replacement stages x and the mask, reads b and writes r
    #     (73 B/node); double-float factors (8 B each)
    classes = [(1, "k_tile<float,PolPQ32> (FCG operator product q = A p with p = z + beta p_prev, FP32)",
                49.0 * nn + 8.0 * nel),
               (2, "k_kron_pass<float> (one axis pass of the Kronecker mass inverse, 17-tap stencil, FP32)",
                (36.0 + 24.0 + 60.0) / 3.0 * nn),
               (0, "k_tile<float,PolCheb> (FP32 Chebyshev-Jacobi smoothing step)", 73.0 * nn + 8.0 * nel),
               (3, "k_tile<df,PolReplace> (FP64-accurate residual replacement: A x in double-float, then "
                   "r = b - A x, r.r and the convergence decision in the epilogue; launches without a due "
                   "replacement exit at once: algorithmic bytes per launch = bytes of a replacement x "
                   "replacements / launches)", 73.0 * nn + 16.0 * nel),
               (4, "k_tile<df,PolProduct> (double-float K or A products of right-hand sides, anchors and adjoint "
                   "steps)", 48.0 * nn + 8.0 * nel)]
    kern = []
    for cls, name, nbytes in classes:
        _lib.check(L.topo_le_kernel_timing(probe.physics._h, cls, 1, None, None), "kernel_timing")
        repl0 = probe.physics.stats()["replacements"]
        design_iteration(probe)
        tot_ms, nlaunch = C.c_double(), C.c_longlong()
        _lib.check(L.topo_le_kernel_timing(probe.physics._h, cls, 0, C.byref(tot_ms), C.byref(nlaunch)),
                   "kernel_timing")
        if nlaunch.value == 0:
            continue
        if cls == 3:  # only launches with a due replacement do the element work
            nbytes *= min(1.0, (probe.physics.stats()["replacements"] - repl0) / nlaunch.value)
        ms_launch = tot_ms.value / nlaunch.value
        ach = nbytes / (ms_launch * 1e-3) / 1e9
        entry = {"kernel": name, "bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                 "frac": ach / peaks["hbm_gbs"], "ms_per_launch": ms_launch, "launches_timed": nlaunch.value,
                 "ms_per_design_iter": tot_ms.value, "algorithmic_bytes": nbytes,
                 "traffic": TRAFFIC.get((args.mesh, name.split(" ")[0]))}
        ninst = ISSUE.get((args.mesh, name.split(" ")[0]))
        if ninst:
            issue_peak = nsm * SMSP_PER_SM * peaks["sm_max_mhz"] * 1e6
            entry["issue"] = {"warp_instructions_per_launch": ninst,
                              "achieved_warp_inst_per_s": ninst / (ms_launch * 1e-3),
                              "peak_warp_inst_per_s": issue_peak,
                              "frac": ninst / (ms_launch * 1e-3) / issue_peak,
                              "note": "instruction-issue bound (double-float arithmetic on the FP32 pipes); "
                                      "peak = SMs x 4 schedulers x max SM clock"}
        kern.append(entry)
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
    return roof


def fd_check(args, opt, xphys0):
    """Central differences (h = args.fd_h) of the objective on args.fd_check
    seeded elements of the filtered initial design against the adjoint
    sensitivities of the mixed path, solved to args.fd_rtol; one object,
    the same checkpointing as the headline.  Over this horizon the response
    decays exponentially away from the loads, so most elements change the
    objective by less than the solves resolve at this h; the seeded elements
    are drawn from those whose sensitivity is at least args.fd_floor of the
    largest."""
    import numpy as np
    t0 = time.perf_counter()
    ph = make_physics(opt, mixed=True, rtol=args.fd_rtol)
    x = xphys0.clone()
    fx, df = evaluate(ph, opt, x)
    dfh = df.cpu().numpy()
    rng = np.random.default_rng(0x7A11 + 32)
    pool = np.flatnonzero(np.abs(dfh) >= args.fd_floor * np.abs(dfh).max())
    els = sorted(int(e) for e in rng.choice(pool, min(args.fd_check, pool.size), replace=False))
    h = args.fd_h
    fd = []
    for e in els:
        x0 = float(x[e])
        x[e] = x0 + h
        fp = evaluate(ph, opt, x)[0]
        x[e] = x0 - h
        fm = evaluate(ph, opt, x)[0]
        x[e] = x0
        fd.append((fp - fm) / (2.0 * h))
    fd = np.array(fd)
    ad = dfh[els]
    dev = np.abs(fd - ad)
    scale = np.abs(ad).max()
    del ph
    return {"elements": len(els), "pool": int(pool.size), "pool_rule": "|dfdx_e| >= %g max|dfdx|" % args.fd_floor,
            "h": h, "rtol": args.fd_rtol, "seed": "0x7A11+32", "objective": fx,
            "max_abs_dev_over_max_abs_dfdx": float(dev.max() / scale),
            "max_rel_dev": float((dev / np.abs(ad)).max()), "median_rel_dev": float(np.median(dev / np.abs(ad))),
            "dfdx_range_sampled": [float(np.abs(ad).min()), float(scale)], "seconds": time.perf_counter() - t0,
            "path": "mixed (FP32 sensitivity element math)"}


def run_e2e(args, wl, flush_l2):
    """The same design iteration through the host-pointer C ABI (VecGetArray
    semantics): design vectors live in host memory; every call copies its
    inputs host->device and results device->host inside the timed region."""
    import numpy as np

    from topopt_in_petsc_transient_gb300 import MMA, Filter, TopOpt
    o = TopOpt(mixed=True, **wl)
    n = o.nel
    ph = make_physics(o)
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
        df *= fscale  # VecScale on the host vector (main.cc:121)
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
            "steps": len(times), "seconds": spread(times),
            "timer": "host wall clock around the synchronous C-ABI calls"}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            hbm = d.get("hbm_gbs") or d.get("hbm_GBps") or d.get("hbm")
            if isinstance(hbm, dict):
                hbm = hbm.get("value")
            if hbm:
                return {"hbm_gbs": float(hbm), "source": "measured (MEASURED_PEAKS.json)",
                        "sm_max_mhz": float(d.get("sm_max_mhz") or 2070.0)}
        except (ValueError, OSError):
            pass
    return {"hbm_gbs": 6800.0, "source": "fallback 6.8 TB/s", "sm_max_mhz": 2070.0}


def oracle_le(wl, steps, dt, rtol):
    """The oracle's LinearElasticity for the workload's physics over `steps`
    Newmark steps in one block."""
    from oracle import oracle as O
    return O.LinearElasticity(wl["nelx"], wl["nely"], wl["nelz"], ncp=1, tsc=steps, t1=dt * steps,
                              objective=wl["objective"], loadsignal=wl["loadsignal"], dalpha=wl["dalpha"],
                              dbeta=wl["dbeta"], rtol=rtol, Emin=wl["Ef"] * wl["Emax"], Emax=wl["Emax"],
                              Rmin=wl["Rf"] * wl["Rmax"], Rmax=wl["Rmax"], load2_node=wl.get("load2_node", -1),
                              load2_phase=wl.get("load2_phase", 0.0))


def oracle_design_x(wl, noise, seed=0x7A11):
    import numpy as np
    n = opt_nel(wl)
    x = np.full(n, wl["V0"])
    if noise > 0.0:
        x += np.random.default_rng(seed).uniform(-noise, noise, n)
    return x


def oracle_physics_seconds(wl, steps, dt, rtol, x):
    le = oracle_le(wl, steps, dt, rtol)
    t0 = time.perf_counter()
    rc, fx, df = le.objective_sensitivities(x)
    return time.perf_counter() - t0, rc, fx, df


def oracle_design_seconds(wl, x):
    """Filter, filter chain rule and MMA of one design iteration in the oracle."""
    import numpy as np

    from oracle import oracle as O
    nx, ny, nz = wl["nelx"], wl["nely"], wl["nelz"]
    n = nx * ny * nz
    t0 = time.perf_counter()
    xt, xp = O.filter_project(nx, ny, nz, x, wl["rmin"], False, 0.1, 0.15, rtol=1e-8)
    O.filter_gradients(nx, ny, nz, xt, np.ones(n), np.full(n, 1.0 / n), wl["rmin"], False, 0.1, 0.15, rtol=1e-8)
    mma = O.MMA(n, 1, x)
    lo, hi = O.MMA.SetOuterMovelimit(0.0, 1.0, 0.2, x)
    mma.Update(x.copy(), np.ones(n) * 1e-3, np.array([0.0]), np.full(n, 1.0 / n), lo, hi)
    return time.perf_counter() - t0


def extrapolated_seconds(wl, nsteps, dt, rtol, x, horizons=(2, 4)):
    """The oracle design evaluation at two short horizons on the full mesh,
    extrapolated linearly to nsteps (every step costs the same)."""
    t = [oracle_physics_seconds(wl, s, dt, rtol, x)[0] for s in horizons]
    per_step = (t[1] - t[0]) / (horizons[1] - horizons[0])
    fixed = t[0] - horizons[0] * per_step
    return fixed + nsteps * per_step, sum(t)


def cpu_baseline(args, wl, horizons=(2, 4)):
    """The oracle (CPU FP64 restatement of the reference path: assembled
    27-point block operators, Jacobi-PCG, the reference's dense 24x24 element
    loops) on the host cores, on a bounded sample of the same workload: the
    design evaluation at horizons of 2 and 4 steps on the full mesh,
    extrapolated linearly to the full horizon, plus filter and MMA at full
    size.  The extrapolation is checked against one full oracle evaluation
    in oracle_accuracy."""
    ncores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(ncores))
    x = oracle_design_x(wl, args.noise)
    t_phys, t_sample = extrapolated_seconds(wl, args.nsteps, args.dt, 1e-10, x, horizons)
    t_design = oracle_design_seconds(wl, x)
    t_iter = t_phys + t_design
    return {"value": 1.0 / t_iter, "unit": UNIT, "cores": int(os.environ.get("OMP_NUM_THREADS", ncores)),
            "kind": "port",
            "sample": "oracle (C, OpenMP, Jacobi-PCG at rtol 1e-10) design evaluation at horizons %s steps on the "
                      "full %s mesh, per-step cost extrapolated to %d steps, + filter/MMA at full size (%.1f s total)"
                      % (list(horizons), args.mesh, args.nsteps, t_sample + t_design),
            "seconds_per_design_iter": t_iter}


def oracle_accuracy(args):
    """Objective and sensitivity error of the mixed and the plain GPU path
    against the FP64 oracle on one full design evaluation (all steps, not
    extrapolated) of the accuracy workload (default: the 96x48x48 cantilever,
    200 steps of dt = 0.005, 5 levels, uniform density 0.12, the same pulse
    and objective), both GPU paths at the headline rtol, the oracle at
    args.oracle_rtol.  The same run times the full oracle design iteration
    and checks the linear extrapolation the CPU baseline uses."""
    import numpy as np
    import torch

    from topopt_in_petsc_transient_gb300 import TopOpt
    ncores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(ncores))
    a = argparse.Namespace(**vars(args))
    a.mesh, a.nsteps, a.dt, a.nlvls, a.ncp = args.oracle_mesh, args.oracle_nsteps, args.oracle_dt, \
        args.oracle_nlvls, 1
    a.noise, a.load2 = 0.0, False
    wl = workload(a)
    o = TopOpt(**wl)
    x = oracle_design_x(wl, 0.0)
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    res = {}
    for name, mixed in (("mixed", True), ("plain", False)):
        ph = make_physics(o, mixed=mixed)
        t0 = time.perf_counter()
        fx, df = evaluate(ph, o, xd)
        torch.cuda.synchronize()
        res[name] = (fx, df.cpu().numpy(), time.perf_counter() - t0)
        del ph
    t_full, rc, fx_o, df_o = oracle_physics_seconds(wl, a.nsteps, a.dt, args.oracle_rtol, x)
    t_ext, _ = extrapolated_seconds(wl, a.nsteps, a.dt, args.oracle_rtol, x)
    t_design = oracle_design_seconds(wl, x)
    out = {"workload": workload_name(a), "oracle_rtol": args.oracle_rtol, "gpu_rtol": args.rtol,
           "oracle_status": rc, "objective_oracle": fx_o,
           "oracle_seconds_full_design_iteration": t_full + t_design,
           "oracle_seconds_extrapolated_from_2_and_4_steps": t_ext + t_design,
           "cores": int(os.environ.get("OMP_NUM_THREADS", ncores))}
    scale = np.abs(df_o).max()
    for name, (fx, df, tg) in res.items():
        out[name] = {"objective": fx, "objective_rel_err_vs_oracle": abs(fx - fx_o) / abs(fx_o),
                     "dfdx_maxrel_err_vs_oracle": float(np.abs(df - df_o).max() / scale),
                     "gpu_seconds_first_evaluation": tg}
    return out


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
        cpu_baseline(args, wl, horizons=(1, 2))
    vals = []
    t0 = time.perf_counter()
    last = None
    for _ in range(args.steps):
        last = cpu_baseline(args, wl, horizons=(1, 2))
        vals.append(last["value"])
    wall = time.perf_counter() - t0
    value = statistics.mean(vals)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic (seeded density noise and second load, analytic load pulse)",
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
    ap.add_argument("--mesh", default="192x96x96")
    ap.add_argument("--nsteps", type=int, default=400)
    ap.add_argument("--dt", type=float, default=0.0025)
    ap.add_argument("--ncp", type=int, default=20)
    ap.add_argument("--nlvls", type=int, default=6)
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
    ap.add_argument("--noise", type=float, default=0.02, help="seeded U(-a, a) noise on the initial design")
    ap.add_argument("--no-load2", dest="load2", action="store_false",
                    help="without the seeded second point load")
    ap.add_argument("--reduction", action="store_true", help="SOMMG reduced-order path")
    ap.add_argument("--basis", type=int, default=8, help="SOMMG basis vectors (with --reduction)")
    ap.add_argument("--omega0", type=float, default=1e-4,
                    help="SOMMG expansion frequency; below the first eigenfrequency for an SPD P0")
    ap.add_argument("--no-graphs", dest="no_graphs", action="store_true",
                    help="launch every kernel directly (profilers see each launch); same kernels")
    ap.add_argument("--plain-steps", dest="plain_steps", type=int, default=None,
                    help="timed plain FP64 iterations (default: --steps)")
    ap.add_argument("--e2e-steps", dest="e2e_steps", type=int, default=2)
    ap.add_argument("--no-cpu", dest="cpu_sample", action="store_false")
    ap.add_argument("--no-roofline", dest="roofline", action="store_false",
                    help="skip the per-kernel-class timing iterations")
    ap.add_argument("--no-oracle-check", dest="oracle_check", action="store_false",
                    help="skip the full oracle evaluation of the accuracy workload")
    ap.add_argument("--oracle-mesh", dest="oracle_mesh", default="96x48x48")
    ap.add_argument("--oracle-nsteps", dest="oracle_nsteps", type=int, default=200)
    ap.add_argument("--oracle-dt", dest="oracle_dt", type=float, default=0.005)
    ap.add_argument("--oracle-nlvls", dest="oracle_nlvls", type=int, default=5)
    ap.add_argument("--oracle-rtol", dest="oracle_rtol", type=float, default=1e-12)
    ap.add_argument("--fd-check", dest="fd_check", type=int, default=32,
                    help="seeded elements of the central finite-difference check (0: skip)")
    ap.add_argument("--fd-h", dest="fd_h", type=float, default=1e-4)
    ap.add_argument("--fd-rtol", dest="fd_rtol", type=float, default=1e-12)
    ap.add_argument("--fd-floor", dest="fd_floor", type=float, default=0.01,
                    help="finite differences on elements with |dfdx| >= this fraction of max|dfdx|")
    args = ap.parse_args()
    if args.plain_steps is None:
        args.plain_steps = args.steps
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
