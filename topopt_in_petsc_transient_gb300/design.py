"""TopOpt-style configuration and the main.cc design iteration on the GPU path.

`TopOpt` holds the parameters TopOpt::SetUp/SetUpOPT read from the PETSc
options database (TopOpt.cc:71-518) and the design vectors as device tensors.
`design_iteration` performs one pass of the optimisation loop of main.cc:82-154
with the same call order: CompleteInitialState, GenerateCheckPoints,
ComputeObjectiveSensitivities, VolumeConstraint, Filter::Gradients, design
output, objective scaling, SetOuterMovelimit, MMA::Update, DesignChange,
IncreaseBeta, Filter::FilterProject; `final_physics_output` is the physics
output of the final design after the loop.
"""
from dataclasses import dataclass, field


@dataclass
class TopOpt:
    nelx: int = 64
    nely: int = 32
    nelz: int = 32
    h: tuple = (1.0, 1.0, 1.0)
    nu: float = 0.3
    nlvls: int = 4
    volfrac: float = 0.3
    V0: float = None
    maxItr: int = 10
    rmin: float = 1.5
    penalK: float = 3.0
    penalM: float = 1.0
    Emax: float = 1e3
    Ef: float = 1e-9
    Rmax: float = 4.16666666667e-4
    Rf: float = 1e-3
    filter: int = 2
    sInt: int = 1
    mInt: int = 0
    Xmin: float = 0.0
    Xmax: float = 1.0
    movlim: float = 0.2
    ti: int = 1
    t1: float = 50.0
    ncp: int = 2
    tsc: int = 25
    dalpha: float = 1e-4
    dbeta: float = 1e-4
    objective: int = 0
    minmax: int = -1
    boundaries: int = 1
    loadloc: int = 1
    optimizationRegion: int = 2
    projectionFilter: bool = True
    beta: float = 0.1
    betaFinal: float = 48.0
    eta: float = 0.15
    loadsignal: int = 0
    m: int = 1
    # GB300 solver controls
    mixed: bool = True
    rtol: float = 1e-10
    filter_rtol: float = 1e-10
    smooth: int = 3
    cheb_ratio: float = 30.0
    use_graphs: bool = True
    coarse_dense_max: int = 4096
    coarse_smooth: int = 12
    sens_fp32: bool = True
    inner_tol: float = 1e-5
    inner_maxit: int = 40
    adaptive_kappa: float = 40.0
    extrapolate: int = 2
    mass_precond: int = 2
    reduction: bool = False  # TopOpt.cc:157-159
    basis: int = 5
    omega0: float = 1.0
    load2_node: int = -1  # workload extensions (second point load, objective 7 output DOF)
    load2_phase: float = 0.0
    out_dof: int = -1
    noise: float = 0.0  # initial design V0 + U(-noise, noise) from a generator seeded with seed
    seed: int = 0x7A11
    mass_precond_smooth: int = 0
    # result files (TopOpt.cc:474-482 -outputDesign/-outputPhysics0/-outputPhysics1,
    # on by default in the reference, opt-in here) under ./workdir (-workdir)
    outputDesign: bool = False
    outputPhysics0: bool = False
    outputPhysics1: bool = False
    workdir: str = None
    xc: tuple = None  # node box (xmin, xmax, ymin, ymax, zmin, zmax); default origin to nel * h
    # state
    fscale: float = 1.0
    itr: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def Emin(self):
        return self.Ef * self.Emax  # TopOpt.cc:472

    @property
    def Rmin(self):
        return self.Rf * self.Rmax  # TopOpt.cc:474

    @property
    def nel(self):
        return self.nelx * self.nely * self.nelz

    def setup(self, device="cuda"):
        """Allocates design vectors (TopOpt::SetUpOPT, TopOpt.cc:495-515) and
        the physics, filter and MMA objects (main.cc:35-58)."""
        import torch

        from .topopt import MMA, Filter, LinearElasticity
        V0 = self.volfrac if self.V0 is None else self.V0
        n = self.nel
        f64 = dict(dtype=torch.float64, device=device)
        self.x = torch.full((n,), V0, **f64)
        if self.noise > 0.0:
            import numpy as np
            rng = np.random.default_rng(self.seed)
            self.x += torch.tensor(rng.uniform(-self.noise, self.noise, n), **f64)
        self.xTilde = torch.full((n,), V0, **f64)
        self.xPhys = torch.full((n,), V0, **f64)
        self.xold = self.x.clone()
        self.dfdx = torch.zeros(n, **f64)
        self.dgdx = torch.zeros(self.m * n, **f64)
        self.xmin = torch.zeros(n, **f64)
        self.xmax = torch.zeros(n, **f64)
        self.physics = LinearElasticity(
            self.nelx, self.nely, self.nelz, nu=self.nu, nlvls=self.nlvls, ncp=self.ncp, tsc=self.tsc, t1=self.t1,
            ti=self.ti, objective=self.objective, stiffnessInterpolation=self.sInt, massInterpolation=self.mInt,
            boundaries=self.boundaries, loadloc=self.loadloc, dalpha=self.dalpha, dbeta=self.dbeta,
            optimizationRegion=self.optimizationRegion, h=self.h, loadsignal=self.loadsignal, mixed=self.mixed,
            rtol=self.rtol, smooth=self.smooth, cheb_ratio=self.cheb_ratio, use_graphs=self.use_graphs,
            coarse_dense_max=self.coarse_dense_max, coarse_smooth=self.coarse_smooth, sens_fp32=self.sens_fp32,
            inner_tol=self.inner_tol, inner_maxit=self.inner_maxit, adaptive_kappa=self.adaptive_kappa,
            extrapolate=self.extrapolate, mass_precond=self.mass_precond,
            mass_precond_smooth=self.mass_precond_smooth, reduction=self.reduction, basis=self.basis,
            omega0=self.omega0, load2_node=self.load2_node, load2_phase=self.load2_phase, out_dof=self.out_dof)
        self.filt = Filter(self.nelx, self.nely, self.nelz, self.filter, self.rmin, h=self.h, rtol=self.filter_rtol)
        # result files (main.cc:38-49): design fields per iteration, the physics
        # of the first iteration and of the final design
        from .topopt import MPIIO
        kw = dict(xc=self.xc, workdir=self.workdir)
        self.output1 = MPIIO(self, 0, "", 3, "x, xTilde, xPhys", "outputDesign_00000.dat", **kw) \
            if self.outputDesign else None
        self.output2 = MPIIO(self, 3, "ux, uy, uz", 1, "xPhys", "outputPhysics0_00000.dat", **kw) \
            if self.outputPhysics0 else None
        self.output3 = MPIIO(self, 3, "ux, uy, uz", 1, "xPhys", "outputPhysics1_00000.dat", **kw) \
            if self.outputPhysics1 else None
        self.firstIterWrite = True  # main.cc:69-70
        self.mma = MMA(n, self.m, self.x)
        self.mma.SetAsymptotes(0.1, 0.6, 1.05)  # main.cc:58
        self.filt.FilterProject(self.x, self.xTilde, self.xPhys, self.projectionFilter, self.beta, self.eta)
        return self


def design_iteration(opt: TopOpt):
    """One iteration of the main.cc optimisation loop (main.cc:76-160);
    returns (fx_true, fx_scaled, gx0, ch, mnd)."""
    from .topopt import VecScale
    opt.itr += 1
    ph = opt.physics
    w, out2 = getattr(opt, "firstIterWrite", False), getattr(opt, "output2", None)
    ph.CompleteInitialState(opt.xPhys, opt.Emin, opt.Emax, opt.Rmin, opt.Rmax, opt.penalK, opt.penalM,
                            write=w, output=out2)
    if opt.ncp > 1:
        ph.GenerateCheckPoints(w, opt.xPhys, out2)
    fx = ph.ComputeObjectiveSensitivities(opt.dfdx, write=w, output=out2)
    gx0 = ph.VolumeConstraint(opt.dgdx, opt.xPhys, opt.volfrac)
    opt.filt.Gradients(opt.x, opt.xTilde, opt.dfdx, opt.m, opt.dgdx, opt.projectionFilter, opt.beta, opt.eta)
    opt.firstIterWrite = False
    if getattr(opt, "output1", None) is not None:  # design output (main.cc:102-105)
        opt.output1.WriteVTK(opt.x, opt.xTilde, opt.xPhys, opt.itr)
    mnd = opt.filt.GetMND(opt.xPhys)
    if opt.itr == 1:
        opt.fscale = 1.0 / fx
    fxs = fx * opt.fscale
    VecScale(opt.dfdx, opt.fscale)
    opt.mma.SetOuterMovelimit(opt.Xmin, opt.Xmax, opt.movlim, opt.x, opt.xmin, opt.xmax)
    if opt.minmax == 1:
        VecScale(opt.dfdx, -1.0)
    opt.mma.Update(opt.x, opt.dfdx, [gx0], opt.dgdx, opt.xmin, opt.xmax)
    ch = opt.mma.DesignChange(opt.x, opt.xold)
    if opt.projectionFilter and (opt.itr >= 200 or ch < 0.01):
        changed, opt.beta = opt.filt.IncreaseBeta(opt.beta, opt.betaFinal, gx0, opt.itr, ch)
        if changed:
            ch = 1.0
    if gx0 > 0:
        ch = 1.0
    opt.filt.FilterProject(opt.x, opt.xTilde, opt.xPhys, opt.projectionFilter, opt.beta, opt.eta)
    return fx, fxs, gx0, ch, mnd


def final_physics_output(opt: TopOpt):
    """The physics of the final design into outputPhysics1 (main.cc:163-176):
    CompleteInitialState, GenerateCheckPoints and ComputeObjectiveSensitivities
    with write set; returns the objective.  Flushes every result file."""
    ph = opt.physics
    out3 = getattr(opt, "output3", None)
    ph.CompleteInitialState(opt.xPhys, opt.Emin, opt.Emax, opt.Rmin, opt.Rmax, opt.penalK, opt.penalM,
                            write=True, output=out3)
    if opt.ncp > 1:
        ph.GenerateCheckPoints(True, opt.xPhys, out3)
    fx = ph.ComputeObjectiveSensitivities(opt.dfdx, write=True, output=out3)
    for out in (getattr(opt, "output1", None), getattr(opt, "output2", None), out3):
        if out is not None:
            out.Flush()
    return fx


def write_restart_files(opt: TopOpt, directory):
    """TopOpt::WriteRestartFiles (TopOpt.cc:678-735): MMA::Restart, then x, xPhys,
    xo1, xo2, U, L into Restart00.dat / Restart01.dat (the two sets alternate)
    and "itr fscale" into Restart0x_itr_f0.dat.  Returns the vector file."""
    import os

    import torch

    from .topopt import write_petsc_vecs
    st = [torch.zeros_like(opt.x) for _ in range(4)]
    opt.mma.Restart(*st)
    opt.flip = not getattr(opt, "flip", True)  # TopOpt.cc:535, :691-695
    tag = "01" if opt.flip else "00"
    vec = os.path.join(directory, "Restart%s.dat" % tag)
    write_petsc_vecs(vec, [opt.x, opt.xPhys] + st)
    with open(os.path.join(directory, "Restart%s_itr_f0.dat" % tag), "w") as f:
        f.write("%d %1.16e\n" % (opt.itr, opt.fscale))
    return vec


def load_restart(opt: TopOpt, vec_file, itr_file=None, only_load_design=False, load_design=0):
    """The -restartFileVec branch of TopOpt::AllocateMMAwithRestart
    (TopOpt.cc:600-670) on a set-up TopOpt: loads x, xPhys, xo1, xo2, U, L.
    With only_load_design the design seeds a fresh MMA (load_design 2: xPhys
    becomes x); otherwise xold = x, itr and fscale come from itr_file and MMA
    continues through its restart constructor."""
    import torch

    from .topopt import MMA, read_petsc_vecs
    st = [torch.zeros_like(opt.x) for _ in range(4)]
    read_petsc_vecs(vec_file, [opt.x, opt.xPhys] + st)
    if only_load_design:
        if load_design == 2:
            opt.x.copy_(opt.xPhys)
        opt.mma = MMA(opt.nel, opt.m, opt.x)
    else:
        opt.xold.copy_(opt.x)
        with open(itr_file) as f:
            tok = f.read().split()
        opt.itr, opt.fscale = int(tok[0]), float(tok[1])
        opt.mma = MMA(opt.nel, opt.m, itr=opt.itr, xo1=st[0], xo2=st[1], U=st[2], L=st[3])
    opt.mma.SetAsymptotes(0.1, 0.6, 1.05)  # main.cc:58
    return opt
