/*
 * topopt_gb300.h -- C ABI of the GB300 transient solve-and-sensitivity path.
 *
 * Drop-in boundary for the classes TopOpt_in_PETSc_Transient's main.cc calls
 * on its hot path (LinearElasticity, PDEFilt/Filter, MMA).  Every entry point
 * takes plain pointers and sizes and returns an int status (0 = TOPO_OK).
 * Host-pointer entry points take arrays exactly as VecGetArray() hands them out
 * on one rank: DMDA natural ordering, node (i,j,k) -> i + nx*(j + ny*k),
 * displacement DOF 3*node + component, element (i,j,k) -> i + (nx-1)*(j + (ny-1)*k).
 * The *_dev variants take device pointers of the same layout.
 * All computation runs on the current CUDA device; there is no CPU fallback:
 * without a usable GPU every compute entry point returns TOPO_ERR_CUDA.
 */
#ifndef TOPOPT_GB300_H
#define TOPOPT_GB300_H
#ifdef __cplusplus
extern "C" {
#endif

/* status codes (PetscErrorCode-compatible: 0 = success) */
#define TOPO_OK 0
#define TOPO_ERR_ARG 1            /* invalid argument / unsupported option       */
#define TOPO_ERR_CUDA 2           /* CUDA runtime error or no device             */
#define TOPO_ERR_OOM 3            /* device allocation failed                    */
#define TOPO_ERR_NOT_CONVERGED 4  /* Krylov solve hit maxit                      */
#define TOPO_ERR_BREAKDOWN 5      /* non-positive curvature in CG                */
#define TOPO_ERR_NAN 6            /* NaN/Inf encountered                         */
#define TOPO_ERR_STATE 7          /* call order violated                         */
#define TOPO_ERR_SYNC_TIMEOUT 8   /* a bounded device-side wait gave up          */

typedef struct topo_le topo_le;
typedef struct topo_pdefilt topo_pdefilt;
typedef struct topo_mma topo_mma;
typedef struct topo_mpiio topo_mpiio;

/* Parameters of LinearElasticity(...) (LinearElasticity.h:29) plus the mesh
 * geometry the reference reads off its DMDA (SetUpBC, LinearElasticity.cc:337-391)
 * and the GB300 solver controls. */
typedef struct topo_le_params {
    int nx, ny, nz;          /* nodes per direction (-nx -ny -nz)                  */
    double hx, hy, hz;       /* element size                                        */
    double nu;               /* Poisson ratio (-nu)                                 */
    int nlvls;               /* multigrid levels (-nlvls)                           */
    int ncp, tsc;            /* checkpoint blocks, steps per block (-ncp -tsc)      */
    double t1;               /* final time (-t1), dt = t1/(ncp*tsc)                 */
    int ti;                  /* 0 backward Euler, 1 Newmark (-ti)                   */
    int objective;           /* 0..6 (-objective)                                   */
    int sInt, mInt;          /* interpolation (-sInt, -massInterpolation)           */
    int boundaries;          /* 0 MBB, 1 cantilever (-boundaries)                   */
    int loadloc;             /* 0 MBB, 1 cantilever (-loadloc)                      */
    int optregion;           /* 0..3 (-optimizationRegion)                          */
    int loadsignal;          /* 0 reference pulse (LinearElasticity.cc:597-606),
                                1 sin(2 pi t) for t < 0.5                          */
    double dalpha, dbeta;    /* Rayleigh damping (-dalph, -dbeta)                   */
    /* GB300 solver controls */
    int mixed;               /* 1: FP32 multigrid inside FP64 flexible CG           */
    double rtol;             /* relative residual of every solve (reference 1e-10)  */
    int maxit;               /* Krylov iteration cap                                */
    int smooth;              /* Chebyshev degree of pre/post smoothing              */
    double cheb_ratio;       /* Chebyshev lower bound = max(lo_bound, hi/ratio)     */
    int use_graphs;          /* 1: CUDA graphs with device-side loop control        */
    int coarse_dense_max;    /* coarsest level solved by a dense inverse from an
                                FP64 Cholesky factor when it has at most this
                                many DOFs, otherwise by Chebyshev-Jacobi
                                smoothing                                         */
    int coarse_smooth;       /* Chebyshev degree of the iterative coarse solve      */
    int sens_fp32;           /* mixed mode: FP32 element math in the sensitivity
                                kernel (state combinations still formed in FP64)  */
    double inner_tol;        /* mixed mode: FP32 recurrence residual reduction
                                between FP64 residual replacements                */
    int inner_maxit;         /* mixed mode: FP32 iterations between replacements    */
    double adaptive_kappa;   /* V-cycle depth: descend only while the Jacobi-scaled
                                operator's condition bound exceeds this; a level
                                below it is solved by a full-spectrum Chebyshev
                                polynomial (mass-dominated Newmark operators need
                                no coarse correction); 0 = always full depth      */
    int extrapolate;         /* initial guesses of the step solves: 0 = the Newmark
                                predictor u + dt v + dt^2/4 a and lambda+;
                                1 = u + dt v + dt^2/2 a (acceleration held) and
                                2 lambda+ - lambda++; 2 = u + dt v + dt^2/4 (3a - a-)
                                (acceleration extrapolated) and
                                3 lambda+ - 3 lambda++ + lambda+++               */
    int mass_precond;        /* preconditioner of the step solves: 0 = multigrid
                                V-cycle with Chebyshev-Jacobi smoothing, 1 =
                                Kronecker mass preconditioner (tensor product of
                                1-D tridiagonal mass solves, density scaled),
                                2 = the Kronecker one whenever the operator's
                                stiffness share is at most mass_precond_share   */
    double mass_precond_share; /* bound on (sK/sM) max_e(kf_e/mf_e) lambda_max(KE,ME)
                                for mass_precond = 2                              */
    int mass_precond_smooth; /* Chebyshev-Jacobi steps (full spectrum of Dinv A)
                                applied after the Kronecker solve; they remove
                                the error of its density scaling where the
                                design varies sharply                             */
    int reduction;           /* 1: SOMMG reduced-order path (-reduction)            */
    int basis;               /* basis vectors of the reduction, 1..32 (-basis)      */
    double omega0;           /* expansion frequency om of P0 = K - om^2 M (-omega0) */
    /* workload extensions with no counterpart in the reference options:
     * a second point load in z at node load2_node (-1: none), signal
     * sin(2 pi t + load2_phase) for t < 0.5 scaled like the line load;
     * objective 7 = sum_t dt/2 u_out^2 of one output DOF (out_dof, -1: the z
     * DOF of the tip-centre node).  Neither combines with reduction = 1. */
    int load2_node;
    double load2_phase;
    int out_dof;
} topo_le_params;

typedef struct topo_le_stats {
    long long cg_iterations;  /* outer Krylov iterations since creation */
    long long solves;         /* linear solves since creation           */
    double device_bytes;      /* HBM held by the object                 */
    double last_fx;           /* last objective                         */
    long long graph_body_launches; /* kernels run inside device-side Krylov loops */
    long long mg_solves;      /* solves preconditioned by the multigrid V-cycle */
    int step_precond;         /* preconditioner of the current design's Newmark
                                 step solves: 0 multigrid V-cycle, 1 Kronecker
                                 mass preconditioner, -1 before the first design */
    long long replacements;   /* FP64-accurate residual replacements of the
                                 mixed-precision solves since creation */
} topo_le_stats;

/* fills p with the reference defaults for a cantilever of nelx x nely x nelz
 * unit elements (TopOpt.cc:75-159) and the GB300 solver defaults */
void topo_le_default_params(topo_le_params *p, int nelx, int nely, int nelz);

/* LinearElasticity::LinearElasticity, LinearElasticity.h:29 / LinearElasticity.cc:13-127 */
int topo_le_create(topo_le **out, const topo_le_params *p);
/* LinearElasticity::~LinearElasticity */
void topo_le_destroy(topo_le *le);

/* LinearElasticity::CompleteInitialState, LinearElasticity.h:81 / .cc:956-1206 */
int topo_le_complete_initial_state(topo_le *le, const double *xPhys, double Emin, double Emax, double Rmin,
                                   double Rmax, double penalK, double penalM);
int topo_le_complete_initial_state_dev(topo_le *le, const double *xPhys_dev, double Emin, double Emax,
                                       double Rmin, double Rmax, double penalK, double penalM);
/* LinearElasticity::GenerateCheckPoints, LinearElasticity.h:83 / .cc:1208-1280 */
int topo_le_generate_checkpoints(topo_le *le);
/* LinearElasticity::ComputeObjectiveSensitivities, LinearElasticity.h:42 / .cc:1625-1908.
 * Overwrites *fx and dfdx (nel values).  Material parameters are the ones of
 * the preceding CompleteInitialState (main.cc passes the same values). */
int topo_le_compute_objective_sensitivities(topo_le *le, double *fx, double *dfdx);
int topo_le_compute_objective_sensitivities_dev(topo_le *le, double *fx, double *dfdx_dev);
/* LinearElasticity::VolumeConstraint, LinearElasticity.h:85 / .cc:1283-1296 */
int topo_le_volume_constraint(topo_le *le, double *gx, double *dgdx, const double *xPhys, double volfrac);
int topo_le_volume_constraint_dev(topo_le *le, double *gx, double *dgdx_dev, const double *xPhys_dev,
                                  double volfrac);

/* Allocation-free volume constraint.  No counterpart in the reference: it
 * computes what LinearElasticity::VolumeConstraint (LinearElasticity.cc:1283-1296)
 * and topo_le_volume_constraint_dev compute, gx = mean(xPhys) - volfrac and
 * dgdx = 1/nel, without a topo_le object and without allocating device memory
 * (its reduction scratch is a fixed 64 KB static device array).  For callers
 * that hold only design vectors and may not allocate.  nel must be in
 * 1..16,777,216 (TOPO_ERR_ARG otherwise).  The first call on a device looks up
 * the scratch address and should come before any stream capture.  Calls that
 * overlap in time on one device share the scratch and race; each call runs on
 * the legacy default stream and returns after gx has been copied to the host.
 * The legacy stream does not wait for work on non-blocking streams: xPhys_dev
 * must be complete (its producing stream synchronised) before the call, as for
 * topo_le_volume_constraint_dev. */
int topo_volume_constraint_noalloc_dev(long long nel, double *gx, double *dgdx_dev, const double *xPhys_dev,
                                       double volfrac);

/* VecScale(dfdx, alpha) of the design loop (main.cc:121, :127: the objective
 * scaling fscale and the sign flip of -minmax 1) on a device vector of n
 * values, x <- alpha x; runs on the legacy default stream and returns after
 * the kernel has finished. */
int topo_vec_scale_dev(double *x_dev, long long n, double alpha);

/* inspection (tests / output): which = 0 U, 1 DU, 2 DDU of step j of the
 * resident block (j = -1: block start state); copies 3*nn values to host */
int topo_le_get_state(topo_le *le, int which, int j, double *out);
/* checkpoint c (0 <= c < ncp: the state at the start of block c; c = 0 the
 * initial state of CompleteInitialState) into host arrays of ndof values: the
 * three vectors the reference writes to cp%04d.dat (LinearElasticity.cc:1134-1136)
 * and GenerateCheckPoints' later files.  Checkpoints 1..ncp-1 are valid after
 * GenerateCheckPoints. */
int topo_le_get_checkpoint(topo_le *le, int c, double *U, double *DU, double *DDU);
/* initial displacement U0 (ndof values, DMDA order) for the next
 * CompleteInitialState instead of rest: LinearElasticity::LoadSolutionAsU0
 * with -onlyLoadDesign -solutionAsU0 (LinearElasticity.cc:2621-2677; U0 is the
 * first record of the -restartFileVecSol file).  U0 = NULL restores u0 = 0.
 * Full path only (the reduced path starts from rest). */
int topo_le_set_initial_displacement(topo_le *le, const double *U0, int on_device);
/* the vectors of LinearElasticity::WriteRestartFiles (RestartSol0x.dat,
 * LinearElasticity.cc:2457-2496) into host arrays of ndof values: DDU0 the
 * initial acceleration, LT the terminal adjoint of the last reverse sweep,
 * DDL0 the adjoint acceleration at t = 0.  Full path only. */
int topo_le_get_restart_state(topo_le *le, double *DDU0, double *LT, double *DDL0);
/* weighted products K x and M x with the current densities (no masking) */
int topo_le_apply_km(topo_le *le, const double *x, double *Kx, double *Mx);
int topo_le_get_stats(topo_le *le, topo_le_stats *out);
/* CUDA-event timing of the matrix-free operator apply on the object's stream:
 * `precision` 0 = FP64, 1 = FP32 residual, 2 = double-float (the FP64-accurate
 * passes of the mixed path), 3 = FP32 Chebyshev smoothing step;
 * `reps` back-to-back launches after `warmup`; returns mean ms per launch */
int topo_le_time_apply(topo_le *le, int precision, int warmup, int reps, double *ms_per_launch);
/* in-solve timing of one fine-grid kernel class: enable = 1 arms CUDA events
 * around each direct launch of that class on the object's stream (launches
 * replayed from CUDA graphs are not seen: create the object with
 * use_graphs = 0); enable = 0 disarms, waits for the stream and returns the
 * summed launch time (ms) and the number of timed launches.  One armed object
 * per process. */
#define TOPO_KT_SMOOTH 0  /* FP32 Chebyshev-Jacobi smoothing step (tile kernel) */
#define TOPO_KT_PQ32 1    /* FP32 FCG operator product q = A p, p.q (tile)    */
#define TOPO_KT_KRON 2    /* one stencil pass of the Kronecker mass inverse   */
#define TOPO_KT_REPLACE 3 /* FP64-accurate residual replacement (tile)        */
#define TOPO_KT_DFPROD 4  /* double-float operator products outside the Krylov
                             loop: right-hand-side, anchor and adjoint products */
int topo_le_kernel_timing(topo_le *le, int kclass, int enable, double *ms_total, long long *launches);
/* SOMMG reduced system of the current design (the public members QQ, Kr,
 * Mr, Pr of SOMMG, SOMMG.h:21-22): Q (basis x 3*nn, row b = basis vector b),
 * Kr, Mr (basis x basis, row-major), Pr (basis); any pointer may be NULL.
 * Requires reduction = 1 and CompleteInitialState. */
int topo_le_reduced_system(topo_le *le, double *Q, double *Kr, double *Mr, double *Pr);
/* SOMMG (SOMMG.h:14-34): the second-order moment-matching reduction model a
 * LinearElasticity object built with reduction = 1 owns (the reference's
 * private member reductionmodel).  topo_sommg_create replaces
 * SOMMG(Vec x, PetscInt order) (SOMMG.cc:11-24): the handle refers to `le`,
 * whose basis must equal order; it does not own `le`. */
typedef struct topo_sommg topo_sommg;
int topo_sommg_create(topo_sommg **out, topo_le *le, int order);
void topo_sommg_destroy(topo_sommg *s);
/* SOMMG::ConstructBasis(K, M, C, P, N, om, ksp) (SOMMG.h:25, SOMMG.cc:40-265):
 * K, M, C, the load P and the Dirichlet mask N are those of le's current
 * design (after CompleteInitialState), the solves use le's solver.  The
 * reduced forward sweep follows, so a later ComputeObjectiveSensitivities
 * integrates in the new basis. */
int topo_sommg_construct_basis(topo_sommg *s, double om);
/* the public members QQ (order x 3*nn, row b = basis vector b), Kr, Mr, Cr
 * (order x order, row-major) and Pr (order) (SOMMG.h:21-22) into host
 * arrays; any pointer may be NULL */
int topo_sommg_get(topo_sommg *s, double *QQ, double *Kr, double *Mr, double *Cr, double *Pr);

/* The Gram product of the reduced matrices (the VecDot(MatMult(A, QQ[j]),
 * QQ[i]) loops of SOMMG.cc:234-251) on the tensor cores, as the reduction of
 * the mixed path computes it: out[a * kb + b] = sum_i Q[a][i] W[b][i] (host
 * array, row-major) for kb <= 32 device rows Q (FP32, row stride ldq) and W
 * (FP64, row stride ldw) of n values.  Operands are split into TF32 pieces
 * that multiply exactly; sums run in FP32 over 64 values in tensor memory,
 * then in double-float and FP64.  Allocates its padded operands. */
int topo_sommg_gram_dev(const float *Q_dev, long long ldq, const double *W_dev, long long ldw, long long n, int kb,
                        double *out);

/* 24x24 box element matrices (E = 1, unit density) as applied by the
 * matrix-free kernels, in the local node order of DMDAGetElements_3D
 * (LinearElasticity.cc:3067-3074), row-major: the Hex8IsoparametricKE/ME
 * products of LinearElasticity.cc:3089-3333.  Pure host arithmetic. */
void topo_box_element_matrices(double hx, double hy, double hz, double nu, double *KE, double *ME);

/* PDEFilt (PDEFilter.h:29-74): Helmholtz filter on the nodal grid */
int topo_pdefilt_create(topo_pdefilt **out, int nx, int ny, int nz, double hx, double hy, double hz, double rmin,
                        double rtol, int maxit);
void topo_pdefilt_destroy(topo_pdefilt *f);
/* PDEFilt::FilterProject (PDEFilter.cc:193-222) == PDEFilt::Gradients (:224) */
int topo_pdefilt_filter_project(topo_pdefilt *f, const double *x, double *xout);
int topo_pdefilt_filter_project_dev(topo_pdefilt *f, const double *x_dev, double *xout_dev);

/* Filter::FilterProject for filter = 2 with optional smoothed Heaviside
 * projection (Filter.cc:60-119, Filter.h:80-83) */
int topo_filter_project(topo_pdefilt *f, const double *x, double *xTilde, double *xPhys, int projection,
                        double beta, double eta);
int topo_filter_project_dev(topo_pdefilt *f, const double *x_dev, double *xTilde_dev, double *xPhys_dev,
                            int projection, double beta, double eta);
/* Filter::Gradients for filter = 2 (Filter.cc:122-206): dfdx and the m
 * constraint gradients dgdx[m*nel] are chain-ruled and filtered in place */
int topo_filter_gradients(topo_pdefilt *f, const double *xTilde, double *dfdx, int m, double *dgdx, int projection,
                          double beta, double eta);
int topo_filter_gradients_dev(topo_pdefilt *f, const double *xTilde_dev, double *dfdx_dev, int m, double *dgdx_dev,
                              int projection, double beta, double eta);
/* Filter::GetMND (Filter.cc:208-227) */
int topo_filter_mnd(topo_pdefilt *f, const double *x, double *mnd);
int topo_filter_mnd_dev(topo_pdefilt *f, const double *x_dev, double *mnd);

/* Filter (Filter.h:34-92) for filterType 0 (sensitivity filter) and 1
 * (density filter): the distance-weighted element filter H of Filter::SetUp
 * (Filter.cc:302-531; identity when its stencil ElemConn is 1) and Hs = H 1 */
typedef struct topo_densfilt topo_densfilt;
int topo_densfilt_create(topo_densfilt **out, int nelx, int nely, int nelz, double hx, double hy, double hz,
                         int filter_type, double rmin);
void topo_densfilt_destroy(topo_densfilt *f);
/* Filter::FilterProject (Filter.cc:60-119): filter 1 xTilde = (H x) ./ Hs,
 * filter 0 xTilde = x; then the optional smoothed Heaviside projection */
int topo_densfilt_filter_project(topo_densfilt *f, const double *x, double *xTilde, double *xPhys, int projection,
                                 double beta, double eta);
int topo_densfilt_filter_project_dev(topo_densfilt *f, const double *x_dev, double *xTilde_dev, double *xPhys_dev,
                                     int projection, double beta, double eta);
/* Filter::Gradients (Filter.cc:122-206): projection chain rule, then
 * filter 1: dfdx and dgdx[m*nel] <- H (v ./ Hs); filter 0: dfdx <- (H (dfdx .* x) ./ Hs) ./ x */
int topo_densfilt_gradients(topo_densfilt *f, const double *x, const double *xTilde, double *dfdx, int m,
                            double *dgdx, int projection, double beta, double eta);
int topo_densfilt_gradients_dev(topo_densfilt *f, const double *x_dev, const double *xTilde_dev, double *dfdx_dev,
                                int m, double *dgdx_dev, int projection, double beta, double eta);
/* Filter::GetMND (Filter.cc:208-227) */
int topo_densfilt_mnd(topo_densfilt *f, const double *x, double *mnd);
int topo_densfilt_mnd_dev(topo_densfilt *f, const double *x_dev, double *mnd);

/* MMA (MMA.h:9-120), design variables resident on the device */
int topo_mma_create(topo_mma **out, int n, int m, const double *a, const double *c, const double *d);
void topo_mma_destroy(topo_mma *mma);
/* restart constructors MMA(n, m, itr, xo1, xo2, U, L[, a, c, d]) (MMA.h:16-19,
 * MMA.cc:6-178): iteration counter and the histories and asymptotes of an
 * earlier run; a, c, d may be NULL (defaults 0, 1000, 0) */
int topo_mma_create_restart(topo_mma **out, int n, int m, int itr, const double *xo1, const double *xo2,
                            const double *U, const double *L, const double *a, const double *c, const double *d);
int topo_mma_create_restart_dev(topo_mma **out, int n, int m, int itr, const double *xo1_dev, const double *xo2_dev,
                                const double *U_dev, const double *L_dev, const double *a, const double *c,
                                const double *d);
/* MMA::Restart (MMA.cc:307-350): xo1, xo2, U, L for a later restart */
int topo_mma_restart(topo_mma *mma, double *xo1, double *xo2, double *U, double *L);
int topo_mma_restart_dev(topo_mma *mma, double *xo1_dev, double *xo2_dev, double *U_dev, double *L_dev);
int topo_mma_set_asymptotes(topo_mma *mma, double init, double decrease, double increase);
/* MMA::SetOuterMovelimit (MMA.cc:374-393) */
int topo_mma_set_outer_movelimit(topo_mma *mma, double Xmin, double Xmax, double movlim, const double *x,
                                 double *xmin, double *xmax);
int topo_mma_set_outer_movelimit_dev(topo_mma *mma, double Xmin, double Xmax, double movlim, const double *x_dev,
                                     double *xmin_dev, double *xmax_dev);
/* MMA::Update (MMA.cc:487-507): xval updated in place; gx has m host values */
int topo_mma_update(topo_mma *mma, double *xval, const double *dfdx, const double *gx, const double *dgdx,
                    const double *xmin, const double *xmax);
int topo_mma_update_dev(topo_mma *mma, double *xval_dev, const double *dfdx_dev, const double *gx,
                        const double *dgdx_dev, const double *xmin_dev, const double *xmax_dev);
/* MMA::DesignChange (MMA.cc:395-414): inf-norm change, xold <- x */
int topo_mma_design_change(topo_mma *mma, const double *x, double *xold, double *ch);
int topo_mma_design_change_dev(topo_mma *mma, const double *x_dev, double *xold_dev, double *ch);
/* MMA::KKTresidual (MMA.cc:416-484) */
int topo_mma_kkt_residual_dev(topo_mma *mma, const double *x_dev, const double *dfdx_dev, const double *fx,
                              const double *dgdx_dev, const double *xmin_dev, const double *xmax_dev, double *norm2,
                              double *normInf);

/* PETSc binary vector records (VecView / VecLoad with a binary viewer): a
 * big-endian int32 class id 1211214, int32 length n, n big-endian doubles.
 * Records are appended to one file (the reference's Restart0x.dat,
 * RestartSol0x.dat and cp%04d.dat: TopOpt.cc:722-727,
 * LinearElasticity.cc:1134-1136, :2482-2484).  on_device: v is a device
 * pointer.  topo_petsc_vec_read reads record `index` (0 = first). */
int topo_petsc_vec_write(const char *path, int append, const double *v, long long n, int on_device);
int topo_petsc_vec_read(const char *path, int index, double *v, long long n, int on_device);

/* Result files in the layout of the reference's MPIIO writer, the input of
 * bin2vtu.py (bin2vtu.py:18-150): one domain of 8-node hexahedra in DMDA
 * natural order.  Replaces MPIIO::MPIIO + Allocate + writePoints + writeCells
 * (MPIIO.cc:32-150, :409-717): topo_mpiio_create truncates `filename` and
 * writes the banner "TopOpt result version 1.1\n\x01", the native uint64
 * header {1, nn, nel, npf, ncf, 8}, the '\x01'-terminated point and cell field
 * names, the float32 node coordinates (uniform on the box xc = {xmin, xmax,
 * ymin, ymax, zmin, zmax} with nx*ny*nz nodes, DMDASetUniformCoordinates)
 * and the uint64 connectivity, offsets and VTK types (12) of the cells.
 * `slots` (>= 2; 0 = 4) datasets may be queued: each is converted to float32
 * on the device straight into mapped pinned host memory and appended by a
 * writer thread while the caller goes on. */
int topo_mpiio_create(topo_mpiio **out, int nx, int ny, int nz, const double *xc, int npf, const char *pnames,
                      int ncf, const char *cnames, const char *filename, int slots);
/* flushes the queued datasets, closes the file */
void topo_mpiio_destroy(topo_mpiio *io);
/* MPIIO::WriteVTK (MPIIO.cc:152-406) = writePointFields + writeCellFields
 * (MPIIO.cc:724-935): appends uint64 itr, the point fields (3 * n_nodal of them:
 * component c of DOF-interleaved nodal vector v is field 3 v + c, nn float32
 * values each) and the cell fields (n_cells arrays of nel float32).  n_nodal = 0
 * repeats the point fields of the previous dataset (zeros before the first):
 * the design-only WriteVTK re-emits its work array.  on_device: the arrays are
 * device pointers read on `stream` (a cudaStream_t, NULL = legacy stream). */
int topo_mpiio_write(topo_mpiio *io, unsigned long long itr, const double *const *nodal, int n_nodal,
                     const double *const *cells, int n_cells, int on_device, void *stream);
/* waits until every queued dataset is in the file */
int topo_mpiio_flush(topo_mpiio *io);
/* attaches (io != NULL) or detaches the physics output of LinearElasticity:
 * the `write, output` arguments of CompleteInitialState (U at itr 0),
 * GenerateCheckPoints (every step tsc*c + j + 1 when ncp > 1) and
 * ComputeObjectiveSensitivities (every step when ncp == 1), each dataset the
 * displacement and xPhys (LinearElasticity.cc:1087-1114, :1220-1252,
 * :1736-1742).  The writer must have 3 point fields and 1 cell field. */
int topo_le_set_output(topo_le *le, topo_mpiio *io);

/* kernels launched by this library so far (direct launches and graph
 * replays; kernels inside device-side Krylov loops are reported per object by
 * topo_le_stats.graph_body_launches) */
long long topo_kernel_launches(void);

/* last error message of the calling thread, and a name for a status code */
const char *topo_last_error(void);
const char *topo_status_str(int status);

#ifdef __cplusplus
}
#endif
#endif
