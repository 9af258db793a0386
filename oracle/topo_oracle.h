/*
 * topo_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU FP64 restatement of the transient solve-and-sensitivity path of
 * TopOpt_in_PETSc_Transient (LinearElasticity, PDEFilt, Filter, MMA, SOMMG).
 * It exists to check the GPU product path; only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it.  Nothing in the shipped library
 * calls into it.
 *
 * Parity status: UNPINNED.  The reference needs PETSc + MPI, which are absent,
 * and ships no golden vectors, so this restatement is anchored on the
 * reference's source (cited per function in topo_oracle.c), on known-answer
 * properties derived from that source, and on finite-difference checks.
 *
 * Linear algebra that the reference delegates to PETSc is restated directly:
 * the AIJ matrices become a node-block 27-point stencil store holding the same
 * non-zeros, and every KSPSolve becomes a Jacobi-preconditioned CG driven to a
 * tight relative residual (the reference's FGMRES+PCMG is only defined at
 * convergence, so parity is defined on converged solutions).
 */
#ifndef TOPO_ORACLE_H
#define TOPO_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nx, ny, nz;          /* nodes per direction (reference -nx -ny -nz)          */
    double hx, hy, hz;       /* element edge lengths                                 */
    double nu;               /* Poisson ratio                                        */
    int ncp, tsc;            /* checkpoint blocks and steps per block                */
    double t1;               /* final time; dt = t1/(ncp*tsc)                        */
    int ti;                  /* 0 backward-Euler-like, 1 Newmark                     */
    int objective;           /* 0..6 (LinearElasticity.cc:1439-1461)                 */
    int sInt, mInt;          /* stiffness / mass interpolation 0 lin, 1 SIMP, 2 RAMP */
    int boundaries;          /* 0 MBB, 1 cantilever                                  */
    int loadloc;             /* 0 MBB line load, 1 cantilever line load              */
    int optregion;           /* 0..3 optimisation (objective) region                 */
    int loadsignal;          /* 0 reference pulse, 1 sin(2 pi t) for t < 0.5         */
    double Emin, Emax, Rmin, Rmax, penalK, penalM, dalpha, dbeta;
    double rtol;             /* relative residual for every CG solve                 */
    int maxit;
    /* workload extensions (not in the reference): a second point load in z at
     * node load2_node (-1: none) with signal sin(2 pi t + load2_phase) for
     * t < 0.5, scaled like the line load; objective 7 = time-integrated
     * dt/2 u^2 of one output DOF (out_dof, -1: z DOF of the tip-centre node) */
    int load2_node;
    double load2_phase;
    int out_dof;
} topo_oracle_params;

typedef struct topo_oracle topo_oracle;

/* element matrices (row-major 24x24), LinearElasticity.cc:3089-3346 */
void oracle_hex8_ke_me(double hx, double hy, double hz, double nu, double *KE, double *ME);

/* LinearElasticity */
topo_oracle *oracle_le_create(const topo_oracle_params *p);
void oracle_le_destroy(topo_oracle *o);
int oracle_le_complete_initial_state(topo_oracle *o, const double *xPhys);
int oracle_le_generate_checkpoints(topo_oracle *o);
int oracle_le_compute_objective_sensitivities(topo_oracle *o, const double *xPhys, double *fx, double *dfdx);
void oracle_le_volume_constraint(int nel, const double *xPhys, double volfrac, double *gx, double *dgdx);
void oracle_le_set_u0(topo_oracle *o, const double *U0);
/* introspection for tests */
int oracle_le_sizes(const topo_oracle *o, int *ndof, int *nel, int *Ts);
void oracle_le_get_vectors(const topo_oracle *o, double *N, double *P, double *RHS0);
void oracle_le_get_newmark(const topo_oracle *o, double *a6, double *dt);
void oracle_le_get_initial_state(const topo_oracle *o, double *U0, double *DU0, double *DDU0);
void oracle_le_get_last_block(const topo_oracle *o, int j, double *U, double *DU, double *DDU);
void oracle_le_get_adjoint0(const topo_oracle *o, double *L1, double *DDL0);
void oracle_le_get_restart_state(const topo_oracle *o, double *DDU0, double *LT, double *DDL0);
long oracle_le_total_cg_iterations(const topo_oracle *o);
/* SOMMG reduced-order path (SOMMG.cc:40-265 and the reduction branches of
 * LinearElasticity.cc): basis of k vectors at expansion frequency omega0,
 * reduced Newmark forward/adjoint, objective and sensitivities on lifted
 * fields.  Q (k x ndof), Kr, Mr (k x k) are returned when non-null. */
int oracle_le_reduced_objective_sensitivities(topo_oracle *o, const double *xPhys, int k, double omega0, double *fx,
                                              double *dfdx, double *Q, double *Kr, double *Mr);
/* y = kfac-weighted K x and mfac-weighted M x (assembled, no masking) */
void oracle_le_apply_KM(const topo_oracle *o, const double *x, double *Kx, double *Mx);
double oracle_load_signal(int which, double t);

/* PDE filter (PDEFilter.cc) on the nodal grid with nx*ny*nz nodes */
void oracle_pde_filter(int nx, int ny, int nz, double hx, double hy, double hz, double rmin,
                       const double *xin, double *xout, double rtol);
void oracle_pde_filter_matrix(double hx, double hy, double hz, double R, double *KF);

/* Filter.h:80-88 and Filter.cc:60-227 */
void oracle_filter_project(int nx, int ny, int nz, double hx, double hy, double hz, double rmin,
                           const double *x, double *xTilde, double *xPhys, int projection,
                           double beta, double eta, double rtol);
void oracle_filter_gradients(int nx, int ny, int nz, double hx, double hy, double hz, double rmin,
                             const double *xTilde, double *dfdx, int m, double *dgdx, int projection,
                             double beta, double eta, double rtol);
double oracle_filter_mnd(int n, const double *x);
/* Filter.cc:60-206 and :302-531 for filterType 0 (sensitivity filter) and 1
 * (density filter) on an ex*ey*ez element grid: H with weights R - dist
 * between element centres, Hs = H 1 */
void oracle_dens_filter_apply(int ex, int ey, int ez, double hx, double hy, double hz, double R, const double *in,
                              double *out);
void oracle_dens_filter_project(int ex, int ey, int ez, double hx, double hy, double hz, int ftype, double R,
                                const double *x, double *xTilde, double *xPhys, int projection, double beta,
                                double eta);
void oracle_dens_filter_gradients(int ex, int ey, int ez, double hx, double hy, double hz, int ftype, double R,
                                  const double *x, const double *xTilde, double *dfdx, int m, double *dgdx,
                                  int projection, double beta, double eta);
int oracle_increase_beta(double *beta, double betaFinal, double gx, int itr, double ch);

/* MMA (MMA.cc) */
typedef struct topo_oracle_mma topo_oracle_mma;
topo_oracle_mma *oracle_mma_create(int n, int m, const double *x, const double *a, const double *c,
                                   const double *d);
void oracle_mma_destroy(topo_oracle_mma *mm);
void oracle_mma_set_asymptotes(topo_oracle_mma *mm, double init, double dec, double inc);
void oracle_mma_set_outer_movelimit(int n, double Xmin, double Xmax, double movlim, const double *x,
                                    double *xmin, double *xmax);
void oracle_mma_update(topo_oracle_mma *mm, double *xval, const double *dfdx, const double *gx,
                       const double *dgdx, const double *xmin, const double *xmax);
double oracle_mma_design_change(int n, const double *x, double *xold);
void oracle_mma_kkt_residual(topo_oracle_mma *mm, const double *x, const double *dfdx, const double *fx,
                             const double *dgdx, const double *xmin, const double *xmax, double *norm2,
                             double *normInf);
void oracle_mma_get_state(const topo_oracle_mma *mm, double *L, double *U, double *lam);

#ifdef __cplusplus
}
#endif
#endif
