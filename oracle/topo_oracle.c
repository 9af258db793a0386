/*
 * topo_oracle.c -- TEST INFRASTRUCTURE ONLY (see topo_oracle.h).
 *
 * CPU FP64 restatement of TopOpt_in_PETSc_Transient's transient
 * solve-and-sensitivity path, single rank, DMDA natural ordering:
 *   node (i,j,k) -> i + nx*(j + ny*k), DOF 3*node + c;
 *   element (i,j,k) -> i + nex*(j + ney*k).
 * Each function cites the reference function it restates.  Parity is
 * UNPINNED (no PETSc/MPI here, no golden vectors in the reference).
 */
#include "topo_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* element matrices                                                     */
/* ------------------------------------------------------------------ */

/* local node order of DMDAGetElements_3D, LinearElasticity.cc:3067-3074 */
static const int LN[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                             {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

/* trilinear shape functions and derivatives on [-1,1]^3,
 * LinearElasticity.cc:3358-3486 (ShapeFunctions, DifferentiatedShapeFunctions) */
static void shape8(double xi, double eta, double zeta, double *S, double *dxi, double *deta, double *dzeta) {
    for (int a = 0; a < 8; a++) {
        double sx = 2.0 * LN[a][0] - 1.0, sy = 2.0 * LN[a][1] - 1.0, sz = 2.0 * LN[a][2] - 1.0;
        S[a] = 0.125 * (1.0 + sx * xi) * (1.0 + sy * eta) * (1.0 + sz * zeta);
        dxi[a] = 0.125 * sx * (1.0 + sy * eta) * (1.0 + sz * zeta);
        deta[a] = 0.125 * sy * (1.0 + sx * xi) * (1.0 + sz * zeta);
        dzeta[a] = 0.125 * sz * (1.0 + sx * xi) * (1.0 + sy * eta);
    }
}

/* 3x3 inverse + determinant, LinearElasticity.cc:3488-3503 */
static double inv3(const double J[3][3], double iJ[3][3]) {
    double det = J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) - J[0][1] * (J[1][0] * J[2][2] - J[2][0] * J[1][2]) +
                 J[0][2] * (J[1][0] * J[2][1] - J[2][0] * J[1][1]);
    iJ[0][0] = (J[1][1] * J[2][2] - J[2][1] * J[1][2]) / det;
    iJ[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) / det;
    iJ[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    iJ[1][0] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]) / det;
    iJ[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    iJ[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) / det;
    iJ[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
    iJ[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) / det;
    iJ[2][2] = (J[0][0] * J[1][1] - J[1][0] * J[0][1]) / det;
    return det;
}

/* Hex8IsoparametricKE / Hex8IsoparametricME, LinearElasticity.cc:3089-3333:
 * 2x2x2 Gauss with the reference's truncated abscissa 0.577350269189626,
 * isotropic D with E = 1, B^T D B det(J), and N^T N det(J) per component. */
void oracle_hex8_ke_me(double hx, double hy, double hz, double nu, double *KE, double *ME) {
    const double gp[2] = {-0.577350269189626, 0.577350269189626};
    double lam = nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), mu = 1.0 / (2.0 * (1.0 + nu));
    double C[6][6] = {{0}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) C[i][j] = lam;
    for (int i = 0; i < 3; i++) C[i][i] = lam + 2.0 * mu;
    C[3][3] = C[4][4] = C[5][5] = mu;
    double X[8], Y[8], Z[8];
    for (int a = 0; a < 8; a++) {
        X[a] = LN[a][0] * hx;
        Y[a] = LN[a][1] * hy;
        Z[a] = LN[a][2] * hz;
    }
    memset(KE, 0, sizeof(double) * 576);
    memset(ME, 0, sizeof(double) * 576);
    for (int ii = 0; ii < 2; ii++)
        for (int jj = 0; jj < 2; jj++)
            for (int kk = 0; kk < 2; kk++) {
                double S[8], dxi[8], deta[8], dzeta[8];
                shape8(gp[ii], gp[jj], gp[kk], S, dxi, deta, dzeta);
                double J[3][3] = {{0}}, iJ[3][3];
                for (int a = 0; a < 8; a++) {
                    J[0][0] += dxi[a] * X[a];
                    J[0][1] += dxi[a] * Y[a];
                    J[0][2] += dxi[a] * Z[a];
                    J[1][0] += deta[a] * X[a];
                    J[1][1] += deta[a] * Y[a];
                    J[1][2] += deta[a] * Z[a];
                    J[2][0] += dzeta[a] * X[a];
                    J[2][1] += dzeta[a] * Y[a];
                    J[2][2] += dzeta[a] * Z[a];
                }
                double w = inv3(J, iJ);
                /* physical derivatives: dN/dx_l = sum_m invJ[l][m] dN/dxi_m */
                double dN[3][8];
                for (int a = 0; a < 8; a++)
                    for (int l = 0; l < 3; l++) dN[l][a] = iJ[l][0] * dxi[a] + iJ[l][1] * deta[a] + iJ[l][2] * dzeta[a];
                double B[6][24];
                memset(B, 0, sizeof(B));
                for (int a = 0; a < 8; a++) {
                    B[0][3 * a + 0] = dN[0][a];
                    B[1][3 * a + 1] = dN[1][a];
                    B[2][3 * a + 2] = dN[2][a];
                    B[3][3 * a + 0] = dN[1][a];
                    B[3][3 * a + 1] = dN[0][a];
                    B[4][3 * a + 1] = dN[2][a];
                    B[4][3 * a + 2] = dN[1][a];
                    B[5][3 * a + 0] = dN[2][a];
                    B[5][3 * a + 2] = dN[0][a];
                }
                double DB[6][24];
                for (int k = 0; k < 6; k++)
                    for (int j = 0; j < 24; j++) {
                        double s = 0.0;
                        for (int l = 0; l < 6; l++) s += C[k][l] * B[l][j];
                        DB[k][j] = s;
                    }
                for (int i = 0; i < 24; i++)
                    for (int j = 0; j < 24; j++) {
                        double s = 0.0;
                        for (int k = 0; k < 6; k++) s += B[k][i] * DB[k][j];
                        KE[24 * i + j] += w * s;
                    }
                for (int a = 0; a < 8; a++)
                    for (int b = 0; b < 8; b++)
                        for (int c = 0; c < 3; c++) ME[24 * (3 * a + c) + 3 * b + c] += w * S[a] * S[b];
            }
}

/* ------------------------------------------------------------------ */
/* structured-grid stencil store (same non-zeros as the DMDA AIJ matrix) */
/* ------------------------------------------------------------------ */

typedef struct {
    int nx, ny, nz, nn, bs; /* bs = DOFs per node (3 elasticity, 1 filter) */
    double *v;              /* [nn][27][bs*bs] */
} stencil_t;

static void st_alloc(stencil_t *s, int nx, int ny, int nz, int bs) {
    s->nx = nx;
    s->ny = ny;
    s->nz = nz;
    s->nn = nx * ny * nz;
    s->bs = bs;
    s->v = (double *)calloc((size_t)s->nn * 27 * bs * bs, sizeof(double));
}
static void st_free(stencil_t *s) { free(s->v); }

/* MatSetValuesLocal(...ADD_VALUES) of w_e * Ee over all elements, element
 * loop order of DMDAGetElements_3D (LinearElasticity.cc:2502-2601). */
static void st_assemble(stencil_t *s, const double *Ee, const double *w) {
    int bs = s->bs, nd = 8 * bs, nex = s->nx - 1, ney = s->ny - 1, nez = s->nz - 1;
    memset(s->v, 0, sizeof(double) * (size_t)s->nn * 27 * bs * bs);
    for (int color = 0; color < 8; color++) {
        int ci = color & 1, cj = (color >> 1) & 1, ck = (color >> 2) & 1;
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = ck; k < nez; k += 2)
            for (int j = cj; j < ney; j += 2)
                for (int i = ci; i < nex; i += 2) {
                    int e = i + nex * (j + ney * k);
                    double we = w[e];
                    for (int a = 0; a < 8; a++) {
                        int na = (i + LN[a][0]) + s->nx * ((j + LN[a][1]) + s->ny * (k + LN[a][2]));
                        for (int b = 0; b < 8; b++) {
                            int o = (LN[b][0] - LN[a][0] + 1) + 3 * (LN[b][1] - LN[a][1] + 1) + 9 * (LN[b][2] - LN[a][2] + 1);
                            double *blk = s->v + ((size_t)na * 27 + o) * bs * bs;
                            for (int c = 0; c < bs; c++)
                                for (int d = 0; d < bs; d++) blk[c * bs + d] += we * Ee[nd * (bs * a + c) + bs * b + d];
                        }
                    }
                }
    }
}

/* MatMult */
static void st_mult(const stencil_t *s, const double *x, double *y) {
    int bs = s->bs, nx = s->nx, ny = s->ny, nz = s->nz;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                int n = i + nx * (j + ny * k);
                double acc[3] = {0, 0, 0};
                for (int dk = -1; dk <= 1; dk++) {
                    int kk = k + dk;
                    if (kk < 0 || kk >= nz) continue;
                    for (int dj = -1; dj <= 1; dj++) {
                        int jj = j + dj;
                        if (jj < 0 || jj >= ny) continue;
                        for (int di = -1; di <= 1; di++) {
                            int ii = i + di;
                            if (ii < 0 || ii >= nx) continue;
                            int m = ii + nx * (jj + ny * kk);
                            int o = (di + 1) + 3 * (dj + 1) + 9 * (dk + 1);
                            const double *blk = s->v + ((size_t)n * 27 + o) * bs * bs;
                            for (int c = 0; c < bs; c++)
                                for (int d = 0; d < bs; d++) acc[c] += blk[c * bs + d] * x[bs * m + d];
                        }
                    }
                }
                for (int c = 0; c < bs; c++) y[bs * n + c] = acc[c];
            }
}

/* Two MatMults with matrices of the same pattern in one sweep: kx = K x and
 * mx = M x, each summed in the order st_mult uses (bitwise the same values). */
static void st_mult2(const stencil_t *K, const stencil_t *M, const double *x, double *kx, double *mx) {
    int nx = K->nx, ny = K->ny, nz = K->nz;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                int n = i + nx * (j + ny * k);
                double ak[3] = {0, 0, 0}, am[3] = {0, 0, 0};
                for (int dk = -1; dk <= 1; dk++) {
                    int kk = k + dk;
                    if (kk < 0 || kk >= nz) continue;
                    for (int dj = -1; dj <= 1; dj++) {
                        int jj = j + dj;
                        if (jj < 0 || jj >= ny) continue;
                        for (int di = -1; di <= 1; di++) {
                            int ii = i + di;
                            if (ii < 0 || ii >= nx) continue;
                            int m = ii + nx * (jj + ny * kk);
                            int o = (di + 1) + 3 * (dj + 1) + 9 * (dk + 1);
                            const double *bk = K->v + ((size_t)n * 27 + o) * 9;
                            const double *bm = M->v + ((size_t)n * 27 + o) * 9;
                            for (int c = 0; c < 3; c++)
                                for (int d = 0; d < 3; d++) {
                                    ak[c] += bk[c * 3 + d] * x[3 * m + d];
                                    am[c] += bm[c * 3 + d] * x[3 * m + d];
                                }
                        }
                    }
                }
                for (int c = 0; c < 3; c++) {
                    kx[3 * n + c] = ak[c];
                    mx[3 * n + c] = am[c];
                }
            }
}

static void st_diag(const stencil_t *s, double *dg) {
    int bs = s->bs;
    for (int n = 0; n < s->nn; n++)
        for (int c = 0; c < bs; c++) dg[bs * n + c] = s->v[((size_t)n * 27 + 13) * bs * bs + c * bs + c];
}

/* ------------------------------------------------------------------ */
/* vector helpers                                                       */
/* ------------------------------------------------------------------ */
static double vdot(int n, const double *a, const double *b) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}
static double *vnew(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }

/* Jacobi-preconditioned CG on an SPD operator: stands in for KSPSolve.  The
 * reference's own settings (FGMRES(100)+PCMG, rtol 1e-10,
 * LinearElasticity.cc:2750-2757) only define the solution up to that
 * tolerance; this solver is driven tighter (params rtol). */
typedef void (*op_fn)(void *ctx, const double *x, double *y);
static int pcg(op_fn op, void *ctx, const double *dinv, int n, const double *b, double *x, double rtol, int maxit,
               long *iters) {
    double *r = vnew(n), *z = vnew(n), *p = vnew(n), *q = vnew(n);
    memset(x, 0, sizeof(double) * n); /* KSPSetInitialGuessNonzero(FALSE), LinearElasticity.cc:2778-2781 */
    memcpy(r, b, sizeof(double) * n);
    double bn = sqrt(vdot(n, b, b));
    int it = 0, ok = 1;
    if (bn > 0.0) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; i++) z[i] = dinv[i] * r[i];
        memcpy(p, z, sizeof(double) * n);
        double rz = vdot(n, r, z);
        for (it = 1; it <= maxit; it++) {
            op(ctx, p, q);
            double alpha = rz / vdot(n, p, q);
#pragma omp parallel for schedule(static)
            for (int i = 0; i < n; i++) {
                x[i] += alpha * p[i];
                r[i] -= alpha * q[i];
            }
            double rn = sqrt(vdot(n, r, r));
            if (rn <= rtol * bn) break;
#pragma omp parallel for schedule(static)
            for (int i = 0; i < n; i++) z[i] = dinv[i] * r[i];
            double rz2 = vdot(n, r, z);
            double beta = rz2 / rz;
            rz = rz2;
#pragma omp parallel for schedule(static)
            for (int i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
        }
        if (it > maxit) ok = 0;
    }
    if (iters) *iters += it;
    free(r);
    free(z);
    free(p);
    free(q);
    return ok ? 0 : 1;
}

/* ------------------------------------------------------------------ */
/* LinearElasticity                                                     */
/* ------------------------------------------------------------------ */

struct topo_oracle {
    topo_oracle_params p;
    int nx, ny, nz, nex, ney, nez, nn, nel, ndof, Ts;
    double KE[576], ME[576], CE[576], a[6], dt;
    double *N, *P, *RHS0, *RHS;
    double *kfac, *dkfac, *mfac, *dmfac;
    stencil_t K, M;
    stencil_t A; /* N Keff N + (I - N), the masked step operator of solve_eff */
    double *dinv_eff, *dinv_m;
    double *U0, *DU0, *DDU0, *U0init, *DU0init;
    double *cp; /* (ncp+1) x {U,DU,DDU}: cp%04d.dat held in memory */
    double *U, *DU, *DDU, *L, *DL, *DDL;
    double *Lp1, *DLp1, *DDLp1, *LT, *DDL0;
    double *HDU, *HDDU, *HDDDU, *R, *t1, *t2, *t3, *t4;
    long cg_iters;
    int last_block;
};

/* Load(t), LinearElasticity.cc:593-615 (which = 0); which = 1 is the
 * half-period sine pulse used by the synthetic cantilever workloads. */
double oracle_load_signal(int which, double t) {
    if (which == 1) return (t < 0.5) ? sin(2.0 * M_PI * t) : 0.0;
    double t0 = 8.0, c = 1.1;
    return exp(-pow(t - t0, 2) / pow(2 * c, 2)) * cos(4.0 * (t - t0)) * cos(5.0 * (t - t0)) * cos(6.0 * (t - t0)) *
           cos(7.0 * (t - t0));
}

/* InterpolateStiffness / InterpolateMass, LinearElasticity.cc:1580-1623 */
static void interp(int type, double vmax, double vmin, double pen, double x, double *f, double *df) {
    switch (type) {
    case 0:
        *f = vmin + x * (vmax - vmin);
        *df = vmax - vmin;
        break;
    case 1:
        *f = vmin + pow(x, pen) * (vmax - vmin);
        *df = pen * pow(x, pen - 1) * (vmax - vmin);
        break;
    default:
        *f = vmin + x / (1 + pen * (1 - x)) * (vmax - vmin);
        *df = (1 + pen) / pow(1 + pen * (1 - x), 2) * (vmax - vmin);
        break;
    }
}

static inline int node_id(const topo_oracle *o, int i, int j, int k) { return i + o->nx * (j + o->ny * k); }

static void edofs(const topo_oracle *o, int e, int *ed) {
    int i = e % o->nex, j = (e / o->nex) % o->ney, k = e / (o->nex * o->ney);
    for (int a = 0; a < 8; a++) {
        int n = node_id(o, i + LN[a][0], j + LN[a][1], k + LN[a][2]);
        for (int c = 0; c < 3; c++) ed[3 * a + c] = 3 * n + c;
    }
}

topo_oracle *oracle_le_create(const topo_oracle_params *p) {
    topo_oracle *o = (topo_oracle *)calloc(1, sizeof(topo_oracle));
    o->p = *p;
    o->nx = p->nx;
    o->ny = p->ny;
    o->nz = p->nz;
    o->nex = p->nx - 1;
    o->ney = p->ny - 1;
    o->nez = p->nz - 1;
    o->nn = p->nx * p->ny * p->nz;
    o->nel = o->nex * o->ney * o->nez;
    o->ndof = 3 * o->nn;
    /* constructor, LinearElasticity.cc:93-97 */
    o->Ts = p->ncp * p->tsc + 1;
    o->dt = p->t1 / (o->Ts - 1);
    double dt = o->dt;
    /* SetUpTimeIntegration, LinearElasticity.cc:185-219 */
    if (p->ti == 0) {
        o->a[0] = 0.0;
        o->a[1] = 0.0;
        o->a[2] = 1.0 / dt;
        o->a[3] = 1.0 / dt;
        o->a[4] = 0.0;
        o->a[5] = 1.0 / (dt * dt);
    } else {
        double b = 0.25, g = 0.5;
        o->a[0] = 1.0 - g / b;
        o->a[1] = (1.0 - g / (2.0 * b)) * dt;
        o->a[2] = g / (b * dt);
        o->a[3] = 1 / (b * dt);
        o->a[4] = 1 / (2.0 * b) - 1.0;
        o->a[5] = 1.0 / (b * dt * dt);
    }
    /* element matrices, LinearElasticity.cc:514-519 and Hex8IsoparametricCE :3335-3346 */
    oracle_hex8_ke_me(p->hx, p->hy, p->hz, p->nu, o->KE, o->ME);
    for (int i = 0; i < 576; i++) o->CE[i] = p->dalpha * o->ME[i] + p->dbeta * o->KE[i];

    int nd = o->ndof;
    o->N = vnew(nd);
    o->P = vnew(o->nel);
    o->RHS0 = vnew(nd);
    o->RHS = vnew(nd);
    /* SetUpBC, LinearElasticity.cc:337-591: Dirichlet vector */
    double xc[6] = {0, o->nex * p->hx, 0, o->ney * p->hy, 0, o->nez * p->hz};
    double epsi = fmin(p->hx * 0.05, fmin(p->hy * 0.05, p->hz * 0.05));
    for (int i = 0; i < nd; i++) o->N[i] = 1.0;
    for (int k = 0; k < o->nz; k++)
        for (int j = 0; j < o->ny; j++)
            for (int i = 0; i < o->nx; i++) {
                int n = node_id(o, i, j, k);
                double x = i * p->hx, y = j * p->hy, z = k * p->hz;
                (void)y;
                if (p->boundaries == 0) {
                    if (fabs(x - xc[0]) < epsi) o->N[3 * n] = o->N[3 * n + 1] = 0.0;
                    if (fabs(x - xc[1]) < epsi && fabs(z - xc[4]) < epsi) o->N[3 * n + 1] = o->N[3 * n + 2] = 0.0;
                } else {
                    if (fabs(x - xc[0]) < epsi) o->N[3 * n] = o->N[3 * n + 1] = o->N[3 * n + 2] = 0.0;
                }
                /* LoadLocation, LinearElasticity.cc:616-675 */
                if (p->loadloc == 0) {
                    if (fabs(x - xc[0]) < epsi && fabs(z - xc[5]) < epsi) {
                        o->RHS0[3 * n + 2] = 1.0;
                        if (fabs(y - xc[2]) < epsi || fabs(y - xc[3]) < epsi) o->RHS0[3 * n + 2] = 0.5;
                    }
                } else {
                    if (fabs(x - xc[1]) < epsi && fabs(z - xc[5] / 2.0) < epsi) {
                        o->RHS0[3 * n + 2] = 1.0;
                        if (fabs(y - xc[2]) < epsi || fabs(y - xc[3]) < epsi) o->RHS0[3 * n + 2] = 0.5;
                    }
                }
            }
    /* SetUpOptimizationRegion, LinearElasticity.cc:222-335 (element centres) */
    for (int e = 0; e < o->nel; e++) {
        int i = e % o->nex, j = (e / o->nex) % o->ney, k = e / (o->nex * o->ney);
        double ex = (i + 0.5) * p->hx, ey = (j + 0.5) * p->hy, ez = (k + 0.5) * p->hz;
        double v = 0.0;
        switch (p->optregion) {
        case 0:
            v = (ez > xc[5] - 1 && ex < xc[0] + 1) ? 1.0 : 0.0;
            break;
        case 1:
            v = (ez > xc[5] / 2.0 - 0.5 && ez < xc[5] / 2.0 + 0.5 && ex < xc[1] - 1) ? 1.0 : 0.0;
            break;
        case 2:
            v = 1.0;
            break;
        default:
            v = (ex > 0.75 * xc[1] - 2.5 && ex < 0.75 * xc[1] + 2.5 && ey > 0.5 * xc[3] - 2.5 &&
                 ey < 0.5 * xc[3] + 2.5 && ez > 0.5 * xc[5] - 2.5 && ez < 0.5 * xc[5] + 2.5)
                    ? 1.0
                    : 0.0;
        }
        o->P[e] = v;
    }
    o->kfac = vnew(o->nel);
    o->dkfac = vnew(o->nel);
    o->mfac = vnew(o->nel);
    o->dmfac = vnew(o->nel);
    st_alloc(&o->K, o->nx, o->ny, o->nz, 3);
    st_alloc(&o->M, o->nx, o->ny, o->nz, 3);
    st_alloc(&o->A, o->nx, o->ny, o->nz, 3);
    o->dinv_eff = vnew(nd);
    o->dinv_m = vnew(nd);
    o->U0 = vnew(nd);
    o->DU0 = vnew(nd);
    o->DDU0 = vnew(nd);
    o->U0init = vnew(nd); /* VecSet(U0,0), VecSet(DU0,0), masked: LinearElasticity.cc:521-587 */
    o->DU0init = vnew(nd);
    o->cp = vnew((size_t)(p->ncp + 1) * 3 * nd);
    size_t blk = (size_t)p->tsc * nd;
    o->U = vnew(blk);
    o->DU = vnew(blk);
    o->DDU = vnew(blk);
    o->L = vnew(blk);
    o->DL = vnew(blk);
    o->DDL = vnew(blk);
    o->Lp1 = vnew(nd);
    o->DLp1 = vnew(nd);
    o->DDLp1 = vnew(nd);
    o->LT = vnew(nd);
    o->DDL0 = vnew(nd);
    o->HDU = vnew(nd);
    o->HDDU = vnew(nd);
    o->HDDDU = vnew(nd);
    o->R = vnew(nd);
    o->t1 = vnew(nd);
    o->t2 = vnew(nd);
    o->t3 = vnew(nd);
    o->t4 = vnew(nd);
    return o;
}

void oracle_le_destroy(topo_oracle *o) {
    if (!o) return;
    double *ptrs[] = {o->N,    o->P,     o->RHS0,  o->RHS,  o->kfac,   o->dkfac, o->mfac, o->dmfac, o->dinv_eff,
                      o->dinv_m, o->U0,  o->DU0,   o->DDU0, o->U0init, o->DU0init, o->cp,  o->U,     o->DU,
                      o->DDU,  o->L,     o->DL,    o->DDL,  o->Lp1,    o->DLp1,  o->DDLp1, o->LT,    o->DDL0,
                      o->HDU,  o->HDDU,  o->HDDDU, o->R,    o->t1,     o->t2,    o->t3,   o->t4};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
    st_free(&o->K);
    st_free(&o->M);
    st_free(&o->A);
    free(o);
}

/* Load(t): RHS = RHS0 * signal / (ny-1), LinearElasticity.cc:593-615 */
static void load(topo_oracle *o, double t) {
    double s = oracle_load_signal(o->p.loadsignal, t) / (o->ny - 1);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o->ndof; i++) o->RHS[i] = o->RHS0[i] * s;
    /* second point load (workload extension, not in the reference) */
    if (o->p.load2_node >= 0 && o->N[3 * o->p.load2_node + 2] != 0.0)
        o->RHS[3 * o->p.load2_node + 2] += ((t < 0.5) ? sin(2.0 * M_PI * t + o->p.load2_phase) : 0.0) / (o->ny - 1);
}
/* output DOF of objective 7: the z DOF of the tip-centre node by default */
static int out_dof(const topo_oracle *o) {
    if (o->p.out_dof >= 0) return o->p.out_dof;
    return 3 * (o->nx - 1 + o->nx * ((o->ny - 1) / 2 + o->ny * ((o->nz - 1) / 2))) + 2;
}

/* Keff x with Keff = K + a5 M + a2 C (= -A before masking), C = alpha M + beta K,
 * AssembleDampingMatrix LinearElasticity.cc:2605-2619 and the A build :1022-1026 */
typedef struct {
    topo_oracle *o;
    int mass_only;
} opctx;
static void op_masked(void *vctx, const double *x, double *y) {
    opctx *c = (opctx *)vctx;
    topo_oracle *o = c->o;
    int nd = o->ndof;
    double *xm = o->t3, *kx = o->t4;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nd; i++) xm[i] = o->N[i] * x[i];
    if (c->mass_only) {
        st_mult(&o->M, xm, y);
    } else {
        double cK = 1.0 + o->a[2] * o->p.dbeta, cM = o->a[5] + o->a[2] * o->p.dalpha;
        st_mult2(&o->K, &o->M, xm, kx, y);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nd; i++) y[i] = cK * kx[i] + cM * y[i];
    }
    /* dRdS = N A N + (I - N): MatDiagonalScale + MatDiagonalSet, LinearElasticity.cc:1118-1122 */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nd; i++) y[i] = o->N[i] * y[i] + (1.0 - o->N[i]) * x[i];
}

/* The same masked step operator N (cK K + cM M) N + (I - N), assembled once
 * per design into one stencil (MatAXPY + MatDiagonalScale + MatDiagonalSet,
 * LinearElasticity.cc:1022-1026, :1118-1122): one sweep per Krylov iteration.
 * The mask entries are exactly 0 or 1, so masking the stored blocks equals
 * masking the vectors; only the combination cK k + cM m rounds differently
 * from cK (K x) + cM (M x). */
static void assemble_masked_eff(topo_oracle *o) {
    double cK = 1.0 + o->a[2] * o->p.dbeta, cM = o->a[5] + o->a[2] * o->p.dalpha;
    int nx = o->nx, ny = o->ny, nz = o->nz;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                int n = i + nx * (j + ny * k);
                for (int oo = 0; oo < 27; oo++) {
                    int di = oo % 3 - 1, dj = (oo / 3) % 3 - 1, dk = oo / 9 - 1;
                    int ii = i + di, jj = j + dj, kk = k + dk;
                    double *ba = o->A.v + ((size_t)n * 27 + oo) * 9;
                    if (ii < 0 || ii >= nx || jj < 0 || jj >= ny || kk < 0 || kk >= nz) {
                        memset(ba, 0, 9 * sizeof(double));
                        continue;
                    }
                    int m = ii + nx * (jj + ny * kk);
                    const double *bk = o->K.v + ((size_t)n * 27 + oo) * 9;
                    const double *bm = o->M.v + ((size_t)n * 27 + oo) * 9;
                    for (int c = 0; c < 3; c++)
                        for (int d = 0; d < 3; d++) {
                            double v = o->N[3 * n + c] * (cK * bk[3 * c + d] + cM * bm[3 * c + d]) * o->N[3 * m + d];
                            if (oo == 13 && c == d) v += 1.0 - o->N[3 * n + c];
                            ba[3 * c + d] = v;
                        }
                }
            }
}
static void op_eff(void *vctx, const double *x, double *y) {
    opctx *c = (opctx *)vctx;
    st_mult(&c->o->A, x, y);
}

/* KSPSolve with operator N A N + (I-N), A = -Keff (LinearElasticity.cc:1118-1126):
 * on free rows -(Keff x) = R, on Dirichlet rows x = R. */
static int solve_eff(topo_oracle *o, const double *R, double *x) {
    opctx c = {o, 0};
    double *rhs = o->t1;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o->ndof; i++) rhs[i] = (o->N[i] != 0.0) ? -R[i] : R[i];
    return pcg(op_eff, &c, o->dinv_eff, o->ndof, rhs, x, o->p.rtol, o->p.maxit, &o->cg_iters);
}
/* KSPSolve with operator N M N + (I-N) (LinearElasticity.cc:1063-1078, :763-776) */
static int solve_mass(topo_oracle *o, const double *R, double *x) {
    opctx c = {o, 1};
    return pcg(op_masked, &c, o->dinv_m, o->ndof, R, x, o->p.rtol, o->p.maxit, &o->cg_iters);
}

/* y = N (cM M + cK K) N x : the B1/B2/B3 MatMults (LinearElasticity.cc:1028-1044) */
static void bmult(topo_oracle *o, double cM, double cK, const double *x, double *y) {
    int nd = o->ndof;
    double *xm = o->t3, *kx = o->t4;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nd; i++) xm[i] = o->N[i] * x[i];
    st_mult2(&o->K, &o->M, xm, kx, y);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nd; i++) y[i] = o->N[i] * (cM * y[i] + cK * kx[i]);
}

void oracle_le_apply_KM(const topo_oracle *o, const double *x, double *Kx, double *Mx) {
    st_mult(&o->K, x, Kx);
    st_mult(&o->M, x, Mx);
}

/* CompleteInitialState, LinearElasticity.cc:956-1206 (non-reduced branch) */
int oracle_le_complete_initial_state(topo_oracle *o, const double *xPhys) {
    const topo_oracle_params *p = &o->p;
    int nd = o->ndof, rc = 0;
    for (int e = 0; e < o->nel; e++) {
        interp(p->sInt, p->Emax, p->Emin, p->penalK, xPhys[e], &o->kfac[e], &o->dkfac[e]);
        interp(p->mInt, p->Rmax, p->Rmin, p->penalM, xPhys[e], &o->mfac[e], &o->dmfac[e]);
    }
    /* AssembleMassMatrix / AssembleStiffnessMatrix, LinearElasticity.cc:2502-2603 */
    st_assemble(&o->M, o->ME, o->mfac);
    st_assemble(&o->K, o->KE, o->kfac);
    assemble_masked_eff(o);
    double *dk = o->t1, *dm = o->t2;
    st_diag(&o->K, dk);
    st_diag(&o->M, dm);
    double cK = 1.0 + o->a[2] * p->dbeta, cM = o->a[5] + o->a[2] * p->dalpha;
    for (int i = 0; i < nd; i++) {
        double de = o->N[i] * (cK * dk[i] + cM * dm[i]) + (1.0 - o->N[i]);
        double dmm = o->N[i] * dm[i] + (1.0 - o->N[i]);
        o->dinv_eff[i] = 1.0 / de;
        o->dinv_m[i] = 1.0 / dmm;
    }
    memcpy(o->U0, o->U0init, sizeof(double) * nd);
    memcpy(o->DU0, o->DU0init, sizeof(double) * nd);
    /* R = N (f(0) - C DU0 - K U0), LinearElasticity.cc:1049-1066 */
    double *kx = o->t3, *mx = o->t4;
    load(o, 0.0);
    st_mult(&o->K, o->DU0, kx);
    st_mult(&o->M, o->DU0, mx);
    for (int i = 0; i < nd; i++) o->R[i] = o->RHS[i] - o->N[i] * (p->dalpha * mx[i] + p->dbeta * kx[i]);
    st_mult(&o->K, o->U0, kx);
    for (int i = 0; i < nd; i++) o->R[i] = o->N[i] * (o->R[i] - o->N[i] * kx[i]);
    double *rr = vnew(nd);
    memcpy(rr, o->R, sizeof(double) * nd);
    rc |= solve_mass(o, rr, o->DDU0);
    free(rr);
    /* write cp0000 (LinearElasticity.cc:1128-1137) */
    memcpy(o->cp, o->U0, sizeof(double) * nd);
    memcpy(o->cp + nd, o->DU0, sizeof(double) * nd);
    memcpy(o->cp + 2 * nd, o->DDU0, sizeof(double) * nd);
    return rc;
}

/* SolveStateBlock, LinearElasticity.cc:1298-1397 */
static int solve_state_block(topo_oracle *o, int c) {
    const topo_oracle_params *p = &o->p;
    int nd = o->ndof, rc = 0;
    double *a = o->a;
    double *b1 = vnew(nd), *b2 = vnew(nd), *b3 = vnew(nd), *rr = vnew(nd);
    for (int j = 0; j < p->tsc; j++) {
        int t = p->tsc * c + j + 1;
        double *Uj = o->U + (size_t)j * nd, *DUj = o->DU + (size_t)j * nd, *DDUj = o->DDU + (size_t)j * nd;
        const double *UM1 = j ? o->U + (size_t)(j - 1) * nd : o->U0;
        const double *DUM1 = j ? o->DU + (size_t)(j - 1) * nd : o->DU0;
        const double *DDUM1 = j ? o->DDU + (size_t)(j - 1) * nd : o->DDU0;
        load(o, t * o->dt);
        bmult(o, a[5] + a[2] * p->dalpha, a[2] * p->dbeta, UM1, b1);
        bmult(o, a[3] - a[0] * p->dalpha, -a[0] * p->dbeta, DUM1, b2);
        bmult(o, a[4] - a[1] * p->dalpha, -a[1] * p->dbeta, DDUM1, b3);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nd; i++) rr[i] = o->N[i] * (-(o->RHS[i] + b1[i] + b2[i] + b3[i]));
        rc |= solve_eff(o, rr, Uj);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nd; i++) {
            double du = Uj[i] - UM1[i];
            DUj[i] = a[0] * DUM1[i] + a[1] * DDUM1[i] + a[2] * du;
            DDUj[i] = -a[3] * DUM1[i] - a[4] * DDUM1[i] + a[5] * du;
        }
    }
    free(b1);
    free(b2);
    free(b3);
    free(rr);
    o->last_block = c;
    return rc;
}

/* GenerateCheckPoints, LinearElasticity.cc:1208-1280 */
int oracle_le_generate_checkpoints(topo_oracle *o) {
    int nd = o->ndof, rc = 0, tsc = o->p.tsc;
    if (o->p.ncp <= 1) return 0;
    for (int c = 0; c < o->p.ncp; c++) {
        rc |= solve_state_block(o, c);
        memcpy(o->U0, o->U + (size_t)(tsc - 1) * nd, sizeof(double) * nd);
        memcpy(o->DU0, o->DU + (size_t)(tsc - 1) * nd, sizeof(double) * nd);
        memcpy(o->DDU0, o->DDU + (size_t)(tsc - 1) * nd, sizeof(double) * nd);
        double *cpc = o->cp + (size_t)(c + 1) * 3 * nd;
        memcpy(cpc, o->U0, sizeof(double) * nd);
        memcpy(cpc + nd, o->DU0, sizeof(double) * nd);
        memcpy(cpc + 2 * nd, o->DDU0, sizeof(double) * nd);
    }
    return rc;
}

/* EvaluateObjective, LinearElasticity.cc:1416-1465 (s = 1, EvaluateObjectiveScale :1400-1414) */
static double eval_objective(int obj, double dt, double kfac, double uKu, double mfac, double duMdu, double uu,
                             double dudu, double dduddu, double duCdu) {
    switch (obj) {
    case 0: return dt * 0.5 * uu;
    case 1: return dt * 0.5 * dudu;
    case 2: return dt * 0.5 * dduddu;
    case 3: return dt * 0.5 * (kfac * uKu);
    case 4: return dt * 0.5 * (mfac * duMdu);
    case 5: return dt * 0.5 * (kfac * uKu + mfac * duMdu);
    default: return dt * 0.5 * duCdu;
    }
}
/* EvaluateObjectiveGradient, LinearElasticity.cc:1469-1514 */
static double eval_objective_gradient(int obj, double dt, double dkfac, double uKu, double dmfac, double duMdu,
                                     double DxduCdu) {
    switch (obj) {
    case 3: return dt * 0.5 * (dkfac * uKu);
    case 4: return dt * 0.5 * (dmfac * duMdu);
    case 5: return dt * 0.5 * (dkfac * uKu + dmfac * duMdu);
    case 6: return dt * 0.5 * DxduCdu;
    default: return 0.0;
    }
}

/* ComputeObjectiveElementLoop, LinearElasticity.cc:2359-2452 */
static double objective_loop(topo_oracle *o, const double *up, const double *dup, const double *ddup) {
    const topo_oracle_params *p = &o->p;
    if (p->objective == 7) { /* extension: dt/2 u_out^2 */
        double v = up[out_dof(o)];
        return o->dt * 0.5 * v * v;
    }
    double *he = vnew(o->nel);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < o->nel; e++) {
        int ed[24];
        edofs(o, e, ed);
        double kf = o->kfac[e], mf = o->mfac[e];
        double uKu = 0, duMdu = 0, duCdu = 0, uu = 0, dudu = 0, dduddu = 0;
        for (int k = 0; k < 24; k++) {
            for (int h = 0; h < 24; h++) {
                uKu += up[ed[k]] * o->KE[k * 24 + h] * up[ed[h]];
                duMdu += dup[ed[k]] * o->ME[k * 24 + h] * dup[ed[h]];
                duCdu += dup[ed[k]] * (p->dalpha * mf * o->ME[k * 24 + h] + p->dbeta * kf * o->KE[k * 24 + h]) *
                         dup[ed[h]];
            }
            uu += up[ed[k]] * up[ed[k]];
            dudu += dup[ed[k]] * dup[ed[k]];
            dduddu += ddup[ed[k]] * ddup[ed[k]];
        }
        he[e] = eval_objective(p->objective, o->dt, kf, uKu, mf, duMdu, uu, dudu, dduddu, duCdu) * o->P[e];
    }
    double fx = 0.0;
    for (int e = 0; e < o->nel; e++) fx += he[e];
    free(he);
    return fx;
}

/* ComputeGradientObjectiveElementLoop + GradObjectiveWrtState,
 * LinearElasticity.cc:2206-2356 and :1516-1576: scatter of P_e * s * dh/d(u,du,ddu). */
static void gradient_objective_loop(topo_oracle *o, const double *up, const double *dup, const double *ddup) {
    const topo_oracle_params *p = &o->p;
    int nd = o->ndof;
    memset(o->HDU, 0, sizeof(double) * nd);
    memset(o->HDDU, 0, sizeof(double) * nd);
    memset(o->HDDDU, 0, sizeof(double) * nd);
    double dt = o->dt;
    if (p->objective == 7) {
        o->HDU[out_dof(o)] = dt * up[out_dof(o)];
        return;
    }
    for (int color = 0; color < 8; color++) {
        int ci = color & 1, cj = (color >> 1) & 1, ck = (color >> 2) & 1;
#pragma omp parallel for collapse(2) schedule(static)
        for (int k = ck; k < o->nez; k += 2)
            for (int j = cj; j < o->ney; j += 2)
                for (int i = ci; i < o->nex; i += 2) {
                    int e = i + o->nex * (j + o->ney * k);
                    int ed[24];
                    edofs(o, e, ed);
                    double kf = o->kfac[e], mf = o->mfac[e], w = o->P[e] * 1.0;
                    for (int kk = 0; kk < 24; kk++) {
                        double h1 = 0, h2 = 0, h3 = 0;
                        switch (p->objective) {
                        case 0: h1 = dt * up[ed[kk]]; break;
                        case 1: h2 = dt * dup[ed[kk]]; break;
                        case 2: h3 = dt * ddup[ed[kk]]; break;
                        case 3:
                            for (int h = 0; h < 24; h++) h1 += dt * kf * o->KE[kk * 24 + h] * up[ed[h]];
                            break;
                        case 4:
                            for (int h = 0; h < 24; h++) h2 += dt * mf * o->ME[kk * 24 + h] * dup[ed[h]];
                            break;
                        case 5:
                            for (int h = 0; h < 24; h++) {
                                h1 += dt * kf * o->KE[kk * 24 + h] * up[ed[h]];
                                h2 += dt * mf * o->ME[kk * 24 + h] * dup[ed[h]];
                            }
                            break;
                        default:
                            for (int h = 0; h < 24; h++)
                                h2 += dt * (p->dalpha * mf * o->ME[kk * 24 + h] + p->dbeta * kf * o->KE[kk * 24 + h]) *
                                      dup[ed[h]];
                        }
                        o->HDU[ed[kk]] += w * h1;
                        o->HDDU[ed[kk]] += w * h2;
                        o->HDDDU[ed[kk]] += w * h3;
                    }
                }
    }
}

/* SolveLagrangen, LinearElasticity.cc:808-954 */
static int solve_lagrangen(topo_oracle *o, int c) {
    const topo_oracle_params *p = &o->p;
    int nd = o->ndof, tsc = p->tsc, rc = 0;
    double *a = o->a;
    double *b1 = vnew(nd), *b2 = vnew(nd), *b3 = vnew(nd), *r1 = vnew(nd);
    for (int j = tsc - 1; j >= 0; j--) {
        int t = tsc * c + j + 1;
        double *Lj = o->L + (size_t)j * nd, *DLj = o->DL + (size_t)j * nd, *DDLj = o->DDL + (size_t)j * nd;
        gradient_objective_loop(o, o->U + (size_t)j * nd, o->DU + (size_t)j * nd, o->DDU + (size_t)j * nd);
        if (t == o->Ts - 1) {
#pragma omp parallel for schedule(static)
            for (int i = 0; i < nd; i++) {
                DLj[i] = -o->HDDU[i];
                DDLj[i] = -o->HDDDU[i];
                r1[i] = o->N[i] * (-(o->HDU[i] - a[2] * DLj[i] - a[5] * DDLj[i]));
            }
            rc |= solve_eff(o, r1, Lj);
            memcpy(o->LT, Lj, sizeof(double) * nd);
        } else {
            bmult(o, a[5] + a[2] * p->dalpha, a[2] * p->dbeta, o->Lp1, b1);
            bmult(o, a[3] - a[0] * p->dalpha, -a[0] * p->dbeta, o->Lp1, b2);
            bmult(o, a[4] - a[1] * p->dalpha, -a[1] * p->dbeta, o->Lp1, b3);
#pragma omp parallel for schedule(static)
            for (int i = 0; i < nd; i++) {
                DLj[i] = -(o->HDDU[i] + b2[i] - a[0] * o->DLp1[i] + a[3] * o->DDLp1[i]);
                DDLj[i] = -(o->HDDDU[i] + b3[i] + a[4] * o->DDLp1[i]);
                double v = -(o->HDU[i] + b1[i] + a[2] * o->DLp1[i] + a[5] * o->DDLp1[i]) + a[2] * DLj[i] + a[5] * DDLj[i];
                r1[i] = o->N[i] * v;
            }
            rc |= solve_eff(o, r1, Lj);
        }
        memcpy(o->Lp1, Lj, sizeof(double) * nd);
        memcpy(o->DLp1, DLj, sizeof(double) * nd);
        memcpy(o->DDLp1, DDLj, sizeof(double) * nd);
    }
    free(b1);
    free(b2);
    free(b3);
    free(r1);
    return rc;
}

/* SolveLagrange0, LinearElasticity.cc:678-804 */
static int solve_lagrange0(topo_oracle *o) {
    const topo_oracle_params *p = &o->p;
    int nd = o->ndof;
    double *a = o->a;
    double *b3 = vnew(nd), *r3 = vnew(nd);
    gradient_objective_loop(o, o->U0, o->DU0, o->DDU0);
    bmult(o, a[4] - a[1] * p->dalpha, -a[1] * p->dbeta, o->Lp1, b3);
    for (int i = 0; i < nd; i++)
        r3[i] = o->N[i] * (-(o->HDDDU[i] + b3[i] - a[1] * o->DLp1[i] + a[4] * o->DDLp1[i]));
    int rc = solve_mass(o, r3, o->DDL0);
    free(b3);
    free(r3);
    return rc;
}

/* ComputeSensitivitiesElementLoopn, LinearElasticity.cc:1911-2077 */
static void sens_loop_n(topo_oracle *o, double *df, const double *up, const double *dup, const double *lp,
                        const double *ubp, const double *dubp, const double *ddubp) {
    const topo_oracle_params *p = &o->p;
    double *a = o->a, dt = o->dt;
#pragma omp parallel for schedule(static)
    for (int e = 0; e < o->nel; e++) {
        int ed[24];
        edofs(o, e, ed);
        double dkf = o->dkfac[e], dmf = o->dmfac[e];
        double t3 = 0, uKu = 0, duMdu = 0, DxduCdu = 0;
        for (int k = 0; k < 24; k++) {
            for (int h = 0; h < 24; h++) {
                double dme = dmf * o->ME[k * 24 + h];
                double dke = dkf * o->KE[k * 24 + h];
                double dce = p->dalpha * dme + p->dbeta * dke;
                double dAdx = -dke - a[5] * dme - a[2] * dce;
                double dBdx1 = a[5] * dme + a[2] * dce;
                double dBdx2 = a[3] * dme - a[0] * dce;
                double dBdx3 = a[4] * dme - a[1] * dce;
                double dAdxu = dAdx * up[ed[h]];
                double dBdxu = dBdx1 * ubp[ed[h]] + dBdx2 * dubp[ed[h]] + dBdx3 * ddubp[ed[h]];
                t3 += lp[ed[k]] * (dAdxu + dBdxu);
                uKu += up[ed[k]] * o->KE[k * 24 + h] * up[ed[h]];
                duMdu += dup[ed[k]] * o->ME[k * 24 + h] * dup[ed[h]];
                DxduCdu += dup[ed[k]] * dce * dup[ed[h]];
            }
        }
        double dfx0 = eval_objective_gradient(p->objective, dt, dkf, uKu, dmf, duMdu, DxduCdu);
        df[e] += o->P[e] * (dfx0 * 1.0) + t3;
    }
}

/* ComputeSensitivitiesElementLoop0, LinearElasticity.cc:2080-2204 */
static void sens_loop_0(topo_oracle *o, double *df) {
    const topo_oracle_params *p = &o->p;
    double dt = o->dt;
    const double *up = o->U0, *dup = o->DU0, *ddup = o->DDU0, *ddlp = o->DDL0;
#pragma omp parallel for schedule(static)
    for (int e = 0; e < o->nel; e++) {
        int ed[24];
        edofs(o, e, ed);
        double dkf = o->dkfac[e], dmf = o->dmfac[e];
        double t2 = 0, uKu = 0, duMdu = 0, DxduCdu = 0;
        for (int k = 0; k < 24; k++) {
            for (int h = 0; h < 24; h++) {
                double dme = dmf * o->ME[k * 24 + h];
                double dke = dkf * o->KE[k * 24 + h];
                double dce = p->dalpha * dme + p->dbeta * dke;
                t2 += ddlp[ed[k]] * dke * up[ed[h]] + ddlp[ed[k]] * dce * dup[ed[h]] + ddlp[ed[k]] * dme * ddup[ed[h]];
                uKu += up[ed[k]] * o->KE[k * 24 + h] * up[ed[h]];
                duMdu += dup[ed[k]] * o->ME[k * 24 + h] * dup[ed[h]];
                DxduCdu += dup[ed[k]] * dce * dup[ed[h]];
            }
        }
        double dfx0 = eval_objective_gradient(p->objective, dt, dkf, uKu, dmf, duMdu, DxduCdu);
        df[e] += o->P[e] * dfx0 + t2;
    }
}

/* ComputeObjectiveSensitivities, LinearElasticity.cc:1625-1908 */
int oracle_le_compute_objective_sensitivities(topo_oracle *o, const double *xPhys, double *fx, double *dfdx) {
    (void)xPhys; /* interpolation factors come from CompleteInitialState's xPhys (same vector in main.cc) */
    int nd = o->ndof, tsc = o->p.tsc, rc = 0;
    memset(dfdx, 0, sizeof(double) * o->nel);
    double f = 0.0;
    for (int c = o->p.ncp - 1; c >= 0; c--) {
        double *cpc = o->cp + (size_t)c * 3 * nd;
        memcpy(o->U0, cpc, sizeof(double) * nd);
        memcpy(o->DU0, cpc + nd, sizeof(double) * nd);
        memcpy(o->DDU0, cpc + 2 * nd, sizeof(double) * nd);
        rc |= solve_state_block(o, c);
        rc |= solve_lagrangen(o, c);
        for (int tc = 0; tc < tsc; tc++)
            f += objective_loop(o, o->U + (size_t)tc * nd, o->DU + (size_t)tc * nd, o->DDU + (size_t)tc * nd);
        if (c == 0) f += objective_loop(o, o->U0, o->DU0, o->DDU0);
        for (int tc = 0; tc < tsc; tc++) {
            const double *ub = tc ? o->U + (size_t)(tc - 1) * nd : o->U0;
            const double *dub = tc ? o->DU + (size_t)(tc - 1) * nd : o->DU0;
            const double *ddub = tc ? o->DDU + (size_t)(tc - 1) * nd : o->DDU0;
            sens_loop_n(o, dfdx, o->U + (size_t)tc * nd, o->DU + (size_t)tc * nd, o->L + (size_t)tc * nd, ub, dub,
                        ddub);
        }
        if (c == 0) {
            rc |= solve_lagrange0(o);
            sens_loop_0(o, dfdx);
        }
    }
    *fx = f;
    return rc;
}

/* VolumeConstraint, LinearElasticity.cc:1283-1296 */
void oracle_le_volume_constraint(int nel, const double *xPhys, double volfrac, double *gx, double *dgdx) {
    double s = 0.0;
    for (int e = 0; e < nel; e++) s += xPhys[e];
    *gx = s / nel - volfrac;
    for (int e = 0; e < nel; e++) dgdx[e] = 1.0 / nel;
}

/* LoadSolutionAsU0 (LinearElasticity.cc:2621-2677, called at :523 after
 * VecSet(U0, 0)): the initial displacement of every CompleteInitialState;
 * NULL restores rest */
void oracle_le_set_u0(topo_oracle *o, const double *U0) {
    if (U0)
        memcpy(o->U0init, U0, sizeof(double) * o->ndof);
    else
        memset(o->U0init, 0, sizeof(double) * o->ndof);
}

int oracle_le_sizes(const topo_oracle *o, int *ndof, int *nel, int *Ts) {
    *ndof = o->ndof;
    *nel = o->nel;
    *Ts = o->Ts;
    return 0;
}
void oracle_le_get_vectors(const topo_oracle *o, double *N, double *P, double *RHS0) {
    memcpy(N, o->N, sizeof(double) * o->ndof);
    memcpy(P, o->P, sizeof(double) * o->nel);
    memcpy(RHS0, o->RHS0, sizeof(double) * o->ndof);
}
void oracle_le_get_newmark(const topo_oracle *o, double *a6, double *dt) {
    memcpy(a6, o->a, sizeof(double) * 6);
    *dt = o->dt;
}
void oracle_le_get_initial_state(const topo_oracle *o, double *U0, double *DU0, double *DDU0) {
    int nd = o->ndof;
    memcpy(U0, o->cp, sizeof(double) * nd);
    memcpy(DU0, o->cp + nd, sizeof(double) * nd);
    memcpy(DDU0, o->cp + 2 * nd, sizeof(double) * nd);
}
void oracle_le_get_last_block(const topo_oracle *o, int j, double *U, double *DU, double *DDU) {
    size_t nd = o->ndof;
    memcpy(U, o->U + j * nd, sizeof(double) * nd);
    memcpy(DU, o->DU + j * nd, sizeof(double) * nd);
    memcpy(DDU, o->DDU + j * nd, sizeof(double) * nd);
}
void oracle_le_get_adjoint0(const topo_oracle *o, double *L1, double *DDL0) {
    memcpy(L1, o->Lp1, sizeof(double) * o->ndof);
    memcpy(DDL0, o->DDL0, sizeof(double) * o->ndof);
}
/* the three vectors of WriteRestartFiles (LinearElasticity.cc:2457-2496):
 * the initial acceleration (checkpoint 0), the terminal adjoint of the last
 * reverse sweep and the adjoint acceleration at t = 0 */
void oracle_le_get_restart_state(const topo_oracle *o, double *DDU0, double *LT, double *DDL0) {
    memcpy(DDU0, o->cp + 2 * (size_t)o->ndof, sizeof(double) * o->ndof);
    memcpy(LT, o->LT, sizeof(double) * o->ndof);
    memcpy(DDL0, o->DDL0, sizeof(double) * o->ndof);
}
long oracle_le_total_cg_iterations(const topo_oracle *o) { return o->cg_iters; }

/* ------------------------------------------------------------------ */
/* PDE filter (PDEFilter.cc)                                            */
/* ------------------------------------------------------------------ */

/* 8x8 Helmholtz element matrix R^2 * int grad Ni . grad Nj + int Ni Nj on an
 * hx*hy*hz box; PDEFilter.cc:485-578 writes the same matrix in closed form. */
void oracle_pde_filter_matrix(double hx, double hy, double hz, double R, double *KF) {
    const double gp[2] = {-0.577350269189626, 0.577350269189626};
    memset(KF, 0, sizeof(double) * 64);
    double det = hx * hy * hz / 8.0;
    for (int ii = 0; ii < 2; ii++)
        for (int jj = 0; jj < 2; jj++)
            for (int kk = 0; kk < 2; kk++) {
                double S[8], dxi[8], deta[8], dzeta[8];
                shape8(gp[ii], gp[jj], gp[kk], S, dxi, deta, dzeta);
                for (int a = 0; a < 8; a++)
                    for (int b = 0; b < 8; b++) {
                        double g = (2 / hx) * (2 / hx) * dxi[a] * dxi[b] + (2 / hy) * (2 / hy) * deta[a] * deta[b] +
                                   (2 / hz) * (2 / hz) * dzeta[a] * dzeta[b];
                        KF[8 * a + b] += det * (R * R * g + S[a] * S[b]);
                    }
            }
}

typedef struct {
    stencil_t *s;
} sctx;
static void op_scalar(void *c, const double *x, double *y) { st_mult(((sctx *)c)->s, x, y); }

/* PDEFilt::FilterProject, PDEFilter.cc:193-222:  U = K^-1 (elemVol T x), xout = T^T U */
void oracle_pde_filter(int nx, int ny, int nz, double hx, double hy, double hz, double rmin, const double *xin,
                       double *xout, double rtol) {
    int nex = nx - 1, ney = ny - 1, nez = nz - 1, nn = nx * ny * nz, nel = nex * ney * nez;
    double R = rmin / 2.0 / sqrt(3.0); /* PDEFilter.cc:32 */
    double KF[64];
    oracle_pde_filter_matrix(hx, hy, hz, R, KF);
    stencil_t s;
    st_alloc(&s, nx, ny, nz, 1);
    double *ones = vnew(nel);
    for (int e = 0; e < nel; e++) ones[e] = 1.0;
    st_assemble(&s, KF, ones);
    double *rhs = vnew(nn), *u = vnew(nn), *dinv = vnew(nn);
    st_diag(&s, dinv);
    for (int i = 0; i < nn; i++) dinv[i] = 1.0 / dinv[i];
    double vol = hx * hy * hz;
    /* MatMult(T, x): T = 0.125 per element node (PDEFilter.cc:580-588) */
    for (int e = 0; e < nel; e++) {
        int i = e % nex, j = (e / nex) % ney, k = e / (nex * ney);
        for (int a = 0; a < 8; a++) rhs[(i + LN[a][0]) + nx * ((j + LN[a][1]) + ny * (k + LN[a][2]))] += 0.125 * xin[e];
    }
    for (int i = 0; i < nn; i++) rhs[i] *= vol;
    sctx c = {&s};
    pcg(op_scalar, &c, dinv, nn, rhs, u, rtol, 100000, NULL);
    for (int e = 0; e < nel; e++) {
        int i = e % nex, j = (e / nex) % ney, k = e / (nex * ney);
        double acc = 0.0;
        for (int a = 0; a < 8; a++) acc += 0.125 * u[(i + LN[a][0]) + nx * ((j + LN[a][1]) + ny * (k + LN[a][2]))];
        xout[e] = acc;
    }
    free(rhs);
    free(u);
    free(dinv);
    free(ones);
    st_free(&s);
}

/* Filter.h:80-88 */
static double smooth_projection(double x, double beta, double eta) {
    return (tanh(beta * eta) + tanh(beta * (x - eta))) / (tanh(beta * eta) + tanh(beta * (1.0 - eta)));
}
static double chainrule_smooth_projection(double x, double beta, double eta) {
    return beta * (1.0 - pow(tanh(beta * (x - eta)), 2.0)) / (tanh(beta * eta) + tanh(beta * (1.0 - eta)));
}

/* Filter::FilterProject, filterType 2, Filter.cc:60-119 */
void oracle_filter_project(int nx, int ny, int nz, double hx, double hy, double hz, double rmin, const double *x,
                           double *xTilde, double *xPhys, int projection, double beta, double eta, double rtol) {
    int nel = (nx - 1) * (ny - 1) * (nz - 1);
    oracle_pde_filter(nx, ny, nz, hx, hy, hz, rmin, x, xTilde, rtol);
    for (int i = 0; i < nel; i++) {
        if (xTilde[i] < 0.0) xTilde[i] = 0.0;
        if (xTilde[i] > 1.0) xTilde[i] = 1.0;
    }
    for (int i = 0; i < nel; i++) xPhys[i] = projection ? smooth_projection(xTilde[i], beta, eta) : xTilde[i];
}

/* Filter::Gradients, filterType 2, Filter.cc:122-206 */
void oracle_filter_gradients(int nx, int ny, int nz, double hx, double hy, double hz, double rmin,
                             const double *xTilde, double *dfdx, int m, double *dgdx, int projection, double beta,
                             double eta, double rtol) {
    int nel = (nx - 1) * (ny - 1) * (nz - 1);
    if (projection) {
        for (int i = 0; i < nel; i++) {
            double d = chainrule_smooth_projection(xTilde[i], beta, eta);
            dfdx[i] *= d;
            for (int j = 0; j < m; j++) dgdx[(size_t)j * nel + i] *= d;
        }
    }
    double *tmp = vnew(nel);
    oracle_pde_filter(nx, ny, nz, hx, hy, hz, rmin, dfdx, tmp, rtol);
    memcpy(dfdx, tmp, sizeof(double) * nel);
    for (int j = 0; j < m; j++) {
        oracle_pde_filter(nx, ny, nz, hx, hy, hz, rmin, dgdx + (size_t)j * nel, tmp, rtol);
        memcpy(dgdx + (size_t)j * nel, tmp, sizeof(double) * nel);
    }
    free(tmp);
}

/* Filter::SetUp, filterType 0/1 (Filter.cc:302-531): out = H in.  The
 * stencil half-width is ElemConn = max_a(ceil(R/h_a) - 1), at least 1; the
 * neighbour range along axis a is [max(i - ElemConn, 0),
 * min(i + ElemConn, n_a - 1, i + ceil(R/h_a) - 1)] (:467-469); entries
 * R - dist for element-centre distances dist < R (:478-490); with
 * ElemConn == 1 H is the identity (:451-459). */
void oracle_dens_filter_apply(int ex, int ey, int ez, double hx, double hy, double hz, double R, const double *in,
                              double *out) {
    int cx = (int)ceil(R / hx) - 1, cy = (int)ceil(R / hy) - 1, cz = (int)ceil(R / hz) - 1;
    int sw = cx > cy ? cx : cy;
    if (cz > sw) sw = cz;
    if (sw == 0) sw = 1;
    long long nel = (long long)ex * ey * ez;
    if (sw == 1) {
        for (long long e = 0; e < nel; e++) out[e] = in[e];
        return;
    }
    for (int k = 0; k < ez; k++)
        for (int j = 0; j < ey; j++)
            for (int i = 0; i < ex; i++) {
                double acc = 0.0;
                int k1 = k + sw < ez - 1 ? k + sw : ez - 1, j1 = j + sw < ey - 1 ? j + sw : ey - 1,
                    i1 = i + sw < ex - 1 ? i + sw : ex - 1;
                if (k + cz < k1) k1 = k + cz;
                if (j + cy < j1) j1 = j + cy;
                if (i + cx < i1) i1 = i + cx;
                for (int k2 = (k - sw > 0 ? k - sw : 0); k2 <= k1; k2++)
                    for (int j2 = (j - sw > 0 ? j - sw : 0); j2 <= j1; j2++)
                        for (int i2 = (i - sw > 0 ? i - sw : 0); i2 <= i1; i2++) {
                            /* element centres h/2 + i h (DMDASetUniformCoordinates, :420) */
                            double d0 = (hx / 2 + i * hx) - (hx / 2 + i2 * hx);
                            double d1 = (hy / 2 + j * hy) - (hy / 2 + j2 * hy);
                            double d2 = (hz / 2 + k * hz) - (hz / 2 + k2 * hz);
                            double dist = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                            if (dist < R) acc += (R - dist) * in[i2 + (long long)ex * (j2 + (long long)ey * k2)];
                        }
                out[i + (long long)ex * (j + (long long)ey * k)] = acc;
            }
}

/* Filter::FilterProject, filterType 0/1 (Filter.cc:60-119) */
void oracle_dens_filter_project(int ex, int ey, int ez, double hx, double hy, double hz, int ftype, double R,
                                const double *x, double *xTilde, double *xPhys, int projection, double beta,
                                double eta) {
    long long nel = (long long)ex * ey * ez;
    if (ftype == 1) {
        double *one = vnew(nel), *hs = vnew(nel);
        for (long long e = 0; e < nel; e++) one[e] = 1.0;
        oracle_dens_filter_apply(ex, ey, ez, hx, hy, hz, R, one, hs);
        oracle_dens_filter_apply(ex, ey, ez, hx, hy, hz, R, x, xTilde);
        for (long long e = 0; e < nel; e++) xTilde[e] /= hs[e];
        free(one);
        free(hs);
    } else {
        memcpy(xTilde, x, sizeof(double) * nel);
    }
    for (long long e = 0; e < nel; e++) xPhys[e] = projection ? smooth_projection(xTilde[e], beta, eta) : xTilde[e];
}

/* Filter::Gradients, filterType 0/1 (Filter.cc:122-206) */
void oracle_dens_filter_gradients(int ex, int ey, int ez, double hx, double hy, double hz, int ftype, double R,
                                  const double *x, const double *xTilde, double *dfdx, int m, double *dgdx,
                                  int projection, double beta, double eta) {
    long long nel = (long long)ex * ey * ez;
    if (projection) {
        for (long long e = 0; e < nel; e++) {
            double d = chainrule_smooth_projection(xTilde[e], beta, eta);
            dfdx[e] *= d;
            for (int j = 0; j < m; j++) dgdx[(size_t)j * nel + e] *= d;
        }
    }
    double *one = vnew(nel), *hs = vnew(nel), *tmp = vnew(nel);
    for (long long e = 0; e < nel; e++) one[e] = 1.0;
    oracle_dens_filter_apply(ex, ey, ez, hx, hy, hz, R, one, hs);
    if (ftype == 0) { /* sensitivities only: (H (df .* x) ./ Hs) ./ x */
        for (long long e = 0; e < nel; e++) tmp[e] = dfdx[e] * x[e];
        oracle_dens_filter_apply(ex, ey, ez, hx, hy, hz, R, tmp, dfdx);
        for (long long e = 0; e < nel; e++) dfdx[e] = (dfdx[e] / hs[e]) / x[e];
    } else { /* H (v ./ Hs) for df and every dg */
        for (int j = -1; j < m; j++) {
            double *v = j < 0 ? dfdx : dgdx + (size_t)j * nel;
            for (long long e = 0; e < nel; e++) tmp[e] = v[e] / hs[e];
            oracle_dens_filter_apply(ex, ey, ez, hx, hy, hz, R, tmp, v);
        }
    }
    free(one);
    free(hs);
    free(tmp);
}

/* Filter::GetMND, Filter.cc:208-227 */
double oracle_filter_mnd(int n, const double *x) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += 4 * x[i] * (1.0 - x[i]);
    return s / n;
}

/* Filter::IncreaseBeta, Filter.cc:274-300 */
int oracle_increase_beta(double *beta, double betaFinal, double gx, int itr, double ch) {
    int change = 0;
    if ((ch < 0.01 || itr % 10 == 0) && beta[0] < betaFinal && gx <= 0.0) {
        change = 1;
        if (beta[0] < 7)
            beta[0] = beta[0] + 1;
        else
            beta[0] = beta[0] * 1.2;
        if (beta[0] > betaFinal) {
            beta[0] = betaFinal;
            change = 0;
        }
    }
    return change;
}

/* ------------------------------------------------------------------ */
/* MMA (MMA.cc)                                                          */
/* ------------------------------------------------------------------ */
struct topo_oracle_mma {
    int n, m, k;
    double asyminit, asymdec, asyminc;
    double *a, *c, *d, *y, z, *lam, *mu, *s, *b, *grad, *Hess;
    double *L, *U, *alpha, *beta, *p0, *q0, *pij, *qij, *xo1, *xo2;
};

/* MMA(n, m, x, a, c, d), MMA.cc:180-229 */
topo_oracle_mma *oracle_mma_create(int n, int m, const double *x, const double *a, const double *c,
                                   const double *d) {
    topo_oracle_mma *mm = (topo_oracle_mma *)calloc(1, sizeof(topo_oracle_mma));
    mm->n = n;
    mm->m = m;
    mm->k = 0;
    mm->asyminit = 0.5;
    mm->asymdec = 0.7;
    mm->asyminc = 1.2;
    mm->a = vnew(m);
    mm->c = vnew(m);
    mm->d = vnew(m);
    memcpy(mm->a, a, sizeof(double) * m);
    memcpy(mm->c, c, sizeof(double) * m);
    memcpy(mm->d, d, sizeof(double) * m);
    mm->y = vnew(m);
    mm->lam = vnew(m);
    mm->mu = vnew(m);
    mm->s = vnew(2 * m);
    mm->b = vnew(m);
    mm->grad = vnew(m);
    mm->Hess = vnew((size_t)m * m);
    mm->L = vnew(n);
    mm->U = vnew(n);
    mm->alpha = vnew(n);
    mm->beta = vnew(n);
    mm->p0 = vnew(n);
    mm->q0 = vnew(n);
    mm->pij = vnew((size_t)n * m);
    mm->qij = vnew((size_t)n * m);
    mm->xo1 = vnew(n);
    mm->xo2 = vnew(n);
    (void)x;
    return mm;
}
void oracle_mma_destroy(topo_oracle_mma *mm) {
    if (!mm) return;
    double *ptrs[] = {mm->a,  mm->c,    mm->d,    mm->y,  mm->lam, mm->mu,  mm->s,   mm->b,   mm->grad, mm->Hess,
                      mm->L, mm->U, mm->alpha, mm->beta, mm->p0, mm->q0,  mm->pij, mm->qij, mm->xo1, mm->xo2};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
    free(mm);
}
/* MMA::SetAsymptotes, MMA.cc:350-358 */
void oracle_mma_set_asymptotes(topo_oracle_mma *mm, double init, double dec, double inc) {
    mm->asyminit = init;
    mm->asymdec = dec;
    mm->asyminc = inc;
}
/* MMA::SetOuterMovelimit, MMA.cc:374-393 */
void oracle_mma_set_outer_movelimit(int n, double Xmin, double Xmax, double movlim, const double *x, double *xmin,
                                    double *xmax) {
    for (int i = 0; i < n; i++) {
        xmax[i] = fmin(Xmax, x[i] + movlim);
        xmin[i] = fmax(Xmin, x[i] - movlim);
    }
}
/* MMA::DesignChange, MMA.cc:395-414 */
double oracle_mma_design_change(int n, const double *x, double *xold) {
    double ch = 0.0;
    for (int i = 0; i < n; i++) {
        ch = fmax(ch, fabs(x[i] - xold[i]));
        xold[i] = x[i];
    }
    return ch;
}
static double dmax(double a, double b) { return a > b ? a : b; }
static double dmin(double a, double b) { return a < b ? a : b; }

/* MMA::GenSub, MMA.cc:510-637 (RobustAsymptotesType 0, no constraint modification) */
static void mma_gensub(topo_oracle_mma *mm, const double *xv, const double *dfdx, const double *gx, const double *dgdx,
                       const double *xmin, const double *xmax) {
    int n = mm->n, m = mm->m;
    mm->k++;
    if (mm->k < 3) {
        for (int i = 0; i < n; i++) {
            mm->L[i] = xv[i] - mm->asyminit * (xmax[i] - xmin[i]);
            mm->U[i] = xv[i] + mm->asyminit * (xmax[i] - xmin[i]);
        }
    }
    if (mm->k > 2) {
        for (int i = 0; i < n; i++) {
            double helpvar = (xv[i] - mm->xo1[i]) * (mm->xo1[i] - mm->xo2[i]);
            double gamma = helpvar < 0.0 ? mm->asymdec : (helpvar > 0.0 ? mm->asyminc : 1.0);
            mm->L[i] = xv[i] - gamma * (mm->xo1[i] - mm->L[i]);
            mm->U[i] = xv[i] + gamma * (mm->U[i] - mm->xo1[i]);
            double xmi = dmax(1.0e-5, xmax[i] - xmin[i]);
            mm->L[i] = dmax(mm->L[i], xv[i] - 10.0 * xmi);
            mm->L[i] = dmin(mm->L[i], xv[i] - 0.01 * xmi);
            mm->U[i] = dmax(mm->U[i], xv[i] + 0.01 * xmi);
            mm->U[i] = dmin(mm->U[i], xv[i] + 10.0 * xmi);
        }
    }
    double feps = 1.0e-6;
    for (int i = 0; i < n; i++) {
        mm->alpha[i] = dmax(xmin[i], 0.9 * mm->L[i] + 0.1 * xv[i]);
        mm->beta[i] = dmin(xmax[i], 0.9 * mm->U[i] + 0.1 * xv[i]);
        double dfp = dmax(0.0, dfdx[i]), dfm = dmax(0.0, -1.0 * dfdx[i]);
        mm->p0[i] = pow(mm->U[i] - xv[i], 2.0) * (dfp + 0.001 * fabs(dfdx[i]) + 0.5 * feps / (mm->U[i] - mm->L[i]));
        mm->q0[i] = pow(xv[i] - mm->L[i], 2.0) * (dfm + 0.001 * fabs(dfdx[i]) + 0.5 * feps / (mm->U[i] - mm->L[i]));
        for (int j = 0; j < m; j++) {
            double g = dgdx[(size_t)j * n + i];
            mm->pij[(size_t)j * n + i] = pow(mm->U[i] - xv[i], 2.0) * dmax(0.0, g);
            mm->qij[(size_t)j * n + i] = pow(xv[i] - mm->L[i], 2.0) * dmax(0.0, -1.0 * g);
        }
    }
    for (int j = 0; j < m; j++) {
        double s = 0.0;
        for (int i = 0; i < n; i++)
            s += mm->pij[(size_t)j * n + i] / (mm->U[i] - xv[i]) + mm->qij[(size_t)j * n + i] / (xv[i] - mm->L[i]);
        mm->b[j] = s - gx[j];
    }
}

/* MMA::XYZofLAMBDA, MMA.cc:678-728 */
static void mma_xyz(topo_oracle_mma *mm, double *x) {
    int n = mm->n, m = mm->m;
    double lamai = 0.0;
    for (int i = 0; i < m; i++) {
        if (mm->lam[i] < 0.0) mm->lam[i] = 0;
        mm->y[i] = dmax(0.0, mm->lam[i] - mm->c[i]);
        lamai += mm->lam[i] * mm->a[i];
    }
    mm->z = dmax(0.0, 10.0 * (lamai - 1.0));
    for (int i = 0; i < n; i++) {
        double pj = mm->p0[i], qj = mm->q0[i];
        for (int j = 0; j < m; j++) {
            pj += mm->pij[(size_t)j * n + i] * mm->lam[j];
            qj += mm->qij[(size_t)j * n + i] * mm->lam[j];
        }
        x[i] = (sqrt(pj) * mm->L[i] + sqrt(qj) * mm->U[i]) / (sqrt(pj) + sqrt(qj));
        if (x[i] < mm->alpha[i]) x[i] = mm->alpha[i];
        if (x[i] > mm->beta[i]) x[i] = mm->beta[i];
    }
}
/* MMA::DualGrad, MMA.cc:730-765 */
static void mma_dualgrad(topo_oracle_mma *mm, const double *x) {
    int n = mm->n, m = mm->m;
    for (int j = 0; j < m; j++) {
        double s = 0.0;
        for (int i = 0; i < n; i++)
            s += mm->pij[(size_t)j * n + i] / (mm->U[i] - x[i]) + mm->qij[(size_t)j * n + i] / (x[i] - mm->L[i]);
        mm->grad[j] = s - mm->b[j] - mm->a[j] * mm->z - mm->y[j];
    }
}
/* MMA::DualHess, MMA.cc:767-868 */
static void mma_dualhess(topo_oracle_mma *mm, const double *x) {
    int n = mm->n, m = mm->m;
    double *df2 = vnew(n), *PQ = vnew((size_t)n * m);
    for (int i = 0; i < n; i++) {
        double pj = mm->p0[i], qj = mm->q0[i];
        for (int j = 0; j < m; j++) {
            pj += mm->pij[(size_t)j * n + i] * mm->lam[j];
            qj += mm->qij[(size_t)j * n + i] * mm->lam[j];
            PQ[(size_t)i * m + j] = mm->pij[(size_t)j * n + i] / pow(mm->U[i] - x[i], 2.0) -
                                    mm->qij[(size_t)j * n + i] / pow(x[i] - mm->L[i], 2.0);
        }
        df2[i] = -1.0 / (2.0 * pj / pow(mm->U[i] - x[i], 3.0) + 2.0 * qj / pow(x[i] - mm->L[i], 3.0));
        double xp = (sqrt(pj) * mm->L[i] + sqrt(qj) * mm->U[i]) / (sqrt(pj) + sqrt(qj));
        if (xp < mm->alpha[i]) df2[i] = 0.0;
        if (xp > mm->beta[i]) df2[i] = 0.0;
    }
    for (int i = 0; i < m; i++)
        for (int j = 0; j < m; j++) {
            double s = 0.0;
            for (int k = 0; k < n; k++) s += PQ[(size_t)k * m + i] * df2[k] * PQ[(size_t)k * m + j];
            mm->Hess[i * m + j] = s;
        }
    double lamai = 0.0;
    for (int j = 0; j < m; j++) {
        if (mm->lam[j] < 0.0) mm->lam[j] = 0.0;
        lamai += mm->lam[j] * mm->a[j];
        if (mm->lam[j] > mm->c[j]) mm->Hess[j * m + j] += -1.0;
        mm->Hess[j * m + j] += -mm->mu[j] / mm->lam[j];
    }
    if (lamai > 0.0)
        for (int j = 0; j < m; j++)
            for (int k = 0; k < m; k++) mm->Hess[j * m + k] += -10.0 * mm->a[j] * mm->a[k];
    double tr = 0.0;
    for (int i = 0; i < m; i++) tr += mm->Hess[i * m + i];
    double corr = 1e-4 * tr / m;
    if (-1.0 * corr < 1.0e-7) corr = -1.0e-7;
    for (int i = 0; i < m; i++) mm->Hess[i * m + i] += corr;
    free(df2);
    free(PQ);
}
/* MMA::Factorize / MMA::Solve, MMA.cc:936-969 */
static void mma_factorize_solve(double *K, double *x, int nn) {
    for (int ss = 0; ss < nn - 1; ss++)
        for (int i = ss + 1; i < nn; i++) {
            K[i * nn + ss] = K[i * nn + ss] / K[ss * nn + ss];
            for (int j = ss + 1; j < nn; j++) K[i * nn + j] = K[i * nn + j] - K[i * nn + ss] * K[ss * nn + j];
        }
    for (int i = 1; i < nn; i++) {
        double a = 0.0;
        for (int j = 0; j < i; j++) a = a - K[i * nn + j] * x[j];
        x[i] = x[i] + a;
    }
    x[nn - 1] = x[nn - 1] / K[(nn - 1) * nn + (nn - 1)];
    for (int i = nn - 2; i >= 0; i--) {
        double a = x[i];
        for (int j = i + 1; j < nn; j++) a = a - K[i * nn + j] * x[j];
        x[i] = a / K[i * nn + i];
    }
}
/* MMA::DualLineSearch, MMA.cc:870-888 */
static void mma_linesearch(topo_oracle_mma *mm) {
    int m = mm->m;
    double theta = 1.005;
    for (int i = 0; i < m; i++) {
        if (theta < -1.01 * mm->s[i] / mm->lam[i]) theta = -1.01 * mm->s[i] / mm->lam[i];
        if (theta < -1.01 * mm->s[i + m] / mm->mu[i]) theta = -1.01 * mm->s[i + m] / mm->mu[i];
    }
    theta = 1.0 / theta;
    for (int i = 0; i < m; i++) {
        mm->lam[i] = mm->lam[i] + theta * mm->s[i];
        mm->mu[i] = mm->mu[i] + theta * mm->s[i + m];
    }
}
/* MMA::DualResidual, MMA.cc:890-934 */
static double mma_dualresidual(topo_oracle_mma *mm, const double *x, double epsi) {
    int n = mm->n, m = mm->m;
    double nrI = 0.0;
    for (int j = 0; j < m; j++) {
        double s = 0.0;
        for (int i = 0; i < n; i++)
            s += mm->pij[(size_t)j * n + i] / (mm->U[i] - x[i]) + mm->qij[(size_t)j * n + i] / (x[i] - mm->L[i]);
        double r1 = s - mm->b[j] - mm->a[j] * mm->z - mm->y[j] + mm->mu[j];
        double r2 = mm->mu[j] * mm->lam[j] - epsi;
        if (nrI < fabs(r1)) nrI = fabs(r1);
        if (nrI < fabs(r2)) nrI = fabs(r2);
    }
    return nrI;
}
/* MMA::SolveDIP, MMA.cc:639-676 */
static void mma_solvedip(topo_oracle_mma *mm, double *x) {
    int m = mm->m, n = mm->n;
    for (int j = 0; j < m; j++) {
        mm->lam[j] = mm->c[j] / 2.0;
        mm->mu[j] = 1.0;
    }
    double tol = 1.0e-9 * sqrt(m + n), epsi = 1.0, err = 1.0;
    while (epsi > tol) {
        int loop = 0;
        while (err > 0.9 * epsi && loop < 100) {
            loop++;
            mma_xyz(mm, x);
            mma_dualgrad(mm, x);
            for (int j = 0; j < m; j++) mm->grad[j] = -1.0 * mm->grad[j] - epsi / mm->lam[j];
            mma_dualhess(mm, x);
            mma_factorize_solve(mm->Hess, mm->grad, m);
            for (int j = 0; j < m; j++) mm->s[j] = mm->grad[j];
            for (int i = 0; i < m; i++)
                mm->s[m + i] = -mm->mu[i] + epsi / mm->lam[i] - mm->s[i] * mm->mu[i] / mm->lam[i];
            mma_linesearch(mm);
            mma_xyz(mm, x);
            err = mma_dualresidual(mm, x, epsi);
        }
        epsi = epsi * 0.1;
    }
}
/* MMA::Update, MMA.cc:487-507 */
void oracle_mma_update(topo_oracle_mma *mm, double *xval, const double *dfdx, const double *gx, const double *dgdx,
                       const double *xmin, const double *xmax) {
    mma_gensub(mm, xval, dfdx, gx, dgdx, xmin, xmax);
    memcpy(mm->xo2, mm->xo1, sizeof(double) * mm->n);
    memcpy(mm->xo1, xval, sizeof(double) * mm->n);
    mma_solvedip(mm, xval);
}
/* MMA::KKTresidual, MMA.cc:416-484 */
void oracle_mma_kkt_residual(topo_oracle_mma *mm, const double *x, const double *dfdx, const double *fx,
                             const double *dgdx, const double *xmin, const double *xmax, double *norm2,
                             double *normInf) {
    int n = mm->n, m = mm->m;
    double n2 = 0.0, nI = 0.0;
    for (int i = 0; i < n; i++) {
        double ri = dfdx[i];
        for (int j = 0; j < m; j++) ri += mm->lam[j] * dgdx[(size_t)j * n + i];
        double mu_min = (x[i] < xmin[i] + 1.0e-5 && ri > 0.0) ? ri : 0.0;
        double mu_max = (x[i] > xmax[i] - 1.0e-5 && ri < 0.0) ? -ri : 0.0;
        ri += -mu_min + mu_max;
        n2 += ri * ri;
        nI = dmax(fabs(ri), nI);
        double resi = mu_min * (x[i] - xmin[i]);
        n2 += resi * resi;
        nI = dmax(fabs(resi), nI);
        resi = mu_max * (xmax[i] - x[i]);
        n2 += resi * resi;
        nI = dmax(fabs(resi), nI);
    }
    double ri = 0.0;
    for (int j = 0; j < m; j++) ri += mm->lam[j] * (mm->a[j] * mm->z + mm->y[j] - fx[j]);
    n2 += ri * ri;
    nI = dmax(fabs(ri), nI);
    *norm2 = sqrt(n2);
    *normInf = nI;
}
void oracle_mma_get_state(const topo_oracle_mma *mm, double *L, double *U, double *lam) {
    memcpy(L, mm->L, sizeof(double) * mm->n);
    memcpy(U, mm->U, sizeof(double) * mm->n);
    memcpy(lam, mm->lam, sizeof(double) * mm->m);
}

/* ------------------------------------------------------------------ */
/* SOMMG reduced-order path: SOMMG::ConstructBasis (SOMMG.cc:40-265) and   */
/* the reduction branches of LinearElasticity.cc (:404-458, :993-1008,     */
/* :1089-1107, :1225-1243, :1683-1774, :1850-1868, :2318-2336).            */
/* ------------------------------------------------------------------ */

/* P0 = K - om^2 M with Dirichlet rows: N P0 N + (I - N) (SOMMG.cc:58-72) */
typedef struct {
    topo_oracle *o;
    double om2;
} p0ctx;
static void op_p0(void *vctx, const double *x, double *y) {
    p0ctx *c = (p0ctx *)vctx;
    topo_oracle *o = c->o;
    int nd = o->ndof;
    double *xm = o->t3, *kx = o->t4;
    for (int i = 0; i < nd; i++) xm[i] = o->N[i] * x[i];
    st_mult(&o->K, xm, kx);
    st_mult(&o->M, xm, y);
    for (int i = 0; i < nd; i++) y[i] = o->N[i] * (kx[i] - c->om2 * y[i]) + (1.0 - o->N[i]) * x[i];
}

/* dense k x k solve A x = b, LU with partial pivoting (stands in for the
 * reference's PCLU on the SeqDense reduced matrices, SetUpSolver2) */
static void dense_solve(int k, const double *A, const double *b, double *x) {
    double *LU = (double *)malloc(sizeof(double) * k * k);
    int *piv = (int *)malloc(sizeof(int) * k);
    memcpy(LU, A, sizeof(double) * k * k);
    for (int i = 0; i < k; i++) piv[i] = i;
    for (int c = 0; c < k; c++) {
        int pr = c;
        for (int r = c + 1; r < k; r++)
            if (fabs(LU[r * k + c]) > fabs(LU[pr * k + c])) pr = r;
        if (pr != c) {
            for (int j = 0; j < k; j++) {
                double t = LU[c * k + j];
                LU[c * k + j] = LU[pr * k + j];
                LU[pr * k + j] = t;
            }
            int t = piv[c];
            piv[c] = piv[pr];
            piv[pr] = t;
        }
        for (int r = c + 1; r < k; r++) {
            double f = LU[r * k + c] / LU[c * k + c];
            LU[r * k + c] = f;
            for (int j = c + 1; j < k; j++) LU[r * k + j] -= f * LU[c * k + j];
        }
    }
    for (int i = 0; i < k; i++) {
        double s = b[piv[i]];
        for (int j = 0; j < i; j++) s -= LU[i * k + j] * x[j];
        x[i] = s;
    }
    for (int i = k - 1; i >= 0; i--) {
        double s = x[i];
        for (int j = i + 1; j < k; j++) s -= LU[i * k + j] * x[j];
        x[i] = s / LU[i * k + i];
    }
    free(LU);
    free(piv);
}
static void dgemv_k(int k, const double *A, const double *x, double *y) {
    for (int i = 0; i < k; i++) {
        double s = 0.0;
        for (int j = 0; j < k; j++) s += A[i * k + j] * x[j];
        y[i] = s;
    }
}
/* full = sum_k r[k] Q_k (the VecAXPY lifts of LinearElasticity.cc:1089-1107) */
static void lift(const topo_oracle *o, int k, const double *Q, const double *r, double *full) {
    int nd = o->ndof;
    memset(full, 0, sizeof(double) * nd);
    for (int b = 0; b < k; b++)
        for (int i = 0; i < nd; i++) full[i] += r[b] * Q[(size_t)b * nd + i];
}

int oracle_le_reduced_objective_sensitivities(topo_oracle *o, const double *xPhys, int k, double omega0, double *fx,
                                              double *dfdx, double *Qout, double *Kr_out, double *Mr_out) {
    const topo_oracle_params *p = &o->p;
    int nd = o->ndof, Ts = o->Ts, rc = 0;
    double *a = o->a, dt = o->dt, al = p->dalpha, be = p->dbeta;
    rc |= oracle_le_complete_initial_state(o, xPhys); /* AssembleMass/Stiffness with xPhys */
    /* ---- ConstructBasis (SOMMG.cc:40-214) ---- */
    double *Q = vnew((size_t)k * nd), *Pv = vnew(nd), *f = vnew(nd), *mq = vnew(nd), *dinv = vnew(nd);
    double *Ut = vnew((size_t)k * k);
    double om2 = omega0 * omega0;
    for (int i = 0; i < nd; i++) Pv[i] = o->N[i] * o->RHS0[i]; /* VecPointwiseMult(P, P, N), :75 */
    {
        double *dk = o->t1, *dm = o->t2;
        st_diag(&o->K, dk);
        st_diag(&o->M, dm);
        for (int i = 0; i < nd; i++) dinv[i] = 1.0 / (o->N[i] * (dk[i] - om2 * dm[i]) + (1.0 - o->N[i]));
    }
    p0ctx pc = {o, om2};
    for (int j = 0; j < k; j++) {
        double *Qj = Q + (size_t)j * nd;
        if (j == 0) {
            rc |= pcg(op_p0, &pc, dinv, nd, Pv, Qj, p->rtol, p->maxit, &o->cg_iters); /* :78-80 */
        } else {
            /* fvec = 2 om M Q_{j-1} (:109-111) with M diagonally scaled by N (:68);
             * the moment-matching correction (:113-176) is scaled by the comma
             * expression (-1,0) == 0 at :176 and so contributes nothing */
            const double *Qm = Q + (size_t)(j - 1) * nd;
            for (int i = 0; i < nd; i++) mq[i] = o->N[i] * Qm[i];
            st_mult(&o->M, mq, f);
            for (int i = 0; i < nd; i++) f[i] = o->N[i] * (2.0 * omega0 * o->N[i] * f[i]); /* :181 */
            rc |= pcg(op_p0, &pc, dinv, nd, f, Qj, p->rtol, p->maxit, &o->cg_iters);       /* :185 */
            /* modified Gram-Schmidt against the accepted vectors (:195-202) */
            for (int i = 0; i < j; i++) {
                const double *Qi = Q + (size_t)i * nd;
                double u = vdot(nd, Qi, Qj);
                Ut[i * k + j] = u;
                for (int q = 0; q < nd; q++) Qj[q] -= u * Qi[q];
            }
        }
        double nrm = sqrt(vdot(nd, Qj, Qj)); /* :92, :206 */
        Ut[j * k + j] = nrm;
        for (int q = 0; q < nd; q++) Qj[q] /= nrm;
    }
    /* ---- reduced matrices and load (SOMMG.cc:228-252); Q vanishes on clamped
     * DOFs, so the masked and unmasked products agree ---- */
    double *Kr = vnew((size_t)k * k), *Mr = vnew((size_t)k * k), *Cr = vnew((size_t)k * k), *Pr = vnew(k);
    double *kq = vnew(nd), *mqq = vnew(nd);
    for (int j = 0; j < k; j++) {
        const double *Qj = Q + (size_t)j * nd;
        st_mult(&o->K, Qj, kq);
        for (int i = 0; i < nd; i++) mq[i] = o->N[i] * Qj[i];
        st_mult(&o->M, mq, mqq);
        for (int i = 0; i < nd; i++) mqq[i] *= o->N[i];
        for (int i = 0; i < k; i++) {
            const double *Qi = Q + (size_t)i * nd;
            Kr[i * k + j] = vdot(nd, Qi, kq);
            Mr[i * k + j] = vdot(nd, Qi, mqq);
        }
    }
    for (int i = 0; i < k * k; i++) Cr[i] = al * Mr[i] + be * Kr[i]; /* C = alpha M + beta K, :2605-2619 */
    for (int i = 0; i < k; i++) Pr[i] = vdot(nd, Pv, Q + (size_t)i * nd);
    if (Qout) memcpy(Qout, Q, sizeof(double) * k * nd);
    if (Kr_out) memcpy(Kr_out, Kr, sizeof(double) * k * k);
    if (Mr_out) memcpy(Mr_out, Mr, sizeof(double) * k * k);
    /* ---- reduced Newmark (N = 1, :1000-1002), dense operators ---- */
    double *Ke = vnew((size_t)k * k), *B1 = vnew((size_t)k * k), *B2 = vnew((size_t)k * k), *B3 = vnew((size_t)k * k);
    for (int i = 0; i < k * k; i++) {
        Ke[i] = Kr[i] + a[5] * Mr[i] + a[2] * Cr[i];
        B1[i] = a[5] * Mr[i] + a[2] * Cr[i];
        B2[i] = a[3] * Mr[i] - a[0] * Cr[i];
        B3[i] = a[4] * Mr[i] - a[1] * Cr[i];
    }
    size_t hs = (size_t)Ts * k;
    double *Ur = vnew(hs), *DUr = vnew(hs), *DDUr = vnew(hs), *Lr = vnew(hs), *DLr = vnew(hs), *DDLr = vnew(hs);
    double *v1 = vnew(k), *v2 = vnew(k), *v3 = vnew(k), *rr = vnew(k);
    /* CompleteInitialState: U0 = DU0 = 0, M DDU0 = f(0) - C DU0 - K U0 (:1049-1078) */
    double s0 = oracle_load_signal(p->loadsignal, 0.0) / (o->ny - 1);
    for (int i = 0; i < k; i++) rr[i] = Pr[i] * s0;
    dense_solve(k, Mr, rr, DDUr);
    for (int t = 1; t < Ts; t++) { /* SolveStateBlock (:1298-1397) */
        const double *u = Ur + (size_t)(t - 1) * k, *du = DUr + (size_t)(t - 1) * k, *ddu = DDUr + (size_t)(t - 1) * k;
        double st = oracle_load_signal(p->loadsignal, t * dt) / (o->ny - 1);
        dgemv_k(k, B1, u, v1);
        dgemv_k(k, B2, du, v2);
        dgemv_k(k, B3, ddu, v3);
        for (int i = 0; i < k; i++) rr[i] = Pr[i] * st + v1[i] + v2[i] + v3[i];
        double *un = Ur + (size_t)t * k;
        dense_solve(k, Ke, rr, un);
        for (int i = 0; i < k; i++) {
            double d = un[i] - u[i];
            DUr[(size_t)t * k + i] = a[0] * du[i] + a[1] * ddu[i] + a[2] * d;
            DDUr[(size_t)t * k + i] = -a[3] * du[i] - a[4] * ddu[i] + a[5] * d;
        }
    }
    /* ---- objective on the lifted states, every step including t = 0 (:1778-1802) ---- */
    double *uf = vnew(nd), *duf = vnew(nd), *dduf = vnew(nd), *lf = vnew(nd);
    double *ubf = vnew(nd), *dubf = vnew(nd), *ddubf = vnew(nd);
    double fsum = 0.0;
    for (int t = 0; t < Ts; t++) {
        lift(o, k, Q, Ur + (size_t)t * k, uf);
        lift(o, k, Q, DUr + (size_t)t * k, duf);
        lift(o, k, Q, DDUr + (size_t)t * k, dduf);
        fsum += objective_loop(o, uf, duf, dduf);
    }
    /* ---- adjoint in reduced space with projected state gradients (:2318-2336) ---- */
    double *h1 = vnew(k), *h2 = vnew(k), *h3 = vnew(k), *Lp = vnew(k), *DLp = vnew(k), *DDLp = vnew(k);
    for (int t = Ts - 1; t >= 1; t--) {
        lift(o, k, Q, Ur + (size_t)t * k, uf);
        lift(o, k, Q, DUr + (size_t)t * k, duf);
        lift(o, k, Q, DDUr + (size_t)t * k, dduf);
        gradient_objective_loop(o, uf, duf, dduf);
        for (int i = 0; i < k; i++) {
            h1[i] = vdot(nd, o->HDU, Q + (size_t)i * nd);
            h2[i] = vdot(nd, o->HDDU, Q + (size_t)i * nd);
            h3[i] = vdot(nd, o->HDDDU, Q + (size_t)i * nd);
        }
        double *Lt = Lr + (size_t)t * k, *DLt = DLr + (size_t)t * k, *DDLt = DDLr + (size_t)t * k;
        if (t == Ts - 1) { /* :864-889 */
            for (int i = 0; i < k; i++) {
                DLt[i] = -h2[i];
                DDLt[i] = -h3[i];
                rr[i] = h1[i] - a[2] * DLt[i] - a[5] * DDLt[i]; /* -r1: -Keff L = r1 */
            }
        } else { /* :892-924 */
            dgemv_k(k, B1, Lp, v1);
            dgemv_k(k, B2, Lp, v2);
            dgemv_k(k, B3, Lp, v3);
            for (int i = 0; i < k; i++) {
                DLt[i] = -(h2[i] + v2[i] - a[0] * DLp[i] + a[3] * DDLp[i]);
                DDLt[i] = -(h3[i] + v3[i] + a[4] * DDLp[i]);
                double v = -(h1[i] + v1[i] + a[2] * DLp[i] + a[5] * DDLp[i]) + a[2] * DLt[i] + a[5] * DDLt[i];
                rr[i] = -v;
            }
        }
        dense_solve(k, Ke, rr, Lt);
        memcpy(Lp, Lt, sizeof(double) * k);
        memcpy(DLp, DLt, sizeof(double) * k);
        memcpy(DDLp, DDLt, sizeof(double) * k);
    }
    /* ---- sensitivities on the lifted states and adjoints (:1804-1840) ---- */
    memset(dfdx, 0, sizeof(double) * o->nel);
    for (int t = 1; t < Ts; t++) {
        lift(o, k, Q, Ur + (size_t)t * k, uf);
        lift(o, k, Q, DUr + (size_t)t * k, duf);
        lift(o, k, Q, Lr + (size_t)t * k, lf);
        lift(o, k, Q, Ur + (size_t)(t - 1) * k, ubf);
        lift(o, k, Q, DUr + (size_t)(t - 1) * k, dubf);
        lift(o, k, Q, DDUr + (size_t)(t - 1) * k, ddubf);
        sens_loop_n(o, dfdx, uf, duf, lf, ubf, dubf, ddubf);
    }
    /* ---- SolveLagrange0 (:678-804) and the t = 0 sensitivities ---- */
    lift(o, k, Q, Ur, o->U0);
    lift(o, k, Q, DUr, o->DU0);
    lift(o, k, Q, DDUr, o->DDU0);
    gradient_objective_loop(o, o->U0, o->DU0, o->DDU0);
    for (int i = 0; i < k; i++) h3[i] = vdot(nd, o->HDDDU, Q + (size_t)i * nd);
    dgemv_k(k, B3, Lp, v3);
    for (int i = 0; i < k; i++) rr[i] = -(h3[i] + v3[i] - a[1] * DLp[i] + a[4] * DDLp[i]);
    double *ddl0 = vnew(k);
    dense_solve(k, Mr, rr, ddl0);
    lift(o, k, Q, ddl0, o->DDL0);
    sens_loop_0(o, dfdx);
    *fx = fsum;
    free(Q); free(Pv); free(f); free(mq); free(dinv); free(Ut); free(Kr); free(Mr); free(Cr); free(Pr);
    free(kq); free(mqq); free(Ke); free(B1); free(B2); free(B3); free(Ur); free(DUr); free(DDUr);
    free(Lr); free(DLr); free(DDLr); free(v1); free(v2); free(v3); free(rr); free(uf); free(duf); free(dduf);
    free(lf); free(ubf); free(dubf); free(ddubf); free(h1); free(h2); free(h3); free(Lp); free(DLp); free(DDLp);
    free(ddl0);
    return rc;
}
