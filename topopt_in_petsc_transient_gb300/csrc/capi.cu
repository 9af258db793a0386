// capi.cu -- extern "C" boundary (include/topopt_gb300.h) over the GB300
// LinearElasticity, PDE filter and MMA objects.  Host-pointer entry points
// stage through device buffers owned by the handle; *_dev entry points take
// device pointers directly.
#include <cstring>
#include <string>
#include <vector>

#include "filter.h"
#include "kernels.cuh"
#include "le.h"
#include "mma.h"

using namespace topo;

struct topo_le {
    TopoLE *impl;
    double *d_x, *d_df, *d_aux;  // staging for host-pointer calls
    double *part;
    unsigned int *counter;
    long long nel, ndof;
};
struct topo_pdefilt {
    TopoPDEFilt *impl;
    double *d_a, *d_b, *d_c, *d_g;
    long long nel;
    int gcap;  // constraint columns held by d_g
};
struct topo_sommg {
    topo_le *le;  // the LinearElasticity object whose reduction model this is
    int order;
};
struct topo_mma {
    TopoMMA *impl;
    double *d_x, *d_df, *d_dg, *d_lo, *d_hi;
    int n, m;
};

namespace {

int device_ok() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_error("no CUDA device available: the GB300 path has no CPU fallback");
        return TOPO_ERR_CUDA;
    }
    return TOPO_OK;
}

#define ACK(call)                                                            \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) {                                             \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));  \
            return TOPO_ERR_CUDA;                                            \
        }                                                                    \
    } while (0)

__global__ void k_volume(long long n, const double *__restrict__ x, double volfrac, double *dg, Partials<1> part,
                         double *gx) {
    double v[1] = {0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        v[0] += x[i];
        dg[i] = 1.0 / (double)n;
    }
    double tot[1];
    if (grid_reduce<EW, 1>(v, part, tot)) *gx = tot[0] / (double)n - volfrac;
}

__global__ void k_scale(long long n, double *__restrict__ x, double alpha) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] *= alpha;
}

}  // namespace

extern "C" {

void topo_le_default_params(topo_le_params *p, int nelx, int nely, int nelz) {
    memset(p, 0, sizeof(*p));
    p->nx = nelx + 1;
    p->ny = nely + 1;
    p->nz = nelz + 1;
    p->hx = p->hy = p->hz = 1.0;
    p->nu = 0.3;
    p->nlvls = 4;
    p->ncp = 2;
    p->tsc = 25;
    p->t1 = 50.0;
    p->ti = 1;
    p->objective = 0;
    p->sInt = 1;
    p->mInt = 0;
    p->boundaries = 1;
    p->loadloc = 1;
    p->optregion = 2;
    p->loadsignal = 0;
    p->dalpha = 1e-4;
    p->dbeta = 1e-4;
    p->mixed = 1;
    p->rtol = 1e-10;
    p->maxit = 500;
    p->smooth = 3;
    p->cheb_ratio = 30.0;
    p->use_graphs = 1;
    p->coarse_dense_max = 4096;
    p->coarse_smooth = 12;
    p->sens_fp32 = 1;
    p->inner_tol = 1e-5;
    p->inner_maxit = 40;
    p->adaptive_kappa = 40.0;
    p->extrapolate = 2;
    p->mass_precond = 2;
    p->mass_precond_share = 0.25;
    p->mass_precond_smooth = 0;
    p->reduction = 0;
    p->basis = 5;
    p->omega0 = 1.0;
    p->load2_node = -1;
    p->load2_phase = 0.0;
    p->out_dof = -1;
}

int topo_le_create(topo_le **out, const topo_le_params *p) {
    if (!out || !p) return TOPO_ERR_ARG;
    *out = nullptr;
    int rc = device_ok();
    if (rc) return rc;
    TopoLE *impl = nullptr;
    rc = le_create(&impl, p);
    if (rc) return rc;
    topo_le *h = new topo_le();
    h->impl = impl;
    h->nel = le_nel(impl);
    h->ndof = le_ndof(impl);
    bool ok = cudaMalloc(&h->d_x, sizeof(double) * h->nel) == cudaSuccess &&
              cudaMalloc(&h->d_df, sizeof(double) * h->nel) == cudaSuccess &&
              cudaMalloc(&h->d_aux, sizeof(double) * 2 * h->ndof) == cudaSuccess &&
              cudaMalloc(&h->part, sizeof(double) * 65536) == cudaSuccess &&
              cudaMalloc(&h->counter, sizeof(unsigned int) * 4) == cudaSuccess;
    if (!ok || cudaMemset(h->counter, 0, sizeof(unsigned int) * 4) != cudaSuccess) {
        cudaGetLastError();
        topo_le_destroy(h);
        set_error("device allocation of LinearElasticity staging buffers failed");
        return TOPO_ERR_OOM;
    }
    *out = h;
    return TOPO_OK;
}

void topo_le_destroy(topo_le *le) {
    if (!le) return;
    le_destroy(le->impl);
    cudaFree(le->d_x);
    cudaFree(le->d_df);
    cudaFree(le->d_aux);
    cudaFree(le->part);
    cudaFree(le->counter);
    delete le;
}

int topo_le_complete_initial_state_dev(topo_le *le, const double *xPhys_dev, double Emin, double Emax, double Rmin,
                                       double Rmax, double penalK, double penalM) {
    if (!le || !xPhys_dev) return TOPO_ERR_ARG;
    return le_complete_initial_state(le->impl, xPhys_dev, Emin, Emax, Rmin, Rmax, penalK, penalM);
}

int topo_le_complete_initial_state(topo_le *le, const double *xPhys, double Emin, double Emax, double Rmin,
                                   double Rmax, double penalK, double penalM) {
    if (!le || !xPhys) return TOPO_ERR_ARG;
    ACK(cudaMemcpy(le->d_x, xPhys, sizeof(double) * le->nel, cudaMemcpyHostToDevice));
    return topo_le_complete_initial_state_dev(le, le->d_x, Emin, Emax, Rmin, Rmax, penalK, penalM);
}

int topo_le_generate_checkpoints(topo_le *le) {
    if (!le) return TOPO_ERR_ARG;
    return le_generate_checkpoints(le->impl);
}

int topo_le_compute_objective_sensitivities_dev(topo_le *le, double *fx, double *dfdx_dev) {
    if (!le || !fx || !dfdx_dev) return TOPO_ERR_ARG;
    return le_compute_objective_sensitivities(le->impl, fx, dfdx_dev);
}

int topo_le_compute_objective_sensitivities(topo_le *le, double *fx, double *dfdx) {
    if (!le || !fx || !dfdx) return TOPO_ERR_ARG;
    int rc = le_compute_objective_sensitivities(le->impl, fx, le->d_df);
    if (rc) return rc;
    ACK(cudaMemcpy(dfdx, le->d_df, sizeof(double) * le->nel, cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

int topo_le_volume_constraint_dev(topo_le *le, double *gx, double *dgdx_dev, const double *xPhys_dev, double volfrac) {
    if (!le || !gx || !dgdx_dev || !xPhys_dev) return TOPO_ERR_ARG;
    double *gd = le->part + 65535;
    count_launch();
    k_volume<<<red_blocks(le->nel), EW>>>(le->nel, xPhys_dev, volfrac, dgdx_dev, Partials<1>{le->part, le->counter}, gd);
    ACK(cudaMemcpy(gx, gd, sizeof(double), cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

int topo_le_volume_constraint(topo_le *le, double *gx, double *dgdx, const double *xPhys, double volfrac) {
    if (!le || !gx || !dgdx || !xPhys) return TOPO_ERR_ARG;
    ACK(cudaMemcpy(le->d_x, xPhys, sizeof(double) * le->nel, cudaMemcpyHostToDevice));
    int rc = topo_le_volume_constraint_dev(le, gx, le->d_df, le->d_x, volfrac);
    if (rc) return rc;
    ACK(cudaMemcpy(dgdx, le->d_df, sizeof(double) * le->nel, cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

int topo_vec_scale_dev(double *x_dev, long long n, double alpha) {
    if (n < 0 || (n > 0 && !x_dev)) return TOPO_ERR_ARG;
    if (n == 0) return TOPO_OK;
    int rc = device_ok();
    if (rc) return rc;
    count_launch();
    k_scale<<<ew_blocks(n), EW>>>(n, x_dev, alpha);
    ACK(cudaGetLastError());
    ACK(cudaStreamSynchronize(0));
    return TOPO_OK;
}

int topo_le_get_state(topo_le *le, int which, int j, double *out) {
    if (!le || !out) return TOPO_ERR_ARG;
    return le_get_state(le->impl, which, j, out);
}

int topo_le_get_checkpoint(topo_le *le, int c, double *U, double *DU, double *DDU) {
    if (!le || !U || !DU || !DDU) return TOPO_ERR_ARG;
    return le_get_checkpoint(le->impl, c, U, DU, DDU);
}

int topo_le_set_initial_displacement(topo_le *le, const double *U0, int on_device) {
    if (!le) return TOPO_ERR_ARG;
    return le_set_initial_displacement(le->impl, U0, on_device);
}

int topo_le_get_restart_state(topo_le *le, double *DDU0, double *LT, double *DDL0) {
    if (!le || !DDU0 || !LT || !DDL0) return TOPO_ERR_ARG;
    return le_get_restart_state(le->impl, DDU0, LT, DDL0);
}

int topo_le_set_output(topo_le *le, topo_mpiio *io) {
    if (!le) return TOPO_ERR_ARG;
    return le_set_output(le->impl, io);
}

int topo_le_apply_km(topo_le *le, const double *x, double *Kx, double *Mx) {
    if (!le || !x || !Kx || !Mx) return TOPO_ERR_ARG;
    long long nd = le->ndof;
    double *dK = le->d_aux, *dM = le->d_aux + nd, *dx = nullptr;
    ACK(cudaMalloc(&dx, sizeof(double) * nd));
    cudaError_t e = cudaMemcpy(dx, x, sizeof(double) * nd, cudaMemcpyHostToDevice);
    int rc = (e == cudaSuccess) ? le_apply_km(le->impl, dx, dK, dM) : TOPO_ERR_CUDA;
    if (!rc) {
        if (cudaMemcpy(Kx, dK, sizeof(double) * nd, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(Mx, dM, sizeof(double) * nd, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = TOPO_ERR_CUDA;
    }
    cudaFree(dx);
    return rc;
}

int topo_le_get_stats(topo_le *le, topo_le_stats *out) {
    if (!le || !out) return TOPO_ERR_ARG;
    return le_stats(le->impl, out);
}

int topo_le_time_apply(topo_le *le, int precision, int warmup, int reps, double *ms_per_launch) {
    if (!le || !ms_per_launch || reps < 1 || warmup < 0 || precision < 0 || precision > 3) return TOPO_ERR_ARG;
    return le_time_apply(le->impl, precision, warmup, reps, ms_per_launch);
}

int topo_le_reduced_system(topo_le *le, double *Q, double *Kr, double *Mr, double *Pr) {
    if (!le) return TOPO_ERR_ARG;
    return le_reduced_system(le->impl, Q, Kr, Mr, Pr);
}

int topo_le_kernel_timing(topo_le *le, int kclass, int enable, double *ms_total, long long *launches) {
    if (!le) return TOPO_ERR_ARG;
    return le_kernel_timing(le->impl, kclass, enable, ms_total, launches);
}

int topo_sommg_create(topo_sommg **out, topo_le *le, int order) {
    if (!out || !le) return TOPO_ERR_ARG;
    *out = nullptr;
    const int kb = le_basis(le->impl);
    if (kb == 0 || order != kb) {
        set_error("SOMMG(x, order): the LinearElasticity object must be created with reduction = 1 and basis = order");
        return TOPO_ERR_ARG;
    }
    *out = new topo_sommg{le, order};
    return TOPO_OK;
}

void topo_sommg_destroy(topo_sommg *s) { delete s; }

int topo_sommg_gram_dev(const float *Q_dev, long long ldq, const double *W_dev, long long ldw, long long n, int kb,
                        double *out) {
    int rc = device_ok();
    if (rc) return rc;
    return le_gram_tc_dev(Q_dev, ldq, W_dev, ldw, n, kb, out);
}

int topo_sommg_construct_basis(topo_sommg *s, double om) {
    if (!s) return TOPO_ERR_ARG;
    return le_sommg_construct_basis(s->le->impl, om);
}

int topo_sommg_get(topo_sommg *s, double *QQ, double *Kr, double *Mr, double *Cr, double *Pr) {
    if (!s) return TOPO_ERR_ARG;
    const int kb = s->order;
    std::vector<double> k, m;
    if (Cr) {
        k.resize((size_t)kb * kb);
        m.resize((size_t)kb * kb);
    }
    int rc = le_reduced_system(s->le->impl, QQ, Cr ? k.data() : Kr, Cr ? m.data() : Mr, Pr);
    if (rc || !Cr) return rc;
    double alpha, beta;
    le_damping(s->le->impl, &alpha, &beta);
    for (size_t i = 0; i < k.size(); i++) Cr[i] = alpha * m[i] + beta * k[i];  // Q'(alpha M + beta K)Q, SOMMG.cc:246-249
    if (Kr) memcpy(Kr, k.data(), sizeof(double) * k.size());
    if (Mr) memcpy(Mr, m.data(), sizeof(double) * m.size());
    return TOPO_OK;
}

void topo_box_element_matrices(double hx, double hy, double hz, double nu, double *KE, double *ME) {
    // kernels use lexicographic local nodes L = ax + 2ay + 4az; the reference
    // order is (0,0,0),(1,0,0),(1,1,0),(0,1,0),(0,0,1),(1,0,1),(1,1,1),(0,1,1)
    static const int ref2lex[8] = {0, 1, 3, 2, 4, 5, 7, 6};
    double K[576], M[576];
    box_element_matrices(hx, hy, hz, nu, K, M);
    for (int a = 0; a < 8; a++)
        for (int b = 0; b < 8; b++)
            for (int c = 0; c < 3; c++)
                for (int d = 0; d < 3; d++) {
                    int i = 3 * a + c, j = 3 * b + d;
                    int li = 3 * ref2lex[a] + c, lj = 3 * ref2lex[b] + d;
                    KE[i * 24 + j] = K[li * 24 + lj];
                    ME[i * 24 + j] = M[li * 24 + lj];
                }
}

// ---------------------------------------------------------------------------
int topo_pdefilt_create(topo_pdefilt **out, int nx, int ny, int nz, double hx, double hy, double hz, double rmin,
                        double rtol, int maxit) {
    if (!out) return TOPO_ERR_ARG;
    *out = nullptr;
    int rc = device_ok();
    if (rc) return rc;
    TopoPDEFilt *impl = nullptr;
    rc = pdefilt_create(&impl, nx, ny, nz, hx, hy, hz, rmin, rtol, maxit);
    if (rc) return rc;
    topo_pdefilt *h = new topo_pdefilt();
    h->impl = impl;
    h->nel = pdefilt_nel(impl);
    h->gcap = 2;
    bool ok = cudaMalloc(&h->d_a, sizeof(double) * h->nel) == cudaSuccess &&
              cudaMalloc(&h->d_b, sizeof(double) * h->nel) == cudaSuccess &&
              cudaMalloc(&h->d_c, sizeof(double) * h->nel) == cudaSuccess &&
              cudaMalloc(&h->d_g, sizeof(double) * h->nel * h->gcap) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        topo_pdefilt_destroy(h);
        set_error("device allocation of PDE filter staging buffers failed");
        return TOPO_ERR_OOM;
    }
    *out = h;
    return TOPO_OK;
}

void topo_pdefilt_destroy(topo_pdefilt *f) {
    if (!f) return;
    pdefilt_destroy(f->impl);
    cudaFree(f->d_a);
    cudaFree(f->d_b);
    cudaFree(f->d_c);
    cudaFree(f->d_g);
    delete f;
}

int topo_pdefilt_filter_project_dev(topo_pdefilt *f, const double *x_dev, double *xout_dev) {
    if (!f || !x_dev || !xout_dev) return TOPO_ERR_ARG;
    return pdefilt_apply_dev(f->impl, x_dev, xout_dev);
}

int topo_pdefilt_filter_project(topo_pdefilt *f, const double *x, double *xout) {
    if (!f || !x || !xout) return TOPO_ERR_ARG;
    ACK(cudaMemcpy(f->d_a, x, sizeof(double) * f->nel, cudaMemcpyHostToDevice));
    int rc = pdefilt_apply_dev(f->impl, f->d_a, f->d_b);
    if (rc) return rc;
    ACK(cudaMemcpy(xout, f->d_b, sizeof(double) * f->nel, cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

int topo_filter_project_dev(topo_pdefilt *f, const double *x_dev, double *xTilde_dev, double *xPhys_dev,
                            int projection, double beta, double eta) {
    if (!f || !x_dev || !xTilde_dev || !xPhys_dev) return TOPO_ERR_ARG;
    return filter_project_dev(f->impl, x_dev, xTilde_dev, xPhys_dev, projection, beta, eta);
}

int topo_filter_project(topo_pdefilt *f, const double *x, double *xTilde, double *xPhys, int projection, double beta,
                        double eta) {
    if (!f || !x || !xTilde || !xPhys) return TOPO_ERR_ARG;
    size_t b = sizeof(double) * f->nel;
    ACK(cudaMemcpy(f->d_a, x, b, cudaMemcpyHostToDevice));
    int rc = filter_project_dev(f->impl, f->d_a, f->d_b, f->d_c, projection, beta, eta);
    if (rc) return rc;
    ACK(cudaMemcpy(xTilde, f->d_b, b, cudaMemcpyDeviceToHost));
    ACK(cudaMemcpy(xPhys, f->d_c, b, cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

int topo_filter_gradients_dev(topo_pdefilt *f, const double *xTilde_dev, double *dfdx_dev, int m, double *dgdx_dev,
                              int projection, double beta, double eta) {
    if (!f || !xTilde_dev || !dfdx_dev || m < 0 || (m > 0 && !dgdx_dev)) return TOPO_ERR_ARG;
    return filter_gradients_dev(f->impl, xTilde_dev, dfdx_dev, m, dgdx_dev, projection, beta, eta);
}

int topo_filter_gradients(topo_pdefilt *f, const double *xTilde, double *dfdx, int m, double *dgdx, int projection,
                          double beta, double eta) {
    if (!f || !xTilde || !dfdx || m < 0 || m > f->gcap || (m > 0 && !dgdx)) return TOPO_ERR_ARG;
    size_t b = sizeof(double) * f->nel;
    ACK(cudaMemcpy(f->d_a, xTilde, b, cudaMemcpyHostToDevice));
    ACK(cudaMemcpy(f->d_b, dfdx, b, cudaMemcpyHostToDevice));
    if (m) ACK(cudaMemcpy(f->d_g, dgdx, b * m, cudaMemcpyHostToDevice));
    int rc = filter_gradients_dev(f->impl, f->d_a, f->d_b, m, f->d_g, projection, beta, eta);
    if (rc) return rc;
    ACK(cudaMemcpy(dfdx, f->d_b, b, cudaMemcpyDeviceToHost));
    if (m) ACK(cudaMemcpy(dgdx, f->d_g, b * m, cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

int topo_filter_mnd_dev(topo_pdefilt *f, const double *x_dev, double *mnd) {
    if (!f || !x_dev || !mnd) return TOPO_ERR_ARG;
    return filter_mnd_dev(f->impl, x_dev, mnd);
}

int topo_filter_mnd(topo_pdefilt *f, const double *x, double *mnd) {
    if (!f || !x || !mnd) return TOPO_ERR_ARG;
    ACK(cudaMemcpy(f->d_a, x, sizeof(double) * f->nel, cudaMemcpyHostToDevice));
    return filter_mnd_dev(f->impl, f->d_a, mnd);
}

// ---------------------------------------------------------------------------
int topo_mma_create(topo_mma **out, int n, int m, const double *a, const double *c, const double *d) {
    if (!out) return TOPO_ERR_ARG;
    *out = nullptr;
    int rc = device_ok();
    if (rc) return rc;
    TopoMMA *impl = nullptr;
    rc = mma_create(&impl, n, m, a, c, d);
    if (rc) return rc;
    topo_mma *h = new topo_mma();
    h->impl = impl;
    h->n = n;
    h->m = m;
    size_t b = sizeof(double) * (size_t)n;
    bool ok = cudaMalloc(&h->d_x, b) == cudaSuccess && cudaMalloc(&h->d_df, b) == cudaSuccess &&
              cudaMalloc(&h->d_dg, b * m) == cudaSuccess && cudaMalloc(&h->d_lo, b) == cudaSuccess &&
              cudaMalloc(&h->d_hi, b) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        topo_mma_destroy(h);
        set_error("device allocation of MMA staging buffers failed");
        return TOPO_ERR_OOM;
    }
    *out = h;
    return TOPO_OK;
}

int topo_mma_create_restart_dev(topo_mma **out, int n, int m, int itr, const double *xo1_dev, const double *xo2_dev,
                                const double *U_dev, const double *L_dev, const double *a, const double *c,
                                const double *d) {
    if (!out || !xo1_dev || !xo2_dev || !U_dev || !L_dev) return TOPO_ERR_ARG;
    int rc = topo_mma_create(out, n, m, a, c, d);
    if (rc) return rc;
    rc = mma_restart_set_dev((*out)->impl, itr, xo1_dev, xo2_dev, U_dev, L_dev);
    if (rc) {
        topo_mma_destroy(*out);
        *out = nullptr;
    }
    return rc;
}

int topo_mma_create_restart(topo_mma **out, int n, int m, int itr, const double *xo1, const double *xo2,
                            const double *U, const double *L, const double *a, const double *c, const double *d) {
    if (!out || !xo1 || !xo2 || !U || !L) return TOPO_ERR_ARG;
    int rc = topo_mma_create(out, n, m, a, c, d);
    if (rc) return rc;
    topo_mma *h = *out;
    size_t b = sizeof(double) * (size_t)n;
    // staging: x, df, lo, hi and the first constraint-gradient slot hold the four vectors
    if (cudaMemcpy(h->d_x, xo1, b, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->d_df, xo2, b, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->d_lo, U, b, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->d_hi, L, b, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        set_error("MMA restart: host-to-device copy failed");
        topo_mma_destroy(h);
        *out = nullptr;
        return TOPO_ERR_CUDA;
    }
    rc = mma_restart_set_dev(h->impl, itr, h->d_x, h->d_df, h->d_lo, h->d_hi);
    if (rc) {
        topo_mma_destroy(h);
        *out = nullptr;
    }
    return rc;
}

int topo_mma_restart_dev(topo_mma *mma, double *xo1_dev, double *xo2_dev, double *U_dev, double *L_dev) {
    if (!mma || !xo1_dev || !xo2_dev || !U_dev || !L_dev) return TOPO_ERR_ARG;
    return mma_restart_get_dev(mma->impl, xo1_dev, xo2_dev, U_dev, L_dev);
}

int topo_mma_restart(topo_mma *mma, double *xo1, double *xo2, double *U, double *L) {
    if (!mma || !xo1 || !xo2 || !U || !L) return TOPO_ERR_ARG;
    int rc = mma_restart_get_dev(mma->impl, mma->d_x, mma->d_df, mma->d_lo, mma->d_hi);
    if (rc) return rc;
    size_t b = sizeof(double) * (size_t)mma->n;
    ACK(cudaMemcpy(xo1, mma->d_x, b, cudaMemcpyDeviceToHost));
    ACK(cudaMemcpy(xo2, mma->d_df, b, cudaMemcpyDeviceToHost));
    ACK(cudaMemcpy(U, mma->d_lo, b, cudaMemcpyDeviceToHost));
    ACK(cudaMemcpy(L, mma->d_hi, b, cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

void topo_mma_destroy(topo_mma *mma) {
    if (!mma) return;
    mma_destroy(mma->impl);
    cudaFree(mma->d_x);
    cudaFree(mma->d_df);
    cudaFree(mma->d_dg);
    cudaFree(mma->d_lo);
    cudaFree(mma->d_hi);
    delete mma;
}

int topo_mma_set_asymptotes(topo_mma *mma, double init, double decrease, double increase) {
    if (!mma) return TOPO_ERR_ARG;
    return mma_set_asymptotes(mma->impl, init, decrease, increase);
}

int topo_mma_set_outer_movelimit_dev(topo_mma *mma, double Xmin, double Xmax, double movlim, const double *x_dev,
                                     double *xmin_dev, double *xmax_dev) {
    if (!mma || !x_dev || !xmin_dev || !xmax_dev) return TOPO_ERR_ARG;
    return mma_movelimit_dev(mma->impl, Xmin, Xmax, movlim, x_dev, xmin_dev, xmax_dev);
}

int topo_mma_set_outer_movelimit(topo_mma *mma, double Xmin, double Xmax, double movlim, const double *x,
                                 double *xmin, double *xmax) {
    if (!mma || !x || !xmin || !xmax) return TOPO_ERR_ARG;
    size_t b = sizeof(double) * (size_t)mma->n;
    ACK(cudaMemcpy(mma->d_x, x, b, cudaMemcpyHostToDevice));
    int rc = mma_movelimit_dev(mma->impl, Xmin, Xmax, movlim, mma->d_x, mma->d_lo, mma->d_hi);
    if (rc) return rc;
    ACK(cudaMemcpy(xmin, mma->d_lo, b, cudaMemcpyDeviceToHost));
    ACK(cudaMemcpy(xmax, mma->d_hi, b, cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

int topo_mma_design_change(topo_mma *mma, const double *x, double *xold, double *ch) {
    if (!mma || !x || !xold || !ch) return TOPO_ERR_ARG;
    size_t b = sizeof(double) * (size_t)mma->n;
    ACK(cudaMemcpy(mma->d_x, x, b, cudaMemcpyHostToDevice));
    ACK(cudaMemcpy(mma->d_df, xold, b, cudaMemcpyHostToDevice));
    int rc = mma_design_change_dev(mma->impl, mma->d_x, mma->d_df, ch);
    if (rc) return rc;
    ACK(cudaMemcpy(xold, mma->d_df, b, cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

int topo_mma_update_dev(topo_mma *mma, double *xval_dev, const double *dfdx_dev, const double *gx,
                        const double *dgdx_dev, const double *xmin_dev, const double *xmax_dev) {
    if (!mma || !xval_dev || !dfdx_dev || !gx || !dgdx_dev || !xmin_dev || !xmax_dev) return TOPO_ERR_ARG;
    return mma_update_dev(mma->impl, xval_dev, dfdx_dev, gx, dgdx_dev, xmin_dev, xmax_dev);
}

int topo_mma_update(topo_mma *mma, double *xval, const double *dfdx, const double *gx, const double *dgdx,
                    const double *xmin, const double *xmax) {
    if (!mma || !xval || !dfdx || !gx || !dgdx || !xmin || !xmax) return TOPO_ERR_ARG;
    size_t b = sizeof(double) * (size_t)mma->n;
    ACK(cudaMemcpy(mma->d_x, xval, b, cudaMemcpyHostToDevice));
    ACK(cudaMemcpy(mma->d_df, dfdx, b, cudaMemcpyHostToDevice));
    ACK(cudaMemcpy(mma->d_dg, dgdx, b * mma->m, cudaMemcpyHostToDevice));
    ACK(cudaMemcpy(mma->d_lo, xmin, b, cudaMemcpyHostToDevice));
    ACK(cudaMemcpy(mma->d_hi, xmax, b, cudaMemcpyHostToDevice));
    int rc = mma_update_dev(mma->impl, mma->d_x, mma->d_df, gx, mma->d_dg, mma->d_lo, mma->d_hi);
    if (rc) return rc;
    ACK(cudaMemcpy(xval, mma->d_x, b, cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

int topo_mma_design_change_dev(topo_mma *mma, const double *x_dev, double *xold_dev, double *ch) {
    if (!mma || !x_dev || !xold_dev || !ch) return TOPO_ERR_ARG;
    return mma_design_change_dev(mma->impl, x_dev, xold_dev, ch);
}

int topo_mma_kkt_residual_dev(topo_mma *mma, const double *x_dev, const double *dfdx_dev, const double *fx,
                              const double *dgdx_dev, const double *xmin_dev, const double *xmax_dev, double *norm2,
                              double *normInf) {
    if (!mma || !x_dev || !dfdx_dev || !fx || !dgdx_dev || !xmin_dev || !xmax_dev || !norm2 || !normInf)
        return TOPO_ERR_ARG;
    return mma_kkt_dev(mma->impl, x_dev, dfdx_dev, fx, dgdx_dev, xmin_dev, xmax_dev, norm2, normInf);
}

long long topo_kernel_launches(void) { return launch_counter(); }

const char *topo_last_error(void) { return last_error(); }

const char *topo_status_str(int status) {
    switch (status) {
    case TOPO_OK: return "ok";
    case TOPO_ERR_ARG: return "invalid argument";
    case TOPO_ERR_CUDA: return "CUDA error";
    case TOPO_ERR_OOM: return "out of device memory";
    case TOPO_ERR_NOT_CONVERGED: return "linear solve did not converge";
    case TOPO_ERR_BREAKDOWN: return "Krylov breakdown";
    case TOPO_ERR_NAN: return "NaN or Inf encountered";
    case TOPO_ERR_STATE: return "call order violated";
    case TOPO_ERR_SYNC_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
    }
}

}  // extern "C"
