// filter.cu -- PDEFilt (PDEFilter.cc) and the filter-type-2 branch of Filter
// (Filter.cc) on one GPU.
//
// The Helmholtz filter (-R^2 lap + 1) u = T x on the nodal grid has the same
// 8x8 element matrix KF for every element (R^2 * Laplacian + mass of the box,
// PDEFilter.cc:485-578), so its assembled operator is applied node-centrically
// from the element matrix in constant memory; T (0.125 per element node,
// :580-588) and T^t are gathers.  The solve is Jacobi-preconditioned CG in FP64
// with device-resident scalars.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "filter.h"
#include "kernels.cuh"

namespace topo {

#define FCK(call)                                                            \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) {                                             \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));  \
            return TOPO_ERR_CUDA;                                            \
        }                                                                    \
    } while (0)

struct FiltScalars {
    double bb, rr, rz, rz_old, pq, alpha, beta;
    double tol2;
    int it, maxit, done, status;
};

struct TopoPDEFilt {
    GridDesc g;
    double h[3], R, vol, rtol;
    int maxit;
    double KF[64];
    double *rhs, *u, *r, *p, *q, *dinv;
    double *e1, *e2;  // element scratch
    FiltScalars *S;
    double *part;
    unsigned int *counter;
    unsigned long long *mbits;
    std::vector<void *> ptrs;
    cudaStream_t stream;
};

struct KFMat {
    double v[64];
};

// y = K_F x (assembled, natural boundary), red: x.y
__global__ void k_filt_apply(GridDesc g, KFMat KF, const double *__restrict__ x, double *y, Partials<1> part,
                             const FiltScalars *S, int check_done) {
    if (check_done && S->done) return;
    long long nn = g.nn();
    double v[1] = {0.0};
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        lex3(n, g.nx, g.ny, i, j, k);
        double acc = 0.0;
        for (int c = 0; c < 8; c++) {
            int ei = i - (c & 1), ej = j - ((c >> 1) & 1), ek = k - (c >> 2);
            if (ei < 0 || ej < 0 || ek < 0 || ei >= g.ex || ej >= g.ey || ek >= g.ez) continue;
            // node n is local corner c of element e; KF uses the reference local order
            for (int L = 0; L < 8; L++) {
                long long m = (ei + (L & 1)) + (long long)g.nx * ((ej + ((L >> 1) & 1)) + (long long)g.ny * (ek + (L >> 2)));
                acc += KF.v[c * 8 + L] * x[m];
            }
        }
        y[n] = acc;
        v[0] += x[n] * acc;
    }
    double tot[1];
    if (grid_reduce<EW, 1>(v, part, tot)) {
        FiltScalars *Sm = const_cast<FiltScalars *>(S);
        Sm->pq = tot[0];
        Sm->alpha = (tot[0] > 0.0) ? Sm->rz / tot[0] : 0.0;
        if (!(tot[0] > 0.0)) {
            Sm->done = 1;
            Sm->status = isfinite(tot[0]) ? TOPO_ERR_BREAKDOWN : TOPO_ERR_NAN;
        }
    }
}

// rhs = vol * T x  (T = 0.125 per element corner)
__global__ void k_T(GridDesc g, double vol, const double *__restrict__ x, double *rhs) {
    long long nn = g.nn();
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        lex3(n, g.nx, g.ny, i, j, k);
        double acc = 0.0;
        for (int c = 0; c < 8; c++) {
            int ei = i - (c & 1), ej = j - ((c >> 1) & 1), ek = k - (c >> 2);
            if (ei < 0 || ej < 0 || ek < 0 || ei >= g.ex || ej >= g.ey || ek >= g.ez) continue;
            acc += 0.125 * x[ei + (long long)g.ex * (ej + (long long)g.ey * ek)];
        }
        rhs[n] = acc * vol;
    }
}

// xout = T^t u; optional clamp to [0,1] and smoothed Heaviside projection
// (Filter.cc:83-113, Filter.h:80-83)
__global__ void k_Tt(GridDesc g, const double *__restrict__ u, double *xout, double *xphys, int clamp, int projection,
                     double beta, double eta) {
    long long nel = g.nel();
    double den = tanh(beta * eta) + tanh(beta * (1.0 - eta));
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nel; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        lex3(e, g.ex, g.ey, i, j, k);
        double acc = 0.0;
        for (int L = 0; L < 8; L++)
            acc += 0.125 * u[(i + (L & 1)) + (long long)g.nx * ((j + ((L >> 1) & 1)) + (long long)g.ny * (k + (L >> 2)))];
        if (clamp) {
            if (acc < 0.0) acc = 0.0;
            if (acc > 1.0) acc = 1.0;
        }
        xout[e] = acc;
        if (xphys) xphys[e] = projection ? (tanh(beta * eta) + tanh(beta * (acc - eta))) / den : acc;
    }
}

// Filter::Gradients chain rule of the projection (Filter.cc:128-169)
__global__ void k_chain(long long nel, const double *__restrict__ xt, double *df, int m, double *dg, double beta,
                        double eta) {
    double den = tanh(beta * eta) + tanh(beta * (1.0 - eta));
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nel; e += (long long)gridDim.x * blockDim.x) {
        double t = tanh(beta * (xt[e] - eta));
        double d = beta * (1.0 - t * t) / den;
        df[e] *= d;
        for (int j = 0; j < m; j++) dg[(long long)j * nel + e] *= d;
    }
}

__global__ void k_filt_dinv(GridDesc g, KFMat KF, double *dinv) {
    long long nn = g.nn();
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        lex3(n, g.nx, g.ny, i, j, k);
        double acc = 0.0;
        for (int c = 0; c < 8; c++) {
            int ei = i - (c & 1), ej = j - ((c >> 1) & 1), ek = k - (c >> 2);
            if (ei < 0 || ej < 0 || ek < 0 || ei >= g.ex || ej >= g.ey || ek >= g.ez) continue;
            acc += KF.v[c * 8 + c];
        }
        dinv[n] = 1.0 / acc;
    }
}

// r = b (x0 = 0), z = Dinv r, p = z; reductions b.b, r.z
__global__ void k_fpcg_init(long long n, const double *__restrict__ b, const double *__restrict__ dinv, double *x,
                            double *r, double *p, FiltScalars *S, Partials<2> part) {
    double v[2] = {0.0, 0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double bi = b[i];
        x[i] = 0.0;
        r[i] = bi;
        double zi = dinv[i] * bi;
        p[i] = zi;
        v[0] += bi * bi;
        v[1] += bi * zi;
    }
    double tot[2];
    if (grid_reduce<EW, 2>(v, part, tot)) {
        S->bb = tot[0];
        S->rr = tot[0];
        S->rz = tot[1];
        S->it = 0;
        S->status = 0;
        S->done = (tot[0] == 0.0);
    }
}

// x += a p, r -= a q, z = Dinv r, red r.r, r.z -> beta, convergence
__global__ void k_fpcg_update(long long n, const double *__restrict__ dinv, double *x, double *r,
                              const double *__restrict__ p, const double *__restrict__ q, FiltScalars *S,
                              Partials<2> part) {
    if (S->done) return;
    double a = S->alpha;
    double v[2] = {0.0, 0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        x[i] += a * p[i];
        double ri = r[i] - a * q[i];
        r[i] = ri;
        v[0] += ri * ri;
        v[1] += ri * dinv[i] * ri;
    }
    double tot[2];
    if (grid_reduce<EW, 2>(v, part, tot)) {
        S->rr = tot[0];
        S->rz_old = S->rz;
        S->rz = tot[1];
        S->beta = tot[1] / S->rz_old;
        S->it += 1;
        if (!isfinite(tot[0])) {
            S->status = TOPO_ERR_NAN;
            S->done = 1;
        } else if (tot[0] <= S->tol2 * S->bb) {
            S->done = 1;
        } else if (S->it >= S->maxit) {
            S->status = TOPO_ERR_NOT_CONVERGED;
            S->done = 1;
        }
    }
}

__global__ void k_fpcg_p(long long n, const double *__restrict__ dinv, const double *__restrict__ r, double *p,
                         const FiltScalars *S) {
    if (S->done) return;
    double b = S->beta;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = dinv[i] * r[i] + b * p[i];
}

__global__ void k_fprime(FiltScalars *S, double tol2, int maxit) {
    S->tol2 = tol2;
    S->maxit = maxit;
    S->done = 0;
    S->status = 0;
}

// GetMND (Filter.cc:208-227)
__global__ void k_mnd(long long n, const double *__restrict__ x, Partials<1> part, double *out) {
    double v[1] = {0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        v[0] += 4.0 * x[i] * (1.0 - x[i]);
    double tot[1];
    if (grid_reduce<EW, 1>(v, part, tot)) *out = tot[0] / (double)n;
}

// ---------------------------------------------------------------------------
int pdefilt_create(TopoPDEFilt **out, int nx, int ny, int nz, double hx, double hy, double hz, double rmin, double rtol,
                   int maxit) {
    *out = nullptr;
    if (nx < 2 || ny < 2 || nz < 2 || hx <= 0 || hy <= 0 || hz <= 0 || rmin <= 0) {
        set_error("invalid PDE filter parameters");
        return TOPO_ERR_ARG;
    }
    TopoPDEFilt *f = new TopoPDEFilt();
    f->g = GridDesc{nx, ny, nz, nx - 1, ny - 1, nz - 1};
    f->h[0] = hx;
    f->h[1] = hy;
    f->h[2] = hz;
    f->R = rmin / 2.0 / sqrt(3.0);  // PDEFilter.cc:32
    f->vol = hx * hy * hz;
    f->rtol = rtol;
    f->maxit = maxit;
    // KF = R^2 * Laplacian + mass of the box: mode-basis diagonal, mapped back
    // to the reference local node order (PDEFilter.cc:485-578 gives the same
    // matrix in closed form)
    {
        const double w[2] = {0.25, 1.0 / 12.0};
        double V = hx * hy * hz, g2[3] = {4.0 / (hx * hx), 4.0 / (hy * hy), 4.0 / (hz * hz)};
        double dm[8];
        for (int m = 0; m < 8; m++) {
            double Wm = V * w[m & 1] * w[(m >> 1) & 1] * w[(m >> 2) & 1];
            double lap = 0.0;
            for (int a = 0; a < 3; a++)
                if (m & (1 << a)) {
                    int ms = m & ~(1 << a);
                    lap += g2[a] * V * w[ms & 1] * w[(ms >> 1) & 1] * w[(ms >> 2) & 1];
                }
            dm[m] = f->R * f->R * lap + Wm;
        }
        // reference local order node r -> lexicographic L
        const int lex[8] = {0, 1, 3, 2, 4, 5, 7, 6};
        for (int col = 0; col < 8; col++) {
            double v[8] = {0};
            v[col] = 1.0;
            mode_fwd(v);
            for (int m = 0; m < 8; m++) v[m] *= dm[m];
            mode_bwd(v);
            for (int L = 0; L < 8; L++) f->KF[L * 8 + col] = v[L];
        }
        (void)lex;
    }
    cudaError_t e = cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        set_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
        delete f;
        return TOPO_ERR_CUDA;
    }
    long long nn = f->g.nn(), nel = f->g.nel();
    auto get = [&](void **p, size_t b) -> int {
        cudaError_t ee = cudaMalloc(p, b);
        if (ee != cudaSuccess) {
            cudaGetLastError();
            set_error("cudaMalloc failed in PDE filter");
            return TOPO_ERR_OOM;
        }
        cudaMemset(*p, 0, b);
        f->ptrs.push_back(*p);
        return 0;
    };
    int rc = 0;
    rc |= get((void **)&f->rhs, sizeof(double) * nn);
    rc |= get((void **)&f->u, sizeof(double) * nn);
    rc |= get((void **)&f->r, sizeof(double) * nn);
    rc |= get((void **)&f->p, sizeof(double) * nn);
    rc |= get((void **)&f->q, sizeof(double) * nn);
    rc |= get((void **)&f->dinv, sizeof(double) * nn);
    rc |= get((void **)&f->e1, sizeof(double) * nel);
    rc |= get((void **)&f->e2, sizeof(double) * nel);
    rc |= get((void **)&f->S, sizeof(FiltScalars));
    rc |= get((void **)&f->part, sizeof(double) * 2 * 65536);
    rc |= get((void **)&f->counter, sizeof(unsigned int) * 4);
    if (rc) {
        pdefilt_destroy(f);
        return TOPO_ERR_OOM;
    }
    KFMat K;
    memcpy(K.v, f->KF, sizeof(K.v));
    count_launch();
    k_filt_dinv<<<ew_blocks(nn), EW, 0, f->stream>>>(f->g, K, f->dinv);
    e = cudaStreamSynchronize(f->stream);
    if (e != cudaSuccess) {
        set_error(std::string("PDE filter setup: ") + cudaGetErrorString(e));
        pdefilt_destroy(f);
        return TOPO_ERR_CUDA;
    }
    *out = f;
    return TOPO_OK;
}

void pdefilt_destroy(TopoPDEFilt *f) {
    if (!f) return;
    for (void *p : f->ptrs) cudaFree(p);
    if (f->stream) cudaStreamDestroy(f->stream);
    delete f;
}

long long pdefilt_nel(const TopoPDEFilt *f) { return f->g.nel(); }
const double *pdefilt_matrix(const TopoPDEFilt *f) { return f->KF; }

// U = K^-1 (vol T x) by Jacobi PCG; the host polls convergence every 8 iterations
static int helmholtz_solve(TopoPDEFilt *f, const double *x_dev) {
    cudaStream_t s = f->stream;
    long long nn = f->g.nn();
    Partials<1> p1{f->part, f->counter};
    Partials<2> p2{f->part, f->counter};
    KFMat K;
    memcpy(K.v, f->KF, sizeof(K.v));
    count_launch();
    k_T<<<ew_blocks(nn), EW, 0, s>>>(f->g, f->vol, x_dev, f->rhs);
    count_launch();
    k_fprime<<<1, 1, 0, s>>>(f->S, f->rtol * f->rtol, f->maxit);
    count_launch();
    k_fpcg_init<<<red_blocks(nn), EW, 0, s>>>(nn, f->rhs, f->dinv, f->u, f->r, f->p, f->S, p2);
    FiltScalars h;
    for (int outer = 0; outer < 1000000; outer++) {
        for (int it = 0; it < 8; it++) {
            count_launch();
            k_filt_apply<<<red_blocks(nn), EW, 0, s>>>(f->g, K, f->p, f->q, p1, f->S, 1);
            count_launch();
            k_fpcg_update<<<red_blocks(nn), EW, 0, s>>>(nn, f->dinv, f->u, f->r, f->p, f->q, f->S, p2);
            count_launch();
            k_fpcg_p<<<ew_blocks(nn), EW, 0, s>>>(nn, f->dinv, f->r, f->p, f->S);
        }
        FCK(cudaMemcpyAsync(&h, f->S, sizeof(h), cudaMemcpyDeviceToHost, s));
        FCK(cudaStreamSynchronize(s));
        if (h.done) break;
    }
    if (h.status) {
        set_error(std::string("PDE filter solve failed with status ") + std::to_string(h.status));
        return h.status;
    }
    return TOPO_OK;
}

int pdefilt_apply_dev(TopoPDEFilt *f, const double *x_dev, double *xout_dev) {
    int rc = helmholtz_solve(f, x_dev);
    if (rc) return rc;
    count_launch();
    k_Tt<<<ew_blocks(f->g.nel()), EW, 0, f->stream>>>(f->g, f->u, xout_dev, nullptr, 0, 0, 0.0, 0.0);
    FCK(cudaStreamSynchronize(f->stream));
    return TOPO_OK;
}

int filter_project_dev(TopoPDEFilt *f, const double *x_dev, double *xTilde_dev, double *xPhys_dev, int projection,
                       double beta, double eta) {
    int rc = helmholtz_solve(f, x_dev);
    if (rc) return rc;
    count_launch();
    k_Tt<<<ew_blocks(f->g.nel()), EW, 0, f->stream>>>(f->g, f->u, xTilde_dev, xPhys_dev, 1, projection, beta, eta);
    FCK(cudaStreamSynchronize(f->stream));
    return TOPO_OK;
}

int filter_gradients_dev(TopoPDEFilt *f, const double *xTilde_dev, double *dfdx_dev, int m, double *dgdx_dev,
                         int projection, double beta, double eta) {
    long long nel = f->g.nel();
    if (projection) {
        count_launch();
        k_chain<<<ew_blocks(nel), EW, 0, f->stream>>>(nel, xTilde_dev, dfdx_dev, m, dgdx_dev, beta, eta);
    }
    // PDEFilt::Gradients == FilterProject (PDEFilter.cc:224); in place via scratch
    FCK(cudaMemcpyAsync(f->e1, dfdx_dev, sizeof(double) * nel, cudaMemcpyDeviceToDevice, f->stream));
    int rc = pdefilt_apply_dev(f, f->e1, dfdx_dev);
    if (rc) return rc;
    for (int j = 0; j < m; j++) {
        FCK(cudaMemcpyAsync(f->e1, dgdx_dev + (size_t)j * nel, sizeof(double) * nel, cudaMemcpyDeviceToDevice,
                            f->stream));
        rc = pdefilt_apply_dev(f, f->e1, dgdx_dev + (size_t)j * nel);
        if (rc) return rc;
    }
    return TOPO_OK;
}

int filter_mnd_dev(TopoPDEFilt *f, const double *x_dev, double *mnd) {
    long long nel = f->g.nel();
    Partials<1> p1{f->part, f->counter};
    count_launch();
    k_mnd<<<red_blocks(nel), EW, 0, f->stream>>>(nel, x_dev, p1, f->e2);
    FCK(cudaMemcpyAsync(mnd, f->e2, sizeof(double), cudaMemcpyDeviceToHost, f->stream));
    FCK(cudaStreamSynchronize(f->stream));
    return TOPO_OK;
}

}  // namespace topo
