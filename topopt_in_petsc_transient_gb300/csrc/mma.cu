// mma.cu -- the Method of Moving Asymptotes (MMA.cc) with design vectors
// resident on the GPU.
//
// Per design iteration: GenSub (MMA.cc:510-637) is one element-wise kernel
// with a fused reduction of b; SolveDIP (:639-676) runs its epsilon/Newton
// loops with one element-wise pass per dual gradient+Hessian evaluation and
// one per dual residual; the m-sized dual algebra (Hessian corrections, the
// m x m LU of Factorize/Solve, line search) runs in FP64 in a single device
// thread.  The host only reads the loop-control flags.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "mma.h"

namespace topo {

constexpr int MMA_MAXM = 8;

#define MCK(call)                                                            \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) {                                             \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));  \
            return TOPO_ERR_CUDA;                                            \
        }                                                                    \
    } while (0)

struct MMAScalars {
    int m, k;
    double asyminit, asymdec, asyminc;
    double a[MMA_MAXM], c[MMA_MAXM], d[MMA_MAXM];
    double b[MMA_MAXM], y[MMA_MAXM], z, lam[MMA_MAXM], mu[MMA_MAXM], grad[MMA_MAXM], s[2 * MMA_MAXM];
    double Hess[MMA_MAXM * MMA_MAXM];
    double epsi, err;
    int loop;
    double ch, n2, ninf;
};

struct TopoMMA {
    int n, m;
    double *L, *U, *alpha, *beta, *p0, *q0, *pij, *qij, *xo1, *xo2;
    MMAScalars *S;
    double *part;
    unsigned int *counter;
    unsigned long long *bits;
    std::vector<void *> ptrs;
    cudaStream_t stream;
    MMAScalars host;
};

// GenSub element part (RobustAsymptotesType 0, no constraint modification)
__global__ void k_mma_gensub(long long n, int m, const double *__restrict__ xv, const double *__restrict__ dfdx,
                             const double *__restrict__ dgdx, const double *__restrict__ xmin,
                             const double *__restrict__ xmax, double *L, double *U, const double *__restrict__ xo1,
                             const double *__restrict__ xo2, double *alf, double *bet, double *p0, double *q0,
                             double *pij, double *qij, MMAScalars *S, GenSubGx gx, Partials<MMA_MAXM> part) {
    const int k = S->k;  // already incremented on the host side
    const double asyminit = S->asyminit, asymdec = S->asymdec, asyminc = S->asyminc;
    const double feps = 1.0e-6;
    double bsum[MMA_MAXM];
    for (int j = 0; j < MMA_MAXM; j++) bsum[j] = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double x = xv[i], lo = xmin[i], hi = xmax[i], Li, Ui;
        if (k < 3) {
            Li = x - asyminit * (hi - lo);
            Ui = x + asyminit * (hi - lo);
        } else {
            Li = L[i];
            Ui = U[i];
            double x1 = xo1[i], x2 = xo2[i];
            double helpvar = (x - x1) * (x1 - x2);
            double gamma = helpvar < 0.0 ? asymdec : (helpvar > 0.0 ? asyminc : 1.0);
            Li = x - gamma * (x1 - Li);
            Ui = x + gamma * (Ui - x1);
            double xmi = fmax(1.0e-5, hi - lo);
            Li = fmax(Li, x - 10.0 * xmi);
            Li = fmin(Li, x - 0.01 * xmi);
            Ui = fmax(Ui, x + 0.01 * xmi);
            Ui = fmin(Ui, x + 10.0 * xmi);
        }
        L[i] = Li;
        U[i] = Ui;
        alf[i] = fmax(lo, 0.9 * Li + 0.1 * x);
        bet[i] = fmin(hi, 0.9 * Ui + 0.1 * x);
        double df = dfdx[i], dfp = fmax(0.0, df), dfm = fmax(0.0, -df);
        double ux = Ui - x, xl = x - Li;
        p0[i] = ux * ux * (dfp + 0.001 * fabs(df) + 0.5 * feps / (Ui - Li));
        q0[i] = xl * xl * (dfm + 0.001 * fabs(df) + 0.5 * feps / (Ui - Li));
        for (int j = 0; j < m; j++) {
            double g = dgdx[(long long)j * n + i];
            double pv = ux * ux * fmax(0.0, g), qv = xl * xl * fmax(0.0, -g);
            pij[(long long)j * n + i] = pv;
            qij[(long long)j * n + i] = qv;
            bsum[j] += pv / ux + qv / xl;
        }
    }
    double tot[MMA_MAXM];
    if (grid_reduce<EW, MMA_MAXM>(bsum, part, tot))
        for (int j = 0; j < m; j++) S->b[j] = tot[j] - gx.v[j];
}

__global__ void k_mma_shift(long long n, const double *__restrict__ x, double *xo1, double *xo2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        xo2[i] = xo1[i];
        xo1[i] = x[i];
    }
}

// SolveDIP initialisation (MMA.cc:642-650)
__global__ void k_mma_dual_init(MMAScalars *S) {
    for (int j = 0; j < S->m; j++) {
        S->lam[j] = S->c[j] / 2.0;
        S->mu[j] = 1.0;
    }
    S->epsi = 1.0;
    S->err = 1.0;
    S->loop = 0;
}

// scalar part of XYZofLAMBDA (MMA.cc:696-703)
__device__ void mma_yz(MMAScalars *S) {
    double lamai = 0.0;
    for (int i = 0; i < S->m; i++) {
        if (S->lam[i] < 0.0) S->lam[i] = 0;
        S->y[i] = fmax(0.0, S->lam[i] - S->c[i]);
        lamai += S->lam[i] * S->a[i];
    }
    S->z = fmax(0.0, 10.0 * (lamai - 1.0));
}
__global__ void k_mma_yz(MMAScalars *S) { mma_yz(S); }

__device__ __forceinline__ double mma_x_of_lambda(int m, long long n, long long i, const double *lam,
                                                  const double *p0, const double *q0, const double *pij,
                                                  const double *qij, const double *L, const double *U,
                                                  const double *alf, const double *bet, double &pj, double &qj,
                                                  double &xraw) {
    pj = p0[i];
    qj = q0[i];
    for (int j = 0; j < m; j++) {
        pj += pij[(long long)j * n + i] * lam[j];
        qj += qij[(long long)j * n + i] * lam[j];
    }
    double sp = sqrt(pj), sq = sqrt(qj);
    xraw = (sp * L[i] + sq * U[i]) / (sp + sq);
    double x = xraw;
    if (x < alf[i]) x = alf[i];
    if (x > bet[i]) x = bet[i];
    return x;
}

// x = x(lambda) written out; sums of DualGrad (MMA.cc:738-743) and the
// Hessian products (MMA.cc:790-818) in one pass: NV = m + m*m <= 72 doubles.
// Packed as [grad m | hess m*m].
template <int M>
__global__ void k_mma_gradhess(long long n, double *x, const double *__restrict__ p0, const double *__restrict__ q0,
                               const double *__restrict__ pij, const double *__restrict__ qij,
                               const double *__restrict__ L, const double *__restrict__ U,
                               const double *__restrict__ alf, const double *__restrict__ bet, MMAScalars *S,
                               Partials<M + M * M> part) {
    double lam[M];
    for (int j = 0; j < M; j++) lam[j] = S->lam[j];
    double acc[M + M * M];
    for (int j = 0; j < M + M * M; j++) acc[j] = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double pj, qj, xr;
        double xi = mma_x_of_lambda(M, n, i, lam, p0, q0, pij, qij, L, U, alf, bet, pj, qj, xr);
        x[i] = xi;
        double ux = U[i] - xi, xl = xi - L[i];
        double PQ[M];
        for (int j = 0; j < M; j++) {
            double pv = pij[(long long)j * n + i], qv = qij[(long long)j * n + i];
            acc[j] += pv / ux + qv / xl;
            PQ[j] = pv / (ux * ux) - qv / (xl * xl);
        }
        double df2 = -1.0 / (2.0 * pj / (ux * ux * ux) + 2.0 * qj / (xl * xl * xl));
        if (xr < alf[i] || xr > bet[i]) df2 = 0.0;
        for (int a = 0; a < M; a++)
            for (int b = 0; b < M; b++) acc[M + a * M + b] += PQ[a] * df2 * PQ[b];
    }
    double tot[M + M * M];
    if (grid_reduce<EW, M + M * M>(acc, part, tot)) {
        // DualGrad completion, then the Newton step of SolveDIP (MMA.cc:658-670)
        for (int j = 0; j < M; j++) S->grad[j] = tot[j] - S->b[j] - S->a[j] * S->z - S->y[j];
        for (int j = 0; j < M; j++) S->grad[j] = -1.0 * S->grad[j] - S->epsi / S->lam[j];
        double *H = S->Hess;
        for (int a = 0; a < M * M; a++) H[a] = tot[M + a];
        // DualHess corrections (MMA.cc:829-858)
        double lamai = 0.0;
        for (int j = 0; j < M; j++) {
            if (S->lam[j] < 0.0) S->lam[j] = 0.0;
            lamai += S->lam[j] * S->a[j];
            if (S->lam[j] > S->c[j]) H[j * M + j] += -1.0;
            H[j * M + j] += -S->mu[j] / S->lam[j];
        }
        if (lamai > 0.0)
            for (int j = 0; j < M; j++)
                for (int kk = 0; kk < M; kk++) H[j * M + kk] += -10.0 * S->a[j] * S->a[kk];
        double tr = 0.0;
        for (int j = 0; j < M; j++) tr += H[j * M + j];
        double corr = 1e-4 * tr / M;
        if (-1.0 * corr < 1.0e-7) corr = -1.0e-7;
        for (int j = 0; j < M; j++) H[j * M + j] += corr;
        // Factorize / Solve (MMA.cc:936-969)
        double *g = S->grad;
        for (int ss = 0; ss < M - 1; ss++)
            for (int ii = ss + 1; ii < M; ii++) {
                H[ii * M + ss] = H[ii * M + ss] / H[ss * M + ss];
                for (int jj = ss + 1; jj < M; jj++) H[ii * M + jj] = H[ii * M + jj] - H[ii * M + ss] * H[ss * M + jj];
            }
        for (int ii = 1; ii < M; ii++) {
            double aa = 0.0;
            for (int jj = 0; jj < ii; jj++) aa = aa - H[ii * M + jj] * g[jj];
            g[ii] = g[ii] + aa;
        }
        g[M - 1] = g[M - 1] / H[(M - 1) * M + (M - 1)];
        for (int ii = M - 2; ii >= 0; ii--) {
            double aa = g[ii];
            for (int jj = ii + 1; jj < M; jj++) aa = aa - H[ii * M + jj] * g[jj];
            g[ii] = aa / H[ii * M + ii];
        }
        for (int j = 0; j < M; j++) S->s[j] = g[j];
        for (int j = 0; j < M; j++) S->s[M + j] = -S->mu[j] + S->epsi / S->lam[j] - S->s[j] * S->mu[j] / S->lam[j];
        // DualLineSearch (MMA.cc:870-888)
        double theta = 1.005;
        for (int j = 0; j < M; j++) {
            if (theta < -1.01 * S->s[j] / S->lam[j]) theta = -1.01 * S->s[j] / S->lam[j];
            if (theta < -1.01 * S->s[j + M] / S->mu[j]) theta = -1.01 * S->s[j + M] / S->mu[j];
        }
        theta = 1.0 / theta;
        for (int j = 0; j < M; j++) {
            S->lam[j] = S->lam[j] + theta * S->s[j];
            S->mu[j] = S->mu[j] + theta * S->s[j + M];
        }
        // XYZofLAMBDA scalar part for the new lambda
        mma_yz(S);
    }
}

// x(lambda) and DualResidual (MMA.cc:890-934); also advances the loop control
template <int M>
__global__ void k_mma_resid(long long n, double *x, const double *__restrict__ p0, const double *__restrict__ q0,
                            const double *__restrict__ pij, const double *__restrict__ qij, const double *__restrict__ L,
                            const double *__restrict__ U, const double *__restrict__ alf, const double *__restrict__ bet,
                            MMAScalars *S, Partials<M> part) {
    double lam[M];
    for (int j = 0; j < M; j++) lam[j] = S->lam[j];
    double acc[M];
    for (int j = 0; j < M; j++) acc[j] = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double pj, qj, xr;
        double xi = mma_x_of_lambda(M, n, i, lam, p0, q0, pij, qij, L, U, alf, bet, pj, qj, xr);
        x[i] = xi;
        for (int j = 0; j < M; j++)
            acc[j] += pij[(long long)j * n + i] / (U[i] - xi) + qij[(long long)j * n + i] / (xi - L[i]);
    }
    double tot[M];
    if (grid_reduce<EW, M>(acc, part, tot)) {
        double nrI = 0.0;
        for (int j = 0; j < M; j++) {
            double r1 = tot[j] - S->b[j] - S->a[j] * S->z - S->y[j] + S->mu[j];
            double r2 = S->mu[j] * S->lam[j] - S->epsi;
            nrI = fmax(nrI, fmax(fabs(r1), fabs(r2)));
        }
        S->err = nrI;
        S->loop += 1;
    }
}

__global__ void k_mma_movelimit(long long n, double Xmin, double Xmax, double movlim, const double *__restrict__ x,
                                double *xmin, double *xmax) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        xmax[i] = fmin(Xmax, x[i] + movlim);
        xmin[i] = fmax(Xmin, x[i] - movlim);
    }
}

__global__ void k_mma_change(long long n, const double *__restrict__ x, double *xold, unsigned long long *bits) {
    double ch = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        ch = fmax(ch, fabs(x[i] - xold[i]));
        xold[i] = x[i];
    }
    for (int o = 16; o > 0; o >>= 1) ch = fmax(ch, __shfl_xor_sync(0xffffffffu, ch, o));
    if ((threadIdx.x & 31) == 0) atomicMax(bits, (unsigned long long)__double_as_longlong(ch));
}

// KKTresidual (MMA.cc:416-484): sums and maxima over elements
__global__ void k_mma_kkt(long long n, int m, const double *__restrict__ x, const double *__restrict__ dfdx,
                          const double *__restrict__ dgdx, const double *__restrict__ xmin,
                          const double *__restrict__ xmax, const MMAScalars *S, Partials<1> part,
                          unsigned long long *bits, double *n2out) {
    double v[1] = {0.0}, ninf = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double ri = dfdx[i];
        for (int j = 0; j < m; j++) ri += S->lam[j] * dgdx[(long long)j * n + i];
        double mu_min = (x[i] < xmin[i] + 1.0e-5 && ri > 0.0) ? ri : 0.0;
        double mu_max = (x[i] > xmax[i] - 1.0e-5 && ri < 0.0) ? -ri : 0.0;
        ri += -mu_min + mu_max;
        double r2 = mu_min * (x[i] - xmin[i]), r3 = mu_max * (xmax[i] - x[i]);
        v[0] += ri * ri + r2 * r2 + r3 * r3;
        ninf = fmax(ninf, fmax(fabs(ri), fmax(fabs(r2), fabs(r3))));
    }
    for (int o = 16; o > 0; o >>= 1) ninf = fmax(ninf, __shfl_xor_sync(0xffffffffu, ninf, o));
    if ((threadIdx.x & 31) == 0) atomicMax(bits, (unsigned long long)__double_as_longlong(ninf));
    double tot[1];
    if (grid_reduce<EW, 1>(v, part, tot)) *n2out = tot[0];
}

// ---------------------------------------------------------------------------
int mma_create(TopoMMA **out, int n, int m, const double *a, const double *c, const double *d) {
    *out = nullptr;
    if (n < 1 || m < 1 || m > 2) {
        set_error("MMA: n >= 1 and 1 <= m <= 2 supported");
        return TOPO_ERR_ARG;
    }
    TopoMMA *mm = new TopoMMA();
    mm->n = n;
    mm->m = m;
    if (cudaStreamCreateWithFlags(&mm->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete mm;
        set_error("MMA: stream creation failed");
        return TOPO_ERR_CUDA;
    }
    auto get = [&](void **p, size_t b) -> int {
        if (cudaMalloc(p, b) != cudaSuccess) {
            cudaGetLastError();
            return TOPO_ERR_OOM;
        }
        cudaMemset(*p, 0, b);
        mm->ptrs.push_back(*p);
        return 0;
    };
    int rc = 0;
    size_t vb = sizeof(double) * (size_t)n;
    rc |= get((void **)&mm->L, vb);
    rc |= get((void **)&mm->U, vb);
    rc |= get((void **)&mm->alpha, vb);
    rc |= get((void **)&mm->beta, vb);
    rc |= get((void **)&mm->p0, vb);
    rc |= get((void **)&mm->q0, vb);
    rc |= get((void **)&mm->pij, vb * m);
    rc |= get((void **)&mm->qij, vb * m);
    rc |= get((void **)&mm->xo1, vb);
    rc |= get((void **)&mm->xo2, vb);
    rc |= get((void **)&mm->S, sizeof(MMAScalars));
    rc |= get((void **)&mm->part, sizeof(double) * 8 * 65536);
    rc |= get((void **)&mm->counter, sizeof(unsigned int) * 4);
    rc |= get((void **)&mm->bits, sizeof(unsigned long long) * 2);
    if (rc) {
        set_error("MMA: device allocation failed");
        mma_destroy(mm);
        return TOPO_ERR_OOM;
    }
    // MMA::MMA(n, m, x, a, c, d), MMA.cc:180-229
    MMAScalars &h = mm->host;
    memset(&h, 0, sizeof(h));
    h.m = m;
    h.k = 0;
    h.asyminit = 0.5;
    h.asymdec = 0.7;
    h.asyminc = 1.2;
    for (int j = 0; j < m; j++) {
        h.a[j] = a ? a[j] : 0.0;
        h.c[j] = c ? c[j] : 1000.0;
        h.d[j] = d ? d[j] : 0.0;
    }
    if (cudaMemcpy(mm->S, &h, sizeof(h), cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("MMA: upload failed");
        mma_destroy(mm);
        return TOPO_ERR_CUDA;
    }
    *out = mm;
    return TOPO_OK;
}

void mma_destroy(TopoMMA *mm) {
    if (!mm) return;
    for (void *p : mm->ptrs) cudaFree(p);
    if (mm->stream) cudaStreamDestroy(mm->stream);
    delete mm;
}

int mma_set_asymptotes(TopoMMA *mm, double init, double dec, double inc) {
    mm->host.asyminit = init;
    mm->host.asymdec = dec;
    mm->host.asyminc = inc;
    MCK(cudaMemcpyAsync(&mm->S->asyminit, &mm->host.asyminit, 3 * sizeof(double), cudaMemcpyHostToDevice,
                        mm->stream));
    MCK(cudaStreamSynchronize(mm->stream));
    return TOPO_OK;
}

int mma_movelimit_dev(TopoMMA *mm, double Xmin, double Xmax, double movlim, const double *x, double *xmin,
                      double *xmax) {
    count_launch();
    k_mma_movelimit<<<ew_blocks(mm->n), EW, 0, mm->stream>>>(mm->n, Xmin, Xmax, movlim, x, xmin, xmax);
    MCK(cudaStreamSynchronize(mm->stream));
    return TOPO_OK;
}

template <int M>
static int solve_dip(TopoMMA *mm, double *x) {
    cudaStream_t s = mm->stream;
    long long n = mm->n;
    unsigned nb = red_blocks(n);
    Partials<M + M * M> pgh{mm->part, mm->counter};
    Partials<M> pr{mm->part, mm->counter};
    count_launch();
    k_mma_dual_init<<<1, 1, 0, s>>>(mm->S);
    double epsi = 1.0, err = 1.0;
    const double tol = 1.0e-9 * sqrt((double)(mm->m + mm->n));
    // SolveDIP loop structure (MMA.cc:651-674)
    count_launch();
    k_mma_yz<<<1, 1, 0, s>>>(mm->S);
    while (epsi > tol) {
        int loop = 0;
        while (err > 0.9 * epsi && loop < 100) {
            loop++;
            count_launch();
            k_mma_gradhess<M><<<nb, EW, 0, s>>>(n, x, mm->p0, mm->q0, mm->pij, mm->qij, mm->L, mm->U, mm->alpha,
                                                mm->beta, mm->S, pgh);
            count_launch();
            k_mma_resid<M><<<nb, EW, 0, s>>>(n, x, mm->p0, mm->q0, mm->pij, mm->qij, mm->L, mm->U, mm->alpha,
                                             mm->beta, mm->S, pr);
            MCK(cudaMemcpyAsync(&err, &mm->S->err, sizeof(double), cudaMemcpyDeviceToHost, s));
            MCK(cudaStreamSynchronize(s));
            if (!std::isfinite(err)) {
                set_error("MMA dual solve produced a non-finite residual");
                return TOPO_ERR_NAN;
            }
        }
        epsi = epsi * 0.1;
        MCK(cudaMemcpyAsync(&mm->S->epsi, &epsi, sizeof(double), cudaMemcpyHostToDevice, s));
    }
    MCK(cudaStreamSynchronize(s));
    return TOPO_OK;
}

int mma_update_dev(TopoMMA *mm, double *xval, const double *dfdx, const double *gx, const double *dgdx,
                   const double *xmin, const double *xmax) {
    cudaStream_t s = mm->stream;
    long long n = mm->n;
    mm->host.k += 1;
    MCK(cudaMemcpyAsync(&mm->S->k, &mm->host.k, sizeof(int), cudaMemcpyHostToDevice, s));
    GenSubGx g;
    memset(&g, 0, sizeof(g));
    for (int j = 0; j < mm->m; j++) g.v[j] = gx[j];
    Partials<MMA_MAXM> pb{mm->part, mm->counter};
    count_launch();
    k_mma_gensub<<<red_blocks(n), EW, 0, s>>>(n, mm->m, xval, dfdx, dgdx, xmin, xmax, mm->L, mm->U, mm->xo1, mm->xo2,
                                             mm->alpha, mm->beta, mm->p0, mm->q0, mm->pij, mm->qij, mm->S, g, pb);
    count_launch();
    k_mma_shift<<<ew_blocks(n), EW, 0, s>>>(n, xval, mm->xo1, mm->xo2);
    int rc = (mm->m == 1) ? solve_dip<1>(mm, xval) : solve_dip<2>(mm, xval);
    if (rc) return rc;
    MCK(cudaGetLastError());
    return TOPO_OK;
}

int mma_design_change_dev(TopoMMA *mm, const double *x, double *xold, double *ch) {
    MCK(cudaMemsetAsync(mm->bits, 0, sizeof(unsigned long long), mm->stream));
    count_launch();
    k_mma_change<<<ew_blocks(mm->n), EW, 0, mm->stream>>>(mm->n, x, xold, mm->bits);
    unsigned long long b = 0;
    MCK(cudaMemcpyAsync(&b, mm->bits, sizeof(b), cudaMemcpyDeviceToHost, mm->stream));
    MCK(cudaStreamSynchronize(mm->stream));
    double v;
    memcpy(&v, &b, sizeof(v));
    *ch = v;
    return TOPO_OK;
}

int mma_kkt_dev(TopoMMA *mm, const double *x, const double *dfdx, const double *fx, const double *dgdx,
                const double *xmin, const double *xmax, double *norm2, double *normInf) {
    cudaStream_t s = mm->stream;
    MCK(cudaMemsetAsync(mm->bits, 0, sizeof(unsigned long long), s));
    double *n2d = mm->part + 8 * 65536 - 1;
    Partials<1> p1{mm->part, mm->counter};
    count_launch();
    k_mma_kkt<<<red_blocks(mm->n), EW, 0, s>>>(mm->n, mm->m, x, dfdx, dgdx, xmin, xmax, mm->S, p1, mm->bits, n2d);
    unsigned long long b = 0;
    double n2 = 0.0;
    MMAScalars h;
    MCK(cudaMemcpyAsync(&b, mm->bits, sizeof(b), cudaMemcpyDeviceToHost, s));
    MCK(cudaMemcpyAsync(&n2, n2d, sizeof(double), cudaMemcpyDeviceToHost, s));
    MCK(cudaMemcpyAsync(&h, mm->S, sizeof(h), cudaMemcpyDeviceToHost, s));
    MCK(cudaStreamSynchronize(s));
    double ninf;
    memcpy(&ninf, &b, sizeof(ninf));
    double ri = 0.0;
    for (int j = 0; j < mm->m; j++) ri += h.lam[j] * (h.a[j] * h.z + h.y[j] - fx[j]);
    n2 += ri * ri;
    ninf = fmax(fabs(ri), ninf);
    *norm2 = sqrt(n2);
    *normInf = ninf;
    return TOPO_OK;
}

int mma_restart_set_dev(TopoMMA *mm, int itr, const double *xo1, const double *xo2, const double *U,
                        const double *L) {
    if (itr < 0) {
        set_error("MMA restart: negative iteration counter");
        return TOPO_ERR_ARG;
    }
    // the reference accepts itr < 3 with a warning ("NOT A LEGAL RESTART POINT")
    const size_t b = sizeof(double) * (size_t)mm->n;
    cudaStream_t s = mm->stream;
    MCK(cudaMemcpyAsync(mm->xo1, xo1, b, cudaMemcpyDeviceToDevice, s));
    MCK(cudaMemcpyAsync(mm->xo2, xo2, b, cudaMemcpyDeviceToDevice, s));
    MCK(cudaMemcpyAsync(mm->U, U, b, cudaMemcpyDeviceToDevice, s));
    MCK(cudaMemcpyAsync(mm->L, L, b, cudaMemcpyDeviceToDevice, s));
    mm->host.k = itr;
    MCK(cudaMemcpyAsync(&mm->S->k, &mm->host.k, sizeof(int), cudaMemcpyHostToDevice, s));
    MCK(cudaStreamSynchronize(s));
    return TOPO_OK;
}

int mma_restart_get_dev(TopoMMA *mm, double *xo1, double *xo2, double *U, double *L) {
    const size_t b = sizeof(double) * (size_t)mm->n;
    cudaStream_t s = mm->stream;
    MCK(cudaMemcpyAsync(xo1, mm->xo1, b, cudaMemcpyDeviceToDevice, s));
    MCK(cudaMemcpyAsync(xo2, mm->xo2, b, cudaMemcpyDeviceToDevice, s));
    MCK(cudaMemcpyAsync(U, mm->U, b, cudaMemcpyDeviceToDevice, s));
    MCK(cudaMemcpyAsync(L, mm->L, b, cudaMemcpyDeviceToDevice, s));
    MCK(cudaStreamSynchronize(s));
    return TOPO_OK;
}

int mma_n(const TopoMMA *mm) { return mm->n; }
int mma_m(const TopoMMA *mm) { return mm->m; }
void *mma_stream(TopoMMA *mm) { return mm->stream; }

}  // namespace topo
