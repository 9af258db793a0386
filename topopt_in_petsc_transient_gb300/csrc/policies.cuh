// policies.cuh -- fused epilogues for the matrix-free tile kernel (tile.cuh).
//
// Masking convention: the Dirichlet vector N of the reference
// (LinearElasticity.cc:552-574) is stored as a per-node bitmask `fixed`
// (bit c set <=> DOF 3n+c is clamped).  Every system operator is the
// reference's  N A N + (I - N)  (MatDiagonalScale + MatDiagonalSet,
// LinearElasticity.cc:1118-1122), applied as: zero clamped inputs, apply the
// element operator, zero clamped outputs, add the identity on clamped DOFs.
#pragma once
#include "df.cuh"
#include "tile.cuh"

namespace topo {

template <class T>
__device__ __forceinline__ void mask3(uint8_t f, T v[3]) {
    if (f & 1) v[0] = T(0);
    if (f & 2) v[1] = T(0);
    if (f & 4) v[2] = T(0);
}

// scalars of one Krylov solve, resident in device memory
struct SolveScalars {
    double bb, rr, rho, rho_old, alpha, beta, pq, gam;
    double tol2;      // rtol^2
    int it, maxit;
    int status;       // 0 running/converged, TOPO_ERR_* on failure
    int done;         // 1 once converged / failed: later body kernels return
    int zero_x;       // rhs was exactly zero: solution is zero
    int total_it;     // accumulated iterations over all solves (diagnostics)
    // reliable-update mixed precision (FP32 recurrence, FP64 replacements)
    double rr_ref, tau2;
    int need_replace, restart, inner_it, kmax;
    int replacements, breakdowns32;
    // the FP32 recurrence runs on r32 = sigma * r (sigma = 1/rms(r) at the
    // last FP64 residual), so FP32 never sees the absolute scale of the state
    double sigma, ndof;
    int rescale;
    float beta32;     // beta of the FP32 recurrence in FP32 (read per staged node by PolPQ32)
    float alpha32;    // alpha of the FP32 recurrence in FP32 and alpha / sigma (the
    double alpha_x;   // step of the unscaled FP64 x): set once with alpha by PolPQ32
};

// ---------------------------------------------------------------------------
// element weights: ck = sK * kf[e] (* P[e]), cm = sM * mf[e] (* P[e])
// ---------------------------------------------------------------------------
template <class T>
struct Weights {
    const T *kf, *mf;  // per-element density factors (may be null when s == 0)
    const double *P;   // optional region mask
    T sK, sM;
    __device__ __forceinline__ void get(long long e, T &ck, T &cm) const {
        ck = kf ? sK * kf[e] : T(0);
        cm = mf ? sM * mf[e] : T(0);
        if (P) {  // region mask: only when the caller passes one
            const T w = (T)P[e];
            ck = ck * w;
            cm = cm * w;
        }
    }
};

// solver state after the initial residual (t[0] = b.b, t[1] = r.r)
__device__ __forceinline__ void init_finish(SolveScalars *S, const double t[2], bool has_r32,
                                            cudaGraphConditionalHandle cond, int has_cond, bool accept_x0 = true) {
    S->bb = t[0];
    S->rr = t[1];
    S->it = 0;
    S->status = 0;
    S->zero_x = (t[0] == 0.0);
    S->done = (t[0] == 0.0) || (accept_x0 && t[1] <= S->tol2 * t[0]);
    S->need_replace = 0;
    S->restart = 1;
    S->inner_it = 0;
    S->sigma = (t[1] > 0.0) ? sqrt(S->ndof / t[1]) : 1.0;
    S->rr_ref = t[1] * S->sigma * S->sigma;
    S->rescale = has_r32;
    if (!isfinite(t[1])) {
        S->status = TOPO_ERR_NAN;
        S->done = 1;
    }
    if (has_cond) cudaGraphSetConditional(cond, S->done ? 0u : 1u);
}

// ---------------------------------------------------------------------------
// FCG initial residual: r = b - (N A N + I - N) x0, reductions b.b and r.r
// ---------------------------------------------------------------------------
template <class T>
struct PolInitResid {
    static constexpr int NIN = 1, NRED = 2;
    static constexpr bool HAS_K = true, HAS_M = true;
    const uint8_t *fixed;
    Weights<T> w;
    const double *x, *b;
    double *r;
    float *r32;  // optional FP32 copy for the mixed-precision preconditioner
    SolveScalars *S;
    cudaGraphConditionalHandle cond;
    int has_cond;
    Partials<2> part;
    __device__ void load(long long n, T v[1][3]) const {
        v[0][0] = T(x[3 * n]);
        v[0][1] = T(x[3 * n + 1]);
        v[0][2] = T(x[3 * n + 2]);
        mask3(fixed[n], v[0]);
    }
    __device__ void coef(long long e, T &ck, T &cm) const { w.get(e, ck, cm); }
    __device__ void epilogue(long long n, int, int, int, const T y[3], double red[2]) const {
        uint8_t f = fixed[n];
        for (int c = 0; c < 3; c++) {
            double xv = x[3 * n + c], bv = b[3 * n + c];
            double ax = ((f >> c) & 1) ? xv : todbl(y[c]);
            double rv = bv - ax;
            r[3 * n + c] = rv;
            red[0] += bv * bv;
            red[1] += rv * rv;
        }
    }
    __device__ void finish(const double t[2]) const { init_finish(S, t, r32 != nullptr, cond, has_cond); }
};

// ---------------------------------------------------------------------------
// FCG operator product: q = (N A N + I - N) p, reduction p.q -> alpha
// ---------------------------------------------------------------------------
template <class T>
struct PolPQ {
    static constexpr int NIN = 1, NRED = 1;
    static constexpr bool HAS_K = true, HAS_M = true;
    const uint8_t *fixed;
    Weights<T> w;
    const T *p;
    T *q;
    SolveScalars *S;
    Partials<1> part;
    __device__ void load(long long n, T v[1][3]) const {
        v[0][0] = p[3 * n];
        v[0][1] = p[3 * n + 1];
        v[0][2] = p[3 * n + 2];
        mask3(fixed[n], v[0]);
    }
    __device__ void coef(long long e, T &ck, T &cm) const { w.get(e, ck, cm); }
    __device__ void epilogue(long long n, int, int, int, const T y[3], double red[1]) const {
        uint8_t f = fixed[n];
        for (int c = 0; c < 3; c++) {
            T pv = p[3 * n + c];
            T qv = ((f >> c) & 1) ? pv : y[c];
            q[3 * n + c] = qv;
            red[0] += (double)pv * (double)qv;
        }
    }
    __device__ void finish(const double t[1]) const {
        S->pq = t[0];
        if (!(t[0] > 0.0) || !isfinite(t[0])) {
            S->status = isfinite(t[0]) ? TOPO_ERR_BREAKDOWN : TOPO_ERR_NAN;
            S->alpha = 0.0;
            S->done = 1;
        } else {
            S->alpha = S->rho / t[0];
        }
    }
};

// ---------------------------------------------------------------------------
// Mixed precision (reliable updates): the Krylov recurrence runs on FP32
// vectors with the FP32 operator; FP64 is used for the iterate x, the dot
// products and the true residual r = b - A x, recomputed ("replaced") with
// the FP64 operator whenever the FP32 recurrence residual has dropped by
// inner_tol or after inner_maxit iterations.  Convergence is decided on the
// FP64 residual only, so the tolerance means the same as in the plain path.
// ---------------------------------------------------------------------------
struct PolPQ32 {
    // q = (N A N + I - N) p and p.q, with the FCG direction update
    // p = z + beta p_prev (k_mfcg_p) done while staging: p_prev is read from
    // pb[it & 1] and the new p written to pb[(it + 1) & 1], so no CTA
    // overwrites a halo value another CTA still stages
    static constexpr int NIN = 1, NRED = 1;
    static constexpr bool HAS_K = true, HAS_M = true;
    const uint8_t *fixed;
    Weights<float> w;
    const float *z;
    float *pb[2];
    float *q;
    SolveScalars *S;
    Partials<1> part;
    __device__ __forceinline__ void pnew(long long n, float v[3]) const {
        const float beta = S->beta32;
        const float *pp = (S->it & 1) ? pb[1] : pb[0];  // a select: no local copy of pb
        for (int c = 0; c < 3; c++) v[c] = (beta == 0.0f) ? z[3 * n + c] : z[3 * n + c] + beta * pp[3 * n + c];
    }
    __device__ void load(long long n, float v[1][3]) const {
        pnew(n, v[0]);
        mask3(fixed[n], v[0]);
    }
    __device__ void coef(long long e, float &ck, float &cm) const { w.get(e, ck, cm); }
    struct Pre {
        float p[3];
        uint8_t f;
    };
    __device__ Pre pre(long long n) const {
        Pre r;
        pnew(n, r.p);
        r.f = fixed[n];
        return r;
    }
    using Red = float;  // p.q summed per thread in FP32 (about a dozen nodes), widened once
    __device__ void epilogue(long long n, int, int, int, const float y[3], float red[1], const Pre &r) const {
        float *pout = (S->it & 1) ? pb[0] : pb[1];
        float s = 0.0f;
        for (int c = 0; c < 3; c++) {
            float pv = r.p[c];
            float qv = ((r.f >> c) & 1) ? pv : y[c];
            pout[3 * n + c] = pv;
            q[3 * n + c] = qv;
            s += pv * qv;
        }
        red[0] += s;
    }
    __device__ void finish(const double t[1]) const {
        S->pq = t[0];
        if (!(t[0] > 0.0) || !isfinite(t[0])) {
            S->alpha = 0.0;  // FP32 breakdown: restart from the true residual
            S->need_replace = 1;
            S->breakdowns32 += 1;
        } else {
            S->alpha = S->rho / t[0];
        }
        S->alpha32 = (float)S->alpha;
        S->alpha_x = S->alpha / S->sigma;
    }
};

// solver state after a residual replacement with true residual norm^2 rr
__device__ __forceinline__ void replace_finish(SolveScalars *S, double rr, cudaGraphConditionalHandle cond,
                                               int has_cond) {
    S->rr = rr;
    S->need_replace = 0;
    S->restart = 1;
    S->inner_it = 0;
    S->replacements += 1;
    S->sigma = (rr > 0.0) ? sqrt(S->ndof / rr) : 1.0;
    S->rr_ref = rr * S->sigma * S->sigma;
    S->rescale = 1;
    if (!isfinite(rr)) {
        S->status = TOPO_ERR_NAN;
        S->done = 1;
    } else if (rr <= S->tol2 * S->bb) {
        S->done = 1;
    } else if (S->it >= S->maxit) {
        S->status = TOPO_ERR_NOT_CONVERGED;
        S->done = 1;
    }
    if (has_cond) cudaGraphSetConditional(cond, S->done ? 0u : 1u);
}

// Residual replacement of the mixed FCG, only when one is due (the whole grid
// exits otherwise): y = (N A N) x FP64-accurate (T = double-float), then in
// the epilogue r = b - y on free DOFs and b - x on clamped ones, r.r and the
// convergence decision (replace_finish), which drives the graph condition.
// b, x and the mask of the output node are loaded before the element phase.
// Every CTA reads the replacement flag before it can reach the grid
// reduction whose last CTA clears it.
template <class T>
struct PolReplace {
    static constexpr int NIN = 1, NRED = 1;
    static constexpr bool HAS_K = true, HAS_M = true;
    const uint8_t *fixed;
    Weights<T> w;
    const double *x;
    const double *b;
    double *r;
    SolveScalars *S;
    cudaGraphConditionalHandle cond;
    int has_cond;
    Partials<1> part;
    __device__ bool skip() const { return S->need_replace == 0; }
    __device__ void load(long long n, T v[1][3]) const {
        v[0][0] = T(x[3 * n]);
        v[0][1] = T(x[3 * n + 1]);
        v[0][2] = T(x[3 * n + 2]);
        mask3(fixed[n], v[0]);
    }
    // asynchronous staging (tile.cuh): x and the clamp mask
    using Src = double;
    static constexpr int NSRC = 1;
    static constexpr bool MASK = true;
    __device__ const double *src(int) const { return x; }
    __device__ void xform(const double raw[][3], uint8_t f, T v[1][3]) const {
        for (int c = 0; c < 3; c++) v[0][c] = T(raw[0][c]);
        mask3(f, v[0]);
    }
    __device__ void coef(long long e, T &ck, T &cm) const { w.get(e, ck, cm); }
    struct Pre {
        double b[3], x[3];
        uint8_t f;
    };
    __device__ Pre pre(long long n) const {
        Pre q;
        for (int c = 0; c < 3; c++) {
            q.b[c] = b[3 * n + c];
            q.x[c] = x[3 * n + c];
        }
        q.f = fixed[n];
        return q;
    }
    __device__ void epilogue(long long n, int, int, int, const T yv[3], double red[1], const Pre &q) const {
        for (int c = 0; c < 3; c++) {
            const double rv = q.b[c] - (((q.f >> c) & 1) ? q.x[c] : todbl(yv[c]));
            r[3 * n + c] = rv;
            red[0] += rv * rv;
        }
    }
    __device__ void finish(const double t[1]) const { replace_finish(S, t[0], cond, has_cond); }
};

// ---------------------------------------------------------------------------
// Chebyshev-Jacobi smoothing step (one operator application):
//   r = b - (N A N + I - N) x_in ;  d = c1 d + c2 Dinv r ;  x_out = x_in + d
// Coefficients from the device-resident spectrum bounds [lo, hi] of Dinv A.
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void cheb_coeffs(const double *lohi, int k, T &c1, T &c2) {
    double lo = lohi[0], hi = lohi[1];
    double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
    if (k == 0) {
        c1 = T(0);
        c2 = (T)(1.0 / theta);
        return;
    }
    double rho_prev = 1.0 / sigma, rho = rho_prev;
    for (int i = 1; i <= k; i++) {
        rho_prev = rho;
        rho = 1.0 / (2.0 * sigma - rho_prev);
    }
    c1 = (T)(rho * rho_prev);
    c2 = (T)(2.0 * rho / delta);
}

template <class T>
struct PolCheb {
    static constexpr int NIN = 1, NRED = 0;
    static constexpr bool HAS_K = true, HAS_M = true;
    const uint8_t *fixed;
    Weights<T> w;
    const T *x_in, *b, *dinv;
    T *x_out, *d;
    const double *ctab;  // Chebyshev table [k][2] = (c1, c2), built once per design
    int k;
    Partials<1> part;
    __device__ void load(long long n, T v[1][3]) const {
        v[0][0] = x_in[3 * n];
        v[0][1] = x_in[3 * n + 1];
        v[0][2] = x_in[3 * n + 2];
        mask3(fixed[n], v[0]);
    }
    __device__ void coef(long long e, T &ck, T &cm) const { w.get(e, ck, cm); }
    struct Pre {
        T x[3], b[3], di[3], d[3];
        uint8_t f;
    };
    __device__ Pre pre(long long n) const {
        Pre q;
        for (int c = 0; c < 3; c++) {
            q.x[c] = x_in[3 * n + c];
            q.b[c] = b[3 * n + c];
            q.di[c] = dinv[3 * n + c];
            q.d[c] = (k == 0) ? T(0) : d[3 * n + c];
        }
        q.f = fixed[n];
        return q;
    }
    __device__ void epilogue(long long n, int, int, int, const T y[3], double *, const Pre &q) const {
        const T c1 = (T)ctab[2 * k], c2 = (T)ctab[2 * k + 1];
        for (int c = 0; c < 3; c++) {
            T rv = q.b[c] - (((q.f >> c) & 1) ? q.x[c] : y[c]);
            T dv = c1 * q.d[c] + c2 * q.di[c] * rv;
            d[3 * n + c] = dv;
            x_out[3 * n + c] = q.x[c] + dv;
        }
    }
    __device__ void finish(const double *) const {}
};

// The last fine-level smoothing step of the FP32 preconditioner in the mixed
// FCG, fused with the FCG dot products of its output z (the preconditioned
// residual): z.r32 -> rho, z.q32 -> gamma, beta = -gamma / (p.q)  (k_mfcg_dot).
// Here b is r32.
struct PolChebDot {
    static constexpr int NIN = 1, NRED = 2;
    static constexpr bool HAS_K = true, HAS_M = true;
    const uint8_t *fixed;
    Weights<float> w;
    const float *x_in, *b, *dinv;
    float *x_out, *d;
    const double *ctab;
    int k;
    const float *q32;
    SolveScalars *S;
    Partials<2> part;
    __device__ void load(long long n, float v[1][3]) const {
        v[0][0] = x_in[3 * n];
        v[0][1] = x_in[3 * n + 1];
        v[0][2] = x_in[3 * n + 2];
        mask3(fixed[n], v[0]);
    }
    __device__ void coef(long long e, float &ck, float &cm) const { w.get(e, ck, cm); }
    struct Pre {
        float x[3], b[3], di[3], d[3], q[3];
        uint8_t f;
    };
    __device__ Pre pre(long long n) const {
        Pre r;
        for (int c = 0; c < 3; c++) {
            r.x[c] = x_in[3 * n + c];
            r.b[c] = b[3 * n + c];
            r.di[c] = dinv[3 * n + c];
            r.d[c] = (k == 0) ? 0.0f : d[3 * n + c];
            r.q[c] = q32[3 * n + c];
        }
        r.f = fixed[n];
        return r;
    }
    using Red = float;  // the dot products summed per thread in FP32, widened once
    __device__ void epilogue(long long n, int, int, int, const float y[3], float red[2], const Pre &q) const {
        const float c1 = (float)ctab[2 * k], c2 = (float)ctab[2 * k + 1];
        float s0 = 0.0f, s1 = 0.0f;
        for (int c = 0; c < 3; c++) {
            float rv = q.b[c] - (((q.f >> c) & 1) ? q.x[c] : y[c]);
            float dv = c1 * q.d[c] + c2 * q.di[c] * rv;
            float zv = q.x[c] + dv;
            d[3 * n + c] = dv;
            x_out[3 * n + c] = zv;
            s0 += zv * q.b[c];
            s1 += zv * q.q[c];
        }
        red[0] += s0;
        red[1] += s1;
    }
    __device__ void finish(const double t[2]) const {
        S->rho = t[0];
        S->gam = t[1];
        S->beta = S->restart ? 0.0 : -t[1] / S->pq;
        if (!isfinite(S->beta)) S->beta = 0.0;
        S->beta32 = (float)S->beta;
        S->rescale = 0;
    }
};

// residual only: r = b - (N A N + I - N) x   (before restriction)
template <class T>
struct PolResid {
    static constexpr int NIN = 1, NRED = 0;
    static constexpr bool HAS_K = true, HAS_M = true;
    const uint8_t *fixed;
    Weights<T> w;
    const T *x, *b;
    T *r;
    Partials<1> part;
    __device__ void load(long long n, T v[1][3]) const {
        v[0][0] = x[3 * n];
        v[0][1] = x[3 * n + 1];
        v[0][2] = x[3 * n + 2];
        mask3(fixed[n], v[0]);
    }
    __device__ void coef(long long e, T &ck, T &cm) const { w.get(e, ck, cm); }
    __device__ void epilogue(long long n, int, int, int, const T y[3], double *) const {
        uint8_t f = fixed[n];
        for (int c = 0; c < 3; c++) {
            T xv = x[3 * n + c];
            r[3 * n + c] = b[3 * n + c] - (((f >> c) & 1) ? xv : y[c]);
        }
    }
    __device__ void finish(const double *) const {}
};

// plain weighted product y = sum_e (ck KE + cm ME) x_e, no masking
template <class T, bool HK, bool HM>
struct PolProduct {
    static constexpr int NIN = 1, NRED = 0;
    static constexpr bool HAS_K = HK, HAS_M = HM;
    Weights<T> w;
    const double *x;
    double *y;
    Partials<1> part;
    __device__ void load(long long n, T v[1][3]) const {
        v[0][0] = T(x[3 * n]);
        v[0][1] = T(x[3 * n + 1]);
        v[0][2] = T(x[3 * n + 2]);
    }
    // asynchronous staging (tile.cuh): x, no mask
    using Src = double;
    static constexpr int NSRC = 1;
    static constexpr bool MASK = false;
    __device__ const double *src(int) const { return x; }
    __device__ void xform(const double raw[][3], uint8_t, T v[1][3]) const {
        for (int c = 0; c < 3; c++) v[0][c] = T(raw[0][c]);
    }
    __device__ void coef(long long e, T &ck, T &cm) const { w.get(e, ck, cm); }
    __device__ void epilogue(long long n, int, int, int, const T yv[3], double *) const {
        y[3 * n] = todbl(yv[0]);
        y[3 * n + 1] = todbl(yv[1]);
        y[3 * n + 2] = todbl(yv[2]);
    }
    __device__ void finish(const double *) const {}
};

// ---------------------------------------------------------------------------
// forward time stepping (SolveStateBlock, LinearElasticity.cc:1317-1385)
// ---------------------------------------------------------------------------
struct StepCtx {   // device-resident time-stepping state
    int block;     // checkpoint block c
    int j;         // step within block
    int tsc;
    int nadj;      // adjoint steps completed in the current reverse sweep
    double dt;
    double fx;     // objective accumulator
};

// second point load of the extended workloads: sin(2 pi t + phase) for t < 0.5
__device__ __forceinline__ double load2_signal(double phase, double t) {
    return (t < 0.5) ? sin(2.0 * 3.14159265358979323846 * t + phase) : 0.0;
}

__device__ __forceinline__ double load_signal(int which, double t) {
    if (which == 1) return (t < 0.5) ? sin(2.0 * 3.14159265358979323846 * t) : 0.0;
    // LinearElasticity.cc:597-606
    const double t0 = 8.0, c = 1.1;
    double s = t - t0;
    return exp(-(s * s) / ((2 * c) * (2 * c))) * cos(4.0 * s) * cos(5.0 * s) * cos(6.0 * s) * cos(7.0 * s);
}

// Load(t) / (ny - 1) and the second load's signal at every time step t dt,
// t = 0 .. Ts - 1, tabulated once per object by the same device functions: the
// right-hand-side kernels read two doubles instead of evaluating exp/sin/cos
// in FP64 per thread or per node (GB300 runs FP64 at 1/64 of the FP32 rate)
static __global__ void k_load_table(int Ts, double dt, int which, double scale, double phase, double *sig,
                                    double *sig2) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < Ts; t += gridDim.x * blockDim.x) {
        sig[t] = load_signal(which, t * dt) * scale;
        sig2[t] = load2_signal(phase, t * dt) * scale;
    }
}

// ---------------------------------------------------------------------------
// Newmark right-hand side of one forward step (plain FP64 path):
//   b = N (f(t) + B1 u- + B2 du- + B3 ddu-),  B_i = N (cMi M + cKi K) N
// staged as vK = sum cKi (u-,du-,ddu-)_i and vM = sum cMi (...)_i so that one
// element pass gives K vK + M vM.  Also writes the initial guess x0 (the
// Newmark predictor, see fwd_prep_args).
// ---------------------------------------------------------------------------
template <class T>
struct PolRhsFwd {
    static constexpr int NIN = 2, NRED = 0;
    static constexpr bool HAS_K = true, HAS_M = true;
    const uint8_t *fixed;
    Weights<T> w;
    const double *cp;                   // checkpoints: block start state (j == 0)
    const double *Uh, *DUh, *DDUh;      // block history [tsc][ndof]
    long long ndof;
    const double *rhs0;                 // RHSLocation (LoadLocation, LinearElasticity.cc:616-675)
    const double *sig, *sig2;           // Load(t)/(ny-1) and the second load's signal per step (k_load_table)
    long long load2_dof;                // z DOF of the second point load (-1: none)
    double cK[3], cM[3];                // combination coefficients of (u-, du-, ddu-)
    double pred[3];                     // predictor coefficients (u-, du-, ddu-)
    double pred2[2];                    // with an older acceleration ddu--: (ddu-, ddu--)
    int use_pred2;                      // 1: x0 = u- + dt du- + pred2 . (ddu-, ddu--) when ddu-- exists
    const StepCtx *st;
    double *b, *x0;
    Partials<1> part;
    __device__ __forceinline__ void prev(const double *&u, const double *&du, const double *&ddu) const {
        int j = st->j;
        if (j == 0) {
            const double *base = cp + (long long)st->block * 3 * ndof;
            u = base;
            du = base + ndof;
            ddu = base + 2 * ndof;
        } else {
            u = Uh + (long long)(j - 1) * ndof;
            du = DUh + (long long)(j - 1) * ndof;
            ddu = DDUh + (long long)(j - 1) * ndof;
        }
    }
    __device__ void load(long long n, T v[2][3]) const {
        const double *u, *du, *ddu;
        prev(u, du, ddu);
        for (int c = 0; c < 3; c++) {
            double a = u[3 * n + c], bb = du[3 * n + c], cc = ddu[3 * n + c];
            v[0][c] = T(cK[0] * a + cK[1] * bb + cK[2] * cc);
            v[1][c] = T(cM[0] * a + cM[1] * bb + cM[2] * cc);
        }
        mask3(fixed[n], v[0]);
        mask3(fixed[n], v[1]);
    }
    __device__ void coef(long long e, T &ck, T &cm) const { w.get(e, ck, cm); }
    __device__ void epilogue(long long n, int, int, int, const T y[3], double *) const {
        const double *u, *du, *ddu;
        prev(u, du, ddu);
        // acceleration one step further back: history slot j-2, or the block
        // start state for j = 1; none for j = 0
        const double *ddu2 = nullptr;
        if (use_pred2 && st->j >= 2)
            ddu2 = DDUh + (long long)(st->j - 2) * ndof;
        else if (use_pred2 && st->j == 1)
            ddu2 = cp + (long long)st->block * 3 * ndof + 2 * ndof;
        int t = st->tsc * st->block + st->j + 1;
        const double s = sig[t];
        uint8_t f = fixed[n];
        for (int c = 0; c < 3; c++) {
            bool fx = (f >> c) & 1;
            const double f2 = (3 * n + c == load2_dof) ? sig2[t] : 0.0;
            b[3 * n + c] = fx ? 0.0 : (rhs0[3 * n + c] * s + f2 + todbl(y[c]));
            double xv = pred[0] * u[3 * n + c] + pred[1] * du[3 * n + c];
            if (ddu2)
                xv += pred2[0] * ddu[3 * n + c] + pred2[1] * ddu2[3 * n + c];
            else
                xv += pred[2] * ddu[3 * n + c];
            x0[3 * n + c] = fx ? 0.0 : xv;
        }
    }
    __device__ void finish(const double *) const {}
};

}  // namespace topo
