// kernels.cuh -- element-wise, transfer, coarse-solve, Krylov-scalar,
// time-integration and sensitivity kernels of the transient path.
#pragma once
#include "policies.cuh"

namespace topo {

constexpr int EW = 256;  // threads of element-wise kernels

__host__ inline unsigned ew_blocks(long long n) {
    long long b = (n + EW - 1) / EW;
    return (unsigned)(b < 1 ? 1 : (b > 65535LL * 64 ? 65535LL * 64 : b));
}

// grid of the element-wise kernels that end in a grid reduction: a single
// wave of grid-stride CTAs (many short CTAs each doing a block reduction,
// fence and counter atomic are latency-bound)
__host__ inline unsigned red_blocks(long long n) {
    unsigned b = ew_blocks(n);
    return b < 608u ? b : 608u;
}

// Chebyshev coefficients (c1, c2) of steps k = 0..kmax-1 from the device-side
// spectrum bounds; computed once per design iteration so that no kernel
// repeats the FP64 divisions per thread
static __global__ void k_cheb_table(const double *lohi, int kmax, double *coef) {
    double c1, c2;
    for (int k = 0; k < kmax; k++) {
        cheb_coeffs<double>(lohi, k, c1, c2);
        coef[2 * k] = c1;
        coef[2 * k + 1] = c2;
    }
}

// ---------------------------------------------------------------------------
// material interpolation, InterpolateStiffness / InterpolateMass
// (LinearElasticity.cc:1580-1623)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void interp_dev(int type, double vmax, double vmin, double pen, double x, double &f,
                                           double &df) {
    if (type == 0) {
        f = vmin + x * (vmax - vmin);
        df = vmax - vmin;
    } else if (type == 1) {
        f = vmin + pow(x, pen) * (vmax - vmin);
        df = pen * pow(x, pen - 1) * (vmax - vmin);
    } else {
        f = vmin + x / (1 + pen * (1 - x)) * (vmax - vmin);
        double q = 1 + pen * (1 - x);
        df = (1 + pen) / (q * q) * (vmax - vmin);
    }
}

struct MatParams {
    int sInt, mInt;
    double Emin, Emax, penalK, Rmin, Rmax, penalM;
};

static __global__ void k_interp(long long nel, const double *__restrict__ x, MatParams mp, double *kf, double *dkf, double *mf,
                         double *dmf, float *kff, float *mff, df *kfx, df *mfx) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nel; e += (long long)gridDim.x * blockDim.x) {
        double k, dk, m, dm;
        interp_dev(mp.sInt, mp.Emax, mp.Emin, mp.penalK, x[e], k, dk);
        interp_dev(mp.mInt, mp.Rmax, mp.Rmin, mp.penalM, x[e], m, dm);
        kf[e] = k;
        dkf[e] = dk;
        mf[e] = m;
        dmf[e] = dm;
        kff[e] = (float)k;
        mff[e] = (float)m;
        kfx[e] = df(k);
        mfx[e] = df(m);
    }
}

// coarse element density factors: mean of the 8 children (rediscretised
// coarse operators of the geometric multigrid)
static __global__ void k_coarsen(GridDesc gf, GridDesc gc, const double *__restrict__ kf, const double *__restrict__ mf,
                          double *kc, double *mc, float *kcf, float *mcf) {
    long long nel = gc.nel();
    for (long long E = blockIdx.x * (long long)blockDim.x + threadIdx.x; E < nel; E += (long long)gridDim.x * blockDim.x) {
        int I = (int)(E % gc.ex), J = (int)((E / gc.ex) % gc.ey), K = (int)(E / ((long long)gc.ex * gc.ey));
        double sk = 0.0, sm = 0.0;
        for (int c = 0; c < 8; c++) {
            long long e = (2 * I + (c & 1)) + (long long)gf.ex * ((2 * J + ((c >> 1) & 1)) + (long long)gf.ey * (2 * K + (c >> 2)));
            sk += kf[e];
            sm += mf[e];
        }
        kc[E] = 0.125 * sk;
        mc[E] = 0.125 * sm;
        kcf[E] = (float)(0.125 * sk);
        mcf[E] = (float)(0.125 * sm);
    }
}

// inverse of the assembled diagonal of (N A N + I - N), A = sum_e (sK kf_e KE + sM mf_e ME)
static __global__ void k_dinv(GridDesc g, const uint8_t *__restrict__ fixed, const double *__restrict__ kf,
                       const double *__restrict__ mf, double sK, double sM, double dK0, double dK1, double dK2, double dM,
                       double *dinvd, float *dinvf) {
    long long nn = g.nn();
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        lex3(n, g.nx, g.ny, i, j, k);
        double sk = 0.0, sm = 0.0;
        for (int c = 0; c < 8; c++) {
            int ei = i - (c & 1), ej = j - ((c >> 1) & 1), ek = k - (c >> 2);
            if (ei < 0 || ej < 0 || ek < 0 || ei >= g.ex || ej >= g.ey || ek >= g.ez) continue;
            long long e = ei + (long long)g.ex * (ej + (long long)g.ey * ek);
            if (kf) sk += kf[e];
            sm += mf[e];
        }
        uint8_t f = fixed[n];
        const double dK[3] = {dK0, dK1, dK2};
        for (int c = 0; c < 3; c++) {
            double d = sK * sk * dK[c] + sM * sm * dM;
            double v = ((f >> c) & 1) ? 1.0 : 1.0 / d;
            dinvd[3 * n + c] = v;
            dinvf[3 * n + c] = (float)v;
        }
    }
}

// Spectrum bounds of Dinv A from the element-wise Rayleigh-quotient argument:
// x'Ax = sum_e x_e'(ck KE + cm ME)x_e <= sum_e sum_i x_ei^2 (ck lamK dK_i + cm lamM dM)
// so lambda_max(Dinv A) <= max_{e,i} (ck lamK dK_i + cm lamMhi dM)/(ck dK_i + cm dM),
// lambda_min(Dinv A) >= min_{e,i} cm lamMlo dM / (ck dK_i + cm dM)  (lamK_min = 0).
// The lower bound is negative for a negative mass coefficient (the shifted
// operator K - om^2 M), so the atomics act on an order-preserving image of the
// doubles (exact and order independent).
// order-preserving map of doubles to unsigned integers (negative values
// included), so that atomicMin / atomicMax on the image order like the values
__device__ __forceinline__ unsigned long long ord_bits(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_value(unsigned long long u) {
    const unsigned long long b = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
    return __longlong_as_double((long long)b);
}

static __global__ void k_bounds(long long nel, const double *__restrict__ kf, const double *__restrict__ mf, double sK,
                         double sM, double dK0, double dK1, double dK2, double dM, double lamK, double lamMlo,
                         double lamMhi, unsigned long long *bits /* [0]=max hi, [1]=min lo */) {
    double hi = 0.0, lo = 1e300;
    const double dK[3] = {dK0, dK1, dK2};
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nel; e += (long long)gridDim.x * blockDim.x) {
        double ck = kf ? sK * kf[e] : 0.0, cm = sM * mf[e];
        // a negative mass coefficient (the shifted operator K - om^2 M) takes
        // the mass bounds in the opposite order
        const double mhi = cm >= 0.0 ? lamMhi : lamMlo, mlo = cm >= 0.0 ? lamMlo : lamMhi;
        for (int c = 0; c < 3; c++) {
            double den = ck * dK[c] + cm * dM;
            if (den <= 0.0) continue;
            hi = fmax(hi, (ck * lamK * dK[c] + cm * mhi * dM) / den);
            lo = fmin(lo, (cm * mlo * dM) / den);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    }
    if ((threadIdx.x & 31) == 0) {  // lo is negative for the shifted operator K - om^2 M
        atomicMax(&bits[0], ord_bits(hi));
        atomicMin(&bits[1], ord_bits(lo));
    }
}

static __global__ void k_bounds_init(unsigned long long *bits) {
    bits[0] = ord_bits(0.0);
    bits[1] = ord_bits(1e300);
}

// Chebyshev interval: [max(lo_bound, hi/ratio), hi]; the Dirichlet identity
// rows contribute eigenvalue 1 and are kept inside the interval.
// lohi[0..1]: smoothing interval, lohi[2..3]: full-spectrum bounds
// lohi[4]: the element-wise lower bound itself.  A bound <= 0 (it cannot show
// the shifted operator K - om^2 M positive) keeps the level out of the
// well-conditioned test, and the full-spectrum table then uses the smoothing
// interval.
static __global__ void k_bounds_final(const unsigned long long *bits, double ratio, double *lohi) {
    double hi = ord_value(bits[0]);
    double lo = ord_value(bits[1]);
    hi = fmax(hi, 1.0);
    double l = fmax(lo, hi / ratio);
    l = fmin(l, 1.0);
    lohi[0] = l;
    lohi[1] = hi;
    lohi[2] = lo > 0.0 ? fmin(lo, 1.0) : l;
    lohi[3] = hi;
    lohi[4] = lo;
}

// first Chebyshev step from a zero initial guess: d = Dinv b / theta, x = d
template <class T>
static __global__ void k_cheb0(long long ndof, const T *__restrict__ b, const T *__restrict__ dinv, const double *coef,
                               T *x, T *d) {
    const T c2 = (T)coef[1];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x) {
        T v = c2 * dinv[i] * b[i];
        d[i] = v;
        x[i] = v;
    }
}

// The fine-level first Chebyshev step of the mixed-precision FCG.  After a
// residual replacement (S->rescale) the FP32 right-hand side is re-formed
// here as r32 = sigma r from the scaled FP64 residual before the step uses it.
static __global__ void k_cheb0_rescale(long long ndof, const double *__restrict__ r, float *b,
                                       const float *__restrict__ dinv, const double *coef, float *x, float *d,
                                       const SolveScalars *S) {
    const float c2 = (float)coef[1];
    const bool rs = S->rescale != 0;
    const ScaleF64 sg = scale_split(S->sigma);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x) {
        float bv;
        if (rs) {
            bv = scaled_f32(r[i], sg);
            b[i] = bv;
        } else {
            bv = b[i];
        }
        float v = c2 * dinv[i] * bv;
        d[i] = v;
        x[i] = v;
    }
}

// Restriction = transpose of trilinear prolongation (the DMDA Q1
// interpolation of DMCreateInterpolation, LinearElasticity.cc:2838-2842):
// coarse node gathers fine nodes 2I-1..2I+1 with weights 1/2, 1, 1/2 per axis.
template <class T>
static __global__ void k_restrict(GridDesc gf, GridDesc gc, const uint8_t *__restrict__ fixc, const T *__restrict__ rf, T *bc) {
    long long nn = gc.nn();
    for (long long N = blockIdx.x * (long long)blockDim.x + threadIdx.x; N < nn; N += (long long)gridDim.x * blockDim.x) {
        int I = (int)(N % gc.nx), J = (int)((N / gc.nx) % gc.ny), K = (int)(N / ((long long)gc.nx * gc.ny));
        T acc[3] = {T(0), T(0), T(0)};
        for (int dk = -1; dk <= 1; dk++) {
            int k = 2 * K + dk;
            if (k < 0 || k >= gf.nz) continue;
            T wk = dk ? T(0.5) : T(1);
            for (int dj = -1; dj <= 1; dj++) {
                int j = 2 * J + dj;
                if (j < 0 || j >= gf.ny) continue;
                T wj = wk * (dj ? T(0.5) : T(1));
                for (int di = -1; di <= 1; di++) {
                    int i = 2 * I + di;
                    if (i < 0 || i >= gf.nx) continue;
                    T w = wj * (di ? T(0.5) : T(1));
                    long long n = i + (long long)gf.nx * (j + (long long)gf.ny * k);
                    acc[0] += w * rf[3 * n];
                    acc[1] += w * rf[3 * n + 1];
                    acc[2] += w * rf[3 * n + 2];
                }
            }
        }
        mask3(fixc[N], acc);
        bc[3 * N] = acc[0];
        bc[3 * N + 1] = acc[1];
        bc[3 * N + 2] = acc[2];
    }
}

// x_f += P x_c (trilinear), clamped DOFs untouched
template <class T>
static __global__ void k_prolong(GridDesc gf, GridDesc gc, const uint8_t *__restrict__ fixf, const T *__restrict__ xc, T *xf) {
    long long nn = gf.nn();
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        int i = (int)(n % gf.nx), j = (int)((n / gf.nx) % gf.ny), k = (int)(n / ((long long)gf.nx * gf.ny));
        int I0 = i >> 1, J0 = j >> 1, K0 = k >> 1;
        int I1 = I0 + (i & 1), J1 = J0 + (j & 1), K1 = K0 + (k & 1);
        T acc[3] = {T(0), T(0), T(0)};
        for (int c = 0; c < 8; c++) {
            int I = (c & 1) ? I1 : I0, J = ((c >> 1) & 1) ? J1 : J0, K = (c >> 2) ? K1 : K0;
            // duplicate corners (even index) carry weight 1 split over the two equal picks
            T w = T(0.125);
            long long N = I + (long long)gc.nx * (J + (long long)gc.ny * K);
            acc[0] += w * xc[3 * N];
            acc[1] += w * xc[3 * N + 1];
            acc[2] += w * xc[3 * N + 2];
        }
        uint8_t f = fixf[n];
        for (int c = 0; c < 3; c++)
            if (!((f >> c) & 1)) xf[3 * n + c] += acc[c];
    }
}

// y = A x for the explicit coarse inverse (one warp per row)
template <class T>
static __global__ void k_gemv(int n, const T *__restrict__ A, const T *__restrict__ x, T *y) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    const T *row = A + (size_t)warp * n;
    T acc = T(0);
    for (int j = lane; j < n; j += 32) acc += row[j] * x[j];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[warp] = acc;
}

// dense coarsest-level operator, one thread per entry: sum over the (at most 8)
// elements shared by the two nodes, fixed order (deterministic).  Element
// matrices KE/ME are the 24x24 box matrices in lexicographic local order.
static __global__ void k_coarse_assemble(GridDesc g, const uint8_t *__restrict__ fixed, const double *__restrict__ kf,
                                  const double *__restrict__ mf, double sK, double sM, const double *__restrict__ KE,
                                  const double *__restrict__ ME, double *A) {
    long long nd = 3 * g.nn();
    long long tot = nd * nd;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
        long long r = t / nd, s = t % nd;
        long long nr = r / 3, ns = s / 3;
        int cr = (int)(r % 3), cs = (int)(s % 3);
        int ir, jr, kr;
        lex3(nr, g.nx, g.ny, ir, jr, kr);
        int is, js, ks;
        lex3(ns, g.nx, g.ny, is, js, ks);
        bool fr = (fixed[nr] >> cr) & 1, fs = (fixed[ns] >> cs) & 1;
        double v = 0.0;
        if (fr || fs) {
            v = (r == s) ? 1.0 : 0.0;
        } else if (abs(ir - is) <= 1 && abs(jr - js) <= 1 && abs(kr - ks) <= 1) {
            for (int c = 0; c < 8; c++) {
                int ei = ir - (c & 1), ej = jr - ((c >> 1) & 1), ek = kr - (c >> 2);
                if (ei < 0 || ej < 0 || ek < 0 || ei >= g.ex || ej >= g.ey || ek >= g.ez) continue;
                int ax = is - ei, ay = js - ej, az = ks - ek;
                if (ax < 0 || ax > 1 || ay < 0 || ay > 1 || az < 0 || az > 1) continue;
                int La = c, Lb = ax + 2 * ay + 4 * az;
                long long e = ei + (long long)g.ex * (ej + (long long)g.ey * ek);
                int ia = 3 * La + cr, ib = 3 * Lb + cs;
                double ck = kf ? sK * kf[e] : 0.0, cm = sM * mf[e];
                v += ck * KE[ia * 24 + ib] + cm * ME[ia * 24 + ib];
            }
        }
        A[t] = v;
    }
}

// Dense coarsest-level operator (SPD, FP64).  Cholesky factor A = L L' in
// place in the lower triangle, right-looking, one column per step in two
// passes: the updated column k is saved (k_chol_save), then scaled into
// L(:, k) and the trailing lower triangle updated, A(i, j) -= L(i, k) L(j, k)
// (k_chol_update).  Then W = L^-1 by forward substitution (row i of W scaled
// by 1 / L(i, i), then subtracted from the rows below) and A^-1 = W' W, so the
// V-cycle's coarse solve stays one dense matrix-vector product.
static __global__ void k_chol_save(const double *A, int n, int k, double *col) {
    for (int t = k + blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        col[t] = A[(size_t)t * n + k];
}
static __global__ void k_chol_update(double *A, int n, int k, const double *__restrict__ col) {
    const long long m = n - k;
    const double p = col[k], d = sqrt(p);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < m * m; t += (long long)gridDim.x * blockDim.x) {
        const int i = k + (int)(t / m), j = k + (int)(t % m);
        if (j > i) continue;
        double &a = A[(size_t)i * n + j];
        if (j == k)
            a = (i == k) ? d : col[i] / d;
        else
            a -= (col[i] / p) * col[j];  // L(i, k) L(j, k) = col_i col_j / col_k
    }
}
static __global__ void k_chol_identity(double *W, int n) {
    const long long tot = (long long)n * n;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x)
        W[t] = (t / n == t % n) ? 1.0 : 0.0;
}
// forward substitution step i: row i of W (columns <= i) divided by L(i, i)
static __global__ void k_chol_trsv_scale(const double *L, double *W, int n, int i) {
    const double d = L[(size_t)i * n + i];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c <= i; c += gridDim.x * blockDim.x) W[(size_t)i * n + c] /= d;
}
// rows r > i of W (columns <= i) minus L(r, i) times row i
static __global__ void k_chol_trsv_update(const double *L, double *W, int n, int i) {
    const long long w = i + 1, tot = (long long)(n - i - 1) * w;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
        const int r = i + 1 + (int)(t / w), c = (int)(t % w);
        W[(size_t)r * n + c] -= L[(size_t)r * n + i] * W[(size_t)i * n + c];
    }
}
// A^-1 = W' W with W = L^-1 lower triangular: Ainv(i, j) = sum over r >= max(i, j) of W(r, i) W(r, j)
static __global__ void k_chol_gram(const double *__restrict__ W, int n, double *Ainv) {
    const long long tot = (long long)n * n;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t / n), j = (int)(t % n);
        double s = 0.0;
        for (int r = i > j ? i : j; r < n; r++) s += W[(size_t)r * n + i] * W[(size_t)r * n + j];
        Ainv[t] = s;
    }
}

static __global__ void k_d2f(long long n, const double *__restrict__ a, float *b) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

static __global__ void k_copy(long long n, const double *__restrict__ a, double *b) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = a[i];
}

// ---------------------------------------------------------------------------
// flexible CG (Notay's FCG(1)): p_{k+1} = z_{k+1} - (z_{k+1}.q_k / p_k.q_k) p_k
// ---------------------------------------------------------------------------
template <class TZ>
static __global__ void k_fcg_dot(long long ndof, const TZ *__restrict__ z, const double *__restrict__ r,
                          const double *__restrict__ q, SolveScalars *S, Partials<2> part) {
    double v[2] = {0.0, 0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x) {
        double zi = (double)z[i];
        v[0] += zi * r[i];
        v[1] += zi * q[i];
    }
    double tot[2];
    if (grid_reduce<EW, 2>(v, part, tot)) {
        S->rho = tot[0];
        S->gam = tot[1];
        S->beta = (S->it == 0) ? 0.0 : -tot[1] / S->pq;
        if (!isfinite(tot[0])) {
            S->status = TOPO_ERR_NAN;
            S->done = 1;
        }
    }
}

template <class TZ>
static __global__ void k_fcg_p(long long ndof, const TZ *__restrict__ z, double *p, const SolveScalars *S) {
    double beta = S->beta;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x)
        p[i] = (beta == 0.0) ? (double)z[i] : (double)z[i] + beta * p[i];
}

static __global__ void k_fcg_update(long long ndof, double *x, double *r, float *r32, const double *__restrict__ p,
                             const double *__restrict__ q, SolveScalars *S, Partials<1> part,
                             cudaGraphConditionalHandle cond, int has_cond) {
    double alpha = S->alpha;
    double v[1] = {0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        double rv = r[i] - alpha * q[i];
        r[i] = rv;
        if (r32) r32[i] = (float)rv;
        v[0] += rv * rv;
    }
    double tot[1];
    if (grid_reduce<EW, 1>(v, part, tot)) {
        S->rr = tot[0];
        S->it += 1;
        S->total_it += 1;
        S->rho_old = S->rho;
        if (!isfinite(tot[0])) {
            S->status = TOPO_ERR_NAN;
            S->done = 1;
        } else if (tot[0] <= S->tol2 * S->bb) {
            S->done = 1;
        } else if (S->it >= S->maxit) {
            S->status = TOPO_ERR_NOT_CONVERGED;
            S->done = 1;
        }
        if (has_cond) cudaGraphSetConditional(cond, S->done ? 0u : 1u);
    }
}

// mixed-precision FCG pieces (FP32 vectors, FP64 scalars and iterate)
// r32 = sigma * r after an FP64 residual (init or replacement)
static __global__ void k_mfcg_scale(long long ndof, const double *__restrict__ r, float *r32, const SolveScalars *S) {
    if (!S->rescale) return;
    const ScaleF64 sg = scale_split(S->sigma);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x)
        r32[i] = scaled_f32(r[i], sg);
}

static __global__ void k_mfcg_dot(long long ndof, const float *__restrict__ z, const float *__restrict__ r32,
                                  const float *__restrict__ q32, SolveScalars *S, Partials<2> part) {
    float s0 = 0.0f, s1 = 0.0f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x) {
        float zi = z[i];
        s0 += zi * r32[i];
        s1 += zi * q32[i];
    }
    const float v[2] = {s0, s1};
    double tot[2];
    if (grid_reduce<EW, 2>(v, part, tot)) {
        S->rho = tot[0];
        S->gam = tot[1];
        S->beta = S->restart ? 0.0 : -tot[1] / S->pq;
        if (!isfinite(S->beta)) S->beta = 0.0;
        S->beta32 = (float)S->beta;
        S->rescale = 0;
    }
}

// p is double-buffered (PolPQ32 reads the previous p from pb[it & 1] and
// writes the new one to pb[(it + 1) & 1])
static __global__ void k_mfcg_update(long long ndof, double *__restrict__ x, float *__restrict__ r32,
                                     const float *pb0, const float *pb1, const float *__restrict__ q, SolveScalars *S,
                                     Partials<1> part) {
    const float *__restrict__ p = ((S->it + 1) & 1) ? pb1 : pb0;
    // alpha in FP32 and in unscaled units, formed once by PolPQ32 (an FP64
    // division per thread would cost more FP64-pipe time than the x update)
    const float af = S->alpha32;
    const double ax = S->alpha_x;
    float s = 0.0f;
    // four grid strides per trip: all loads of a trip are issued before its stores
    const long long st = (long long)gridDim.x * blockDim.x;
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; i + 3 * st < ndof; i += 4 * st) {
        double xv[4];
        float pv[4], rv[4], qv[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            xv[u] = x[i + u * st];
            pv[u] = p[i + u * st];
            rv[u] = r32[i + u * st];
            qv[u] = q[i + u * st];
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            x[i + u * st] = fma(ax, f32_to_f64(pv[u]), xv[u]);
            const float r = rv[u] - af * qv[u];
            r32[i + u * st] = r;
            s += r * r;
        }
    }
    for (; i < ndof; i += st) {
        x[i] = fma(ax, f32_to_f64(p[i]), x[i]);
        float rv = r32[i] - af * q[i];
        r32[i] = rv;
        s += rv * rv;
    }
    const float v[1] = {s};
    double tot[1];
    if (grid_reduce<EW, 1>(v, part, tot)) {
        S->it += 1;
        S->total_it += 1;
        S->inner_it += 1;
        S->restart = 0;
        // replace when the recurrence residual has dropped by inner_tol, or
        // when it says the solve has converged (the replacement then checks
        // that on the true residual)
        const double est = tot[0] / (S->sigma * S->sigma);
        if (!isfinite(tot[0]) || tot[0] <= S->tau2 * S->rr_ref || est <= S->tol2 * S->bb || S->inner_it >= S->kmax ||
            S->it >= S->maxit)
            S->need_replace = 1;
    }
}

// almost always a no-op (the solve zeroes x only for a zero right-hand side):
// launched as one wave of grid-stride CTAs, so the check costs one wave
static __global__ void k_fcg_zero_x(long long ndof, double *x, const SolveScalars *S) {
    if (!S->zero_x) return;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x)
        x[i] = 0.0;
}

// ---------------------------------------------------------------------------
// Newmark corrector (SolveStateBlock, LinearElasticity.cc:1363-1375):
//   du = a0 du- + a1 ddu- + a2 (u - u-),  ddu = -a3 du- - a4 ddu- + a5 (u - u-)
// writes step j of the block history
// ---------------------------------------------------------------------------
struct Newmark {
    double a[6];
    df da[6];  // the same as double-float pairs (k_newmark_track)
};

static __global__ void k_newmark(long long ndof, const double *__restrict__ x, const StepCtx *st, const double *cp, double *Uh,
                          double *DUh, double *DDUh, Newmark nm) {
    int j = st->j;
    const double *u, *du, *ddu;
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
    double *uo = Uh + (long long)j * ndof, *duo = DUh + (long long)j * ndof, *dduo = DDUh + (long long)j * ndof;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x) {
        double un = x[i], dU = un - u[i];
        uo[i] = un;
        duo[i] = nm.a[0] * du[i] + nm.a[1] * ddu[i] + nm.a[2] * dU;
        dduo[i] = -nm.a[3] * du[i] - nm.a[4] * ddu[i] + nm.a[5] * dU;
    }
}

// ---------------------------------------------------------------------------
// Mixed forward sweep: tracked products and next-step preparation.
// With A = sK K + sM M the step operator and s = (u, du, ddu) a state, the
// tracked products T = (A u, A du, A ddu) give the next step's
//   KS = sum_i c'_i s_i              (the only operator input: b needs K KS)
//   BT = sum_i cA_i T_i              (b = f + BT + K KS)
//   X0 = predictor . s,  AX = predictor . T   (r0 = b - AX)
// (c'_i = cK_i - cM_i sK/sM, cA_i = cM_i/sM; SolveStateBlock,
// LinearElasticity.cc:1317-1361).  X0, BT and AX are written into the solver
// vectors x, b and r of the next solve, which reads them in its first pass.
// ---------------------------------------------------------------------------
struct FwdPrep {
    double ck[3], cA[3];   // c'_i and cA_i
    double pred[3];        // predictor u + pred1 du + pred2 ddu (no older acceleration)
    double pred2[2];       // with ddu--: u + pred1 du + pred2[0] ddu + pred2[1] ddu--
    int use_pred2;
    double *KS, *X0, *BT, *AX;
    // the coefficients as double-float pairs, split on the host
    df dck[3], dcA[3], dpred[3], dpred2[2];
};
// in double-float arithmetic (FP32 pipes): GB300 runs FP64 at about two FMAs
// per clock and SM, and the FP64 form of these combinations set the time of
// the kernels that call this; one FP64 addition per output joins hi + lo
__device__ __forceinline__ void fwd_prep(long long i, df u, df du, df ddu, df ddu_prev, bool has_prev, df au, df av,
                                         df aa, df aa_prev, const FwdPrep &P) {
    P.KS[i] = todbl(P.dck[0] * u + P.dck[1] * du + P.dck[2] * ddu);
    P.BT[i] = todbl(P.dcA[0] * au + P.dcA[1] * av + P.dcA[2] * aa);
    // the predictor's coefficient of u is 1 (fwd_prep_args)
    df x = P.dpred[1] * du + u, ax = P.dpred[1] * av + au;
    if (has_prev && P.use_pred2) {
        x += P.dpred2[0] * ddu + P.dpred2[1] * ddu_prev;
        ax += P.dpred2[0] * aa + P.dpred2[1] * aa_prev;
    } else {
        x += P.dpred[2] * ddu;
        ax += P.dpred[2] * aa;
    }
    P.X0[i] = todbl(x);
    P.AX[i] = todbl(ax);
}

// after a forward solve (Newmark corrector, LinearElasticity.cc:1363-1375):
// the new state into history slot j; the tracked products of the new state,
// A u = b - r (the solve's final, FP64-accurate residual; 0 when the solve
// zeroed x), A du and A ddu by the same linear corrector; then the next
// step's KS, X0 (into x), BT (into b) and AX (into r).
// The differences that cancel (u+ - u, b - r, A u+ - A u) are formed in FP64;
// the combinations run in double-float arithmetic on the FP32 pipes, with the
// FP64 inputs split on the integer pipes (f64_to_df) and one FP64 addition
// per output: GB300 issues about two FP64 FMAs per clock and SM, and the
// all-FP64 form (23 FP64 operations per DOF) was bound by that rate at
// about twice its DRAM time.
// STD: Newmark beta = 1/4, gamma = 1/2 (a0 = -1, a1 = 0).
template <bool STD>
static __global__ void __launch_bounds__(EW, 4) k_newmark_track(long long ndof, double *x, const StepCtx *st, const double *cp, double *Uh,
                                       double *DUh, double *DDUh, Newmark nm, double *b, double *r,
                                       const SolveScalars *S, double *AU, double *AV, double *AA, FwdPrep P) {
    const int j = st->j;
    const double *u, *du, *ddu;
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
    double *uo = Uh + (long long)j * ndof, *duo = DUh + (long long)j * ndof, *dduo = DDUh + (long long)j * ndof;
    const bool zx = S->zero_x != 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x) {
        // every input is loaded before the first store: the outputs may alias
        // the inputs as far as the compiler knows, so a load after a store
        // would wait for a second memory round trip (the kernel is bound by
        // load latency, not by bandwidth)
        const double un64 = x[i], u64 = u[i], du64 = du[i], ddu64 = ddu[i];
        const double b64 = b[i], r64 = r[i], au64 = AU[i], av64 = AV[i], aa64 = AA[i];
        const df un(un64), dU(un64 - u64), dup(du64), ddup(ddu64);
        const df dun = STD ? nm.da[2] * dU - dup : nm.da[0] * dup + nm.da[1] * ddup + nm.da[2] * dU;
        const df ddun = nm.da[5] * dU - nm.da[3] * dup - nm.da[4] * ddup;
        uo[i] = un64;
        duo[i] = todbl(dun);
        dduo[i] = todbl(ddun);
        const double aun64 = zx ? 0.0 : b64 - r64;
        const df aun(aun64), d(aun64 - au64), av(av64), aa(aa64);
        const df avn = STD ? nm.da[2] * d - av : nm.da[0] * av + nm.da[1] * aa + nm.da[2] * d;
        const df aan = nm.da[5] * d - nm.da[3] * av - nm.da[4] * aa;
        AU[i] = aun64;
        AV[i] = todbl(avn);
        AA[i] = todbl(aan);
        fwd_prep(i, un, dun, ddun, ddup, true, aun, avn, aan, aa, P);
    }
}

// next-step preparation from given states and tracked products (block start:
// no older acceleration; re-anchoring: ddu_prev and A ddu_prev given)
static __global__ void k_fwd_prep(long long ndof, const double *__restrict__ u, const double *__restrict__ du,
                                  const double *__restrict__ ddu, const double *__restrict__ ddu_prev,
                                  const double *__restrict__ AU, const double *__restrict__ AV,
                                  const double *__restrict__ AA, const double *__restrict__ AAprev, FwdPrep P) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x)
        fwd_prep(i, df(u[i]), df(du[i]), df(ddu[i]), df(ddu_prev ? ddu_prev[i] : 0.0), ddu_prev != nullptr,
                 df(AU[i]), df(AV[i]), df(AA[i]), df(AAprev ? AAprev[i] : 0.0), P);
}

// Mixed forward step, after the K-only double-float product y = K KS:
// b = f(t) + BT + y and r0 = b - A x0 on free DOFs (0 on clamped ones), b.b,
// r.r and the FCG set-up; BT arrives in b and A x0 in r (k_newmark_track /
// k_fwd_prep).  x0 is never accepted without a true residual: A u+ = b - r
// must hold for the stored u+ and r0 rests on tracked products.  A streaming
// kernel at full occupancy: the tile kernel's epilogue runs one CTA per SM in
// double-float (SolveStateBlock, LinearElasticity.cc:1317-1361).
struct RhsLoad {
    const double *rhs0;
    const double *sig, *sig2;  // per-step load signals (k_load_table)
    long long load2_dof;
};
static __global__ void __launch_bounds__(EW, 4) k_rhs_finish(long long ndof, const uint8_t *__restrict__ fixed, const double *__restrict__ y,
                                    RhsLoad L, const StepCtx *st, double *__restrict__ b, double *__restrict__ r,
                                    SolveScalars *S, cudaGraphConditionalHandle cond, int has_cond, Partials<2> part) {
    const int t = st->tsc * st->block + st->j + 1;
    const double s = L.sig[t];
    double red[2] = {0.0, 0.0};
    // the load terms are nonzero on a few DOFs only: tested on the bit
    // patterns (integer pipes), formed in FP64 where present
    auto one = [&](long long i, uint8_t f, double bi, double yi, double f0, double ri) {
        const int c = (int)(i % 3);
        if ((f >> c) & 1) {
            b[i] = 0.0;
            r[i] = 0.0;
            return;
        }
        double bv = bi + yi;
        if (__double_as_longlong(f0) << 1) bv += f0 * s;
        if (i == L.load2_dof) bv += L.sig2[t];
        const double rv = bv - ri;
        b[i] = bv;
        r[i] = rv;
        red[0] += bv * bv;
        red[1] += rv * rv;
    };
    // four grid strides per trip: all loads of a trip are issued before the
    // FP64 reductions that depend on them
    const long long gs = (long long)gridDim.x * blockDim.x;
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; i + 3 * gs < ndof; i += 4 * gs) {
        uint8_t f[4];
        double bi[4], yi[4], fi[4], ri[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const long long k = i + u * gs;
            f[u] = fixed[k / 3];
            bi[u] = b[k];
            yi[u] = y[k];
            fi[u] = L.rhs0[k];
            ri[u] = r[k];
        }
#pragma unroll
        for (int u = 0; u < 4; u++) one(i + u * gs, f[u], bi[u], yi[u], fi[u], ri[u]);
    }
    for (; i < ndof; i += gs) one(i, fixed[i / 3], b[i], y[i], L.rhs0[i], r[i]);
    double tot[2];
    if (grid_reduce<EW, 2>(red, part, tot)) init_finish(S, tot, true, cond, has_cond, false);
}

static __global__ void k_step_set(StepCtx *st, int block, int j) {
    st->block = block;
    st->j = j;
}
static __global__ void k_step_add(StepCtx *st, int delta) {
    st->j += delta;
    if (delta < 0) st->nadj += 1;
}

}  // namespace topo
