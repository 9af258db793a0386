// kron.cuh -- Kronecker (tensor-product) mass preconditioner.
//
// On a box grid the consistent hex8 mass of a uniform density is exactly a
// Kronecker product of 1-D assembled masses,
//   M_unit = Tx (x) Ty (x) Tz,   T = assembled h/6 [2 1; 1 2] (tridiagonal),
// so its inverse is three sweeps of independent tridiagonal solves, one along
// every grid line of each axis.  The Newmark effective operator of the
// transient path, Keff = sK K(kf) + sM M(mf), is dominated by its mass part
// whenever sK kf / (sM mf) times the largest generalized eigenvalue of the
// element pair (KE, ME) is small -- the case for the time steps of the
// transient cantilever workloads -- and then
//   P^-1 = N S (Tx^-1 (x) Ty^-1 (x) Tz^-1) S N + (I - N),
//   S = diag(1 / sqrt(sM w_n)),  w_n = mean mass factor of the elements at n,
// is an accurate preconditioner for the masked operator N Keff N + I - N
// (exact for the mass part of a uniform design).  Dirichlet planes that clamp
// a component on a whole face decouple the end node of that component's 1-D
// factor; other clamped DOFs are handled by the masking N alone.
//
// The 1-D inverses are formed on the host (Thomas elimination of the
// tridiagonal T for every unit vector) and applied as banded rows below.
#pragma once
#include "kernels.cuh"

namespace topo {

// node scaling s_n = 1 / sqrt(sM * mean_{e at n} mf_e)
template <class T>
static __global__ void k_kron_scale(GridDesc g, const double *__restrict__ mf, double sM, T *scale) {
    long long nn = g.nn();
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        int i = (int)(n % g.nx), j = (int)((n / g.nx) % g.ny), k = (int)(n / ((long long)g.nx * g.ny));
        double s = 0.0;
        int cnt = 0;
        for (int c = 0; c < 8; c++) {
            int ei = i - (c & 1), ej = j - ((c >> 1) & 1), ek = k - (c >> 2);
            if (ei < 0 || ej < 0 || ek < 0 || ei >= g.ex || ej >= g.ey || ek >= g.ez) continue;
            s += mf[ei + (long long)g.ex * (ej + (long long)g.ey * ek)];
            cnt++;
        }
        double w = sM * s / (double)(cnt > 0 ? cnt : 1);
        scale[n] = (T)(w > 0.0 ? 1.0 / sqrt(w) : 0.0);
    }
}

// max_e kf_e / mf_e (positive doubles: their bit patterns order like unsigned)
static __global__ void k_ratio_max(long long nel, const double *__restrict__ kf, const double *__restrict__ mf,
                                   unsigned long long *bits) {
    double m = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nel; e += (long long)gridDim.x * blockDim.x)
        if (mf[e] > 0.0) m = fmax(m, kf[e] / mf[e]);
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(bits, (unsigned long long)__double_as_longlong(m));
}

// Banded application of the 1-D inverses.  T^-1 of the 1-D mass decays like
// (2 - sqrt(3))^|i-j| = 0.268^|i-j| away from the diagonal, so each axis pass
// applies the exact inverse rows truncated to |i - j| <= KRON_B (truncation
// 0.268^9 < 1e-5 relative, well below the error of the density scaling): a
// 17-tap stencil along that axis with position dependent taps, data-parallel
// over all DOFs.  Tap table per axis a and component c: [a][c][n_a][2 KRON_B + 1].
constexpr int KRON_B = 8;
constexpr int KRON_W = 2 * KRON_B + 1;

template <class T>
struct KronBand {
    const T *t;  // [3][3][nmax][KRON_W]
    int nmax;
    __device__ __forceinline__ const T *row(int a, int c, int i) const {
        return t + (((size_t)(a * 3 + c) * nmax) + i) * KRON_W;
    }
};

// t = S N r (masked, node-scaled input of the x pass).  In the mixed FCG it
// also re-forms r32 = sigma r after a residual replacement (S->rescale).
template <class T, class R>
static __global__ void __launch_bounds__(256) k_kron_prep(GridDesc g, const uint8_t *__restrict__ fixed, R *r,
                                                          const double *__restrict__ r64, const SolveScalars *S,
                                                          const T *__restrict__ scale, T *t) {
    const unsigned nd = 3u * (unsigned)g.nn();
    const unsigned q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nd) return;
    const unsigned n = q / 3u, c = q - 3u * n;
    R rv;
    if (S && S->rescale) {
        rv = (R)(S->sigma * r64[q]);
        r[q] = rv;
    } else {
        rv = r[q];
    }
    t[q] = ((fixed[n] >> c) & 1) ? T(0) : (T)rv * scale[n];
}

// one axis pass: out_q = sum_{|d| <= KRON_B} tap[pos][d] in_{q + d stride},
// flat grid over the 3 nn DOFs (32-bit index arithmetic: 3 nn < 2^32).
// Positions at least KRON_B from both ends read their taps' inputs directly;
// the others clamp indices past the line end (their taps are zero).  AXIS 2
// finishes P^-1: out = S x on free DOFs, r on clamped ones; with DOT it also
// forms the FCG dot products z.r and z.q of its output (the role of
// k_mfcg_dot).
struct KronDot {
    const float *q32;
    SolveScalars *S;
    Partials<2> part;
};

template <class T, class R, int AXIS, bool DOT>
static __global__ void __launch_bounds__(256) k_kron_pass(GridDesc g, const uint8_t *__restrict__ fixed,
                                                          const R *__restrict__ r, const T *__restrict__ scale,
                                                          KronBand<T> B, const T *__restrict__ in, T *out, KronDot kd) {
    const unsigned nd = 3u * (unsigned)g.nn();
    const unsigned q = blockIdx.x * blockDim.x + threadIdx.x;
    double red[2] = {0.0, 0.0};
    if (q < nd) {
        const unsigned n = q / 3u, c = q - 3u * n;
        const unsigned nx = (unsigned)g.nx, nxy = nx * (unsigned)g.ny;
        const unsigned k = n / nxy, rem = n - k * nxy, j = rem / nx, i = rem - j * nx;
        const int pos = AXIS == 0 ? (int)i : (AXIS == 1 ? (int)j : (int)k);
        const int len = AXIS == 0 ? g.nx : (AXIS == 1 ? g.ny : g.nz);
        const int stride = AXIS == 0 ? 3 : (AXIS == 1 ? 3 * (int)nx : 3 * (int)nxy);
        const T *tap = B.row(AXIS, (int)c, pos);
        const T *src = in + q;
        T acc = T(0);
        if (pos >= KRON_B && pos < len - KRON_B) {
#pragma unroll
            for (int d = -KRON_B; d <= KRON_B; d++) acc += tap[d + KRON_B] * src[d * stride];
        } else {
#pragma unroll
            for (int d = -KRON_B; d <= KRON_B; d++) {
                int p = pos + d;
                p = p < 0 ? 0 : (p > len - 1 ? len - 1 : p);
                acc += tap[d + KRON_B] * src[(p - pos) * stride];
            }
        }
        if (AXIS == 2) {
            const bool fx = (fixed[n] >> c) & 1;
            const T z = fx ? (T)r[q] : scale[n] * acc;
            out[q] = z;
            if (DOT) {
                red[0] = (double)((float)z * (float)r[q]);
                red[1] = (double)((float)z * kd.q32[q]);
            }
        } else {
            out[q] = acc;
        }
    }
    if constexpr (DOT) {
        double tot[2];
        if (grid_reduce<256, 2>(red, kd.part, tot)) {
            SolveScalars *S = kd.S;
            S->rho = tot[0];
            S->gam = tot[1];
            S->beta = S->restart ? 0.0 : -tot[1] / S->pq;
            if (!isfinite(S->beta)) S->beta = 0.0;
            S->rescale = 0;
        }
    }
}

}  // namespace topo
