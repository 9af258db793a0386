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

// The three axis passes stage whole grid lines in shared memory: each input
// value is read from global memory once per pass and the 17 taps read the
// staged line.  Pass outputs: out_q = sum_{|d| <= KRON_B} tap[pos][d] v_{pos+d}
// with indices past a line end clamped (their taps are zero).
struct KronDot {
    const float *q32;
    SolveScalars *S;
    Partials<2> part;
};

// x pass: KX_LINES x-lines (3 nx consecutive values each) per CTA.  The
// staged input is the masked, node-scaled residual t = S N r; in the mixed
// FCG the staging also re-forms r32 = sigma r after a residual replacement
// (S->rescale).
constexpr int KX_LINES = 4;
constexpr int KRON_THREADS = 256;

template <class T, class R>
static __global__ void __launch_bounds__(KRON_THREADS)
    k_kron_x(GridDesc g, const uint8_t *__restrict__ fixed, R *r, const double *__restrict__ r64,
             const SolveScalars *S, const T *__restrict__ scale, KronBand<T> B, T *out) {
    extern __shared__ __align__(16) unsigned char kron_smem[];
    T *tile = reinterpret_cast<T *>(kron_smem);  // [KX_LINES][3 nx]
    const int row = 3 * g.nx;
    const long long nlines = (long long)g.ny * g.nz;
    const long long line0 = (long long)blockIdx.x * KX_LINES;
    const int nl = (int)(nlines - line0 < KX_LINES ? nlines - line0 : KX_LINES);
    const bool rs = S != nullptr && S->rescale != 0;
    const double sg = rs ? S->sigma : 1.0;
    for (int t = threadIdx.x; t < nl * row; t += blockDim.x) {
        const int l = t / row, w = t - l * row, c = w % 3;
        const long long q = (line0 + l) * row + w;
        const long long n = (line0 + l) * g.nx + w / 3;
        R rv;
        if (rs) {
            rv = (R)(sg * r64[q]);
            r[q] = rv;
        } else {
            rv = r[q];
        }
        tile[t] = ((fixed[n] >> c) & 1) ? T(0) : (T)rv * scale[n];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nl * row; t += blockDim.x) {
        const int l = t / row, w = t - l * row, i = w / 3, c = w - 3 * i;
        const T *tap = B.row(0, c, i);
        const T *v = tile + l * row + c;
        T acc = T(0);
        if (i >= KRON_B && i < g.nx - KRON_B) {
#pragma unroll
            for (int d = -KRON_B; d <= KRON_B; d++) acc += tap[d + KRON_B] * v[3 * (i + d)];
        } else {
#pragma unroll
            for (int d = -KRON_B; d <= KRON_B; d++) {
                int p = i + d;
                p = p < 0 ? 0 : (p > g.nx - 1 ? g.nx - 1 : p);
                acc += tap[d + KRON_B] * v[3 * p];
            }
        }
        out[(line0 + l) * row + w] = acc;
    }
}

// y pass (AXIS 1) and z pass (AXIS 2): a CTA stages a chunk of KW values of
// one x-row (consecutive in memory) at every position along the line.  The
// z pass finishes P^-1: out = S x on free DOFs, r on clamped ones; with DOT it
// also forms the FCG dot products z.r and z.q of its output.
constexpr int KW = 32;

__host__ inline unsigned kron_yz_blocks(const GridDesc &g, int axis) {
    const int nchunk = (3 * g.nx + KW - 1) / KW;
    return (unsigned)nchunk * (unsigned)(axis == 1 ? g.nz : g.ny);
}

template <class T, class R, int AXIS, bool DOT>
static __global__ void __launch_bounds__(KRON_THREADS)
    k_kron_yz(GridDesc g, const uint8_t *__restrict__ fixed, const R *__restrict__ r, const T *__restrict__ scale,
              KronBand<T> B, const T *__restrict__ in, T *out, KronDot kd) {
    extern __shared__ __align__(16) unsigned char kron_smem[];
    T *tile = reinterpret_cast<T *>(kron_smem);  // [len][KW]
    const int row = 3 * g.nx;
    const int nchunk = (row + KW - 1) / KW;
    const int chunk = blockIdx.x % nchunk, other = blockIdx.x / nchunk;
    const int w0 = chunk * KW, wn = (row - w0 < KW) ? row - w0 : KW;
    const int len = AXIS == 1 ? g.ny : g.nz;
    const long long S = AXIS == 1 ? (long long)row : (long long)row * g.ny;
    const long long base = AXIS == 1 ? (long long)other * row * g.ny + w0 : (long long)other * row + w0;
    for (int t = threadIdx.x; t < len * KW; t += blockDim.x) {
        const int p = t / KW, w = t - p * KW;
        if (w < wn) tile[t] = in[base + p * S + w];
    }
    __syncthreads();
    double red[2] = {0.0, 0.0};
    for (int t = threadIdx.x; t < len * KW; t += blockDim.x) {
        const int p = t / KW, w = t - p * KW;
        if (w >= wn) continue;
        const int c = (w0 + w) % 3;
        const T *tap = B.row(AXIS, c, p);
        const T *v = tile + w;
        T acc = T(0);
        if (p >= KRON_B && p < len - KRON_B) {
#pragma unroll
            for (int d = -KRON_B; d <= KRON_B; d++) acc += tap[d + KRON_B] * v[(p + d) * KW];
        } else {
#pragma unroll
            for (int d = -KRON_B; d <= KRON_B; d++) {
                int pp = p + d;
                pp = pp < 0 ? 0 : (pp > len - 1 ? len - 1 : pp);
                acc += tap[d + KRON_B] * v[pp * KW];
            }
        }
        const long long q = base + p * S + w;
        if (AXIS == 2) {
            const long long n = q / 3;
            const T z = ((fixed[n] >> c) & 1) ? (T)r[q] : scale[n] * acc;
            out[q] = z;
            if (DOT) {
                red[0] += (double)((float)z * (float)r[q]);
                red[1] += (double)((float)z * kd.q32[q]);
            }
        } else {
            out[q] = acc;
        }
    }
    if constexpr (DOT) {
        double tot[2];
        if (grid_reduce<KRON_THREADS, 2>(red, kd.part, tot)) {
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
