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

// masked node scaling per DOF: ms[3n + c] = 1 / sqrt(sM * mean_{e at n} mf_e)
// on free DOFs and -1 on clamped ones (the mask N and the scaling S of P^-1
// in one array laid out like the residual)
template <class T>
static __global__ void k_kron_scale(GridDesc g, const uint8_t *__restrict__ fixed, const double *__restrict__ mf,
                                    double sM, T *ms) {
    long long nn = g.nn();
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        lex3(n, g.nx, g.ny, i, j, k);
        double s = 0.0;
        int cnt = 0;
        for (int c = 0; c < 8; c++) {
            int ei = i - (c & 1), ej = j - ((c >> 1) & 1), ek = k - (c >> 2);
            if (ei < 0 || ej < 0 || ek < 0 || ei >= g.ex || ej >= g.ey || ek >= g.ez) continue;
            s += mf[ei + (long long)g.ex * (ej + (long long)g.ey * ek)];
            cnt++;
        }
        double w = sM * s / (double)(cnt > 0 ? cnt : 1);
        const T sc = (T)(w > 0.0 ? 1.0 / sqrt(w) : 0.0);
        const uint8_t f = fixed[n];
        for (int c = 0; c < 3; c++) ms[3 * n + c] = ((f >> c) & 1) ? T(-1) : sc;
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
// value is read from global memory once per pass, with every load of a
// thread issued before the CTA's barrier.  A thread computes KRON_MP
// consecutive outputs of one line from a register window of KRON_MP + 2 KRON_B
// staged values (3 shared-memory reads per output instead of 17).  Positions
// at least KRON_B from both line ends use the interior taps, staged once per
// CTA (the interior rows of the exact inverse agree with them to
// 0.268^(2 KRON_B) relative) and held in registers for a group of interior
// outputs; the others use their exact rows, which are zero past the line end,
// so the window clamps indices there.
struct KronDot {
    const float *q32;
    SolveScalars *S;
    Partials<2> part;
};

constexpr int KRON_THREADS = 256;
constexpr size_t KRON_SMEM_MAX = 200 * 1024;    // per-CTA staging limit (the selection checks it)
constexpr int KRON_MP = 8;                      // outputs per thread along a line
constexpr int KRON_WIN = KRON_MP + 2 * KRON_B;  // register window

// interior taps of one axis for the three components: the exact row at the
// middle of the line (lines shorter than 2 KRON_B + 1 have no interior)
template <class T>
__device__ __forceinline__ void kron_stage_interior(const KronBand<T> &B, int axis, int len, T *tint) {
    for (int t = threadIdx.x; t < 3 * KRON_W; t += blockDim.x) {
        const int c = t / KRON_W, d = t - c * KRON_W;
        tint[t] = B.row(axis, c, len / 2)[d];
    }
}

// KRON_MP outputs at positions p0.. of a staged line (value at position p is
// src[p * sstride]); outputs past the line end are computed but not used
template <class T>
__device__ __forceinline__ void kron_line(const T *src, int sstride, int len, int p0, const T *tint,
                                          const KronBand<T> &B, int axis, int c, T out[KRON_MP]) {
    T win[KRON_WIN];
#pragma unroll
    for (int k = 0; k < KRON_WIN; k++) {
        int p = p0 - KRON_B + k;
        p = p < 0 ? 0 : (p > len - 1 ? len - 1 : p);
        win[k] = src[p * sstride];
    }
    if (p0 >= KRON_B && p0 + KRON_MP <= len - KRON_B) {  // interior group: taps in registers
        T tap[KRON_W];
#pragma unroll
        for (int d = 0; d < KRON_W; d++) tap[d] = tint[c * KRON_W + d];
#pragma unroll
        for (int k = 0; k < KRON_MP; k++) {
            T acc = T(0);
#pragma unroll
            for (int d = 0; d < KRON_W; d++) acc += tap[d] * win[k + d];
            out[k] = acc;
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < KRON_MP; k++) {
        const int pos = p0 + k;
        const T *tp = (pos >= KRON_B && pos < len - KRON_B) ? tint + c * KRON_W
                                                            : B.row(axis, c, pos < len ? pos : len - 1);
        T acc = T(0);
#pragma unroll
        for (int d = 0; d < KRON_W; d++) acc += tp[d] * win[k + d];
        out[k] = acc;
    }
}

// x pass: kx lines (3 nx consecutive values each) per CTA.  The staged input
// is the masked, node-scaled residual t = S N r; in the mixed FCG the staging
// also re-forms r32 = sigma r after a residual replacement (S->rescale).
// Shared layout [line][component][position] with an odd pitch (conflict-free
// windows); the outputs go through shared memory so that the global stores
// are coalesced.
__host__ __device__ inline int kx_pitch(int nx) { return nx | 1; }
__host__ inline int kx_lines(const GridDesc &g, size_t elem) {
    const size_t per_line = elem * 2 * 3 * (size_t)kx_pitch(g.nx);
    int L = (int)((size_t)(48 * 1024) / per_line);
    return L < 1 ? 1 : (L > 8 ? 8 : L);
}
__host__ inline size_t kron_x_smem(const GridDesc &g, size_t elem, int kx = 0) {
    return elem * ((size_t)(kx > 0 ? kx : kx_lines(g, elem)) * 2 * 3 * kx_pitch(g.nx) + 3 * KRON_W);
}
// lines per CTA for a launch: the shared-memory cap, lowered so that the grid
// still fills one wave of `slots` resident CTAs
__host__ inline int kx_lines_launch(const GridDesc &g, size_t elem, long long slots) {
    const long long nlines = (long long)g.ny * g.nz;
    const long long want = (nlines + slots - 1) / slots;
    const int cap = kx_lines(g, elem);
    return (int)(want < 1 ? 1 : (want > cap ? cap : want));
}

template <class T, class R>
__device__ __forceinline__ void kron_x_body(const GridDesc &g, int kx, R *r, const double *__restrict__ r64,
                                            const SolveScalars *S, const T *__restrict__ ms, const KronBand<T> &B,
                                            T *out) {
    TOPO_DYNAMIC_SMEM(unsigned char, kron_smem);
    const int LP = kx_pitch(g.nx);
    T *tile = reinterpret_cast<T *>(kron_smem);  // [kx][3][LP]
    T *otile = tile + kx * 3 * LP;               // [kx][3][LP]
    T *tint = otile + kx * 3 * LP;               // [3][KRON_W]
    const int row = 3 * g.nx;
    const long long nlines = (long long)g.ny * g.nz;
    const long long line0 = (long long)blockIdx.x * kx;
    const int nl = (int)(nlines - line0 < kx ? nlines - line0 : kx);
    const bool rs = S != nullptr && S->rescale != 0;
    const ScaleF64 sg = scale_split(rs ? S->sigma : 1.0);
    kron_stage_interior(B, 0, g.nx, tint);
    const long long q0 = line0 * row;
    const int nv = nl * row;
    // t / row by a multiply-high with ceil(2^32 / row), exact for t < 2^32 / row
    // (nv is a few thousand): no integer division sequence per value
    const unsigned mrow = (unsigned)((0x100000000ull + (unsigned)row - 1) / (unsigned)row);
#pragma unroll 4
    for (int t = threadIdx.x; t < nv; t += KRON_THREADS) {
        const int l = (int)__umulhi((unsigned)t, mrow), w = t - l * row;  // line and position of value t
        const int i = w / 3, c = w - 3 * i;
        const long long q = q0 + t;
        R rv;
        if (rs) {
            rv = (R)scaled_f32(r64[q], sg);
            r[q] = rv;
        } else {
            rv = r[q];
        }
        const T m = ms[q];
        tile[(l * 3 + c) * LP + i] = m < T(0) ? T(0) : (T)rv * m;
    }
    __syncthreads();
    const int ngrp = (g.nx + KRON_MP - 1) / KRON_MP;
    const int nrows = nl * 3;
    for (int t = threadIdx.x; t < nrows * ngrp; t += KRON_THREADS) {
        const int rw = t % nrows, grp = t / nrows;
        const int c = rw % 3;
        const int p0 = grp * KRON_MP;
        T o[KRON_MP];
        kron_line(tile + rw * LP, 1, g.nx, p0, tint, B, 0, c, o);
#pragma unroll
        for (int k = 0; k < KRON_MP; k++)
            if (p0 + k < g.nx) otile[rw * LP + p0 + k] = o[k];
    }
    __syncthreads();
#pragma unroll 4
    for (int t = threadIdx.x; t < nv; t += KRON_THREADS) {
        const int l = (int)__umulhi((unsigned)t, mrow), w = t - l * row;
        const int i = w / 3, c = w - 3 * i;
        out[q0 + t] = otile[(l * 3 + c) * LP + i];
    }
}

template <class T, class R>
static __global__ void __launch_bounds__(KRON_THREADS)
    k_kron_x(GridDesc g, int kx, R *r, const double *__restrict__ r64, const SolveScalars *S, const T *__restrict__ ms,
             KronBand<T> B, T *out) {
    kron_x_body<T, R>(g, kx, r, r64, S, ms, B, out);
}
// y pass (AXIS 1) and z pass (AXIS 2): a CTA stages a chunk of KW values of
// one x-row (consecutive in memory) at every position along the line.  The
// z pass finishes P^-1: out = S x on free DOFs, r on clamped ones; with DOT it
// also forms the FCG dot products z.r and z.q of its output.  The z pass
// stages its epilogue operands (r, the masked scale, q) with the input, so
// that no global load waits inside the output loop.
constexpr int KW = 32;

__host__ inline unsigned kron_yz_blocks(const GridDesc &g, int axis) {
    const int nchunk = (3 * g.nx + KW - 1) / KW;
    return (unsigned)nchunk * (unsigned)(axis == 1 ? g.nz : g.ny);
}
__host__ inline size_t kron_yz_smem(const GridDesc &g, int axis, size_t elem, bool dot = false) {
    const size_t len = (size_t)(axis == 1 ? g.ny : g.nz);
    return elem * (KW * len * (axis == 2 ? 3 : 1) + 3 * KRON_W) + (dot ? sizeof(float) * KW * len : 0);
}

template <class T, class R, int AXIS, bool DOT>
static __global__ void __launch_bounds__(KRON_THREADS, sizeof(T) == 4 ? 4 : 2)
    k_kron_yz(GridDesc g, const R *__restrict__ r, const T *__restrict__ ms, KronBand<T> B, const T *__restrict__ in,
              T *out, KronDot kd) {
    TOPO_DYNAMIC_SMEM(unsigned char, kron_smem);
    const int len = AXIS == 1 ? g.ny : g.nz;
    T *tile = reinterpret_cast<T *>(kron_smem);  // [len][KW]
    T *tint = tile + (size_t)len * KW;           // [3][KRON_W]
    T *rt = tint + 3 * KRON_W;                   // AXIS 2: r [len][KW]
    T *mt = rt + (size_t)len * KW;               // AXIS 2: masked scale [len][KW]
    float *qt = reinterpret_cast<float *>(mt + (size_t)len * KW);  // DOT: q [len][KW]
    const int row = 3 * g.nx;
    const int nchunk = (row + KW - 1) / KW;
    const int chunk = blockIdx.x % nchunk, other = blockIdx.x / nchunk;
    const int w0 = chunk * KW, wn = (row - w0 < KW) ? row - w0 : KW;
    const long long S = AXIS == 1 ? (long long)row : (long long)row * g.ny;
    const long long base = AXIS == 1 ? (long long)other * row * g.ny + w0 : (long long)other * row + w0;
    kron_stage_interior(B, AXIS, len, tint);
    // the staging is a pure copy: cp.async puts every copy of the chunk in
    // flight at once, with no register round trip
    static_assert(std::is_same<T, R>::value, "staged r is copied, not converted");
    for (int t = threadIdx.x; t < len * KW; t += KRON_THREADS) {
        const int p = t / KW, w = t - p * KW;
        if (w < wn) {
            const long long q = base + p * S + w;
            cp_async<(int)sizeof(T)>(tile + t, in + q);
            if (AXIS == 2) {
                cp_async<(int)sizeof(T)>(rt + t, r + q);
                cp_async<(int)sizeof(T)>(mt + t, ms + q);
                if (DOT) cp_async<4>(qt + t, kd.q32 + q);
            }
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    // the FCG dot products: FP32 per thread (at most a few dozen terms), FP64
    // across threads (GB300 runs FP64 at 1/64 of the FP32 rate)
    float sr = 0.0f, sq = 0.0f;
    const int ngrp = (len + KRON_MP - 1) / KRON_MP;
    for (int t = threadIdx.x; t < ngrp * KW; t += KRON_THREADS) {
        const int grp = t / KW, w = t - grp * KW;
        if (w >= wn) continue;
        const int c = (w0 + w) % 3;
        const int p0 = grp * KRON_MP;
        T o[KRON_MP];
        kron_line(tile + w, KW, len, p0, tint, B, AXIS, c, o);
#pragma unroll
        for (int k = 0; k < KRON_MP; k++) {
            const int p = p0 + k;
            if (p >= len) break;
            const long long q = base + p * S + w;
            if (AXIS == 2) {
                const int sidx = p * KW + w;
                const T m = mt[sidx], rv = rt[sidx];
                const T z = m < T(0) ? rv : m * o[k];
                out[q] = z;
                if (DOT) {
                    sr += (float)z * (float)rv;
                    sq += (float)z * qt[sidx];
                }
            } else {
                out[q] = o[k];
            }
        }
    }
    if constexpr (DOT) {
        const float red[2] = {sr, sq};
        double tot[2];
        if (grid_reduce<KRON_THREADS, 2>(red, kd.part, tot)) {
            SolveScalars *S = kd.S;
            S->rho = tot[0];
            S->gam = tot[1];
            S->beta = S->restart ? 0.0 : -tot[1] / S->pq;
            if (!isfinite(S->beta)) S->beta = 0.0;
            S->beta32 = (float)S->beta;
            S->rescale = 0;
        }
    }
}

}  // namespace topo
