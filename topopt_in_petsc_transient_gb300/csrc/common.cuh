// common.cuh -- shared device machinery for the GB300 transient topology
// optimisation path: structured-grid descriptors, the hex8 element operator in
// the per-axis sum/difference ("mode") basis, and deterministic reductions.
//
// Data layout (identical to the reference DMDA natural ordering so host
// buffers cross the C ABI without permutation, LinearElasticity.cc:3033-3087):
//   node (i,j,k)    -> n = i + nx*(j + ny*k), displacement DOF 3*n + c
//   element (i,j,k) -> e = i + ex*(j + ey*k)
// Every nodal vector is DOF-interleaved (xyz per node); FP64 for states,
// FP32 copies inside the multigrid preconditioner.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/topopt_gb300.h"

// dynamic shared memory of a kernel: one declaration form for every kernel
// (a host build of the kernel sources for tests may define it otherwise)
#ifndef TOPO_DYNAMIC_SMEM
#define TOPO_DYNAMIC_SMEM(T, name) extern __shared__ __align__(16) T name[]
#endif

namespace topo {

// status codes TOPO_OK / TOPO_ERR_* come from the C ABI header

// host-side count of kernel launches issued by this library (one program-wide
// counter; graph replays are added from their captured kernel counts)
inline long long &launch_counter() {
    static long long c = 0;
    return c;
}
inline void count_launch(long long n = 1) { launch_counter() += n; }
// ---------------------------------------------------------------------------
// one level of the structured node/element grid
// ---------------------------------------------------------------------------
struct GridDesc {
    int nx, ny, nz;  // nodes
    int ex, ey, ez;  // elements = nodes - 1
    __host__ __device__ long long nn() const { return (long long)nx * ny * nz; }
    __host__ __device__ long long nel() const { return (long long)ex * ey * ez; }
};

// Constants of the hex8 element operator on an hx*hy*hz box in the mode basis.
//
// Per axis the two nodal values (v0, v1) of an element edge are mapped to
// s = v0 + v1 and d = v1 - v0; the trilinear field is then
//   u = sum_m U_m psi_p(xi) psi_q(eta) psi_r(zeta),  psi_s = 1/2, psi_d = xi - 1/2,
// with m = p + 2q + 4r (bit set = difference mode).  In this basis the 2x2x2
// Gauss-integrated (exact for a box) mass matrix is diagonal with weights
// W_m = V prod(w), w_s = 1/4, w_d = 1/12, and the isotropic stiffness couples
// only a handful of modes (d/dx psi_d = 2 psi_s).  The element matrices are
// therefore applied with ~290 flops instead of the 1536 of the dense 24x24
// products of LinearElasticity.cc:3089-3333, with identical results up to
// rounding (the reference's truncated Gauss abscissa differs by 2e-16).
// In the mode basis (index i = 8 c + m) the element stiffness Khat has 45
// non-zeros that form symmetric diagonal blocks after a permutation: two 3x3,
// six 2x2 and three 1x1 blocks (rigid translations, modes i = 0, 8, 16, are
// its null space).  The pattern does not depend on the box shape or on nu.
constexpr int KH_NB = 11;
constexpr int KH_NNZ = 45;
__host__ __device__ constexpr int kh_size(int b) { return b < 2 ? 3 : (b < 8 ? 2 : 1); }
__host__ __device__ constexpr int kh_idx(int b, int r) {
    // blocks: {1,10,20} {6,13,19} {2,9} {3,22} {4,17} {5,14} {11,21} {12,18} {7} {15} {23}
    return b == 0 ? (r == 0 ? 1 : r == 1 ? 10 : 20)
         : b == 1 ? (r == 0 ? 6 : r == 1 ? 13 : 19)
         : b == 2 ? (r == 0 ? 2 : 9)
         : b == 3 ? (r == 0 ? 3 : 22)
         : b == 4 ? (r == 0 ? 4 : 17)
         : b == 5 ? (r == 0 ? 5 : 14)
         : b == 6 ? (r == 0 ? 11 : 21)
         : b == 7 ? (r == 0 ? 12 : 18)
         : b == 8 ? 7 : b == 9 ? 15 : 23;
}

template <class T>
struct ElemConst {
    T W[8];      // V * w_p * w_q * w_r
    T g[3];      // 2 / h_a
    T lam, mu;   // Lame parameters for E = 1 (LinearElasticity.cc:3134-3135)
    T K[KH_NNZ]; // Khat blocks, row-major per block, blocks in kh_idx order
};

template <class T>
__host__ __device__ inline ElemConst<T> make_elem_const_base(double hx, double hy, double hz, double nu) {
    ElemConst<T> c;
    double V = hx * hy * hz;
    const double w[2] = {0.25, 1.0 / 12.0};
    for (int m = 0; m < 8; m++) c.W[m] = (T)(V * w[m & 1] * w[(m >> 1) & 1] * w[(m >> 2) & 1]);
    c.g[0] = (T)(2.0 / hx);
    c.g[1] = (T)(2.0 / hy);
    c.g[2] = (T)(2.0 / hz);
    c.lam = (T)(nu / ((1.0 + nu) * (1.0 - 2.0 * nu)));
    c.mu = (T)(1.0 / (2.0 * (1.0 + nu)));
    for (int i = 0; i < KH_NNZ; i++) c.K[i] = (T)0.0;
    return c;
}

// (i, j, k) of lexicographic index n on an nx x ny x . grid with 32-bit
// unsigned divisions: node and element indices stay far below 2^32 on every
// grid that fits in HBM (the 64-bit division sequences cost several times more)
__host__ __device__ __forceinline__ void lex3(long long n, int nx, int ny, int &i, int &j, int &k) {
    const unsigned u = (unsigned)n, q = u / (unsigned)nx;
    i = (int)(u - q * (unsigned)nx);
    k = (int)(q / (unsigned)ny);
    j = (int)(q - (unsigned)k * (unsigned)ny);
}

// sums of the element math; df.cuh overloads them for double-float pairs
__host__ __device__ __forceinline__ float tadd(float a, float b) { return a + b; }
__host__ __device__ __forceinline__ double tadd(double a, double b) { return a + b; }
__host__ __device__ __forceinline__ float tsub(float a, float b) { return a - b; }
__host__ __device__ __forceinline__ double tsub(double a, double b) { return a - b; }
__host__ __device__ __forceinline__ float tmul(float a, float b) { return a * b; }
__host__ __device__ __forceinline__ double tmul(double a, double b) { return a * b; }

// nodal -> mode transform of one component (local node L = ax + 2ay + 4az)
template <class T>
__host__ __device__ __forceinline__ void mode_fwd(T v[8]) {
#pragma unroll
    for (int s = 0; s < 3; s++) {
        const int b = 1 << s;
#pragma unroll
        for (int L = 0; L < 8; L++) {
            if (L & b) continue;
            T a0 = v[L], a1 = v[L | b];
            v[L] = tadd(a0, a1);
            v[L | b] = tsub(a1, a0);
        }
    }
}

// transpose of mode_fwd: mode -> nodal (used for operator outputs y = T^t Y)
template <class T>
__host__ __device__ __forceinline__ void mode_bwd(T v[8]) {
#pragma unroll
    for (int s = 2; s >= 0; s--) {
        const int b = 1 << s;
#pragma unroll
        for (int L = 0; L < 8; L++) {
            if (L & b) continue;
            T sv = v[L], dv = v[L | b];
            v[L] = tsub(sv, dv);
            v[L | b] = tadd(sv, dv);
        }
    }
}

// Y = Khat U : element stiffness (E = 1) in mode space, without density factor.
// G_ab(m) = d u_b / d x_a on modes with bit a clear; strain energy density
// lam (div u)^2 + mu sum g_ab^2 + mu sum g_ab g_ba (isotropic, Voigt C of
// LinearElasticity.cc:3141-3146).
template <class T>
__host__ __device__ __forceinline__ void mode_stiffness(const ElemConst<T> &C, const T U[3][8], T Y[3][8]) {
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int m = 0; m < 8; m++) Y[b][m] = T(0);
    T D[8];
#pragma unroll
    for (int m = 0; m < 8; m++) {
        T acc = T(0);
#pragma unroll
        for (int a = 0; a < 3; a++)
            if (!(m & (1 << a))) acc += C.g[a] * U[a][m | (1 << a)];
        D[m] = acc;
    }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++)
#pragma unroll
            for (int m = 0; m < 8; m++) {
                if (m & (1 << a)) continue;
                T gab = C.g[a] * U[b][m | (1 << a)];
                T sym = gab;
                if (!(m & (1 << b))) sym += C.g[b] * U[a][m | (1 << b)];
                T S = C.mu * sym;
                if (a == b) S += C.lam * D[m];
                Y[b][m | (1 << a)] += C.g[a] * (C.W[m] * S);
            }
}

// element constants including the Khat blocks, evaluated in double by
// applying the exact mode-basis stiffness to unit mode vectors
template <class T>
inline ElemConst<T> make_elem_const(double hx, double hy, double hz, double nu) {
    ElemConst<T> c = make_elem_const_base<T>(hx, hy, hz, nu);
    ElemConst<double> d = make_elem_const_base<double>(hx, hy, hz, nu);
    double Kh[24][24];
    for (int j = 0; j < 24; j++) {
        double U[3][8] = {{0}}, Y[3][8];
        U[j / 8][j % 8] = 1.0;
        mode_stiffness(d, U, Y);
        for (int i = 0; i < 24; i++) Kh[i][j] = Y[i / 8][i % 8];
    }
    int k = 0;
    for (int b = 0; b < KH_NB; b++)
        for (int r = 0; r < kh_size(b); r++)
            for (int s = 0; s < kh_size(b); s++) c.K[k++] = (T)Kh[kh_idx(b, r)][kh_idx(b, s)];
    return c;
}

// Y = Khat U with the block structure (45 multiply-adds); U, Y in [comp][mode]
template <class T>
__host__ __device__ __forceinline__ void mode_khat(const ElemConst<T> &C, const T U[3][8], T Y[3][8]) {
    Y[0][0] = Y[1][0] = Y[2][0] = T(0);
    int k = 0;
#pragma unroll
    for (int b = 0; b < KH_NB; b++) {
        const int n = kh_size(b);
#pragma unroll
        for (int r = 0; r < n; r++) {
            const int ir = kh_idx(b, r);
            T acc = C.K[k + r * n] * U[kh_idx(b, 0) / 8][kh_idx(b, 0) % 8];
#pragma unroll
            for (int s = 1; s < n; s++) acc = tadd(acc, C.K[k + r * n + s] * U[kh_idx(b, s) / 8][kh_idx(b, s) % 8]);
            Y[ir / 8][ir % 8] = acc;
        }
        k += n * n;
    }
}

// Y = ck Khat U + cm W .* U (stiffness + mass in mode space; MASS = false:
// ck Khat U alone); each U entry is consumed by one block, so the live range
// shrinks as blocks complete
template <bool MASS = true, class T>
__host__ __device__ __forceinline__ void mode_khat_mass(const ElemConst<T> &C, T ck, T cm, const T U[3][8],
                                                        T Y[3][8]) {
    T cw[8];
#pragma unroll
    for (int m = 0; m < 8; m++) cw[m] = MASS ? tmul(cm, C.W[m]) : T(0);
    Y[0][0] = MASS ? tmul(cw[0], U[0][0]) : T(0);
    Y[1][0] = MASS ? tmul(cw[0], U[1][0]) : T(0);
    Y[2][0] = MASS ? tmul(cw[0], U[2][0]) : T(0);
    int k = 0;
#pragma unroll
    for (int b = 0; b < KH_NB; b++) {
        const int n = kh_size(b);
#pragma unroll
        for (int r = 0; r < n; r++) {
            const int ir = kh_idx(b, r);
            T acc = tmul(C.K[k + r * n], U[kh_idx(b, 0) / 8][kh_idx(b, 0) % 8]);
#pragma unroll
            for (int s = 1; s < n; s++)
                acc = tadd(acc, tmul(C.K[k + r * n + s], U[kh_idx(b, s) / 8][kh_idx(b, s) % 8]));
            Y[ir / 8][ir % 8] = MASS ? tadd(tmul(ck, acc), tmul(cw[ir % 8], U[ir / 8][ir % 8])) : tmul(ck, acc);
        }
        k += n * n;
    }
}

// ---------------------------------------------------------------------------
// deterministic grid-wide reductions: per-CTA partials, last CTA sums in a
// fixed order (no floating-point atomics, bitwise reproducible)
// ---------------------------------------------------------------------------
template <int NV>
struct Partials {
    double *part;           // [gridDim][NV]
    unsigned int *counter;  // one counter per reduction site, reset by last CTA
};

template <int NT, int NV>
__device__ __forceinline__ void block_reduce(double v[NV], double *smem /* [NV][NT/32] */) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; i++) {
        double x = v[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) smem[i * (NT / 32) + wid] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; i++) {
            double s = 0.0;
            for (int w = 0; w < NT / 32; w++) s += smem[i * (NT / 32) + w];
            v[i] = s;
        }
    }
}

// FP32 partials: the warp-level tree in FP32 (GB300 runs FP64 at 1/64 of the
// FP32 rate, and an FP64 tree costs every thread five FP64 additions per
// value), then the warp sums widened once and added in FP64 by thread 0
template <int NT, int NV>
__device__ __forceinline__ void block_reduce_f32(const float vf[NV], double v[NV], double *smem /* [NV][NT/32] */) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; i++) {
        float x = vf[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) smem[i * (NT / 32) + wid] = (double)x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; i++) {
            double s = 0.0;
            for (int w = 0; w < NT / 32; w++) s += smem[i * (NT / 32) + w];
            v[i] = s;
        }
    }
}

// the grid stage of grid_reduce: v holds the CTA sums in thread 0
template <int NT, int NV>
__device__ __forceinline__ bool grid_reduce_blocks(double v[NV], const Partials<NV> &P, double tot[NV],
                                                   double *sred) {
    __shared__ bool last;
    const unsigned int nblk = gridDim.x * gridDim.y * gridDim.z;
    const unsigned int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; i++) P.part[(size_t)bid * NV + i] = v[i];
        __threadfence();
        unsigned int t = atomicAdd(P.counter, 1u);
        last = (t == nblk - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    // every thread of the last CTA sums a fixed strided subset, then a fixed
    // shuffle tree: the summation order depends only on the grid size
    double s[NV];
#pragma unroll
    for (int i = 0; i < NV; i++) s[i] = 0.0;
    for (unsigned int b = threadIdx.x; b < nblk; b += NT)
#pragma unroll
        for (int i = 0; i < NV; i++) s[i] += ((volatile double *)P.part)[(size_t)b * NV + i];
    __syncthreads();
    block_reduce<NT, NV>(s, sred);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; i++) tot[i] = s[i];
        *P.counter = 0u;
        return true;
    }
    return false;
}

// Called by every thread of every CTA (1D-linearised block id).  Returns true
// in exactly one thread (thread 0 of the last CTA to finish); on that thread
// `tot` holds the grid sums.
template <int NT, int NV>
__device__ __forceinline__ bool grid_reduce(double v[NV], const Partials<NV> &P, double tot[NV]) {
    __shared__ double sred[NV * (NT / 32)];
    block_reduce<NT, NV>(v, sred);
    return grid_reduce_blocks<NT, NV>(v, P, tot, sred);
}
// the same from FP32 per-thread partials (block_reduce_f32)
template <int NT, int NV>
__device__ __forceinline__ bool grid_reduce(const float vf[NV], const Partials<NV> &P, double tot[NV]) {
    __shared__ double sred[NV * (NT / 32)];
    double v[NV];
    block_reduce_f32<NT, NV>(vf, v, sred);
    return grid_reduce_blocks<NT, NV>(v, P, tot, sred);
}

}  // namespace topo
