// tile.cuh -- the matrix-free hex8 operator kernel.
//
// One CTA of 512 threads owns a 7x7x7 brick of output nodes.  It stages the
// 9x9x9 input nodes (brick + one-node halo) in shared memory, lets each thread
// apply the element operator of one of the 8x8x8 elements touching the brick
// (mode-basis form, common.cuh), parks the 24 element outputs in shared memory
// and finally lets each output node gather its 8 element contributions.  No
// atomics: every output is written once, so results are bitwise reproducible.
// Element work on the brick faces is recomputed by the neighbour CTA
// (512/343 = 1.49x redundancy), traded for determinism and zero global
// scatter traffic.
//
// What is staged, how element weights are formed and what happens to the
// assembled value (masking, fused vector updates, dot products) is supplied by
// a policy type; see le.cu for the policies used by the solver.
#pragma once
#include <type_traits>
#include "common.cuh"

namespace topo {

constexpr int TILE = 7;               // output nodes per CTA edge
constexpr int TILE_E = TILE + 1;      // elements per CTA edge
constexpr int TILE_N = TILE + 2;      // staged nodes per CTA edge
constexpr int TILE_THREADS = 512;     // == TILE_E^3
constexpr int TILE_STAGED = TILE_N * TILE_N * TILE_N;  // 729
constexpr int TILE_OUT = TILE * TILE * TILE;            // 343
constexpr int EL_STRIDE = 25;         // padded element-output row (bank spread)

template <class T, class Pol>
constexpr size_t tile_smem_bytes() {
    return sizeof(T) * ((size_t)Pol::NIN * TILE_STAGED * 3 + (size_t)TILE_THREADS * EL_STRIDE);
}

__host__ __device__ inline int tile_count(const GridDesc &g, int &ntx, int &nty) {
    ntx = (g.nx + TILE - 1) / TILE;
    nty = (g.ny + TILE - 1) / TILE;
    return ntx * nty * ((g.nz + TILE - 1) / TILE);
}

// Policy interface:
//   static constexpr int NIN;      staged 3-vectors per node (1: K and M act on
//                                  input 0; 2: K on input 0, M on input 1)
//   static constexpr bool HAS_K, HAS_M;
//   static constexpr int NRED;     grid-reduced doubles (0..4)
//   __device__ void load(long long n, T v[NIN][3]) const;
//   __device__ void coef(long long e, T &ck, T &cm) const;
//   __device__ void epilogue(long long n, int i, int j, int k, const T y[3], double red[]) const;
//   __device__ void finish(const double tot[]) const;   (thread 0 of last CTA)
//   Partials<NRED> part;  (when NRED > 0)
// optional early exit: a policy may define `bool skip() const` (read by every
// thread before any shared-memory or reduction work, so the whole grid exits)
template <class P>
__device__ __forceinline__ auto pol_skip(const P &p, int) -> decltype(p.skip()) {
    return p.skip();
}
template <class P>
__device__ __forceinline__ bool pol_skip(const P &, long) {
    return false;
}

// optional epilogue-operand prefetch: a policy may define `Pre pre(long long n)`
// and `epilogue(n, i, j, k, y, red, const Pre &)`; the kernel issues pre()
// before the element phase so the loads overlap the element arithmetic
struct NoPre {};
template <class P>
__device__ __forceinline__ auto pol_pre(const P &p, long long n, int) -> decltype(p.pre(n)) {
    return p.pre(n);
}
template <class P>
__device__ __forceinline__ NoPre pol_pre(const P &, long long, long) {
    return NoPre{};
}
template <class P, class T, class A, class R>
__device__ __forceinline__ auto pol_epi(const P &p, long long n, int i, int j, int k, const T y[3], A *red,
                                        const R &pre, int) -> decltype(p.epilogue(n, i, j, k, y, red, pre)) {
    return p.epilogue(n, i, j, k, y, red, pre);
}
template <class P, class T, class A, class R>
__device__ __forceinline__ void pol_epi(const P &p, long long n, int i, int j, int k, const T y[3], A *red,
                                        const R &, long) {
    p.epilogue(n, i, j, k, y, red);
}

// per-thread accumulator type of a policy's reductions: `using Red = float;`
// in an FP32 policy keeps the per-node sums on the FP32 pipe (GB300 runs FP64
// at 1/64 of the FP32 rate); the thread's partials widen to FP64 once, for the
// grid reduction
template <class P, class = void>
struct pol_red {
    using type = double;
};
template <class P>
struct pol_red<P, std::void_t<typename P::Red>> {
    using type = typename P::Red;
};
template <class P>
using pol_red_t = typename pol_red<P>::type;

// staged input nodes of brick `tile` held by this thread (at most two)
template <class T, class Pol>
__device__ __forceinline__ void tile_fetch(const Pol &pol, const GridDesc &g, int tile, int ntx, int nty,
                                           T v[2][Pol::NIN][3]) {
    const int i0 = (tile % ntx) * TILE, j0 = ((tile / ntx) % nty) * TILE, k0 = (tile / (ntx * nty)) * TILE;
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const int s = threadIdx.x + it * TILE_THREADS;
        const int lx = s % TILE_N, ly = (s / TILE_N) % TILE_N, lz = s / (TILE_N * TILE_N);
        const int gi = i0 - 1 + lx, gj = j0 - 1 + ly, gk = k0 - 1 + lz;
        if (s < TILE_STAGED && gi >= 0 && gi < g.nx && gj >= 0 && gj < g.ny && gk >= 0 && gk < g.nz) {
            long long n = gi + (long long)g.nx * (gj + (long long)g.ny * gk);
            pol.load(n, v[it]);
        } else {
#pragma unroll
            for (int f = 0; f < Pol::NIN; f++) v[it][f][0] = v[it][f][1] = v[it][f][2] = T(0);
        }
    }
}

// FP32 kernels are persistent: the grid holds as many CTAs as fit on the
// device, each CTA walks the bricks tile = blockIdx.x, + gridDim.x, ... and
// loads the next brick's staged nodes into registers while it computes the
// current one, so the global-load latency of the staging overlaps the element
// arithmetic.  Reductions accumulate over a CTA's bricks in a fixed order and
// are reduced once over the grid.  FP64 and double-float kernels (one CTA of
// 128 registers a thread per SM) launch one CTA per brick: holding the next
// brick's values would spill.
template <class T>
constexpr bool tile_persistent() {
    return sizeof(T) == 4;
}
// one brick: stage (v holds its staged nodes), element phase, gather and
// epilogue; with `next` >= 0 the staged nodes of brick `next` are loaded into
// v while this brick is computed
template <class T, class Pol>
__device__ __forceinline__ void tile_brick(const GridDesc &g, const ElemConst<T> &C, const Pol &pol, T *sIn, T *sEl,
                                           int tile, int next, int ntx, int nty, T v[2][Pol::NIN][3],
                                           pol_red_t<Pol> *red) {
    const int tid = threadIdx.x;
    const int i0 = (tile % ntx) * TILE, j0 = ((tile / ntx) % nty) * TILE, k0 = (tile / (ntx * nty)) * TILE;
    // ---- staged inputs (brick + halo, zero outside the domain) to shared memory ----
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const int s = tid + it * TILE_THREADS;
        if (s < TILE_STAGED) {
#pragma unroll
            for (int f = 0; f < Pol::NIN; f++)
#pragma unroll
                for (int c = 0; c < 3; c++) sIn[(f * TILE_STAGED + s) * 3 + c] = v[it][f][c];
        }
    }
    // output node of this thread and its prefetched epilogue operands
    const int tx = tid % TILE, ty = (tid / TILE) % TILE, tz = tid / (TILE * TILE);
    const int oi = i0 + tx, oj = j0 + ty, ok = k0 + tz;
    const bool has_out = tid < TILE_OUT && oi < g.nx && oj < g.ny && ok < g.nz;
    const long long on = has_out ? oi + (long long)g.nx * (oj + (long long)g.ny * ok) : 0;
    const auto pre = pol_pre(pol, on, 0);
    __syncthreads();
    if (next >= 0) tile_fetch<T>(pol, g, next, ntx, nty, v);

    // ---- one element per thread ----
    {
        const int lx = tid & 7, ly = (tid >> 3) & 7, lz = tid >> 6;
        const int ei = i0 - 1 + lx, ej = j0 - 1 + ly, ek = k0 - 1 + lz;
        T *out = sEl + tid * EL_STRIDE;
        if (ei >= 0 && ei < g.ex && ej >= 0 && ej < g.ey && ek >= 0 && ek < g.ez) {
            long long e = ei + (long long)g.ex * (ej + (long long)g.ey * ek);
            T ck, cm;
            pol.coef(e, ck, cm);
            T U[3][8];
#pragma unroll
            for (int L = 0; L < 8; L++) {
                int s = (lx + (L & 1)) + TILE_N * ((ly + ((L >> 1) & 1)) + TILE_N * (lz + (L >> 2)));
#pragma unroll
                for (int c = 0; c < 3; c++) U[c][L] = sIn[s * 3 + c];
            }
#pragma unroll
            for (int c = 0; c < 3; c++) mode_fwd(U[c]);
            T Y[3][8];
            if (Pol::HAS_K && Pol::HAS_M && Pol::NIN == 1) {
                mode_khat_mass(C, ck, cm, U, Y);
            } else {
                if (Pol::HAS_K) {
                    mode_khat(C, U, Y);
#pragma unroll
                    for (int c = 0; c < 3; c++)
#pragma unroll
                        for (int m = 0; m < 8; m++) Y[c][m] *= ck;
                } else {
#pragma unroll
                    for (int c = 0; c < 3; c++)
#pragma unroll
                        for (int m = 0; m < 8; m++) Y[c][m] = T(0);
                }
                if (Pol::HAS_M) {
#pragma unroll
                    for (int b = 0; b < 3; b++) {
                        T V[8];
                        if (Pol::NIN == 2) {
#pragma unroll
                            for (int L = 0; L < 8; L++) {
                                int s = (lx + (L & 1)) + TILE_N * ((ly + ((L >> 1) & 1)) + TILE_N * (lz + (L >> 2)));
                                V[L] = sIn[((Pol::NIN - 1) * TILE_STAGED + s) * 3 + b];
                            }
                            mode_fwd(V);
                        } else {
#pragma unroll
                            for (int m = 0; m < 8; m++) V[m] = U[b][m];
                        }
#pragma unroll
                        for (int m = 0; m < 8; m++) Y[b][m] += (cm * C.W[m]) * V[m];
                    }
                }
            }
#pragma unroll
            for (int b = 0; b < 3; b++) {
                mode_bwd(Y[b]);
#pragma unroll
                for (int L = 0; L < 8; L++) out[L * 3 + b] = Y[b][L];
            }
        } else {
#pragma unroll
            for (int q = 0; q < 24; q++) out[q] = T(0);
        }
    }
    __syncthreads();

    // ---- gather + policy epilogue ----
    if (has_out) {
        T y[3] = {T(0), T(0), T(0)};
#pragma unroll
        for (int L = 0; L < 8; L++) {
            int ax = L & 1, ay = (L >> 1) & 1, az = L >> 2;
            int le = (tx + 1 - ax) + TILE_E * ((ty + 1 - ay) + TILE_E * (tz + 1 - az));
#pragma unroll
            for (int c = 0; c < 3; c++) y[c] += sEl[le * EL_STRIDE + L * 3 + c];
        }
        pol_epi(pol, on, oi, oj, ok, y, red, pre, 0);
    }
}

template <class T, class Pol>
__global__ void __launch_bounds__(TILE_THREADS, sizeof(T) == 4 ? 2 : 1) k_tile(const GridDesc g, const ElemConst<T> C, const Pol pol) {
    TOPO_DYNAMIC_SMEM(unsigned char, smem_raw);
    T *sIn = reinterpret_cast<T *>(smem_raw);
    T *sEl = sIn + Pol::NIN * TILE_STAGED * 3;
    if (pol_skip(pol, 0)) return;
    static_assert(TILE_STAGED <= 2 * TILE_THREADS, "staging assumes two passes");
    int ntx, nty;
    const int ntiles = tile_count(g, ntx, nty);
    pol_red_t<Pol> red[Pol::NRED > 0 ? Pol::NRED : 1];
#pragma unroll
    for (int r = 0; r < (Pol::NRED > 0 ? Pol::NRED : 1); r++) red[r] = 0;
    T v[2][Pol::NIN][3];
    if constexpr (tile_persistent<T>()) {
        if ((int)blockIdx.x < ntiles) tile_fetch<T>(pol, g, blockIdx.x, ntx, nty, v);
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const int next = tile + (int)gridDim.x < ntiles ? tile + (int)gridDim.x : -1;
            tile_brick<T>(g, C, pol, sIn, sEl, tile, next, ntx, nty, v, red);
            __syncthreads();  // shared memory is restaged for the next brick
        }
    } else {
        tile_fetch<T>(pol, g, blockIdx.x, ntx, nty, v);
        tile_brick<T>(g, C, pol, sIn, sEl, blockIdx.x, -1, ntx, nty, v, red);
    }
    if constexpr (Pol::NRED > 0) {
        double rd[Pol::NRED], tot[Pol::NRED];
#pragma unroll
        for (int r = 0; r < Pol::NRED; r++) rd[r] = (double)red[r];
        if (grid_reduce<TILE_THREADS, Pol::NRED>(rd, pol.part, tot)) pol.finish(tot);
    }
}

}  // namespace topo
