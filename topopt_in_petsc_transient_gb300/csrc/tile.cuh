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

// ---------------------------------------------------------------------------
// element phase and gather, shared by both staging paths
// ---------------------------------------------------------------------------
// one element per thread: the 24 outputs of element (lx, ly, lz) of the brick
// at (i0, j0, k0) from the staged nodes sIn into sEl
template <class T, class Pol>
__device__ __forceinline__ void tile_elements(const GridDesc &g, const ElemConst<T> &C, const Pol &pol, const T *sIn,
                                              T *sEl, int i0, int j0, int k0) {
    const int tid = threadIdx.x;
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
        } else if (Pol::HAS_K && !Pol::HAS_M) {
            mode_khat_mass<false>(C, ck, cm, U, Y);
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
                    for (int m = 0; m < 8; m++) Y[b][m] = tadd(Y[b][m], tmul(tmul(cm, C.W[m]), V[m]));
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

// the output node (tx, ty, tz) of this thread: its 8 element contributions
// from sEl, then the policy epilogue
template <class T, class Pol, class R>
__device__ __forceinline__ void tile_gather(const Pol &pol, const T *sEl, long long on, int oi, int oj, int ok, int tx,
                                            int ty, int tz, const R &pre, pol_red_t<Pol> *red) {
    T y[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int L = 0; L < 8; L++) {
        int ax = L & 1, ay = (L >> 1) & 1, az = L >> 2;
        int le = (tx + 1 - ax) + TILE_E * ((ty + 1 - ay) + TILE_E * (tz + 1 - az));
#pragma unroll
        for (int c = 0; c < 3; c++) y[c] = tadd(y[c], sEl[le * EL_STRIDE + L * 3 + c]);
    }
    pol_epi(pol, on, oi, oj, ok, y, red, pre, 0);
}

// ---------------------------------------------------------------------------
// staging path 1: per-thread loads into registers
// ---------------------------------------------------------------------------
// FP32 kernels are persistent: the grid holds as many CTAs as fit on the
// device, each CTA walks the bricks tile = blockIdx.x, + gridDim.x, ... and
// loads the next brick's staged nodes into registers while it computes the
// current one, so the global-load latency of the staging overlaps the element
// arithmetic.  Reductions accumulate over a CTA's bricks in a fixed order and
// are reduced once over the grid.  FP64 and double-float kernels (one CTA of
// 128 registers a thread per SM) cannot hold the next brick's values: they
// prefetch into shared memory instead (staging path 2) when their policy
// allows it, and otherwise launch one CTA per brick.
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
    tile_elements<T>(g, C, pol, sIn, sEl, i0, j0, k0);
    __syncthreads();
    if (has_out) tile_gather<T>(pol, sEl, on, oi, oj, ok, tx, ty, tz, pre, red);
}

// ---------------------------------------------------------------------------
// staging path 2: per-thread asynchronous copies into shared memory
// ---------------------------------------------------------------------------
// For kernels whose registers are all taken by the element arithmetic (FP64
// and double-float, one CTA of 512 threads per SM) the next brick cannot be
// held in registers.  A policy may then opt in to this path by declaring
//   using Src = float | double;          element type of its raw input arrays
//   static constexpr int NSRC;           raw arrays staged per node (1 or 2)
//   static constexpr bool MASK;          read the clamp bitmask `fixed` too
//   const Src *src(int k) const;         raw array k, 3 values per node
//   void xform(const Src raw[NSRC][3], uint8_t f, T v[1][3]) const;
//                                        staged value from the raw values
// The kernel is then persistent: every thread issues `cp.async` copies of the
// raw values of its own staged nodes of the next brick into its own slots of a
// raw buffer in shared memory (and a plain load of their mask bytes into
// registers) while the current brick is computed, and converts them into the
// staged nodes after waiting for its own copies only.  No register holds the
// prefetched brick, and no barrier guards the raw buffer: each slot is written
// and read by one thread.
//
// (A bulk-copy form, one `cp.async.bulk` per 16-byte-aligned node row of the
// staged brick completing on an mbarrier, was measured slower: 162 to 243
// copies of 32 to 224 bytes per brick keep the copy engine busy for about 28
// cycles each, and the FP32 product took 219 instead of 98 us at 192x96x96.
// The node rows (3 nx values) are not 16-byte multiples, so no tensor map
// describes the bricks.)
template <class P, class = void>
struct pol_async : std::false_type {};
template <class P>
struct pol_async<P, std::void_t<typename P::Src>> : std::true_type {};

// the async path serves the non-persistent (FP64, double-float) kernels; FP32
// kernels keep their register prefetch
template <class T, class Pol>
constexpr bool tile_async() {
    return pol_async<Pol>::value && !tile_persistent<T>();
}

template <class T, class Pol, bool ASYNC = tile_async<T, Pol>()>
struct TileSmem {
    static constexpr size_t bytes = tile_smem_bytes<T, Pol>();
};
template <class T, class Pol>
struct TileSmem<T, Pol, true> {
    using Src = typename Pol::Src;
    static constexpr size_t raw = 0;  // [NSRC][TILE_STAGED][3] Src
    static constexpr size_t in = ((size_t)Pol::NSRC * TILE_STAGED * 3 * sizeof(Src) + 15) / 16 * 16;
    static constexpr size_t el = in + sizeof(T) * (size_t)TILE_STAGED * 3;
    static constexpr size_t bytes = el + sizeof(T) * (size_t)TILE_THREADS * EL_STRIDE;
};

template <int NB>
__device__ __forceinline__ void cp_async(void *dst, const void *src) {
    static_assert(NB == 4 || NB == 8, "cp.async of one FP32 or FP64 value");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src),
                 "n"(NB)
                 : "memory");
}

// this thread's staged nodes of brick `tile`: raw values by cp.async into its
// slots of `raw`, mask bytes into f
template <class T, class Pol>
__device__ __forceinline__ void tile_fetch_async(const Pol &pol, const GridDesc &g, int tile, int ntx, int nty,
                                                 typename Pol::Src *raw, uint8_t f[2]) {
    using Src = typename Pol::Src;
    const int i0 = (tile % ntx) * TILE, j0 = ((tile / ntx) % nty) * TILE, k0 = (tile / (ntx * nty)) * TILE;
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const int s = threadIdx.x + it * TILE_THREADS;
        const int lx = s % TILE_N, ly = (s / TILE_N) % TILE_N, lz = s / (TILE_N * TILE_N);
        const int gi = i0 - 1 + lx, gj = j0 - 1 + ly, gk = k0 - 1 + lz;
        f[it] = 0;
        if (s < TILE_STAGED && gi >= 0 && gi < g.nx && gj >= 0 && gj < g.ny && gk >= 0 && gk < g.nz) {
            const long long n = gi + (long long)g.nx * (gj + (long long)g.ny * gk);
#pragma unroll
            for (int k = 0; k < Pol::NSRC; k++)
#pragma unroll
                for (int c = 0; c < 3; c++)
                    cp_async<(int)sizeof(Src)>(raw + ((size_t)k * TILE_STAGED + s) * 3 + c, pol.src(k) + 3 * n + c);
            if constexpr (Pol::MASK) f[it] = pol.fixed[n];
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

template <class T, class Pol>
__device__ __forceinline__ void tile_run_async(const GridDesc &g, const ElemConst<T> &C, const Pol &pol,
                                               unsigned char *sm, int ntiles, int ntx, int nty, pol_red_t<Pol> *red) {
    using L = TileSmem<T, Pol>;
    using Src = typename Pol::Src;
    static_assert(Pol::NIN == 1, "async staging stages one 3-vector per node");
    const int tid = threadIdx.x;
    Src *raw = reinterpret_cast<Src *>(sm + L::raw);
    T *sIn = reinterpret_cast<T *>(sm + L::in);
    T *sEl = reinterpret_cast<T *>(sm + L::el);
    uint8_t f[2];
    if ((int)blockIdx.x < ntiles) tile_fetch_async<T>(pol, g, blockIdx.x, ntx, nty, raw, f);
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int next = tile + (int)gridDim.x < ntiles ? tile + (int)gridDim.x : -1;
        const int i0 = (tile % ntx) * TILE, j0 = ((tile / ntx) % nty) * TILE, k0 = (tile / (ntx * nty)) * TILE;
        asm volatile("cp.async.wait_group 0;" ::: "memory");  // this thread's copies only
        // raw values -> staged nodes (zero outside the domain)
#pragma unroll
        for (int it = 0; it < 2; it++) {
            const int s = tid + it * TILE_THREADS;
            if (s < TILE_STAGED) {
                const int lx = s % TILE_N, ly = (s / TILE_N) % TILE_N, lz = s / (TILE_N * TILE_N);
                const int gi = i0 - 1 + lx, gj = j0 - 1 + ly, gk = k0 - 1 + lz;
                T v[1][3] = {{T(0), T(0), T(0)}};
                if (gi >= 0 && gi < g.nx && gj >= 0 && gj < g.ny && gk >= 0 && gk < g.nz) {
                    Src rv[Pol::NSRC][3];
#pragma unroll
                    for (int k = 0; k < Pol::NSRC; k++)
#pragma unroll
                        for (int c = 0; c < 3; c++) rv[k][c] = raw[((size_t)k * TILE_STAGED + s) * 3 + c];
                    pol.xform(rv, f[it], v);
                }
#pragma unroll
                for (int c = 0; c < 3; c++) sIn[s * 3 + c] = v[0][c];
            }
        }
        const int tx = tid % TILE, ty = (tid / TILE) % TILE, tz = tid / (TILE * TILE);
        const int oi = i0 + tx, oj = j0 + ty, ok = k0 + tz;
        const bool has_out = tid < TILE_OUT && oi < g.nx && oj < g.ny && ok < g.nz;
        const long long on = has_out ? oi + (long long)g.nx * (oj + (long long)g.ny * ok) : 0;
        const auto pre = pol_pre(pol, on, 0);
        __syncthreads();
        if (next >= 0) tile_fetch_async<T>(pol, g, next, ntx, nty, raw, f);
        tile_elements<T>(g, C, pol, sIn, sEl, i0, j0, k0);
        __syncthreads();
        if (has_out) tile_gather<T>(pol, sEl, on, oi, oj, ok, tx, ty, tz, pre, red);
        __syncthreads();  // shared memory is restaged for the next brick
    }
}

template <class T, class Pol>
__global__ void __launch_bounds__(TILE_THREADS, sizeof(T) == 4 ? 2 : 1) k_tile(const GridDesc g, const ElemConst<T> C, const Pol pol) {
    TOPO_DYNAMIC_SMEM(unsigned char, smem_raw);
    if (pol_skip(pol, 0)) return;
    static_assert(TILE_STAGED <= 2 * TILE_THREADS, "staging assumes two passes");
    int ntx, nty;
    const int ntiles = tile_count(g, ntx, nty);
    pol_red_t<Pol> red[Pol::NRED > 0 ? Pol::NRED : 1];
#pragma unroll
    for (int r = 0; r < (Pol::NRED > 0 ? Pol::NRED : 1); r++) red[r] = 0;
    if constexpr (tile_async<T, Pol>()) {
        tile_run_async<T>(g, C, pol, smem_raw, ntiles, ntx, nty, red);
    } else {
        T *sIn = reinterpret_cast<T *>(smem_raw);
        T *sEl = sIn + Pol::NIN * TILE_STAGED * 3;
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
    }
    if constexpr (Pol::NRED > 0) {
        double tot[Pol::NRED];
        if (grid_reduce<TILE_THREADS, Pol::NRED>(red, pol.part, tot)) pol.finish(tot);
    }
}

}  // namespace topo
