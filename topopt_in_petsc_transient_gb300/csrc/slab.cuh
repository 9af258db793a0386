// slab.cuh -- z-marching form of the matrix-free hex8 operator kernel.
//
// Same policies, same element arithmetic and the same no-atomics gather as the
// brick kernel of tile.cuh, with less recomputation.  A CTA of 256 threads
// owns a 15 x 15 column of output nodes over a range of node layers and
// marches up through it one element layer at a time:
//   - its 16 x 16 threads each compute one element of the current element
//     layer (the elements touching the column, one to each side in x and y);
//   - only the new top node layer (17 x 17 nodes) is staged per step: the
//     bottom corners of an element are the top corners it read one step
//     earlier, carried in registers;
//   - the 24 element outputs go to a ring of two element layers in shared
//     memory, and every output node of layer k gathers its 8 contributions
//     from element layers k - 1 and k.
// Per output node the brick form computes 512/343 = 1.49 elements and stages
// 729/343 = 2.13 nodes; the slab form computes 256/225 = 1.14 elements and
// stages 289/225 = 1.28 nodes (plus one element layer per z-range).  Results
// equal the brick form's up to the summation order of the grid reductions.
#pragma once
#include "tile.cuh"

namespace topo {

constexpr int SLAB_E = 16;                   // elements per CTA edge in x and y
constexpr int SLAB_O = SLAB_E - 1;           // output nodes per CTA edge
constexpr int SLAB_N = SLAB_E + 1;           // staged nodes per CTA edge
constexpr int SLAB_THREADS = SLAB_E * SLAB_E;          // 256, one element each
constexpr int SLAB_STAGED = SLAB_N * SLAB_N;           // 289 nodes per layer
constexpr int SLAB_MIN_LAYERS = 8;           // shortest z-range of a CTA

template <class T, class Pol>
constexpr size_t slab_smem_bytes() {
    return sizeof(T) * ((size_t)Pol::NIN * SLAB_STAGED * 3 + (size_t)2 * SLAB_THREADS * EL_STRIDE);
}

// columns and z-ranges of the launch: the grid is ncx * ncy * nzr CTAs, CTA b
// takes column b % (ncx ncy) and node layers [zr0, zr1) of range b / (ncx ncy)
struct SlabShape {
    int ncx, ncy, nzr, zlen;
};

// z-ranges so that the grid fills about `slots` resident CTAs, each range at
// least SLAB_MIN_LAYERS node layers long
__host__ inline SlabShape slab_shape(const GridDesc &g, long long slots) {
    SlabShape s;
    s.ncx = (g.nx + SLAB_O - 1) / SLAB_O;
    s.ncy = (g.ny + SLAB_O - 1) / SLAB_O;
    const long long cols = (long long)s.ncx * s.ncy;
    long long nzr = (slots + cols - 1) / cols;
    const long long maxr = (g.nz + SLAB_MIN_LAYERS - 1) / SLAB_MIN_LAYERS;
    nzr = nzr < 1 ? 1 : (nzr > maxr ? maxr : nzr);
    s.zlen = (int)((g.nz + nzr - 1) / nzr);
    s.nzr = (g.nz + s.zlen - 1) / s.zlen;
    return s;
}

// node layer gk of the column with node origin (i0 - 1, j0 - 1): the staged
// values this thread holds (positions tid and tid + 256 of the 17 x 17 layer),
// zero outside the domain
template <class T, class Pol>
__device__ __forceinline__ void slab_fetch(const Pol &pol, const GridDesc &g, int i0, int j0, int gk,
                                           T v[2][Pol::NIN][3]) {
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const int s = threadIdx.x + it * SLAB_THREADS;
        const int sx = s % SLAB_N, sy = s / SLAB_N;
        const int gi = i0 - 1 + sx, gj = j0 - 1 + sy;
        if (s < SLAB_STAGED && gi >= 0 && gi < g.nx && gj >= 0 && gj < g.ny && gk >= 0 && gk < g.nz) {
            pol.load(gi + (long long)g.nx * (gj + (long long)g.ny * gk), v[it]);
        } else {
#pragma unroll
            for (int f = 0; f < Pol::NIN; f++) v[it][f][0] = v[it][f][1] = v[it][f][2] = T(0);
        }
    }
}

template <class T, class Pol>
__device__ __forceinline__ void slab_store(T *sN, const T v[2][Pol::NIN][3]) {
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const int s = threadIdx.x + it * SLAB_THREADS;
        if (s < SLAB_STAGED) {
#pragma unroll
            for (int f = 0; f < Pol::NIN; f++)
#pragma unroll
                for (int c = 0; c < 3; c++) sN[(f * SLAB_STAGED + s) * 3 + c] = v[it][f][c];
        }
    }
}

// the 4 corners (x, y bits) of this thread's element in the staged layer
template <class T, class Pol>
__device__ __forceinline__ void slab_corners(const T *sN, int lx, int ly, T q[Pol::NIN][3][4]) {
#pragma unroll
    for (int L = 0; L < 4; L++) {
        const int s = (lx + (L & 1)) + SLAB_N * (ly + (L >> 1));
#pragma unroll
        for (int f = 0; f < Pol::NIN; f++)
#pragma unroll
            for (int c = 0; c < 3; c++) q[f][c][L] = sN[(f * SLAB_STAGED + s) * 3 + c];
    }
}

// element outputs Y (nodal, 8 corners x 3) of the element with corner values
// bot (z bit 0) and top (z bit 1); the arithmetic of the brick kernel
template <class T, class Pol>
__device__ __forceinline__ void slab_element(const ElemConst<T> &C, const Pol &pol, long long e,
                                             const T bot[Pol::NIN][3][4], const T top[Pol::NIN][3][4],
                                             T *out) {
    T ck, cm;
    pol.coef(e, ck, cm);
    T U[3][8];
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int L = 0; L < 4; L++) {
            U[c][L] = bot[0][c][L];
            U[c][L + 4] = top[0][c][L];
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
                    for (int L = 0; L < 4; L++) {
                        V[L] = bot[Pol::NIN - 1][b][L];
                        V[L + 4] = top[Pol::NIN - 1][b][L];
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
}

template <class T, class Pol>
__global__ void __launch_bounds__(SLAB_THREADS, sizeof(T) == 4 ? 3 : 2)
    k_slab(const GridDesc g, const ElemConst<T> C, const Pol pol, const SlabShape sh) {
    TOPO_DYNAMIC_SMEM(unsigned char, smem_raw);
    T *sN = reinterpret_cast<T *>(smem_raw);       // [NIN][289][3] staged top node layer
    T *sEl = sN + Pol::NIN * SLAB_STAGED * 3;      // [2][256][EL_STRIDE] element layers
    if (pol_skip(pol, 0)) return;
    static_assert(SLAB_STAGED <= 2 * SLAB_THREADS, "staging assumes two positions per thread");
    const int tid = threadIdx.x;
    const int col = blockIdx.x % (sh.ncx * sh.ncy), zr = blockIdx.x / (sh.ncx * sh.ncy);
    const int i0 = (col % sh.ncx) * SLAB_O, j0 = (col / sh.ncx) * SLAB_O;
    const int k0 = zr * sh.zlen, k1 = min(k0 + sh.zlen, g.nz);
    const int lx = tid % SLAB_E, ly = tid / SLAB_E;
    const int ei = i0 - 1 + lx, ej = j0 - 1 + ly;
    const bool col_el = ei >= 0 && ei < g.ex && ej >= 0 && ej < g.ey;
    // output node of this thread in every layer of the range
    const int tx = tid % SLAB_E, ty = tid / SLAB_E;
    const int oi = i0 + tx, oj = j0 + ty;
    const bool col_out = tx < SLAB_O && ty < SLAB_O && oi < g.nx && oj < g.ny;
    double red[Pol::NRED > 0 ? Pol::NRED : 1];
#pragma unroll
    for (int r = 0; r < (Pol::NRED > 0 ? Pol::NRED : 1); r++) red[r] = 0.0;

    // bottom node layer of the first element layer k0 - 1
    T v[2][Pol::NIN][3];
    T bot[Pol::NIN][3][4], top[Pol::NIN][3][4];
    slab_fetch<T>(pol, g, i0, j0, k0 - 1, v);
    slab_store<T, Pol>(sN, v);
    slab_fetch<T>(pol, g, i0, j0, k0, v);  // top layer of the first step, in flight
    __syncthreads();
    slab_corners<T, Pol>(sN, lx, ly, bot);
    __syncthreads();  // sN is restaged below

    for (int kk = k0 - 1; kk < k1; kk++) {
        // element layer kk: nodes kk (bot, carried) and kk + 1 (top, staged)
        slab_store<T, Pol>(sN, v);
        const int kout = kk;  // output node layer of this step (kk >= k0)
        const long long on = (col_out && kout >= k0) ? oi + (long long)g.nx * (oj + (long long)g.ny * kout) : 0;
        const auto pre = pol_pre(pol, on, 0);
        __syncthreads();
        slab_corners<T, Pol>(sN, lx, ly, top);
        if (kk + 1 < k1) slab_fetch<T>(pol, g, i0, j0, kk + 2, v);  // next top layer
        T *out = sEl + ((kk & 1) * SLAB_THREADS + tid) * EL_STRIDE;
        if (col_el && kk >= 0 && kk < g.ez) {
            slab_element<T, Pol>(C, pol, ei + (long long)g.ex * (ej + (long long)g.ey * kk), bot, top, out);
        } else {
#pragma unroll
            for (int q = 0; q < 24; q++) out[q] = T(0);
        }
#pragma unroll
        for (int f = 0; f < Pol::NIN; f++)
#pragma unroll
            for (int c = 0; c < 3; c++)
#pragma unroll
                for (int L = 0; L < 4; L++) bot[f][c][L] = top[f][c][L];
        __syncthreads();
        // node layer kout gathers from element layers kout - 1 (top corners)
        // and kout (bottom corners)
        if (kout >= k0 && col_out) {
            T y[3] = {T(0), T(0), T(0)};
#pragma unroll
            for (int L = 0; L < 8; L++) {
                const int ax = L & 1, ay = (L >> 1) & 1, az = L >> 2;
                const int le = (tx + 1 - ax) + SLAB_E * (ty + 1 - ay);
                const int slot = (kout - az) & 1;
#pragma unroll
                for (int c = 0; c < 3; c++) y[c] += sEl[(slot * SLAB_THREADS + le) * EL_STRIDE + L * 3 + c];
            }
            pol_epi(pol, on, oi, oj, kout, y, red, pre, 0);
        }
    }
    if constexpr (Pol::NRED > 0) {
        double tot[Pol::NRED];
        if (grid_reduce<SLAB_THREADS, Pol::NRED>(red, pol.part, tot)) pol.finish(tot);
    }
}

}  // namespace topo
