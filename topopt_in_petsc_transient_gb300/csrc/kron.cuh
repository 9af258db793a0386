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
// 0.268^13 < 4e-8 relative): a 25-tap stencil along that axis with position
// dependent taps, data-parallel over all DOFs.  Tap table per axis a and
// component c: [a][c][n_a][2 KRON_B + 1].
constexpr int KRON_B = 12;
constexpr int KRON_W = 2 * KRON_B + 1;

template <class T>
struct KronBand {
    const T *t;  // [3][3][nmax][KRON_W]
    int nmax;
    __device__ __forceinline__ const T *row(int a, int c, int i) const {
        return t + (((size_t)(a * 3 + c) * nmax) + i) * KRON_W;
    }
};

// one axis pass over every DOF: out_q = sum_d tap[d] v_{q + d stride};
// AXIS 0 reads the residual (masked, node-scaled), AXIS 2 writes S x on free
// DOFs and the residual on clamped ones
template <class T, class R, int AXIS>
static __global__ void __launch_bounds__(256) k_kron_band(GridDesc g, const uint8_t *__restrict__ fixed,
                                                          const R *__restrict__ r, const T *__restrict__ scale,
                                                          KronBand<T> B, const T *__restrict__ in, T *out) {
    const long long nd = 3 * g.nn();
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= nd) return;
    const long long n = q / 3;
    const int c = (int)(q - 3 * n);
    const int i = (int)(n % g.nx), j = (int)((n / g.nx) % g.ny), k = (int)(n / ((long long)g.nx * g.ny));
    const int pos = AXIS == 0 ? i : (AXIS == 1 ? j : k);
    const int len = AXIS == 0 ? g.nx : (AXIS == 1 ? g.ny : g.nz);
    const long long stride = AXIS == 0 ? 1 : (AXIS == 1 ? (long long)g.nx : (long long)g.nx * g.ny);
    const int dlo = pos - KRON_B < 0 ? -pos : -KRON_B;
    const int dhi = pos + KRON_B > len - 1 ? len - 1 - pos : KRON_B;
    const T *tap = B.row(AXIS, c, pos) + KRON_B;
    T acc = T(0);
    for (int d = dlo; d <= dhi; d++) {
        const long long m = n + d * stride;
        T v;
        if (AXIS == 0)
            v = ((fixed[m] >> c) & 1) ? T(0) : (T)r[3 * m + c] * scale[m];
        else
            v = in[3 * m + c];
        acc += tap[d] * v;
    }
    if (AXIS == 2)
        out[q] = ((fixed[n] >> c) & 1) ? (T)r[q] : scale[n] * acc;
    else
        out[q] = acc;
}

}  // namespace topo
