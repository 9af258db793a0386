// df.cuh -- double-float ("FP32 pair") arithmetic for the FP64-accurate
// element passes of the mixed-precision path.
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the element
// operator passes that must be FP64-accurate (true residual replacements, the
// Newmark right-hand side, adjoint products) run on the FP32 pipes with
// unevaluated sums hi + lo of two floats.  Additions use the error-free
// two-sum of the leading parts (Knuth) followed by a fast renormalisation
// (Dekker's quick-two-sum); products use the FMA-based two-product.  The
// absolute error of an addition is ~2^-48 of the larger operand, which is the
// scale that matters for a residual b - A x; the result is converted back to
// FP64 (hi + lo is exact in double).  Stored vectors stay FP64.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace topo {

struct df {
    float hi, lo;
    __host__ __device__ df() : hi(0.0f), lo(0.0f) {}
    __host__ __device__ df(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ df(double v) {
        hi = (float)v;
        lo = (float)(v - (double)hi);
    }
};

__host__ __device__ __forceinline__ double todbl(double v) { return v; }
__host__ __device__ __forceinline__ double todbl(float v) { return (double)v; }
__host__ __device__ __forceinline__ double todbl(df v) { return (double)v.hi + (double)v.lo; }

#ifdef __CUDA_ARCH__
#define DF_ADD(a, b) __fadd_rn((a), (b))
#define DF_SUB(a, b) __fsub_rn((a), (b))
#define DF_MUL(a, b) __fmul_rn((a), (b))
#define DF_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#else
#define DF_ADD(a, b) ((a) + (b))
#define DF_SUB(a, b) ((a) - (b))
#define DF_MUL(a, b) ((a) * (b))
#define DF_FMA(a, b, c) fmaf((a), (b), (c))
#endif

__host__ __device__ __forceinline__ df operator+(df a, df b) {
    float s = DF_ADD(a.hi, b.hi);
    float bb = DF_SUB(s, a.hi);
    float e = DF_ADD(DF_SUB(a.hi, DF_SUB(s, bb)), DF_SUB(b.hi, bb));
    e = DF_ADD(e, DF_ADD(a.lo, b.lo));
    float h = DF_ADD(s, e);
    return df(h, DF_SUB(e, DF_SUB(h, s)));
}
__host__ __device__ __forceinline__ df operator-(df a) { return df(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__host__ __device__ __forceinline__ df operator*(df a, df b) {
    float p = DF_MUL(a.hi, b.hi);
    float e = DF_FMA(a.hi, b.hi, -p);
    e = DF_FMA(a.hi, b.lo, e);
    e = DF_FMA(a.lo, b.hi, e);
    float h = DF_ADD(p, e);
    return df(h, DF_SUB(e, DF_SUB(h, p)));
}
__host__ __device__ __forceinline__ df &operator+=(df &a, df b) { return a = a + b; }
__host__ __device__ __forceinline__ df &operator-=(df &a, df b) { return a = a - b; }
__host__ __device__ __forceinline__ df &operator*=(df &a, df b) { return a = a * b; }

}  // namespace topo
