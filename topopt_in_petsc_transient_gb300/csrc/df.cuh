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

__device__ __forceinline__ float f64_to_f32(double v);
__device__ __forceinline__ double f32_to_f64(float f);

struct df {
    float hi, lo;
    __host__ __device__ df() : hi(0.0f), lo(0.0f) {}
    __host__ __device__ df(float h, float l) : hi(h), lo(l) {}
    // hi = v rounded to FP32, lo = the rest rounded to FP32 (v - hi is exact
    // in FP64).  On the device the conversions run on the integer pipes, one
    // FP64 subtraction remains (magnitudes below 2^-126 flush to zero)
    __host__ __device__ df(double v) {
#ifdef __CUDA_ARCH__
        hi = f64_to_f32(v);
        lo = f64_to_f32(v - f32_to_f64(hi));
#else
        hi = (float)v;
        lo = (float)(v - (double)hi);
#endif
    }
};

// Conversions between FP64 and FP32 on the integer pipes.  GB300 runs FP64
// instructions, conversions included, at about 2 per clock and SM; a
// streaming kernel that converts every value is then bound by them.  These
// rebuild the bit patterns instead:
//  * f64_to_f32: round to nearest (ties away from zero), values below 2^-126
//    in magnitude flush to a signed zero (FP32 element math cannot use them
//    anyway), infinities and NaNs map to their FP32 kinds; finite values
//    above the FP32 range are not expected and become infinities;
//  * f32_to_f64: exact for normal floats, subnormals flush to a signed zero.
__device__ __forceinline__ float f64_to_f32(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7FFu);
    const unsigned sign = hi & 0x80000000u;
    if (e < 897) return __uint_as_float(sign);
    if (e > 1150) return __uint_as_float((e == 2047 && ((hi & 0xFFFFFu) | lo)) ? 0x7FC00000u : (sign | 0x7F800000u));
    const unsigned mag = ((unsigned)(e - 896) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    return __uint_as_float(sign | (mag + ((lo >> 28) & 1u)));
}
__device__ __forceinline__ double f32_to_f64(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned e = (b >> 23) & 0xFFu;
    const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
    if (e == 0) return __longlong_as_double((long long)sign);
    if (e == 255) return (double)f;
    return __longlong_as_double(
        (long long)(sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(b & 0x7FFFFFu) << 29)));
}

__host__ __device__ __forceinline__ double todbl(double v) { return v; }
__host__ __device__ __forceinline__ double todbl(float v) { return (double)v; }
__host__ __device__ __forceinline__ double todbl(df v) {
#ifdef __CUDA_ARCH__
    return f32_to_f64(v.hi) + f32_to_f64(v.lo);
#else
    return (double)v.hi + (double)v.lo;
#endif
}

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
