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
#include <string.h>

namespace topo {

__device__ __forceinline__ float f64_to_f32(double v);
__device__ __forceinline__ double f32_to_f64(float f);
struct df;
__host__ __device__ __forceinline__ df f64_to_df(double v);

struct df {
    float hi, lo;
    __host__ __device__ df() : hi(0.0f), lo(0.0f) {}
    __host__ __device__ df(float h, float l) : hi(h), lo(l) {}
    // hi = v rounded to FP32, lo = the rest rounded to FP32; no FP64
    // instruction (f64_to_df)
    __host__ __device__ df(double v);
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

// FP64 -> double-float split from the bit pattern: hi = v rounded to FP32
// (nearest, ties away, as f64_to_f32); v - hi is exactly R ulp(v) with R a
// 29-bit signed integer (the low mantissa bits, minus 2^29 when hi rounded
// up), so lo = R rounded to FP32 by one int-to-float conversion, scaled by
// ulp(v) in its exponent field.  No FP64 instruction.  |v| below 2^-126
// flushes to zero, as does a lo below 2^-126; finite values above the FP32
// range are not expected and give an infinite hi.
__host__ __device__ __forceinline__ df f64_to_df(double v) {
    unsigned long long b;
    memcpy(&b, &v, sizeof b);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7FFu);
    const unsigned sign = hi & 0x80000000u;
    unsigned hb, lb = 0u;
    if (e < 897) {
        hb = sign;
    } else if (e > 1150) {
        hb = (e == 2047 && ((hi & 0xFFFFFu) | lo)) ? 0x7FC00000u : (sign | 0x7F800000u);
    } else {
        const unsigned mag = ((unsigned)(e - 896) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
        const unsigned rnd = (lo >> 28) & 1u;
        hb = sign | (mag + rnd);
        const int R = (int)(lo & 0x1FFFFFFFu) - (int)(rnd << 29);
        if (R != 0) {
#ifdef __CUDA_ARCH__
            const float fr = __int2float_rn(R);
#else
            const float fr = (float)R;
#endif
            unsigned fb;
            memcpy(&fb, &fr, sizeof fb);
            const int k = e - 1075;  // ulp(v) = 2^k
            if ((int)((fb >> 23) & 0xFFu) + k >= 1) lb = (fb + (unsigned)(k * (1 << 23))) ^ sign;
        }
    }
    df r;
    memcpy(&r.hi, &hb, sizeof hb);
    memcpy(&r.lo, &lb, sizeof lb);
    return r;
}
__host__ __device__ __forceinline__ df::df(double v) { *this = f64_to_df(v); }

// FP32 copies of FP64 values scaled by a positive factor s (the residual
// rescaling r32 = sigma r of the mixed FCG) without FP64 instructions: s is
// split once into 2^k m with m in [1, 2); each value gets k added to its FP64
// exponent field on the integer pipes, is rounded to FP32 (f64_to_f32) and
// multiplied by m in FP32 (two roundings instead of one).  Zero stays zero;
// v 2^k below 2^-126 flushes to zero, as in f64_to_f32, so results below
// 2^-125 may flush (the rescaling brings residuals to unit mean square).
struct ScaleF64 {
    int k;
    float m;
};
__device__ __forceinline__ ScaleF64 scale_split(double s) {
    const long long b = __double_as_longlong(s);
    const int e = (int)((b >> 52) & 0x7FF);
    ScaleF64 r;
    r.k = e - 1023;
    r.m = f64_to_f32(__longlong_as_double((b & 0x800FFFFFFFFFFFFFll) | (1023ll << 52)));
    return r;
}
__device__ __forceinline__ float scaled_f32(double v, ScaleF64 s) {
    long long b = __double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7FF);
    const int en = e + s.k;
    if (e == 0 || en <= 0) return __uint_as_float((unsigned)((unsigned long long)b >> 32) & 0x80000000u);
    if (en >= 2047) b = (b & (long long)0x8000000000000000ull) | (0x7FFll << 52);  // infinity
    else b += (long long)s.k * (1ll << 52);
    return f64_to_f32(__longlong_as_double(b)) * s.m;
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
// a + b without the final renormalisation: Knuth's two-sum of the leading
// parts, with the low parts added to its error term; three FP32 instructions
// fewer than operator+.  The pair may hold |lo| above half an ulp of hi.
// Every df operation and todbl accepts such pairs, and their absolute error
// stays about 2^-48 of the operands, as with operator+.  The sums inside an
// element product (mode transforms, Khat rows, mass terms, the gather of the
// element contributions) use it; the products and todbl that follow absorb
// the difference.
__host__ __device__ __forceinline__ df add_lazy(df a, df b) {
    float s = DF_ADD(a.hi, b.hi);
    float bb = DF_SUB(s, a.hi);
    float e = DF_ADD(DF_SUB(a.hi, DF_SUB(s, bb)), DF_SUB(b.hi, bb));
    return df(s, DF_ADD(e, DF_ADD(a.lo, b.lo)));
}
// the element-math sums and products of tile.cuh / common.cuh: plain for
// float and double; for df, add_lazy sums and renormalised products (products
// without the renormalisation were measured to raise the accuracy floor of
// the stiffness-dominated mixed solves above rtol 1e-11)
__host__ __device__ __forceinline__ df tadd(df a, df b) { return add_lazy(a, b); }
__host__ __device__ __forceinline__ df tsub(df a, df b) { return add_lazy(a, -b); }
__host__ __device__ __forceinline__ df tmul(df a, df b) { return a * b; }

__host__ __device__ __forceinline__ df &operator+=(df &a, df b) { return a = a + b; }
__host__ __device__ __forceinline__ df &operator-=(df &a, df b) { return a = a - b; }
__host__ __device__ __forceinline__ df &operator*=(df &a, df b) { return a = a * b; }

}  // namespace topo
