// conv_check.cu -- the integer-pipe conversions of df.cuh (f64_to_f32,
// f32_to_f64, f64_to_df) against the hardware conversions on random and edge
// values.  Prints "conversions OK" and exits 0 when every value agrees as
// specified: f64_to_f32 equals round-to-nearest except on exact ties (rounded
// away from zero) and below 2^-126 (signed zero); f32_to_f64 is exact for
// normal floats and flushes subnormals to a signed zero; f64_to_df gives the
// hi of f64_to_f32 and lo = v - hi (exact in FP64) rounded to nearest FP32,
// zero below 2^-126; scaled_f32 is within 2^-22 of sigma v (or zero below
// 2^-125).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>

#include "df.cuh"

using namespace topo;

__global__ void k_check(int n, const double *d, const float *f, unsigned *bad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double v = d[i];
        const float got = f64_to_f32(v), ref = __double2float_rn(v);
        const bool tiny = fabs(v) < 1.1754943508222875e-38;
        bool ok;
        if (tiny)
            ok = got == 0.0f && signbit(got) == signbit(v);
        else if (isnan(v))
            ok = isnan(got);
        else
            ok = __float_as_uint(got) == __float_as_uint(ref) ||
                 ((double)got - v == -((double)ref - v));  // an exact tie, rounded the other way
        if (!ok) atomicAdd(&bad[0], 1u);
        const float x = f[i];
        const double w = f32_to_f64(x);
        bool ok2;
        if (x != 0.0f && fabsf(x) < 1.17549435e-38f)
            ok2 = w == 0.0 && signbit(w) == signbit(x);
        else if (isnan(x))
            ok2 = isnan(w);
        else
            ok2 = __double_as_longlong(w) == __double_as_longlong((double)x);
        if (!ok2) atomicAdd(&bad[1], 1u);
        const df sp = f64_to_df(v);
        bool ok3 = __float_as_uint(sp.hi) == __float_as_uint(got);
        if (ok3 && !tiny && isfinite(v) && isfinite(sp.hi)) {
            const double r = v - (double)sp.hi;
            const float lref = fabs(r) < 1.1754943508222875e-38 ? 0.0f : __double2float_rn(r);
            ok3 = (sp.lo == 0.0f && lref == 0.0f) || __float_as_uint(sp.lo) == __float_as_uint(lref);
        } else if (ok3) {
            ok3 = sp.lo == 0.0f;
        }
        if (!ok3) atomicAdd(&bad[2], 1u);
        // scaled_f32: sigma v rounded to FP32 with two roundings (relative
        // error below 2^-22); results below 2^-125 may flush to zero
        if (isfinite(v)) {
            const double sg = ldexp(1.0 + 0.5 * fabs(__sinf((float)i)), (int)(i % 81) - 40);
            const double pr = sg * v;
            const float sf = scaled_f32(v, scale_split(sg));
            bool ok4;
            if (fabs(pr) > 3.0e38)
                ok4 = true;  // outside the FP32 range: not used
            else
                ok4 = fabs((double)sf - pr) <= ldexp(fabs(pr), -22) ||
                      (fabs(pr) < 2.3509887016445750e-38 && sf == 0.0f);
            if (!ok4) atomicAdd(&bad[3], 1u);
        }
    }
}

int main() {
    const int n = 1 << 22;
    double *hd = (double *)malloc(sizeof(double) * n);
    float *hf = (float *)malloc(sizeof(float) * n);
    unsigned long long s = 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        return s;
    };
    for (int i = 0; i < n; i++) {
        unsigned long long r = next();
        double v;
        if (i % 4 == 0) {  // any bit pattern with an exponent in or near the FP32 range
            unsigned long long e = 860 + (r >> 52) % 330;
            unsigned long long b = (r & 0x800FFFFFFFFFFFFFull) | (e << 52);
            memcpy(&v, &b, 8);
        } else {
            v = ((double)(r >> 11) / 9007199254740992.0 - 0.5) * pow(10.0, (double)((int)(r % 60) - 30));
        }
        hd[i] = v;
        unsigned r32 = (unsigned)(next() >> 32);
        float f;
        memcpy(&f, &r32, 4);
        hf[i] = f;
    }
    const double edges[] = {0.0, -0.0, 1.0, -1.0, 1.5, 3.4028234663852886e38, 1.1754943508222875e-38, 1e-40, -1e-300,
                            INFINITY, -INFINITY, NAN, 0.1, 1.0000000596046448 /* a tie between two floats */};
    for (int k = 0; k < (int)(sizeof(edges) / sizeof(edges[0])); k++) hd[k] = edges[k];
    const float fedges[] = {0.0f, -0.0f, 1.0f, 1e-40f, -1e-45f, INFINITY, NAN, 3.4e38f};
    for (int k = 0; k < (int)(sizeof(fedges) / sizeof(fedges[0])); k++) hf[k] = fedges[k];
    double *d;
    float *f;
    unsigned *bad;
    cudaMalloc(&d, sizeof(double) * n);
    cudaMalloc(&f, sizeof(float) * n);
    cudaMalloc(&bad, 4 * sizeof(unsigned));
    cudaMemcpy(d, hd, sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(f, hf, sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemset(bad, 0, 4 * sizeof(unsigned));
    k_check<<<512, 256>>>(n, d, f, bad);
    unsigned hb[4] = {1, 1, 1, 1};
    cudaError_t e = cudaMemcpy(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        printf("CUDA error %s\n", cudaGetErrorString(e));
        return 2;
    }
    printf("f64_to_f32 mismatches %u, f32_to_f64 mismatches %u, f64_to_df mismatches %u, scaled_f32 mismatches %u\n",
           hb[0], hb[1], hb[2], hb[3]);
    if (hb[0] == 0 && hb[1] == 0 && hb[2] == 0 && hb[3] == 0) printf("conversions OK\n");
    return (hb[0] || hb[1] || hb[2] || hb[3]) ? 1 : 0;
}
