// Test-only host stand-in for the CUDA qualifiers and builtins that the
// kernel headers of topopt_in_petsc_transient_gb300/csrc name, so that their
// kernels compile as host C++ and run on host threads (one std::thread per
// CUDA thread, a std::barrier per CTA for __syncthreads).  Atomics and warp
// shuffles are single-thread stand-ins: the emulated kernels run without
// grid reductions.  Never part of the library.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __shared__
#define __align__(n) __attribute__((aligned(n)))
struct emu_uint3 {
    unsigned x = 0, y = 0, z = 0;
};
extern thread_local emu_uint3 threadIdx, blockIdx;
extern emu_uint3 blockDim, gridDim;
void __syncthreads();
inline void __threadfence() {}
inline unsigned atomicAdd(unsigned *p, unsigned v) {
    unsigned o = *p;
    *p += v;
    return o;
}
template <class T>
inline T __shfl_xor_sync(unsigned, T v, int) {
    return v;
}
using std::max;
using std::min;
typedef struct emu_stream *cudaStream_t;
// names kernels.cuh, policies.cuh and kron.cuh use in code the emulation does not run
#include <cstring>
typedef unsigned long long cudaGraphConditionalHandle;
inline void cudaGraphSetConditional(cudaGraphConditionalHandle, unsigned) {}
inline long long __double_as_longlong(double d) {
    long long v;
    std::memcpy(&v, &d, 8);
    return v;
}
inline double __longlong_as_double(long long v) {
    double d;
    std::memcpy(&d, &v, 8);
    return d;
}
template <class T>
inline T atomicMax(T *p, T v) {
    T o = *p;
    if (v > o) *p = v;
    return o;
}
template <class T>
inline T atomicMin(T *p, T v) {
    T o = *p;
    if (v < o) *p = v;
    return o;
}
