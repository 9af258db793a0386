// Test-only host stand-in for the CUDA qualifiers and builtins that the
// kernel headers of topopt_in_petsc_transient_gb300/csrc name, so that their
// kernels compile as host C++ and run on host threads (one std::thread per
// CUDA thread, a std::barrier per CTA for __syncthreads, one CTA at a time).
// Atomics are plain read-modify-writes: only thread 0 of a CTA issues them.
// Never part of the library.
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
// CTAs run one after another, so a static local is the CTA's shared variable
#define __shared__ static
#define __align__(n) __attribute__((aligned(n)))
namespace emu {
extern unsigned char dyn_smem[];  // the dynamic shared memory of the running CTA
}
#define TOPO_DYNAMIC_SMEM(T, name) T *name = reinterpret_cast<T *>(emu::dyn_smem)
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
// every thread of the CTA calls the shuffles of a reduction the same number of
// times: exchange through a CTA-shared buffer between two barriers
template <class T>
inline T __shfl_xor_sync(unsigned, T v, int o) {
    static T buf[1024];
    buf[threadIdx.x] = v;
    __syncthreads();
    const T r = buf[threadIdx.x ^ (unsigned)o];
    __syncthreads();
    return r;
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
