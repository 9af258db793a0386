// noalloc.cu -- the volume constraint of LinearElasticity::VolumeConstraint
// (LinearElasticity.cc:1283-1296) without any device allocation.
//
// topo_le_volume_constraint_dev takes the scratch of its grid-wide sum (one
// partial per CTA plus a completion counter) from a topo_le object, and that
// object allocates HBM when it is created.  Some callers hold no such object
// and must not allocate: an optimiser or filter stage that owns only design
// vectors, running while the state history of a large mesh has committed the
// device memory, or running beside other work on the device that must not be
// held up by the device-wide synchronisation cudaMalloc and cudaFree can
// cause.  This variant keeps its scratch in one fixed file-scope device array
// and touches no allocator, neither CUDA's nor any library's.
//
// Limits, stated once here and checked on every call:
//   * nel is at most NA_SLOTS * EW * NA_ITEMS = 16,777,216 elements (each CTA
//     sums EW * NA_ITEMS elements into its own partial slot);
//   * the scratch is shared by every call on a device: calls that overlap in
//     time (two host threads, or two streams without ordering) race on it and
//     may return wrong sums.  Calls are serialised on the legacy default stream
//     and each returns only after its result has been copied back.
#include <cstdio>
#include <mutex>
#include <string>

#include "kernels.cuh"
#include "le.h"

namespace topo {

constexpr int NA_SLOTS = 8192;  // per-CTA partial sums held by the scratch
constexpr int NA_ITEMS = 8;     // elements summed by each thread
constexpr long long NA_MAX_NEL = (long long)NA_SLOTS * EW * NA_ITEMS;
constexpr int NA_MAX_DEVICES = 64;

// What must start at zero: `counter`.  Static device storage is zero when the
// module is loaded, the first call on a device sets it to zero once more, and
// the last CTA of every launch puts it back to zero after the final sum.
// `part` and `gx` need no initial value: every launch writes a slot before
// reading it.
struct NoAllocScratch {
    double part[NA_SLOTS];
    double gx;
    unsigned int counter;
};
static __device__ __align__(256) NoAllocScratch g_na_scratch;  // 65,552 bytes

static __global__ void __launch_bounds__(EW)
    k_volume_noalloc(long long n, const double *__restrict__ x, double volfrac, double *dg, NoAllocScratch *s) {
    double v[1] = {0.0};
    const long long base = (long long)blockIdx.x * (EW * NA_ITEMS) + threadIdx.x;
#pragma unroll
    for (int k = 0; k < NA_ITEMS; k++) {
        const long long i = base + (long long)k * EW;
        if (i < n) {
            v[0] += x[i];
            dg[i] = 1.0 / (double)n;
        }
    }
    double tot[1];
    if (grid_reduce<EW, 1>(v, Partials<1>{s->part, &s->counter}, tot)) s->gx = tot[0] / (double)n - volfrac;
}

// Device address of the scratch, looked up once per device with that device
// current.  A caller that records CUDA graphs should make its first call
// before it starts recording, so that this lookup is not part of a capture.
static std::mutex g_na_mutex;
static NoAllocScratch *g_na_ptr[NA_MAX_DEVICES] = {};

static int noalloc_scratch(NoAllocScratch **out) {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device available: the GB300 path has no CPU fallback");
        return TOPO_ERR_CUDA;
    }
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        return TOPO_ERR_CUDA;
    }
    if (dev < 0 || dev >= NA_MAX_DEVICES) {
        set_error("device ordinal " + std::to_string(dev) + " beyond the " + std::to_string(NA_MAX_DEVICES) +
                  " devices the allocation-free scratch table covers");
        return TOPO_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_na_scratch);
        if (e != cudaSuccess) {
            set_error(std::string("cudaGetSymbolAddress of the volume-constraint scratch: ") + cudaGetErrorString(e));
            return TOPO_ERR_CUDA;
        }
        NoAllocScratch *s = static_cast<NoAllocScratch *>(p);
        e = cudaMemset(&s->counter, 0, sizeof(s->counter));
        if (e != cudaSuccess) {
            set_error(std::string("zeroing the volume-constraint scratch counter: ") + cudaGetErrorString(e));
            return TOPO_ERR_CUDA;
        }
        g_na_ptr[dev] = s;
    }
    *out = g_na_ptr[dev];
    return TOPO_OK;
}

}  // namespace topo

using namespace topo;

extern "C" int topo_volume_constraint_noalloc_dev(long long nel, double *gx, double *dgdx_dev,
                                                  const double *xPhys_dev, double volfrac) {
    if (!gx || !dgdx_dev || !xPhys_dev) {
        set_error("topo_volume_constraint_noalloc_dev: null pointer argument");
        return TOPO_ERR_ARG;
    }
    if (nel < 1 || nel > NA_MAX_NEL) {
        char msg[200];
        snprintf(msg, sizeof msg,
                 "topo_volume_constraint_noalloc_dev: nel = %lld outside 1..%lld (fixed scratch of %d partial sums "
                 "of %d elements)",
                 nel, NA_MAX_NEL, NA_SLOTS, EW * NA_ITEMS);
        set_error(msg);
        return TOPO_ERR_ARG;
    }
    NoAllocScratch *s = nullptr;
    int rc = noalloc_scratch(&s);
    if (rc) return rc;
    const unsigned blocks = (unsigned)((nel + EW * NA_ITEMS - 1) / (EW * NA_ITEMS));
    count_launch();
    k_volume_noalloc<<<blocks, EW>>>(nel, xPhys_dev, volfrac, dgdx_dev, s);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(gx, &s->gx, sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_error(std::string("topo_volume_constraint_noalloc_dev: ") + cudaGetErrorString(e));
        return TOPO_ERR_CUDA;
    }
    return TOPO_OK;
}
