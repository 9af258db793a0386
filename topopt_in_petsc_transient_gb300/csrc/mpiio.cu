// mpiio.cu -- result files in the layout of the reference's MPIIO writer
// (MPIIO.cc:32-150 mesh, :409-717 header/points/cells, :724-935 datasets), the
// input format of bin2vtu.py (bin2vtu.py:18-150, readHeader :190-205).
//
// File layout, one domain, native byte order (little-endian on x86-64 and
// aarch64 alike, the "native" MPI data representation of the reference):
//   "TopOpt result version 1.1\n\x01"
//   uint64 {nDom = 1, nPointsT, nCellsT, nPFields, nCFields, nodesPerElement = 8}
//   point field names '\x01', cell field names '\x01'   (comma separated)
//   float32 x, y, z per node                            (DMDA natural order)
//   uint64 8 node ids per cell, uint64 offsets 8 (e+1), uint64 types 12
//   per dataset: uint64 itr, float32 point fields (field-major, nn values
//   each), float32 cell fields (field-major, nel values each)
// The node numbering of a cell follows DMDAGetElements_3D (MPIIO.cc:966-1016):
// n0 = (i, j, k), n1 = n0 + x, n2 = n0 + x + y, n3 = n0 + y, n4..n7 = n0..n3 + z.
//
// GB300 design: a dataset is never assembled on the host.  One kernel per
// field array converts FP64 device data to float32 and scatters the
// DOF-interleaved nodal vectors into the field-major record while it stores
// straight into mapped pinned host memory (over NVLink-C2C on Grace); a
// writer thread waits on the dataset's event and appends it to the file, so
// the disk write of block c overlaps the device work of block c + 1.  A ring
// of `slots` such records bounds the pinned memory.
#include <algorithm>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "le.h"
#include "mpiio.h"

namespace {

struct Slot {
    float *h = nullptr;   // host view of the record's float32 values
    float *d = nullptr;   // device view (mapped pinned memory), null without a device
    cudaEvent_t ev = nullptr;
    bool pending_ev = false;  // the record is being produced by device work up to `ev`
    bool busy = false;        // queued for (or being written by) the writer thread
    unsigned long long itr = 0;
};

constexpr int PACK_THREADS = 256;

__global__ void k_pack_nodal(long long nn, const double *__restrict__ u, float *__restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nn; i += (long long)gridDim.x * blockDim.x) {
        const double x = u[3 * i], y = u[3 * i + 1], z = u[3 * i + 2];
        out[i] = (float)x;
        out[nn + i] = (float)y;
        out[2 * nn + i] = (float)z;
    }
}

__global__ void k_pack_cells(long long n, const double *__restrict__ v, float *__restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (float)v[i];
}

}  // namespace

struct topo_mpiio {
    std::string path;
    int nx = 0, ny = 0, nz = 0;
    long long nn = 0, nel = 0;
    int npf = 0, ncf = 0;
    size_t rec = 0;  // float32 values per dataset
    FILE *f = nullptr;
    int device = -1;  // CUDA device the slots are mapped into (-1: host-only writer)
    int grid = 0;
    std::vector<Slot> slots;
    int next = 0, last = -1;
    // writer thread
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<int> q;
    int inflight = 0;
    bool stop = false;
    int werr = TOPO_OK;
    std::string werr_msg;
};

namespace topo {

int mpiio_point_fields(const topo_mpiio *io) { return io->npf; }
int mpiio_cell_fields(const topo_mpiio *io) { return io->ncf; }
long long mpiio_points(const topo_mpiio *io) { return io->nn; }
long long mpiio_cells(const topo_mpiio *io) { return io->nel; }

}  // namespace topo

using namespace topo;

namespace {

void writer_loop(topo_mpiio *io) {
    if (io->device >= 0) cudaSetDevice(io->device);
    for (;;) {
        int s;
        {
            std::unique_lock<std::mutex> lk(io->mu);
            io->cv.wait(lk, [io] { return io->stop || !io->q.empty(); });
            if (io->q.empty()) return;  // stop requested and nothing left
            s = io->q.front();
            io->q.pop_front();
        }
        Slot &sl = io->slots[s];
        int err = TOPO_OK;
        std::string msg;
        if (sl.pending_ev) {
            cudaError_t e = cudaEventSynchronize(sl.ev);
            if (e != cudaSuccess) {
                err = TOPO_ERR_CUDA;
                msg = std::string("MPIIO dataset conversion: ") + cudaGetErrorString(e);
            }
        }
        bool failed_before;
        {
            std::lock_guard<std::mutex> lk(io->mu);
            failed_before = io->werr != TOPO_OK;
        }
        if (!err && !failed_before) {
            const uint64_t itr = sl.itr;
            bool ok = fwrite(&itr, sizeof(itr), 1, io->f) == 1;
            if (ok && io->rec) ok = fwrite(sl.h, sizeof(float), io->rec, io->f) == io->rec;
            if (!ok) {
                err = TOPO_ERR_ARG;
                msg = "MPIIO: write failed on " + io->path;
            }
        }
        {
            std::lock_guard<std::mutex> lk(io->mu);
            if (err && io->werr == TOPO_OK) {
                io->werr = err;
                io->werr_msg = msg;
            }
            sl.busy = false;
            sl.pending_ev = false;
            io->inflight--;
        }
        io->cv.notify_all();
    }
}

int report_writer_error(topo_mpiio *io) {
    std::lock_guard<std::mutex> lk(io->mu);
    if (io->werr != TOPO_OK) set_error(io->werr_msg);
    return io->werr;
}

template <class T>
bool put(FILE *f, const std::vector<T> &v) {
    return v.empty() || fwrite(v.data(), sizeof(T), v.size(), f) == v.size();
}

// banner, header, names, node coordinates and cells (MPIIO.cc:424-717)
bool write_mesh(topo_mpiio *io, const double *xc, const std::string &pnames, const std::string &cnames) {
    FILE *f = io->f;
    const std::string banner = std::string("TopOpt result version 1.1") + "\n\x01";
    bool ok = fwrite(banner.data(), 1, banner.size(), f) == banner.size();
    const uint64_t header[6] = {1, (uint64_t)io->nn, (uint64_t)io->nel, (uint64_t)io->npf, (uint64_t)io->ncf, 8};
    ok = ok && fwrite(header, sizeof(uint64_t), 6, f) == 6;
    const std::string names = pnames + "\x01" + cnames + "\x01";
    ok = ok && fwrite(names.data(), 1, names.size(), f) == names.size();
    const int nx = io->nx, ny = io->ny, nz = io->nz;
    // DMDASetUniformCoordinates: x_i = xmin + i (xmax - xmin) / (nx - 1), in double, stored as float
    const double hx = (xc[1] - xc[0]) / (nx - 1), hy = (xc[3] - xc[2]) / (ny - 1), hz = (xc[5] - xc[4]) / (nz - 1);
    std::vector<float> pts((size_t)3 * nx * ny);
    for (int k = 0; ok && k < nz; k++) {
        size_t c = 0;
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                pts[c++] = (float)(xc[0] + i * hx);
                pts[c++] = (float)(xc[2] + j * hy);
                pts[c++] = (float)(xc[4] + k * hz);
            }
        ok = put(f, pts);
    }
    const int ex = nx - 1, ey = ny - 1, ez = nz - 1;
    const uint64_t sy = (uint64_t)nx, sz = (uint64_t)nx * ny;
    std::vector<uint64_t> conn((size_t)8 * ex * ey);
    for (int k = 0; ok && k < ez; k++) {
        size_t c = 0;
        for (int j = 0; j < ey; j++)
            for (int i = 0; i < ex; i++) {
                const uint64_t n0 = (uint64_t)i + sy * j + sz * k;
                const uint64_t q[4] = {n0, n0 + 1, n0 + 1 + sy, n0 + sy};
                for (int r = 0; r < 4; r++) conn[c + r] = q[r];
                for (int r = 0; r < 4; r++) conn[c + 4 + r] = q[r] + sz;
                c += 8;
            }
        ok = put(f, conn);
    }
    const size_t chunk = (size_t)1 << 20;
    std::vector<uint64_t> buf;
    for (long long e = 0; ok && e < io->nel; e += (long long)chunk) {  // offsets: end of each cell's node list
        const size_t m = (size_t)std::min<long long>((long long)chunk, io->nel - e);
        buf.resize(m);
        for (size_t r = 0; r < m; r++) buf[r] = 8 * (uint64_t)(e + (long long)r + 1);
        ok = put(f, buf);
    }
    for (long long e = 0; ok && e < io->nel; e += (long long)chunk) {  // VTK_HEXAHEDRON
        const size_t m = (size_t)std::min<long long>((long long)chunk, io->nel - e);
        buf.assign(m, 12);
        ok = put(f, buf);
    }
    return ok;
}

void free_slots(topo_mpiio *io) {
    for (Slot &s : io->slots) {
        if (s.ev) cudaEventDestroy(s.ev);
        if (s.h) {
            if (io->device >= 0)
                cudaFreeHost(s.h);
            else
                free(s.h);
        }
        s = Slot();
    }
}

}  // namespace

namespace topo {

int mpiio_write(topo_mpiio *io, unsigned long long itr, const double *const *nodal, int n_nodal,
                const double *const *cells, int n_cells, int on_device, cudaStream_t stream) {
    if (!io || n_nodal < 0 || n_cells != io->ncf || (n_nodal > 0 && 3 * n_nodal != io->npf) ||
        (n_nodal > 0 && !nodal) || (n_cells > 0 && !cells)) {
        set_error("MPIIO WriteVTK: " + std::to_string(n_nodal) + " nodal vectors and " + std::to_string(n_cells) +
                  " cell fields given, the file holds " + std::to_string(io ? io->npf : 0) + " point fields (3 per "
                  "vector, or 0 vectors to repeat the last) and " + std::to_string(io ? io->ncf : 0) + " cell fields");
        return TOPO_ERR_ARG;
    }
    for (int v = 0; v < n_nodal; v++)
        if (!nodal[v]) {
            set_error("MPIIO WriteVTK: null nodal vector");
            return TOPO_ERR_ARG;
        }
    for (int v = 0; v < n_cells; v++)
        if (!cells[v]) {
            set_error("MPIIO WriteVTK: null cell field");
            return TOPO_ERR_ARG;
        }
    if (on_device && io->device < 0) {
        set_error("MPIIO WriteVTK: device arrays given to a writer created without a CUDA device");
        return TOPO_ERR_CUDA;
    }
    int rc = report_writer_error(io);
    if (rc) return rc;
    const int s = io->next;
    Slot &sl = io->slots[s];
    {
        std::unique_lock<std::mutex> lk(io->mu);
        io->cv.wait(lk, [&] { return !sl.busy; });
    }
    const long long nn = io->nn, nel = io->nel;
    float *cellbase_h = sl.h + (size_t)io->npf * nn;
    if (n_nodal == 0 && io->npf > 0) {  // repeat the previous dataset's point fields (zeros before the first)
        if (io->last < 0) {
            memset(sl.h, 0, sizeof(float) * (size_t)io->npf * nn);
        } else {
            Slot &pv = io->slots[io->last];
            if (pv.ev) {  // its conversion may still be running on the device (no-op if never recorded)
                cudaError_t e = cudaEventSynchronize(pv.ev);
                if (e != cudaSuccess) {
                    set_error(std::string("MPIIO WriteVTK: ") + cudaGetErrorString(e));
                    return TOPO_ERR_CUDA;
                }
            }
            memcpy(sl.h, pv.h, sizeof(float) * (size_t)io->npf * nn);
        }
    }
    bool used_device = false;
    if (on_device) {
        float *cellbase_d = sl.d + (size_t)io->npf * nn;
        const int gn = (int)std::min<long long>((nn + PACK_THREADS - 1) / PACK_THREADS, io->grid);
        const int gc = (int)std::min<long long>((nel + PACK_THREADS - 1) / PACK_THREADS, io->grid);
        for (int v = 0; v < n_nodal; v++) {
            count_launch();
            k_pack_nodal<<<gn, PACK_THREADS, 0, stream>>>(nn, nodal[v], sl.d + (size_t)3 * v * nn);
        }
        for (int v = 0; v < n_cells; v++) {
            count_launch();
            k_pack_cells<<<gc, PACK_THREADS, 0, stream>>>(nel, cells[v], cellbase_d + (size_t)v * nel);
        }
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(sl.ev, stream);
        if (e != cudaSuccess) {
            set_error(std::string("MPIIO WriteVTK: ") + cudaGetErrorString(e));
            return TOPO_ERR_CUDA;
        }
        used_device = n_nodal + n_cells > 0;
    } else {
        for (int v = 0; v < n_nodal; v++) {
            const double *u = nodal[v];
            float *o = sl.h + (size_t)3 * v * nn;
            for (long long i = 0; i < nn; i++) {
                o[i] = (float)u[3 * i];
                o[nn + i] = (float)u[3 * i + 1];
                o[2 * nn + i] = (float)u[3 * i + 2];
            }
        }
        for (int v = 0; v < n_cells; v++) {
            const double *x = cells[v];
            float *o = cellbase_h + (size_t)v * nel;
            for (long long i = 0; i < nel; i++) o[i] = (float)x[i];
        }
    }
    {
        std::lock_guard<std::mutex> lk(io->mu);
        sl.itr = itr;
        sl.pending_ev = used_device;
        sl.busy = true;
        io->inflight++;
        io->q.push_back(s);
    }
    io->cv.notify_all();
    io->last = s;
    io->next = (s + 1) % (int)io->slots.size();
    return TOPO_OK;
}

}  // namespace topo

extern "C" {

int topo_mpiio_create(topo_mpiio **out, int nx, int ny, int nz, const double *xc, int npf, const char *pnames,
                      int ncf, const char *cnames, const char *filename, int slots) {
    if (!out || !filename || !xc || nx < 2 || ny < 2 || nz < 2 || npf < 0 || ncf < 0 || slots < 0 || slots == 1) {
        set_error("topo_mpiio_create: output pointer, file name, box xc[6], nx, ny, nz >= 2, npf, ncf >= 0 and "
                  "slots = 0 or >= 2 required");
        return TOPO_ERR_ARG;
    }
    *out = nullptr;
    topo_mpiio *io = new topo_mpiio();
    io->path = filename;
    io->nx = nx;
    io->ny = ny;
    io->nz = nz;
    io->nn = (long long)nx * ny * nz;
    io->nel = (long long)(nx - 1) * (ny - 1) * (nz - 1);
    io->npf = npf;
    io->ncf = ncf;
    io->rec = (size_t)npf * io->nn + (size_t)ncf * io->nel;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        io->device = -1;
    } else {
        cudaGetDevice(&io->device);
        int nsm = 0;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, io->device);
        io->grid = (nsm > 0 ? nsm : 1) * 8;
    }
    io->f = fopen(filename, "wb");
    if (!io->f) {
        set_error(std::string("topo_mpiio_create: cannot open ") + filename);
        delete io;
        return TOPO_ERR_ARG;
    }
    if (!write_mesh(io, xc, pnames ? pnames : "", cnames ? cnames : "")) {
        set_error(std::string("topo_mpiio_create: write failed on ") + filename);
        fclose(io->f);
        delete io;
        return TOPO_ERR_ARG;
    }
    io->slots.resize(slots ? slots : 4);
    const size_t bytes = sizeof(float) * (io->rec ? io->rec : 1);
    for (Slot &s : io->slots) {
        if (io->device >= 0) {
            void *h = nullptr, *d = nullptr;
            cudaError_t e = cudaHostAlloc(&h, bytes, cudaHostAllocMapped | cudaHostAllocPortable);
            if (e == cudaSuccess) e = cudaHostGetDevicePointer(&d, h, 0);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming);
            s.h = (float *)h;
            s.d = (float *)d;
            if (e != cudaSuccess) {
                set_error(std::string("topo_mpiio_create: pinned dataset buffers: ") + cudaGetErrorString(e));
                free_slots(io);
                fclose(io->f);
                delete io;
                return TOPO_ERR_OOM;
            }
        } else {
            s.h = (float *)malloc(bytes);
            if (!s.h) {
                set_error("topo_mpiio_create: out of host memory");
                free_slots(io);
                fclose(io->f);
                delete io;
                return TOPO_ERR_OOM;
            }
        }
    }
    io->th = std::thread(writer_loop, io);
    *out = io;
    return TOPO_OK;
}

int topo_mpiio_flush(topo_mpiio *io) {
    if (!io) {
        set_error("topo_mpiio_flush: null writer");
        return TOPO_ERR_ARG;
    }
    {
        std::unique_lock<std::mutex> lk(io->mu);
        io->cv.wait(lk, [io] { return io->inflight == 0; });
    }
    if (fflush(io->f) != 0) {
        set_error("MPIIO: flush failed on " + io->path);
        return TOPO_ERR_ARG;
    }
    return report_writer_error(io);
}

void topo_mpiio_destroy(topo_mpiio *io) {
    if (!io) return;
    {
        std::unique_lock<std::mutex> lk(io->mu);
        io->cv.wait(lk, [io] { return io->inflight == 0; });
        io->stop = true;
    }
    io->cv.notify_all();
    if (io->th.joinable()) io->th.join();
    fclose(io->f);
    free_slots(io);
    delete io;
}

int topo_mpiio_write(topo_mpiio *io, unsigned long long itr, const double *const *nodal, int n_nodal,
                     const double *const *cells, int n_cells, int on_device, void *stream) {
    return mpiio_write(io, itr, nodal, n_nodal, cells, n_cells, on_device, (cudaStream_t)stream);
}

}  // extern "C"
