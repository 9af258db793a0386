// petscio.cu -- PETSc binary vector records (the format VecView / VecLoad use
// with a binary viewer): a big-endian int32 class id 1211214, a big-endian
// int32 length n, then n big-endian doubles; several records are appended
// to one file (Restart0x.dat, RestartSol0x.dat, cp%04d.dat of the reference:
// TopOpt.cc:722-727, LinearElasticity.cc:1134-1136, :2482-2484).  Vectors are
// in DMDA natural order, the order every array of this library uses.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "le.h"

namespace topo {

static const int PETSC_VEC_CLASSID = 1211214;

static void put_be32(unsigned char *p, unsigned int v) {
    p[0] = (unsigned char)(v >> 24);
    p[1] = (unsigned char)(v >> 16);
    p[2] = (unsigned char)(v >> 8);
    p[3] = (unsigned char)v;
}
static unsigned int get_be32(const unsigned char *p) {
    return ((unsigned int)p[0] << 24) | ((unsigned int)p[1] << 16) | ((unsigned int)p[2] << 8) | (unsigned int)p[3];
}
static void put_be64(unsigned char *p, double d) {
    unsigned long long v;
    memcpy(&v, &d, 8);
    for (int i = 0; i < 8; i++) p[i] = (unsigned char)(v >> (56 - 8 * i));
}
static double get_be64(const unsigned char *p) {
    unsigned long long v = 0;
    for (int i = 0; i < 8; i++) v = (v << 8) | p[i];
    double d;
    memcpy(&d, &v, 8);
    return d;
}

// host copy of n values (device arrays are copied out first)
static int host_values(const double *v, long long n, int on_device, std::vector<double> &tmp, const double **out) {
    if (!on_device) {
        *out = v;
        return TOPO_OK;
    }
    tmp.resize((size_t)n);
    cudaError_t e = cudaMemcpy(tmp.data(), v, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_error(std::string("PETSc vector write: ") + cudaGetErrorString(e));
        return TOPO_ERR_CUDA;
    }
    *out = tmp.data();
    return TOPO_OK;
}

}  // namespace topo

using namespace topo;

extern "C" {

int topo_petsc_vec_write(const char *path, int append, const double *v, long long n, int on_device) {
    if (!path || !v || n < 0 || n > 0x7fffffffLL) {
        set_error("topo_petsc_vec_write: path, values and 0 <= n < 2^31 required");
        return TOPO_ERR_ARG;
    }
    std::vector<double> tmp;
    const double *hv = nullptr;
    int rc = host_values(v, n, on_device, tmp, &hv);
    if (rc) return rc;
    FILE *f = fopen(path, append ? "ab" : "wb");
    if (!f) {
        set_error(std::string("topo_petsc_vec_write: cannot open ") + path);
        return TOPO_ERR_ARG;
    }
    unsigned char head[8];
    put_be32(head, (unsigned int)PETSC_VEC_CLASSID);
    put_be32(head + 4, (unsigned int)n);
    bool ok = fwrite(head, 1, 8, f) == 8;
    std::vector<unsigned char> buf(8 * 4096);
    for (long long i = 0; ok && i < n; i += 4096) {
        const long long m = (n - i < 4096) ? n - i : 4096;
        for (long long k = 0; k < m; k++) put_be64(buf.data() + 8 * k, hv[i + k]);
        ok = fwrite(buf.data(), 8, (size_t)m, f) == (size_t)m;
    }
    ok = (fclose(f) == 0) && ok;
    if (!ok) {
        set_error(std::string("topo_petsc_vec_write: write failed on ") + path);
        return TOPO_ERR_ARG;
    }
    return TOPO_OK;
}

int topo_petsc_vec_read(const char *path, int index, double *v, long long n, int on_device) {
    if (!path || !v || index < 0 || n < 0) {
        set_error("topo_petsc_vec_read: path, output array, index >= 0 and n >= 0 required");
        return TOPO_ERR_ARG;
    }
    FILE *f = fopen(path, "rb");
    if (!f) {
        set_error(std::string("topo_petsc_vec_read: cannot open ") + path);
        return TOPO_ERR_ARG;
    }
    unsigned char head[8];
    long long len = -1;
    for (int r = 0; r <= index; r++) {  // skip the records before `index`
        if (fread(head, 1, 8, f) != 8 || (int)get_be32(head) != PETSC_VEC_CLASSID) {
            fclose(f);
            set_error(std::string("topo_petsc_vec_read: no vector record ") + std::to_string(r) + " in " + path);
            return TOPO_ERR_ARG;
        }
        len = (long long)get_be32(head + 4);
        if (r < index && fseek(f, (long)(8 * len), SEEK_CUR) != 0) {
            fclose(f);
            set_error(std::string("topo_petsc_vec_read: truncated file ") + path);
            return TOPO_ERR_ARG;
        }
    }
    if (len != n) {
        fclose(f);
        set_error("topo_petsc_vec_read: record " + std::to_string(index) + " holds " + std::to_string(len) +
                  " values, " + std::to_string(n) + " expected");
        return TOPO_ERR_ARG;
    }
    std::vector<double> hv((size_t)n);
    std::vector<unsigned char> buf(8 * 4096);
    bool ok = true;
    for (long long i = 0; ok && i < n; i += 4096) {
        const long long m = (n - i < 4096) ? n - i : 4096;
        ok = fread(buf.data(), 8, (size_t)m, f) == (size_t)m;
        for (long long k = 0; ok && k < m; k++) hv[(size_t)(i + k)] = get_be64(buf.data() + 8 * k);
    }
    fclose(f);
    if (!ok) {
        set_error(std::string("topo_petsc_vec_read: truncated file ") + path);
        return TOPO_ERR_ARG;
    }
    if (on_device) {
        cudaError_t e = cudaMemcpy(v, hv.data(), sizeof(double) * (size_t)n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            set_error(std::string("topo_petsc_vec_read: ") + cudaGetErrorString(e));
            return TOPO_ERR_CUDA;
        }
    } else {
        memcpy(v, hv.data(), sizeof(double) * (size_t)n);
    }
    return TOPO_OK;
}

}  // extern "C"
