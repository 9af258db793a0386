// densfilt.cu -- Filter for filterType 0 (sensitivity filter) and 1 (density
// filter), Filter.cc:60-206 and :302-531, on the element grid.
//
// H has entries R - dist between element centres for dist < R inside a box
// stencil: half-width ElemConn = max_a(ceil(R/h_a) - 1) (at least 1), the
// range along axis a running from max(i - ElemConn, 0) to
// min(i + ElemConn, n_a - 1, i + ceil(R/h_a) - 1) (Filter.cc:467-469); with
// ElemConn == 1 H is the identity (:451-459).  Hs = H 1.  The reference
// assembles H as a sparse matrix; here the weights depend only on the element
// offset, so one table of (2 ElemConn + 1)^3 weights and one stencil kernel
// apply H on the fly, summing the neighbours in the reference's column order.
//   filter 1: xTilde = (H x) ./ Hs;  dfdx, dgdx <- H (v ./ Hs)
//   filter 0: xTilde = x;           dfdx <- ((H (dfdx .* x)) ./ Hs) ./ x
// followed / preceded by the smoothed Heaviside projection and its chain rule
// (Filter.h:80-88).
#include <cmath>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "le.h"

namespace topo {

struct TopoDensFilt {
    int ex = 0, ey = 0, ez = 0, ftype = 1, sw = 1;
    int lim[3] = {0, 0, 0};  // upper offsets along x, y, z: min(sw, ceil(R/h_a) - 1)
    bool identity = true;
    long long nel = 0;
    double *w = nullptr;    // (2 sw + 1)^3 weights, offsets (dz, dy, dx) with dx fastest
    double *hs = nullptr;   // row sums of H
    double *tmp = nullptr;  // in-place scratch
    double *part = nullptr;           // per-CTA partial sums of the MND reduction, and its result
    unsigned int *counter = nullptr;
    cudaStream_t stream = nullptr;
};

// pre-scaling of the neighbour value and post-scaling of the sum
enum { DF_PRE_NONE = 0, DF_PRE_DIV_HS = 1, DF_PRE_MUL_X = 2 };
enum { DF_POST_NONE = 0, DF_POST_DIV_HS = 1, DF_POST_DIV_HS_X = 2 };

// y_e = post_e(sum_{e2} w(e2 - e) pre_e2(v_e2))
static __global__ void k_dens_apply(int ex, int ey, int ez, int sw, int lx, int ly, int lz,
                                    const double *__restrict__ w, const double *__restrict__ v,
                                    const double *__restrict__ hs, const double *__restrict__ x, int pre, int post,
                                    double *__restrict__ y) {
    const long long nel = (long long)ex * ey * ez;
    const int S = 2 * sw + 1;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nel; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % ex), j = (int)((e / ex) % ey), k = (int)(e / ((long long)ex * ey));
        const int k0 = -min(sw, k), k1 = min(lz, ez - 1 - k);
        const int j0 = -min(sw, j), j1 = min(ly, ey - 1 - j);
        const int i0 = -min(sw, i), i1 = min(lx, ex - 1 - i);
        double acc = 0.0;
        for (int dk = k0; dk <= k1; dk++)
            for (int dj = j0; dj <= j1; dj++) {
                const double *wr = w + ((dk + sw) * S + (dj + sw)) * S + sw;
                const long long row = (long long)ex * ((j + dj) + (long long)ey * (k + dk)) + i;
                for (int di = i0; di <= i1; di++) {
                    const double wt = wr[di];
                    if (wt == 0.0) continue;
                    const long long e2 = row + di;
                    double val = v[e2];
                    if (pre == DF_PRE_DIV_HS) val = val / hs[e2];
                    else if (pre == DF_PRE_MUL_X) val = val * x[e2];
                    acc += wt * val;
                }
            }
        if (post == DF_POST_DIV_HS) acc = acc / hs[e];
        else if (post == DF_POST_DIV_HS_X) acc = (acc / hs[e]) / x[e];
        y[e] = acc;
    }
}

// identity H (ElemConn == 1): the same scalings with Hs = 1, so only the
// factors x of the sensitivity filter remain
static __global__ void k_dens_identity(long long nel, const double *__restrict__ v, const double *__restrict__ x,
                                       int pre, int post, double *__restrict__ y) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nel; e += (long long)gridDim.x * blockDim.x) {
        double acc = (pre == DF_PRE_MUL_X) ? v[e] * x[e] : v[e];
        if (post == DF_POST_DIV_HS_X) acc = acc / x[e];
        y[e] = acc;
    }
}

// Filter::GetMND (Filter.cc:208-227): mean of 4 x (1 - x)
static __global__ void k_dens_mnd(long long n, const double *__restrict__ x, Partials<1> part, double *out) {
    double v[1] = {0.0};
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        v[0] += 4 * x[e] * (1.0 - x[e]);
    double tot[1];
    if (grid_reduce<EW, 1>(v, part, tot)) *out = tot[0] / (double)n;
}

static __global__ void k_dens_fill(long long n, double v, double *y) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        y[e] = v;
}

// xPhys from xTilde: smoothed Heaviside projection or copy (Filter.cc:110-116)
static __global__ void k_dens_project(long long nel, const double *__restrict__ xt, double *xp, int projection,
                                      double beta, double eta) {
    const double den = tanh(beta * eta) + tanh(beta * (1.0 - eta));
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nel; e += (long long)gridDim.x * blockDim.x)
        xp[e] = projection ? (tanh(beta * eta) + tanh(beta * (xt[e] - eta))) / den : xt[e];
}

// chain rule of the projection (Filter.cc:128-169)
static __global__ void k_dens_chain(long long nel, const double *__restrict__ xt, double *df, int m, double *dg,
                                    double beta, double eta) {
    const double den = tanh(beta * eta) + tanh(beta * (1.0 - eta));
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nel; e += (long long)gridDim.x * blockDim.x) {
        const double t = tanh(beta * (xt[e] - eta));
        const double d = beta * (1.0 - t * t) / den;
        df[e] *= d;
        for (int j = 0; j < m; j++) dg[(long long)j * nel + e] *= d;
    }
}

#define DCK(call)                                                            \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) {                                             \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));  \
            return TOPO_ERR_CUDA;                                            \
        }                                                                    \
    } while (0)

static void dens_apply(TopoDensFilt *f, const double *v, const double *x, int pre, int post, double *y) {
    count_launch();
    if (f->identity)
        k_dens_identity<<<ew_blocks(f->nel), EW, 0, f->stream>>>(f->nel, v, x, pre, post, y);
    else
        k_dens_apply<<<ew_blocks(f->nel), EW, 0, f->stream>>>(f->ex, f->ey, f->ez, f->sw, f->lim[0], f->lim[1],
                                                              f->lim[2], f->w, v, f->hs, x, pre, post, y);
}

static void dens_destroy(TopoDensFilt *f) {
    if (!f) return;
    cudaFree(f->w);
    cudaFree(f->hs);
    cudaFree(f->tmp);
    cudaFree(f->part);
    cudaFree(f->counter);
    if (f->stream) cudaStreamDestroy(f->stream);
    delete f;
}

static int dens_create(TopoDensFilt **out, int ex, int ey, int ez, double hx, double hy, double hz, int ftype,
                       double R) {
    *out = nullptr;
    if (ex < 1 || ey < 1 || ez < 1 || hx <= 0.0 || hy <= 0.0 || hz <= 0.0 || !(R > 0.0) || (ftype != 0 && ftype != 1)) {
        set_error("Filter: filter type 0 or 1, positive element sizes and radius");
        return TOPO_ERR_ARG;
    }
    TopoDensFilt *f = new TopoDensFilt();
    f->ex = ex;
    f->ey = ey;
    f->ez = ez;
    f->ftype = ftype;
    f->nel = (long long)ex * ey * ez;
    const double h[3] = {hx, hy, hz};
    int sw = 0;
    for (int a = 0; a < 3; a++) {
        f->lim[a] = (int)std::ceil(R / h[a]) - 1;
        sw = std::max(sw, f->lim[a]);
    }
    if (sw == 0) sw = 1;  // Filter.cc:396-398
    f->sw = sw;
    f->identity = (sw == 1);  // Filter.cc:451-459
    for (int a = 0; a < 3; a++) f->lim[a] = std::min(f->lim[a], sw);
    const int S = 2 * sw + 1;
    std::vector<double> w((size_t)S * S * S, 0.0);
    for (int dk = -sw; dk <= sw; dk++)
        for (int dj = -sw; dj <= sw; dj++)
            for (int di = -sw; di <= sw; di++) {
                // element centres h/2 + i h (DMDASetUniformCoordinates, Filter.cc:420)
                const double d0 = (hx / 2 + di * hx) - hx / 2, d1 = (hy / 2 + dj * hy) - hy / 2,
                             d2 = (hz / 2 + dk * hz) - hz / 2;
                const double dist = std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                w[((size_t)(dk + sw) * S + (dj + sw)) * S + (di + sw)] = dist < R ? R - dist : 0.0;
            }
    bool ok = cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&f->w, sizeof(double) * w.size()) == cudaSuccess &&
              cudaMalloc(&f->hs, sizeof(double) * f->nel) == cudaSuccess &&
              cudaMalloc(&f->tmp, sizeof(double) * f->nel) == cudaSuccess &&
              cudaMalloc(&f->part, sizeof(double) * (red_blocks(f->nel) + 1)) == cudaSuccess &&
              cudaMalloc(&f->counter, sizeof(unsigned int)) == cudaSuccess &&
              cudaMemset(f->counter, 0, sizeof(unsigned int)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        dens_destroy(f);
        set_error("Filter: device allocation failed");
        return TOPO_ERR_OOM;
    }
    cudaError_t e = cudaMemcpy(f->w, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        count_launch();
        k_dens_fill<<<ew_blocks(f->nel), EW, 0, f->stream>>>(f->nel, 1.0, f->tmp);
        if (f->identity) {
            count_launch();
            k_dens_fill<<<ew_blocks(f->nel), EW, 0, f->stream>>>(f->nel, 1.0, f->hs);
        } else {
            dens_apply(f, f->tmp, nullptr, DF_PRE_NONE, DF_POST_NONE, f->hs);  // Hs = H 1 (Filter.cc:505-509)
        }
        e = cudaStreamSynchronize(f->stream);
    }
    if (e != cudaSuccess) {
        set_error(std::string("Filter set-up: ") + cudaGetErrorString(e));
        dens_destroy(f);
        return TOPO_ERR_CUDA;
    }
    *out = f;
    return TOPO_OK;
}

static int dens_project_dev(TopoDensFilt *f, const double *x, double *xt, double *xp, int projection, double beta,
                            double eta) {
    if (f->ftype == 1)
        dens_apply(f, x, nullptr, DF_PRE_NONE, DF_POST_DIV_HS, xt);
    else
        DCK(cudaMemcpyAsync(xt, x, sizeof(double) * f->nel, cudaMemcpyDeviceToDevice, f->stream));
    count_launch();
    k_dens_project<<<ew_blocks(f->nel), EW, 0, f->stream>>>(f->nel, xt, xp, projection, beta, eta);
    DCK(cudaGetLastError());
    DCK(cudaStreamSynchronize(f->stream));
    return TOPO_OK;
}

static int dens_gradients_dev(TopoDensFilt *f, const double *x, const double *xt, double *df, int m, double *dg,
                              int projection, double beta, double eta) {
    const size_t b = sizeof(double) * f->nel;
    if (projection) {
        count_launch();
        k_dens_chain<<<ew_blocks(f->nel), EW, 0, f->stream>>>(f->nel, xt, df, m, dg, beta, eta);
    }
    if (f->ftype == 0) {  // sensitivity filter: dfdx only (Filter.cc:172-181)
        DCK(cudaMemcpyAsync(f->tmp, df, b, cudaMemcpyDeviceToDevice, f->stream));
        dens_apply(f, f->tmp, x, DF_PRE_MUL_X, DF_POST_DIV_HS_X, df);
    } else {  // density filter: dfdx and every dgdx (Filter.cc:182-195)
        for (int j = -1; j < m; j++) {
            double *v = j < 0 ? df : dg + (size_t)j * f->nel;
            DCK(cudaMemcpyAsync(f->tmp, v, b, cudaMemcpyDeviceToDevice, f->stream));
            dens_apply(f, f->tmp, nullptr, DF_PRE_DIV_HS, DF_POST_NONE, v);
        }
    }
    DCK(cudaGetLastError());
    DCK(cudaStreamSynchronize(f->stream));
    return TOPO_OK;
}

static int dens_mnd_dev(TopoDensFilt *f, const double *x, double *mnd) {
    const unsigned nb = red_blocks(f->nel);
    count_launch();
    k_dens_mnd<<<nb, EW, 0, f->stream>>>(f->nel, x, Partials<1>{f->part, f->counter}, f->part + nb);
    DCK(cudaMemcpyAsync(mnd, f->part + nb, sizeof(double), cudaMemcpyDeviceToHost, f->stream));
    DCK(cudaStreamSynchronize(f->stream));
    return TOPO_OK;
}

}  // namespace topo

using namespace topo;

struct topo_densfilt {
    TopoDensFilt *impl = nullptr;
    long long nel = 0;
    double *d_a = nullptr, *d_b = nullptr, *d_c = nullptr, *d_d = nullptr, *d_g = nullptr;  // host-call staging
    int gcap = 2;
};

extern "C" {

int topo_densfilt_create(topo_densfilt **out, int nelx, int nely, int nelz, double hx, double hy, double hz,
                         int filter_type, double rmin) {
    if (!out) return TOPO_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device available: the GB300 path has no CPU fallback");
        return TOPO_ERR_CUDA;
    }
    TopoDensFilt *impl = nullptr;
    int rc = dens_create(&impl, nelx, nely, nelz, hx, hy, hz, filter_type, rmin);
    if (rc) return rc;
    topo_densfilt *h = new topo_densfilt();
    h->impl = impl;
    h->nel = impl->nel;
    const size_t b = sizeof(double) * h->nel;
    bool ok = cudaMalloc(&h->d_a, b) == cudaSuccess && cudaMalloc(&h->d_b, b) == cudaSuccess &&
              cudaMalloc(&h->d_c, b) == cudaSuccess && cudaMalloc(&h->d_d, b) == cudaSuccess &&
              cudaMalloc(&h->d_g, b * h->gcap) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        topo_densfilt_destroy(h);
        set_error("device allocation of Filter staging buffers failed");
        return TOPO_ERR_OOM;
    }
    *out = h;
    return TOPO_OK;
}

void topo_densfilt_destroy(topo_densfilt *f) {
    if (!f) return;
    dens_destroy(f->impl);
    cudaFree(f->d_a);
    cudaFree(f->d_b);
    cudaFree(f->d_c);
    cudaFree(f->d_d);
    cudaFree(f->d_g);
    delete f;
}

int topo_densfilt_filter_project_dev(topo_densfilt *f, const double *x_dev, double *xTilde_dev, double *xPhys_dev,
                                     int projection, double beta, double eta) {
    if (!f || !x_dev || !xTilde_dev || !xPhys_dev) return TOPO_ERR_ARG;
    return dens_project_dev(f->impl, x_dev, xTilde_dev, xPhys_dev, projection, beta, eta);
}

int topo_densfilt_filter_project(topo_densfilt *f, const double *x, double *xTilde, double *xPhys, int projection,
                                 double beta, double eta) {
    if (!f || !x || !xTilde || !xPhys) return TOPO_ERR_ARG;
    const size_t b = sizeof(double) * f->nel;
    DCK(cudaMemcpy(f->d_a, x, b, cudaMemcpyHostToDevice));
    int rc = dens_project_dev(f->impl, f->d_a, f->d_b, f->d_c, projection, beta, eta);
    if (rc) return rc;
    DCK(cudaMemcpy(xTilde, f->d_b, b, cudaMemcpyDeviceToHost));
    DCK(cudaMemcpy(xPhys, f->d_c, b, cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

int topo_densfilt_gradients_dev(topo_densfilt *f, const double *x_dev, const double *xTilde_dev, double *dfdx_dev,
                                int m, double *dgdx_dev, int projection, double beta, double eta) {
    if (!f || !x_dev || !xTilde_dev || !dfdx_dev || m < 0 || (m > 0 && !dgdx_dev)) return TOPO_ERR_ARG;
    return dens_gradients_dev(f->impl, x_dev, xTilde_dev, dfdx_dev, m, dgdx_dev, projection, beta, eta);
}

int topo_densfilt_gradients(topo_densfilt *f, const double *x, const double *xTilde, double *dfdx, int m,
                            double *dgdx, int projection, double beta, double eta) {
    if (!f || !x || !xTilde || !dfdx || m < 0 || m > f->gcap || (m > 0 && !dgdx)) return TOPO_ERR_ARG;
    const size_t b = sizeof(double) * f->nel;
    DCK(cudaMemcpy(f->d_a, x, b, cudaMemcpyHostToDevice));
    DCK(cudaMemcpy(f->d_b, xTilde, b, cudaMemcpyHostToDevice));
    DCK(cudaMemcpy(f->d_c, dfdx, b, cudaMemcpyHostToDevice));
    if (m) DCK(cudaMemcpy(f->d_g, dgdx, b * m, cudaMemcpyHostToDevice));
    int rc = dens_gradients_dev(f->impl, f->d_a, f->d_b, f->d_c, m, f->d_g, projection, beta, eta);
    if (rc) return rc;
    DCK(cudaMemcpy(dfdx, f->d_c, b, cudaMemcpyDeviceToHost));
    if (m) DCK(cudaMemcpy(dgdx, f->d_g, b * m, cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

int topo_densfilt_mnd_dev(topo_densfilt *f, const double *x_dev, double *mnd) {
    if (!f || !x_dev || !mnd) return TOPO_ERR_ARG;
    return dens_mnd_dev(f->impl, x_dev, mnd);
}

int topo_densfilt_mnd(topo_densfilt *f, const double *x, double *mnd) {
    if (!f || !x || !mnd) return TOPO_ERR_ARG;
    DCK(cudaMemcpy(f->d_a, x, sizeof(double) * f->nel, cudaMemcpyHostToDevice));
    return dens_mnd_dev(f->impl, f->d_a, mnd);
}

}  // extern "C"
