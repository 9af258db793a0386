// Runs the real k_slab and k_tile sources on host threads (one std::thread per
// CUDA thread, a std::barrier per CTA for __syncthreads) with test policies,
// and compares the two forms node by node.
#include <atomic>
#include <barrier>
#include <cstdio>
#include <random>
#include <thread>
#include <vector>

#include "df.cuh"
#include "slab.cuh"

thread_local emu_uint3 threadIdx, blockIdx;
emu_uint3 blockDim, gridDim;
static std::barrier<> *g_bar = nullptr;
void __syncthreads() { g_bar->arrive_and_wait(); }
namespace emu {
unsigned char dyn_smem[256 * 1024] __attribute__((aligned(16)));
}

static std::atomic<long> g_bad{0};

template <class T, int NIN_>
struct PolT {
    static constexpr int NIN = NIN_, NRED = 0;
    static constexpr bool HAS_K = true, HAS_M = true;
    const double *x0, *x1;
    double *y;
    int *writes;
    const double *kf, *mf;
    topo::Partials<1> part;
    struct Pre {
        long long n;
    };
    Pre pre(long long n) const { return Pre{n}; }
    void load(long long n, T v[NIN][3]) const {
        for (int c = 0; c < 3; c++) {
            v[0][c] = T(x0[3 * n + c]);
            if (NIN == 2) v[NIN - 1][c] = T(x1[3 * n + c]);
        }
    }
    void coef(long long e, T &ck, T &cm) const {
        ck = T(kf[e]);
        cm = T(mf[e]);
    }
    void epilogue(long long n, int, int, int, const T yv[3], double *, const Pre &r) const {
        if (r.n != n) g_bad++;
        for (int c = 0; c < 3; c++) y[3 * n + c] = topo::todbl(yv[c]);
        writes[n]++;
    }
    void finish(const double *) const {}
};

// a policy with grid reductions (NRED = 2): sums of y.x0 and y.y through
// grid_reduce, finish() called once by the last CTA
struct RedOut {
    double tot[2];
    int calls;
};
template <class T>
struct PolRed {
    static constexpr int NIN = 1, NRED = 2;
    static constexpr bool HAS_K = true, HAS_M = true;
    const double *x0;
    const double *kf, *mf;
    RedOut *out;
    topo::Partials<2> part;
    void load(long long n, T v[1][3]) const {
        for (int c = 0; c < 3; c++) v[0][c] = T(x0[3 * n + c]);
    }
    void coef(long long e, T &ck, T &cm) const {
        ck = T(kf[e]);
        cm = T(mf[e]);
    }
    void epilogue(long long n, int, int, int, const T yv[3], double red[2]) const {
        for (int c = 0; c < 3; c++) {
            const double y = topo::todbl(yv[c]);
            red[0] += y * x0[3 * n + c];
            red[1] += y * y;
        }
    }
    void finish(const double t[2]) const {
        out->tot[0] = t[0];
        out->tot[1] = t[1];
        out->calls++;
    }
};

template <class Body>
static void run_grid(unsigned grid, unsigned block, Body body) {
    gridDim = {grid, 1, 1};
    blockDim = {block, 1, 1};
    for (unsigned b = 0; b < grid; b++) {
        std::barrier<> bar((std::ptrdiff_t)block);
        g_bar = &bar;
        std::vector<std::thread> th;
        th.reserve(block);
        for (unsigned t = 0; t < block; t++)
            th.emplace_back([=] {
                threadIdx = {t, 0, 0};
                blockIdx = {b, 0, 0};
                body();
            });
        for (auto &x : th) x.join();
    }
}

template <class T, int NIN>
static bool compare(int nx, int ny, int nz, long long slots, unsigned brick_grid) {
    using namespace topo;
    GridDesc g{nx, ny, nz, nx - 1, ny - 1, nz - 1};
    const long long nn = g.nn(), nel = g.nel();
    std::mt19937_64 rng(nx * 1000 + ny * 10 + nz);
    std::uniform_real_distribution<double> U(-1.0, 1.0), P(0.1, 1.0);
    std::vector<double> x0(3 * nn), x1(3 * nn), kf(nel), mf(nel), ya(3 * nn, -7.0), yb(3 * nn, -7.0);
    for (auto &v : x0) v = U(rng);
    for (auto &v : x1) v = U(rng);
    for (auto &v : kf) v = P(rng);
    for (auto &v : mf) v = P(rng);
    std::vector<int> wa(nn, 0), wb(nn, 0);
    const ElemConst<T> C = make_elem_const<T>(1.0, 0.8, 1.25, 0.3);
    PolT<T, NIN> pa{x0.data(), x1.data(), ya.data(), wa.data(), kf.data(), mf.data(), {}};
    PolT<T, NIN> pb{x0.data(), x1.data(), yb.data(), wb.data(), kf.data(), mf.data(), {}};
    // brick form: persistent (FP32) with the given grid, else one CTA per brick
    int ntx, nty;
    const int ntiles = tile_count(g, ntx, nty);
    if (!tile_persistent<T>()) brick_grid = (unsigned)ntiles;
    run_grid(brick_grid, TILE_THREADS, [&] { k_tile<T, PolT<T, NIN>>(g, C, pa); });
    // slab form
    const SlabShape sh = slab_shape(g, slots);
    run_grid((unsigned)(sh.ncx * sh.ncy * sh.nzr), SLAB_THREADS, [&] { k_slab<T, PolT<T, NIN>>(g, C, pb, sh); });
    long diff = 0, wbad = 0;
    double maxd = 0.0;
    for (long long n = 0; n < nn; n++) {
        if (wa[n] != 1 || wb[n] != 1) wbad++;
        for (int c = 0; c < 3; c++) {
            double d = std::fabs(ya[3 * n + c] - yb[3 * n + c]);
            if (d != 0.0) diff++;
            maxd = std::max(maxd, d);
        }
    }
    std::printf("%s NIN=%d grid %dx%dx%d slab %dx%dx%d zlen %d: bitwise differences %ld (max %.3g), bad writes %ld, "
                "pre mismatches %ld\n",
                sizeof(T) == 4 ? "float " : (std::is_same<T, topo::df>::value ? "df    " : "double"), NIN, nx, ny, nz, sh.ncx, sh.ncy, sh.nzr, sh.zlen, diff, maxd,
                wbad, (long)g_bad.load());
    return diff == 0 && wbad == 0 && g_bad.load() == 0;
}

template <class T>
static bool compare_reduction(int nx, int ny, int nz, long long slots, unsigned brick_grid) {
    using namespace topo;
    GridDesc g{nx, ny, nz, nx - 1, ny - 1, nz - 1};
    const long long nn = g.nn(), nel = g.nel();
    std::mt19937_64 rng(nx * 7 + ny * 3 + nz);
    std::uniform_real_distribution<double> U(-1.0, 1.0), P(0.1, 1.0);
    std::vector<double> x0(3 * nn), kf(nel), mf(nel);
    for (auto &v : x0) v = U(rng);
    for (auto &v : kf) v = P(rng);
    for (auto &v : mf) v = P(rng);
    const ElemConst<T> C = make_elem_const<T>(1.0, 1.0, 1.0, 0.3);
    RedOut ra{{0, 0}, 0}, rb{{0, 0}, 0};
    std::vector<double> parts(2 * 65536);
    unsigned counter = 0;
    PolRed<T> pa{x0.data(), kf.data(), mf.data(), &ra, {parts.data(), &counter}};
    PolRed<T> pb{x0.data(), kf.data(), mf.data(), &rb, {parts.data(), &counter}};
    int ntx, nty;
    const int ntiles = tile_count(g, ntx, nty);
    if (!tile_persistent<T>()) brick_grid = (unsigned)ntiles;
    run_grid(brick_grid, TILE_THREADS, [&] { k_tile<T, PolRed<T>>(g, C, pa); });
    const SlabShape sh = slab_shape(g, slots);
    run_grid((unsigned)(sh.ncx * sh.ncy * sh.nzr), SLAB_THREADS, [&] { k_slab<T, PolRed<T>>(g, C, pb, sh); });
    // the same sums on the host in node order, from the slab form's outputs
    std::vector<double> y(3 * nn, 0.0);
    std::vector<int> w(nn, 0);
    PolT<T, 1> py{x0.data(), x0.data(), y.data(), w.data(), kf.data(), mf.data(), {}};
    run_grid((unsigned)(sh.ncx * sh.ncy * sh.nzr), SLAB_THREADS, [&] { k_slab<T, PolT<T, 1>>(g, C, py, sh); });
    double h0 = 0.0, h1 = 0.0;
    for (long long i = 0; i < 3 * nn; i++) {
        h0 += y[i] * x0[i];
        h1 += y[i] * y[i];
    }
    const double tol = 1e-12;
    double err = 0.0;
    for (const RedOut *r : {&ra, &rb})
        err = std::max(err, std::max(std::fabs(r->tot[0] - h0), std::fabs(r->tot[1] - h1)) / h1);
    std::printf("reduction %s grid %dx%dx%d: finish calls %d / %d, relative difference to the host sums %.2e, "
                "counter %u\n", sizeof(T) == 4 ? "float " : "double", nx, ny, nz, ra.calls, rb.calls, err, counter);
    return ra.calls == 1 && rb.calls == 1 && err < tol && counter == 0 && h1 > 0.0;
}

int main() {
    bool ok = true;
    ok &= compare_reduction<double>(20, 18, 21, 12, 0);
    ok &= compare_reduction<float>(17, 16, 12, 3, 4);
    ok &= compare<double, 1>(17, 16, 12, 1, 8);
    ok &= compare<float, 1>(20, 18, 21, 12, 5);
    ok &= compare<double, 2>(31, 16, 9, 64, 12);
    ok &= compare<float, 2>(5, 4, 3, 1, 1);
    ok &= compare<double, 1>(16, 31, 24, 100, 7);
    ok &= compare<float, 1>(33, 9, 17, 5, 3);
    ok &= compare<topo::df, 1>(20, 18, 21, 12, 0);
    ok &= compare<topo::df, 2>(17, 16, 12, 3, 0);
    std::printf(ok ? "slab emulation OK\n" : "slab emulation FAILED\n");
    return ok ? 0 : 1;
}
