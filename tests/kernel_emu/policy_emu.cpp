// Runs the solver's own operator policies (policies.cuh) through the brick
// kernel (tile.cuh) and the slab kernel (slab.cuh) on host threads and
// compares them: the FP32 Krylov product with its direction update and p.q
// (PolPQ32), the double-float replacement product with its early exit
// (PolReplaceProduct), and the double-float K-only product (PolProduct).
#include <barrier>
#include <cstdio>
#include <random>
#include <thread>
#include <vector>

#include "df.cuh"
#include "kernels.cuh"
#include "slab.cuh"

thread_local emu_uint3 threadIdx, blockIdx;
emu_uint3 blockDim, gridDim;
static std::barrier<> *g_bar = nullptr;
void __syncthreads() { g_bar->arrive_and_wait(); }
namespace emu {
unsigned char dyn_smem[256 * 1024] __attribute__((aligned(16)));
}

using namespace topo;

template <class Body>
static void run_grid(unsigned grid, unsigned block, Body body) {
    gridDim = {grid, 1, 1};
    blockDim = {block, 1, 1};
    for (unsigned b = 0; b < grid; b++) {
        std::barrier<> bar((std::ptrdiff_t)block);
        g_bar = &bar;
        std::vector<std::thread> th;
        for (unsigned t = 0; t < block; t++)
            th.emplace_back([=] {
                threadIdx = {t, 0, 0};
                blockIdx = {b, 0, 0};
                body();
            });
        for (auto &x : th) x.join();
    }
}

template <class T, class Pol>
static void run_brick(const GridDesc &g, const ElemConst<T> &C, const Pol &pol, unsigned persistent_grid) {
    int ntx, nty;
    const int ntiles = tile_count(g, ntx, nty);
    const unsigned grid = tile_persistent<T>() ? persistent_grid : (unsigned)ntiles;
    run_grid(grid, TILE_THREADS, [&] { k_tile<T, Pol>(g, C, pol); });
}

template <class T, class Pol>
static void run_slab(const GridDesc &g, const ElemConst<T> &C, const Pol &pol, long long slots) {
    const SlabShape sh = slab_shape(g, slots);
    run_grid((unsigned)(sh.ncx * sh.ncy * sh.nzr), SLAB_THREADS, [&] { k_slab<T, Pol>(g, C, pol, sh); });
}

struct Problem {
    GridDesc g;
    long long nn, nel;
    std::vector<uint8_t> fixed;
    std::vector<double> kf, mf, x;
    Problem(int nx, int ny, int nz) : g{nx, ny, nz, nx - 1, ny - 1, nz - 1} {
        nn = g.nn();
        nel = g.nel();
        std::mt19937_64 rng(nx * 131 + ny * 17 + nz);
        std::uniform_real_distribution<double> U(-1.0, 1.0), P(0.05, 1.0);
        fixed.resize(nn);
        for (long long n = 0; n < nn; n++) fixed[n] = (n % g.nx == 0) ? 7 : ((n % 13 == 0) ? 2 : 0);
        kf.resize(nel);
        mf.resize(nel);
        for (auto &v : kf) v = P(rng);
        for (auto &v : mf) v = P(rng);
        x.resize(3 * nn);
        for (auto &v : x) v = U(rng);
    }
};

static bool pq32(int nx, int ny, int nz, long long slots, unsigned pgrid) {
    Problem pr(nx, ny, nz);
    const long long nd = 3 * pr.nn;
    std::vector<float> kff(pr.nel), mff(pr.nel), z(nd), pprev(nd);
    for (long long e = 0; e < pr.nel; e++) {
        kff[e] = (float)pr.kf[e];
        mff[e] = (float)pr.mf[e];
    }
    for (long long i = 0; i < nd; i++) {
        z[i] = (float)pr.x[i];
        pprev[i] = (float)(0.5 * pr.x[(i * 7) % nd]);
    }
    const ElemConst<float> C = make_elem_const<float>(1.0, 1.0, 1.0, 0.3);
    struct Run {
        std::vector<float> pb0, pb1, q;
        SolveScalars S{};
        std::vector<double> part;
        unsigned counter = 0;
    } a, b;
    for (Run *r : {&a, &b}) {
        r->pb0 = pprev;  // it = 2: p_prev in pb[0], the new p goes to pb[1]
        r->pb1.assign(nd, -7.0f);
        r->q.assign(nd, -7.0f);
        r->S.it = 2;
        r->S.beta = 0.37;
        r->S.rho = 2.5;
        r->part.assign(65536, 0.0);
    }
    auto pol = [&](Run &r) {
        PolPQ32 p{};
        p.fixed = pr.fixed.data();
        p.w = Weights<float>{kff.data(), mff.data(), nullptr, 1.3f, 0.7f};
        p.z = z.data();
        p.pb[0] = r.pb0.data();
        p.pb[1] = r.pb1.data();
        p.q = r.q.data();
        p.S = &r.S;
        p.part = Partials<1>{r.part.data(), &r.counter};
        return p;
    };
    run_brick<float>(pr.g, C, pol(a), pgrid);
    run_slab<float>(pr.g, C, pol(b), slots);
    long diff = 0;
    for (long long i = 0; i < nd; i++)
        if (a.q[i] != b.q[i] || a.pb1[i] != b.pb1[i] || a.q[i] == -7.0f) diff++;
    const double e = std::fabs(a.S.pq - b.S.pq) / std::fabs(a.S.pq);
    std::printf("PolPQ32 grid %dx%dx%d: differences %ld, p.q %.17g vs %.17g (%.1e), alpha %.6g %.6g\n", nx, ny, nz, diff,
                a.S.pq, b.S.pq, e, a.S.alpha, b.S.alpha);
    return diff == 0 && e < 1e-12 && a.S.pq > 0.0 && a.counter == 0 && b.counter == 0;
}

static bool replace_df(int nx, int ny, int nz, long long slots, int need_replace) {
    Problem pr(nx, ny, nz);
    const long long nd = 3 * pr.nn;
    std::vector<df> kfx(pr.nel), mfx(pr.nel);
    for (long long e = 0; e < pr.nel; e++) {
        kfx[e] = df(pr.kf[e]);
        mfx[e] = df(pr.mf[e]);
    }
    const ElemConst<df> C = make_elem_const<df>(1.0, 0.9, 1.1, 0.3);
    std::vector<double> ya(nd, -7.0), yb(nd, -7.0), part(65536, 0.0);
    unsigned counter = 0;
    SolveScalars S{};
    S.need_replace = need_replace;
    auto pol = [&](std::vector<double> &y) {
        PolReplaceProduct<df> p{};
        p.fixed = pr.fixed.data();
        p.w = Weights<df>{kfx.data(), mfx.data(), nullptr, df(1.3), df(40.0)};
        p.x = pr.x.data();
        p.y = y.data();
        p.S = &S;
        p.part = Partials<1>{part.data(), &counter};
        return p;
    };
    run_brick<df>(pr.g, C, pol(ya), 0);
    run_slab<df>(pr.g, C, pol(yb), slots);
    long diff = 0, untouched = 0;
    for (long long i = 0; i < nd; i++) {
        if (ya[i] != yb[i]) diff++;
        if (yb[i] == -7.0) untouched++;
    }
    std::printf("PolReplaceProduct<df> grid %dx%dx%d need_replace %d: differences %ld, untouched %ld\n", nx, ny, nz,
                need_replace, diff, untouched);
    return diff == 0 && (need_replace ? untouched == 0 : untouched == nd);
}

static bool kproduct_df(int nx, int ny, int nz, long long slots) {
    Problem pr(nx, ny, nz);
    const long long nd = 3 * pr.nn;
    std::vector<df> kfx(pr.nel);
    for (long long e = 0; e < pr.nel; e++) kfx[e] = df(pr.kf[e]);
    const ElemConst<df> C = make_elem_const<df>(0.8, 1.0, 1.2, 0.3);
    std::vector<double> ya(nd, -7.0), yb(nd, -7.0);
    auto pol = [&](std::vector<double> &y) {
        return PolProduct<df, true, false>{Weights<df>{kfx.data(), nullptr, nullptr, df(1.0), df(0.0)}, pr.x.data(),
                                           y.data(), {}};
    };
    run_brick<df>(pr.g, C, pol(ya), 0);
    run_slab<df>(pr.g, C, pol(yb), slots);
    long diff = 0;
    for (long long i = 0; i < nd; i++)
        if (ya[i] != yb[i] || yb[i] == -7.0) diff++;
    std::printf("PolProduct<df,K> grid %dx%dx%d: differences %ld\n", nx, ny, nz, diff);
    return diff == 0;
}

int main() {
    bool ok = true;
    ok &= pq32(20, 18, 21, 12, 5);
    ok &= pq32(33, 9, 17, 5, 3);
    ok &= replace_df(17, 16, 12, 3, 1);
    ok &= replace_df(17, 16, 12, 3, 0);
    ok &= kproduct_df(31, 16, 9, 64);
    std::printf(ok ? "policy emulation OK\n" : "policy emulation FAILED\n");
    return ok ? 0 : 1;
}
