// Runs the real k_kron_yz (staged lines) and k_kron_seg (line segments)
// sources on host threads and compares the y and z passes value by value, and
// the two index forms of k_kron_x.
#include <barrier>
#include <cstdio>
#include <random>
#include <thread>
#include <vector>

#include "kron.cuh"

thread_local emu_uint3 threadIdx, blockIdx;
emu_uint3 blockDim, gridDim;
static std::barrier<> *g_bar = nullptr;
void __syncthreads() { g_bar->arrive_and_wait(); }
namespace emu {
unsigned char dyn_smem[256 * 1024] __attribute__((aligned(16)));
}

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

template <int AXIS>
static bool compare(int nx, int ny, int nz) {
    using namespace topo;
    GridDesc g{nx, ny, nz, nx - 1, ny - 1, nz - 1};
    const long long nd = 3 * g.nn();
    const int nmax = std::max(nx, std::max(ny, nz));
    std::mt19937_64 rng(nx * 131 + ny * 7 + nz + AXIS);
    std::uniform_real_distribution<float> U(-1.0f, 1.0f);
    std::vector<float> tab((size_t)9 * nmax * KRON_W), in(nd), r(nd), ms(nd), a(nd, -7.0f), b(nd, -7.0f);
    for (auto &v : tab) v = U(rng);
    for (auto &v : in) v = U(rng);
    for (auto &v : r) v = U(rng);
    for (auto &v : ms) v = U(rng);  // negative entries take the clamped-DOF branch
    KronBand<float> B{tab.data(), nmax};
    run_grid(kron_yz_blocks(g, AXIS), KRON_THREADS,
             [&] { k_kron_yz<float, float, AXIS, false>(g, r.data(), ms.data(), B, in.data(), a.data(), KronDot{}); });
    const unsigned gs = (unsigned)((kron_seg_items(g, AXIS) + KSEG_THREADS - 1) / KSEG_THREADS);
    run_grid(gs, KSEG_THREADS,
             [&] { k_kron_seg<float, float, AXIS, false>(g, r.data(), ms.data(), B, in.data(), b.data(), KronDot{}); });
    long diff = 0, unset = 0;
    for (long long i = 0; i < nd; i++) {
        if (a[i] != b[i]) diff++;
        if (b[i] == -7.0f) unset++;
    }
    std::printf("axis %d grid %dx%dx%d: differences %ld, unwritten %ld\n", AXIS, nx, ny, nz, diff, unset);
    return diff == 0 && unset == 0;
}

// x pass: divided and incremental index forms, with and without the
// replacement rescale (which also rewrites r from the FP64 residual)
static bool compare_x(int nx, int ny, int nz, int kx, bool rescale) {
    using namespace topo;
    GridDesc g{nx, ny, nz, nx - 1, ny - 1, nz - 1};
    const long long nd = 3 * g.nn();
    const int nmax = std::max(nx, std::max(ny, nz));
    std::mt19937_64 rng(nx * 17 + ny * 5 + nz + kx);
    std::uniform_real_distribution<float> U(-1.0f, 1.0f);
    std::vector<float> tab((size_t)9 * nmax * KRON_W), ms(nd), ra(nd), rb(nd), a(nd, -7.0f), b(nd, -7.0f);
    std::vector<double> r64(nd);
    for (auto &v : tab) v = U(rng);
    for (auto &v : ms) v = U(rng);
    for (auto &v : ra) v = U(rng);
    for (auto &v : r64) v = U(rng);
    rb = ra;
    SolveScalars S{};
    S.rescale = rescale ? 1 : 0;
    S.sigma = 1.75;
    KronBand<float> B{tab.data(), nmax};
    const unsigned grid = (unsigned)(((long long)ny * nz + kx - 1) / kx);
    run_grid(grid, KRON_THREADS,
             [&] { k_kron_x<float, float>(g, kx, ra.data(), r64.data(), &S, ms.data(), B, a.data()); });
    run_grid(grid, KRON_THREADS,
             [&] { k_kron_xi<float, float>(g, kx, rb.data(), r64.data(), &S, ms.data(), B, b.data()); });
    long diff = 0, unset = 0;
    for (long long i = 0; i < nd; i++) {
        if (a[i] != b[i] || ra[i] != rb[i]) diff++;
        if (b[i] == -7.0f) unset++;
    }
    std::printf("x pass grid %dx%dx%d, %d lines per CTA%s: differences %ld, unwritten %ld\n", nx, ny, nz, kx,
                rescale ? ", rescale" : "", diff, unset);
    return diff == 0 && unset == 0;
}

int main() {
    bool ok = true;
    ok &= compare_x(5, 4, 3, 3, false);    // row 15 < block: many lines per trip
    ok &= compare_x(97, 6, 5, 8, true);    // row 291 > block
    ok &= compare_x(193, 3, 4, 2, false);  // row 579
    ok &= compare_x(40, 7, 9, 5, true);
    ok &= compare<1>(5, 40, 3);
    ok &= compare<2>(5, 3, 40);
    ok &= compare<1>(11, 17, 9);
    ok &= compare<2>(11, 9, 17);
    ok &= compare<2>(4, 3, 45);
    std::printf(ok ? "kron emulation OK\n" : "kron emulation FAILED\n");
    return ok ? 0 : 1;
}
