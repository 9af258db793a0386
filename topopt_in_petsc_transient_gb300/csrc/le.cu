// le.cu -- GB300 LinearElasticity: transient Newmark forward solves, discrete
// adjoint and element sensitivities of TopOpt_in_PETSc_Transient
// (LinearElasticity.cc), matrix-free on one GPU.
//
// Per design iteration (main.cc:82-90):
//   CompleteInitialState -> element factors, multigrid hierarchy, initial
//     acceleration from the masked mass solve, checkpoint 0
//   GenerateCheckPoints  -> forward blocks 0..ncp-1, checkpoints in HBM
//   ComputeObjectiveSensitivities -> reverse block loop: recompute the block
//     (skipped for the last block, whose history is still resident), adjoint
//     steps with fused element sensitivities/objective, t = 0 mass solve.
// Every linear solve is a flexible CG whose preconditioner is a geometric
// multigrid V-cycle (Chebyshev-Jacobi smoothing, trilinear transfer,
// rediscretised coarse operators, dense coarsest inverse), run either in FP64
// ("plain") or in FP32 inside the FP64 outer iteration ("mixed").
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "le.h"
#include "kron.cuh"
#include "mpiio.h"
#include "sommg.cuh"
#include "gram.cuh"

namespace topo {

#define CK(call)                                                                 \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if (e_ != cudaSuccess) {                                                 \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));      \
            return TOPO_ERR_CUDA;                                                \
        }                                                                        \
    } while (0)

static thread_local std::string g_last_error;

// Function attributes, occupancy and SM counts are properties of a device:
// the one-time caches of the launch helpers are indexed by the ordinal of the
// current device (a second device gets its own attribute calls and grid sizes)
constexpr int MAX_DEVICES = 64;
static int device_slot() {
    int d = 0;
    cudaGetDevice(&d);
    return (d >= 0 && d < MAX_DEVICES) ? d : 0;
}
void set_error(const std::string &s) { g_last_error = s; }
const char *last_error() { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// host helpers: element matrices of a box from the mode operator
// ---------------------------------------------------------------------------
void box_element_matrices(double hx, double hy, double hz, double nu, double *KE, double *ME) {
    ElemConst<double> C = make_elem_const<double>(hx, hy, hz, nu);
    for (int col = 0; col < 24; col++) {
        double u[3][8] = {{0}}, y[3][8];
        u[col % 3][col / 3] = 1.0;
        double U[3][8];
        memcpy(U, u, sizeof(U));
        for (int c = 0; c < 3; c++) mode_fwd(U[c]);
        mode_stiffness(C, U, y);
        for (int c = 0; c < 3; c++) {
            double t[8];
            for (int m = 0; m < 8; m++) t[m] = y[c][m];
            mode_bwd(t);
            for (int L = 0; L < 8; L++) KE[(3 * L + c) * 24 + col] = t[L];
            for (int m = 0; m < 8; m++) t[m] = C.W[m] * U[c][m];
            mode_bwd(t);
            for (int L = 0; L < 8; L++) ME[(3 * L + c) * 24 + col] = t[L];
        }
    }
}

// largest eigenvalue of diag(A)^-1/2 A diag(A)^-1/2 (24x24 SPD) by power iteration
static double jacobi_scaled_lmax(const double *A) {
    double d[24], v[24], w[24];
    for (int i = 0; i < 24; i++) {
        d[i] = 1.0 / sqrt(A[i * 24 + i]);
        v[i] = 1.0 + 0.01 * i;
    }
    double lam = 0.0;
    for (int it = 0; it < 2000; it++) {
        double nrm = 0.0;
        for (int i = 0; i < 24; i++) {
            double s = 0.0;
            for (int j = 0; j < 24; j++) s += d[i] * A[i * 24 + j] * d[j] * v[j];
            w[i] = s;
            nrm += s * s;
        }
        nrm = sqrt(nrm);
        double l = 0.0;
        for (int i = 0; i < 24; i++) l += v[i] * w[i];
        double vn = 0.0;
        for (int i = 0; i < 24; i++) vn += v[i] * v[i];
        lam = l / vn;
        for (int i = 0; i < 24; i++) v[i] = w[i] / nrm;
    }
    return lam;
}

// largest eigenvalue of the generalized problem KE v = mu ME v (ME SPD):
// power iteration on C = L^-1 KE L^-T with ME = L L^T
static double mass_scaled_lmax(const double *KE, const double *ME) {
    double Lc[24][24] = {{0}};
    for (int i = 0; i < 24; i++)
        for (int j = 0; j <= i; j++) {
            double s = ME[i * 24 + j];
            for (int k = 0; k < j; k++) s -= Lc[i][k] * Lc[j][k];
            Lc[i][j] = (i == j) ? sqrt(s) : s / Lc[j][j];
        }
    auto lsolve = [&](const double *b, double *x) {  // L x = b
        for (int i = 0; i < 24; i++) {
            double s = b[i];
            for (int k = 0; k < i; k++) s -= Lc[i][k] * x[k];
            x[i] = s / Lc[i][i];
        }
    };
    auto ltsolve = [&](const double *b, double *x) {  // L^T x = b
        for (int i = 23; i >= 0; i--) {
            double s = b[i];
            for (int k = i + 1; k < 24; k++) s -= Lc[k][i] * x[k];
            x[i] = s / Lc[i][i];
        }
    };
    double v[24], w[24], t[24];
    for (int i = 0; i < 24; i++) v[i] = 1.0 + 0.37 * i - 0.01 * i * i;
    double lam = 0.0;
    for (int it = 0; it < 3000; it++) {
        ltsolve(v, t);
        for (int i = 0; i < 24; i++) {
            double s = 0.0;
            for (int j = 0; j < 24; j++) s += KE[i * 24 + j] * t[j];
            w[i] = s;
        }
        lsolve(w, t);
        double vv = 0.0, vt = 0.0, tt = 0.0;
        for (int i = 0; i < 24; i++) {
            vv += v[i] * v[i];
            vt += v[i] * t[i];
            tt += t[i] * t[i];
        }
        lam = vt / vv;
        double nt = sqrt(tt);
        for (int i = 0; i < 24; i++) v[i] = t[i] / nt;
    }
    return lam;
}

// Rows of the inverse of the assembled 1-D mass h/6 [2 1; 1 2] on n nodes
// (a Dirichlet end decouples that node: identity row), truncated to the band
// |i - j| <= KRON_B: tap[i][KRON_B + d] = (T^-1)_{i, i+d}.  Thomas
// elimination per unit right-hand side.
static void kron_band_1d(int n, double h, bool d0, bool d1, double *tap) {
    std::vector<double> d(n), off(n, 0.0), l(n), im(n), y(n), x(n);
    for (int i = 0; i < n; i++) d[i] = (i == 0 || i == n - 1) ? h / 3.0 : 2.0 * h / 3.0;
    for (int i = 0; i + 1 < n; i++) off[i] = h / 6.0;
    if (d0) {
        d[0] = 1.0;
        off[0] = 0.0;
    }
    if (d1) {
        d[n - 1] = 1.0;
        off[n - 2] = 0.0;
    }
    double m = d[0];
    l[0] = 0.0;
    im[0] = 1.0 / m;
    for (int i = 1; i < n; i++) {
        l[i] = off[i - 1] / m;
        m = d[i] - l[i] * off[i - 1];
        im[i] = 1.0 / m;
    }
    for (int i = 0; i < n * KRON_W; i++) tap[i] = 0.0;
    for (int col = 0; col < n; col++) {  // column col of T^-1 (T symmetric: also row col)
        for (int i = 0; i < n; i++) y[i] = (i == col ? 1.0 : 0.0) - (i > 0 ? l[i] * y[i - 1] : 0.0);
        for (int i = n - 1; i >= 0; i--) x[i] = (y[i] - (i < n - 1 ? off[i] * x[i + 1] : 0.0)) * im[i];
        for (int i = std::max(0, col - KRON_B); i <= std::min(n - 1, col + KRON_B); i++)
            tap[(size_t)i * KRON_W + KRON_B + (col - i)] = x[i];
    }
}

// ---------------------------------------------------------------------------
// device memory arena: every allocation of an object, released together
// ---------------------------------------------------------------------------
struct Arena {
    std::vector<void *> ptrs;
    size_t bytes = 0;
    template <class T>
    int get(T **p, size_t n) {
        void *q = nullptr;
        size_t b = sizeof(T) * (n ? n : 1);
        cudaError_t e = cudaMalloc(&q, b);
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error(std::string("cudaMalloc of ") + std::to_string(b) + " bytes failed: " + cudaGetErrorString(e));
            return TOPO_ERR_OOM;
        }
        cudaMemset(q, 0, b);
        ptrs.push_back(q);
        bytes += b;
        *p = (T *)q;
        return TOPO_OK;
    }
    void release() {
        for (void *p : ptrs) cudaFree(p);
        ptrs.clear();
        bytes = 0;
    }
};

#define AG(p, n)                                 \
    do {                                         \
        int rc_ = arena.get(&(p), (size_t)(n));  \
        if (rc_) return rc_;                     \
    } while (0)

// In-solve timing of one kernel class on the fine grid (`nn` nodes): when
// armed, every direct launch of that class is bracketed by a pair of CUDA
// events on its stream.  Launches recorded into a CUDA graph are not timed.
// Classes: TOPO_KT_SMOOTH (PolCheb / PolChebDot in FP32), TOPO_KT_PQ32,
// TOPO_KT_KRON (each Kronecker stencil pass), TOPO_KT_REPLACE (the residual
// replacement pass, FP64-accurate), TOPO_KT_DFPROD (double-float products of
// the right-hand sides, anchors and adjoint steps).
struct LaunchTimer {
    int cls = -1;
    long long nn = -1;
    std::vector<cudaEvent_t> ev;
    size_t used = 0;
};
static LaunchTimer *g_timer = nullptr;

static bool timer_begin(int cls, long long nn, cudaStream_t s) {
    if (!g_timer || g_timer->cls != cls || g_timer->nn != nn) return false;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cs);
    if (cs != cudaStreamCaptureStatusNone) return false;
    while (g_timer->ev.size() < g_timer->used + 2) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return false;
        g_timer->ev.push_back(e);
    }
    cudaEventRecord(g_timer->ev[g_timer->used], s);
    return true;
}
static void timer_end(bool timed, cudaStream_t s) {
    if (!timed) return;
    cudaEventRecord(g_timer->ev[g_timer->used + 1], s);
    g_timer->used += 2;
}

template <class T, class Pol>
constexpr int tile_class() {
    return (std::is_same<Pol, PolCheb<float>>::value || std::is_same<Pol, PolChebDot>::value) ? TOPO_KT_SMOOTH
           : std::is_same<Pol, PolPQ32>::value                                                 ? TOPO_KT_PQ32
           : std::is_same<Pol, PolReplace<T>>::value                                           ? TOPO_KT_REPLACE
           : (std::is_same<T, df>::value && std::is_same<Pol, PolProduct<df, Pol::HAS_K, Pol::HAS_M>>::value)
               ? TOPO_KT_DFPROD
                                                                                               : -1;
}

// FP32 tile kernels and kernels staged by asynchronous copies are persistent: as many
// CTAs as are resident on the device at once (occupancy of this instantiation
// x SM count), capped by the brick count; the others launch one CTA per brick
template <class T, class Pol>
static void launch_tile(const GridDesc &g, const ElemConst<T> &C, const Pol &pol, cudaStream_t s) {
    static int resident_dev[MAX_DEVICES] = {};
    int &resident = resident_dev[device_slot()];
    const size_t sm = TileSmem<T, Pol>::bytes;
    if (!resident) {
        cudaFuncSetAttribute(k_tile<T, Pol>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        int dev = 0, nsm = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile<T, Pol>, TILE_THREADS, sm);
        resident = std::max(1, per_sm) * std::max(1, nsm);
    }
    int ntx, nty;
    const int ntiles = tile_count(g, ntx, nty);
    const bool timed = tile_class<T, Pol>() >= 0 && timer_begin(tile_class<T, Pol>(), g.nn(), s);
    count_launch();
    const int grid = (tile_persistent<T>() || tile_async<T, Pol>()) ? std::min(ntiles, resident) : ntiles;
    k_tile<T, Pol><<<(unsigned)grid, TILE_THREADS, sm, s>>>(g, C, pol);
    timer_end(timed, s);
}

// ---------------------------------------------------------------------------
// multigrid hierarchy
// ---------------------------------------------------------------------------
struct TopoLE;
template <class A>
static Weights<A> fine_weights(TopoLE *le, bool hk, bool hm, const double *P, double sK, double sM);
template <class A>
static const ElemConst<A> &fine_const(TopoLE *le);

struct Level {
    GridDesc g;
    double h[3];
    ElemConst<double> Cd;
    ElemConst<float> Cf;
    double dK[3], dM, lamK;
    uint8_t *fixed = nullptr;
    double *kfd = nullptr, *mfd = nullptr;  // density factors on this level
    float *kff = nullptr, *mff = nullptr;
    // V-cycle work vectors
    float *fb = nullptr, *fxa = nullptr, *fxb = nullptr, *fd = nullptr, *fr = nullptr;
    double *db = nullptr, *dxa = nullptr, *dxb = nullptr, *dd = nullptr, *dr = nullptr;
};

struct OpLevel {
    double *dinvd = nullptr;
    float *dinvf = nullptr;
    double *lohi = nullptr;  // device [5]: smoothing interval, full-spectrum interval, raw lower bound
    double *cheb = nullptr;   // device [kmax][2] Chebyshev step coefficients (smoothing)
    double *chebf = nullptr;  // same over the full spectrum (smoother-as-solver level)
    double hlohi[5] = {0, 0, 0, 0, 0};
};

struct Operator {
    double sK = 0.0, sM = 1.0;  // A = sK * K(kf) + sM * M(mf)
    int depth = 1;              // levels the V-cycle descends (adaptive)
    std::vector<OpLevel> lv;
    double *Ainv_d = nullptr;
    float *Ainv_f = nullptr;
    // Kronecker mass preconditioner: node scaling and whether it is in use
    bool kron = false;
    double share = 0.0;  // stiffness share (sK/sM) max(kf/mf) lambda_max(KE, ME)
    double *kscale_d = nullptr;
    float *kscale_f = nullptr;
};

struct TopoLE {
    LEParams p;
    GridDesc g;
    long long nn = 0, nel = 0, ndof = 0;
    int Ts = 0;
    double dt = 0.0, a[6] = {0};
    int nlev = 1;
    std::vector<Level> L;
    Operator ops[3];  // 0: Newmark effective operator, 1: mass, 2: SOMMG P0 = K - om^2 M
    int nops = 2;
    // SOMMG reduced path (reduction = 1): basis Q [kb][ndof]; reduced
    // matrices Kr, Mr, Kp, Mp, Gc, Ut [kb*kb each], Pr [kb], fx; reduced
    // history [Ts][3][kb]; accumulators S [4][kb*kb]; Phi [4][kb][ndof]
    long long out_dof = -1;    // objective 7 output DOF
    // K, M products of the two previous adjoint iterates (initial residual of
    // the adjoint solves without an operator pass); ax0_pending: the next
    // solve takes (N A N + I - N) x0 from ax0 (= sq)
    double *KLh1 = nullptr, *MLh1 = nullptr, *KLh2 = nullptr, *MLh2 = nullptr;
    bool ax0_pending = false;
    // mixed forward sweep: tracked products A u-, A du-, A ddu- of the
    // previous state, AApt scratch for A ddu-- when re-anchoring, KSt the
    // next step's K-pass input; fwd_init_pending: the next solve's initial
    // residual comes from the K-only right-hand-side pass (fwd_rhs_init)
    double *AUt = nullptr, *AVt = nullptr, *AAt = nullptr, *AApt = nullptr, *KSt = nullptr;
    bool fwd_init_pending = false;
    int kb = 0;
    bool fp64_solves = false;  // the SOMMG basis solves run the FP64 FCG in either mode
    double *Q = nullptr, *red = nullptr, *rhist = nullptr, *Sacc = nullptr, *Phi = nullptr, *mdpart = nullptr;
    int *rstatus = nullptr;
    // mixed path: the basis in FP32 (rows of qld >= ndof values, a multiple of
    // GR_KC, zero padded), Phi in FP32, the products W = A Q_j as FP32 pairs
    // (Wh, Wl) for the tensor-core Gram (gram.cuh), its per-CTA partials and
    // an FP64 scratch row qd
    bool basis32 = false;
    long long qld = 0;
    float *Q32 = nullptr, *Phi32 = nullptr, *Wh = nullptr, *Wl = nullptr;
    double *gpart = nullptr, *qd = nullptr;
    int gram_blocks = 0;
    Arena arena;
    cudaStream_t stream = nullptr;
    topo_mpiio *out = nullptr;  // attached physics output (topo_le_set_output), not owned

    // fine-level data
    double *N_host_dummy = nullptr;
    double *rhs0 = nullptr, *P = nullptr, *xPhys = nullptr;
    double *sigtab = nullptr;  // [2][Ts]: Load(t)/(ny-1) and the second load's signal per step
    double *kf = nullptr, *dkf = nullptr, *mf = nullptr, *dmf = nullptr;
    df *kfx = nullptr, *mfx = nullptr;  // double-float copies for the mixed path
    ElemConst<df> Cx;
    float *cntP = nullptr;
    double *cp = nullptr;                   // (ncp+1) x 3 x ndof
    double *Uh = nullptr, *DUh = nullptr, *DDUh = nullptr;  // tsc x ndof
    double *Lp1 = nullptr, *DLp1 = nullptr, *DDLp1 = nullptr, *DLc = nullptr, *DDLc = nullptr, *Lp2 = nullptr, *Lp3 = nullptr;
    double *KL = nullptr, *ML = nullptr, *hK = nullptr, *hM = nullptr;
    double *DDL0 = nullptr;
    // restart vectors: LT the terminal adjoint of the last reverse sweep
    // (RestartSol0x.dat), u0init a loaded initial displacement (-solutionAsU0;
    // null: u0 = 0)
    double *LT = nullptr, *u0init = nullptr;
    double *df = nullptr;
    // per-node sensitivity combinations: FP64 (2 x ndof) or FP32 (5 x ndof)
    double *sw64 = nullptr;
    float *sw32 = nullptr;
    // solver vectors
    double *sx = nullptr, *sb = nullptr, *sr = nullptr, *sp = nullptr, *sq = nullptr, *sz = nullptr;
    float *sr32 = nullptr, *sp32 = nullptr, *sp32b = nullptr, *sq32 = nullptr;
    int coarse_dense = 1;
    // coarse assembly scratch
    double *KEc = nullptr, *MEc = nullptr, *chol_w = nullptr, *chol_col = nullptr;  // coarse Cholesky scratch
    int ncoarse = 0;
    // control block
    SolveScalars *S = nullptr;
    StepCtx *st = nullptr;
    double *part = nullptr;
    unsigned int *counter = nullptr;
    unsigned long long *bbits = nullptr;
    // Kronecker mass preconditioner tables
    double *kron_d = nullptr;  // banded 1-D inverses [3][3][nmax][KRON_W]
    float *kron_f = nullptr;
    int kron_nmax = 0;
    double mu_KM = 0.0;  // largest generalized eigenvalue of (KE, ME), fine box
    int *err = nullptr;
    long long nsolves = 0;
    long long mg_solves = 0;  // solves whose preconditioner is the V-cycle
    long long step_kernels[2] = {0, 0}, body_kernels = 0, direct_iters = 0;
    // graphs
    cudaGraphExec_t gx_fwd = nullptr, gx_adj = nullptr;
    int graphs_ok = 0;
    int captured_depth = -1;  // V-cycle depth baked into the step graphs
    // diagnostics
    LEStats stats;
    int last_block_resident = -1;
    int design_ready = 0;
    // checkpoints 1..ncp-1 belong to the current design (GenerateCheckPoints
    // ran after the last CompleteInitialState; always true for ncp = 1)
    int checkpoints_ready = 0;
};

static Partials<1> P1(TopoLE *le) { return Partials<1>{le->part, le->counter}; }

// fine-level element weights / constants for the FP64-accurate passes:
// native double (plain path) or double-float (mixed path)
template <>
Weights<double> fine_weights<double>(TopoLE *le, bool hk, bool hm, const double *P, double sK, double sM) {
    return Weights<double>{hk ? le->kf : nullptr, hm ? le->mf : nullptr, P, sK, sM};
}
template <>
Weights<df> fine_weights<df>(TopoLE *le, bool hk, bool hm, const double *P, double sK, double sM) {
    return Weights<df>{hk ? le->kfx : nullptr, hm ? le->mfx : nullptr, P, df(sK), df(sM)};
}
template <>
Weights<float> fine_weights<float>(TopoLE *le, bool hk, bool hm, const double *P, double sK, double sM) {
    return Weights<float>{hk ? le->L[0].kff : nullptr, hm ? le->L[0].mff : nullptr, P, (float)sK, (float)sM};
}
template <>
const ElemConst<float> &fine_const<float>(TopoLE *le) { return le->L[0].Cf; }
template <>
const ElemConst<double> &fine_const<double>(TopoLE *le) { return le->L[0].Cd; }
template <>
const ElemConst<df> &fine_const<df>(TopoLE *le) { return le->Cx; }
static Partials<2> P2(TopoLE *le) { return Partials<2>{le->part, le->counter}; }

// ---------------------------------------------------------------------------
// creation
// ---------------------------------------------------------------------------
int le_create(TopoLE **out, const LEParams *pp) {
    *out = nullptr;
    const LEParams &p = *pp;
    if (p.nx < 2 || p.ny < 2 || p.nz < 2 || p.ncp < 1 || p.tsc < 1 || p.nlvls < 1 || p.hx <= 0 || p.hy <= 0 ||
        p.hz <= 0 || p.t1 <= 0 || p.objective < 0 || p.objective > 7 ||
        p.load2_node >= (long long)p.nx * p.ny * p.nz || p.out_dof >= 3LL * p.nx * p.ny * p.nz) {
        set_error("invalid LinearElasticity parameters");
        return TOPO_ERR_ARG;
    }
    if (p.reduction && (p.objective == 7 || p.load2_node >= 0)) {
        set_error("the SOMMG reduction does not take the output-DOF objective or the second point load");
        return TOPO_ERR_ARG;
    }
    if (p.reduction && (p.basis < 1 || p.basis > KB_MAX || !(p.omega0 > 0.0))) {
        set_error("SOMMG reduction needs 1 <= basis <= " + std::to_string(KB_MAX) +
                  " and omega0 > 0 (the basis recursion scales by omega0)");
        return TOPO_ERR_ARG;
    }
    // multigrid divisibility (TopOpt::SetUpMESH, TopOpt.cc:200-219)
    int div = 1 << (p.nlvls - 1);
    if ((p.nx - 1) % div || (p.ny - 1) % div || (p.nz - 1) % div) {
        set_error("mesh dimension not compatible with the number of multigrid levels");
        return TOPO_ERR_ARG;
    }
    TopoLE *le = new TopoLE();
    le->p = p;
    le->g = GridDesc{p.nx, p.ny, p.nz, p.nx - 1, p.ny - 1, p.nz - 1};
    le->nn = le->g.nn();
    le->nel = le->g.nel();
    le->ndof = 3 * le->nn;
    // constructor, LinearElasticity.cc:93-97; SetUpTimeIntegration :185-219
    le->Ts = p.ncp * p.tsc + 1;
    le->out_dof = p.out_dof >= 0 ? p.out_dof
                                 : 3 * ((p.nx - 1) + (long long)p.nx * ((p.ny - 1) / 2 + (long long)p.ny * ((p.nz - 1) / 2))) + 2;
    le->dt = p.t1 / (le->Ts - 1);
    double dt = le->dt;
    if (p.ti == 0) {
        double a[6] = {0.0, 0.0, 1.0 / dt, 1.0 / dt, 0.0, 1.0 / (dt * dt)};
        memcpy(le->a, a, sizeof(a));
    } else {
        double b = 0.25, gm = 0.5;
        double a[6] = {1.0 - gm / b, (1.0 - gm / (2.0 * b)) * dt, gm / (b * dt), 1 / (b * dt), 1 / (2.0 * b) - 1.0,
                       1.0 / (b * dt * dt)};
        memcpy(le->a, a, sizeof(a));
    }
    int rc = le_alloc(le);
    if (rc) {
        le_destroy(le);
        return rc;
    }
    *out = le;
    return TOPO_OK;
}

int le_alloc(TopoLE *le) {
    const LEParams &p = le->p;
    Arena &arena = le->arena;
    CK(cudaStreamCreateWithFlags(&le->stream, cudaStreamNonBlocking));
    long long nd = le->ndof, ne = le->nel, nn = le->nn;
    AG(le->rhs0, nd);
    AG(le->P, ne);
    AG(le->xPhys, ne);
    AG(le->kf, ne);
    AG(le->dkf, ne);
    AG(le->mf, ne);
    AG(le->dmf, ne);
    AG(le->kfx, ne);
    AG(le->mfx, ne);
    AG(le->cntP, nn);
    AG(le->cp, (size_t)(p.ncp + 1) * 3 * nd);
    // the reduced path keeps its history in reduced coordinates
    const size_t hsteps = p.reduction ? 1 : (size_t)p.tsc;
    AG(le->Uh, hsteps * nd);
    AG(le->DUh, hsteps * nd);
    AG(le->DDUh, hsteps * nd);
    AG(le->Lp1, nd);
    AG(le->DLp1, nd);
    AG(le->DDLp1, nd);
    AG(le->Lp2, nd);
    AG(le->Lp3, nd);
    if (p.mixed && !p.reduction) {  // tracked products of the forward state
        AG(le->AUt, nd);
        AG(le->AVt, nd);
        AG(le->AAt, nd);
        AG(le->AApt, nd);
        AG(le->KSt, nd);
    }
    if (!p.reduction) {
        AG(le->KLh1, nd);
        AG(le->MLh1, nd);
        AG(le->KLh2, nd);
        AG(le->MLh2, nd);
    }
    AG(le->DLc, nd);
    AG(le->DDLc, nd);
    AG(le->KL, nd);
    AG(le->ML, nd);
    AG(le->hK, nd);
    AG(le->hM, nd);
    AG(le->DDL0, nd);
    AG(le->LT, nd);
    AG(le->df, ne);
    if (p.mixed && p.sens_fp32)
        AG(le->sw32, 5 * nd);
    else
        AG(le->sw64, 2 * nd);
    AG(le->sx, nd);
    AG(le->sb, nd);
    AG(le->sr, nd);
    AG(le->sp, nd);
    AG(le->sq, nd);
    AG(le->sz, nd);
    AG(le->sr32, nd);
    AG(le->sp32, nd);
    AG(le->sp32b, nd);
    AG(le->sq32, nd);
    AG(le->S, 1);
    AG(le->st, 1);
    {
        // per-CTA partials: tile kernels (<= 4 sums per CTA) and the
        // Kronecker pass with the fused dot products (2 sums per CTA)
        const long long kron_blocks = (long long)((3 * p.nx + KW - 1) / KW) * std::max(p.ny, p.nz);
        AG(le->part, std::max(4LL * 65536, 2 * kron_blocks));
    }
    AG(le->counter, 4);
    AG(le->bbits, 4);
    AG(le->err, 1);

    // ---- host-side geometry: masks, load location, region (SetUpBC,
    // LoadLocation, SetUpOptimizationRegion: LinearElasticity.cc:222-675) ----
    std::vector<uint8_t> fixed(nn, 0);
    std::vector<double> rhs0(nd, 0.0), P(ne, 0.0);
    double xc[6] = {0, (p.nx - 1) * p.hx, 0, (p.ny - 1) * p.hy, 0, (p.nz - 1) * p.hz};
    double epsi = std::fmin(p.hx * 0.05, std::fmin(p.hy * 0.05, p.hz * 0.05));
    for (int k = 0; k < p.nz; k++)
        for (int j = 0; j < p.ny; j++)
            for (int i = 0; i < p.nx; i++) {
                long long n = i + (long long)p.nx * (j + (long long)p.ny * k);
                double x = i * p.hx, y = j * p.hy, z = k * p.hz;
                if (p.boundaries == 0) {
                    if (std::fabs(x - xc[0]) < epsi) fixed[n] |= 1 | 2;
                    if (std::fabs(x - xc[1]) < epsi && std::fabs(z - xc[4]) < epsi) fixed[n] |= 2 | 4;
                } else {
                    if (std::fabs(x - xc[0]) < epsi) fixed[n] |= 7;
                }
                double zl = (p.loadloc == 0) ? xc[5] : xc[5] / 2.0;
                double xl = (p.loadloc == 0) ? xc[0] : xc[1];
                if (std::fabs(x - xl) < epsi && std::fabs(z - zl) < epsi) {
                    rhs0[3 * n + 2] = 1.0;
                    if (std::fabs(y - xc[2]) < epsi || std::fabs(y - xc[3]) < epsi) rhs0[3 * n + 2] = 0.5;
                }
            }
    for (long long e = 0; e < ne; e++) {
        int i = (int)(e % le->g.ex), j = (int)((e / le->g.ex) % le->g.ey), k = (int)(e / ((long long)le->g.ex * le->g.ey));
        double ex = (i + 0.5) * p.hx, ey = (j + 0.5) * p.hy, ez = (k + 0.5) * p.hz, v = 0.0;
        switch (p.optregion) {
        case 0: v = (ez > xc[5] - 1 && ex < xc[0] + 1) ? 1.0 : 0.0; break;
        case 1: v = (ez > xc[5] / 2.0 - 0.5 && ez < xc[5] / 2.0 + 0.5 && ex < xc[1] - 1) ? 1.0 : 0.0; break;
        case 2: v = 1.0; break;
        default:
            v = (ex > 0.75 * xc[1] - 2.5 && ex < 0.75 * xc[1] + 2.5 && ey > 0.5 * xc[3] - 2.5 && ey < 0.5 * xc[3] + 2.5 &&
                 ez > 0.5 * xc[5] - 2.5 && ez < 0.5 * xc[5] + 2.5)
                    ? 1.0
                    : 0.0;
        }
        P[e] = v;
    }
    {
        StepCtx sc;
        memset(&sc, 0, sizeof(sc));
        sc.tsc = p.tsc;
        sc.dt = le->dt;
        CK(cudaMemcpy(le->st, &sc, sizeof(sc), cudaMemcpyHostToDevice));
    }
    AG(le->sigtab, 2 * (size_t)le->Ts);
    count_launch();
    k_load_table<<<(le->Ts + 255) / 256, 256, 0, le->stream>>>(le->Ts, le->dt, p.loadsignal, 1.0 / (p.ny - 1),
                                                                p.load2_phase, le->sigtab, le->sigtab + le->Ts);
    CK(cudaMemcpy(le->rhs0, rhs0.data(), sizeof(double) * nd, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(le->P, P.data(), sizeof(double) * ne, cudaMemcpyHostToDevice));
    count_launch();
    k_count_region<<<ew_blocks(nn), EW, 0, le->stream>>>(le->g, le->P, le->cntP);

    // ---- Kronecker mass preconditioner: banded 1-D inverses per axis and
    // component; a face plane clamped for a component decouples that end ----
    {
        const int n3[3] = {p.nx, p.ny, p.nz};
        const double h3[3] = {p.hx, p.hy, p.hz};
        const int nmax = std::max(p.nx, std::max(p.ny, p.nz));
        le->kron_nmax = nmax;
        std::vector<double> tab((size_t)9 * nmax * KRON_W, 0.0);
        auto plane_fixed = [&](int a, int idx, int c) {
            const int u = (a + 1) % 3, v = (a + 2) % 3;
            for (int jv = 0; jv < n3[v]; jv++)
                for (int ju = 0; ju < n3[u]; ju++) {
                    int ijk[3];
                    ijk[a] = idx;
                    ijk[u] = ju;
                    ijk[v] = jv;
                    long long n = ijk[0] + (long long)p.nx * (ijk[1] + (long long)p.ny * ijk[2]);
                    if (!((fixed[n] >> c) & 1)) return false;
                }
            return true;
        };
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++)
                kron_band_1d(n3[a], h3[a], plane_fixed(a, 0, c), plane_fixed(a, n3[a] - 1, c),
                             tab.data() + (size_t)(a * 3 + c) * nmax * KRON_W);
        std::vector<float> tabf(tab.begin(), tab.end());
        AG(le->kron_d, tab.size());
        AG(le->kron_f, tab.size());
        CK(cudaMemcpy(le->kron_d, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(le->kron_f, tabf.data(), sizeof(float) * tabf.size(), cudaMemcpyHostToDevice));
        double KE[576], ME[576];
        box_element_matrices(p.hx, p.hy, p.hz, p.nu, KE, ME);
        le->mu_KM = mass_scaled_lmax(KE, ME);
        le->nops = p.reduction ? 3 : 2;
        for (int o = 0; o < le->nops; o++) {
            AG(le->ops[o].kscale_d, 3 * nn);  // masked scale, one value per DOF
            AG(le->ops[o].kscale_f, 3 * nn);
        }
    }

    // ---- multigrid levels ----
    le->nlev = p.nlvls;
    le->L.resize(le->nlev);
    for (int l = 0; l < le->nlev; l++) {
        Level &lv = le->L[l];
        int f = 1 << l;
        lv.g = GridDesc{(p.nx - 1) / f + 1, (p.ny - 1) / f + 1, (p.nz - 1) / f + 1, (p.nx - 1) / f, (p.ny - 1) / f,
                        (p.nz - 1) / f};
        lv.h[0] = p.hx * f;
        lv.h[1] = p.hy * f;
        lv.h[2] = p.hz * f;
        lv.Cd = make_elem_const<double>(lv.h[0], lv.h[1], lv.h[2], p.nu);
        lv.Cf = make_elem_const<float>(lv.h[0], lv.h[1], lv.h[2], p.nu);
        double KE[576], ME[576];
        box_element_matrices(lv.h[0], lv.h[1], lv.h[2], p.nu, KE, ME);
        for (int c = 0; c < 3; c++) lv.dK[c] = KE[c * 24 + c];
        lv.dM = ME[0];
        lv.lamK = jacobi_scaled_lmax(KE);
        long long lnn = lv.g.nn(), lnel = lv.g.nel(), lnd = 3 * lnn;
        AG(lv.fixed, lnn);
        std::vector<uint8_t> fl(lnn);
        for (int k = 0; k < lv.g.nz; k++)
            for (int j = 0; j < lv.g.ny; j++)
                for (int i = 0; i < lv.g.nx; i++)
                    fl[i + (long long)lv.g.nx * (j + (long long)lv.g.ny * k)] =
                        fixed[(i * f) + (long long)p.nx * ((j * f) + (long long)p.ny * (k * f))];
        CK(cudaMemcpy(lv.fixed, fl.data(), lnn, cudaMemcpyHostToDevice));
        if (l > 0) {
            AG(lv.kfd, lnel);
            AG(lv.mfd, lnel);
            AG(lv.kff, lnel);
            AG(lv.mff, lnel);
        }
        AG(lv.fb, lnd);
        AG(lv.fxa, lnd);
        AG(lv.fxb, lnd);
        AG(lv.fd, lnd);
        AG(lv.fr, lnd);
        AG(lv.db, lnd);
        AG(lv.dxa, lnd);
        AG(lv.dxb, lnd);
        AG(lv.dd, lnd);
        AG(lv.dr, lnd);
        if (l == le->nlev - 1) {
            le->ncoarse = (int)lnd;
            le->coarse_dense = (lnd <= (long long)p.coarse_dense_max) && lnd <= 12288;
        }
        if (l == le->nlev - 1 && le->coarse_dense) {
            AG(le->KEc, 576);
            AG(le->MEc, 576);
            CK(cudaMemcpy(le->KEc, KE, sizeof(KE), cudaMemcpyHostToDevice));
            CK(cudaMemcpy(le->MEc, ME, sizeof(ME), cudaMemcpyHostToDevice));
            AG(le->chol_w, (size_t)lnd * lnd);
            AG(le->chol_col, lnd);
        }
    }
    le->L[0].kfd = le->kf;
    le->L[0].mfd = le->mf;
    le->Cx = make_elem_const<df>(p.hx, p.hy, p.hz, p.nu);
    // fine-level float factors
    AG(le->L[0].kff, ne);
    AG(le->L[0].mff, ne);

    // operators: effective Newmark matrix K + a5 M + a2 C = (1 + a2 b) K + (a5 + a2 a) M
    // (the negated A of LinearElasticity.cc:1022-1026), and the mass matrix.
    le->ops[0].sK = 1.0 + le->a[2] * p.dbeta;
    le->ops[0].sM = le->a[5] + le->a[2] * p.dalpha;
    le->ops[1].sK = 0.0;
    le->ops[1].sM = 1.0;
    // SOMMG basis operator P0 = K - om^2 M (SOMMG.cc:58-59)
    le->ops[2].sK = 1.0;
    le->ops[2].sM = -p.omega0 * p.omega0;
    if (p.reduction) {
        le->kb = p.basis;
        const int kb = le->kb;
        le->basis32 = p.mixed != 0;
        if (le->basis32) {
            le->qld = (nd + GR_KC - 1) / GR_KC * GR_KC;
            AG(le->Q32, (size_t)kb * le->qld);
            AG(le->Wh, (size_t)kb * le->qld);
            AG(le->Wl, (size_t)kb * le->qld);
            AG(le->Phi32, (size_t)4 * kb * nd);
            AG(le->qd, nd);
            int dev = 0, nsm = 0;
            CK(cudaGetDevice(&dev));
            CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
            le->gram_blocks = 2 * std::max(1, nsm);
            AG(le->gpart, (size_t)le->gram_blocks * 1024);
        } else {
            AG(le->Q, (size_t)kb * nd);
            AG(le->Phi, (size_t)4 * kb * nd);
        }
        AG(le->red, (size_t)6 * kb * kb + kb + 1);
        AG(le->rhist, (size_t)le->Ts * 3 * kb);
        AG(le->Sacc, (size_t)4 * kb * kb);
        AG(le->mdpart, (size_t)kb * MD_CHUNKS);
        AG(le->rstatus, 1);
    }
    for (int o = 0; o < le->nops; o++) {
        Operator &op = le->ops[o];
        op.lv.resize(le->nlev);
        for (int l = 0; l < le->nlev; l++) {
            long long lnd = 3 * le->L[l].g.nn();
            AG(op.lv[l].dinvd, lnd);
            AG(op.lv[l].dinvf, lnd);
            AG(op.lv[l].lohi, 5);
            AG(op.lv[l].cheb, 2 * 64);
            AG(op.lv[l].chebf, 2 * 64);
        }
        if (le->coarse_dense) {
            AG(op.Ainv_d, (size_t)le->ncoarse * le->ncoarse);
            AG(op.Ainv_f, (size_t)le->ncoarse * le->ncoarse);
        }
    }
    CK(cudaStreamSynchronize(le->stream));
    le->stats.device_bytes = (double)arena.bytes;
    return TOPO_OK;
}

void le_destroy(TopoLE *le) {
    if (!le) return;
    if (le->gx_fwd) cudaGraphExecDestroy(le->gx_fwd);
    if (le->gx_adj) cudaGraphExecDestroy(le->gx_adj);
    if (le->u0init) cudaFree(le->u0init);
    le->arena.release();
    if (le->stream) cudaStreamDestroy(le->stream);
    delete le;
}

// ---------------------------------------------------------------------------
// per-design setup of the hierarchy (densities changed)
// ---------------------------------------------------------------------------
static int cheb_kmax(const TopoLE *le) {
    int k = le->p.smooth > le->p.coarse_smooth ? le->p.smooth : le->p.coarse_smooth;
    return k < 1 ? 1 : (k > 64 ? 64 : k);
}

static int setup_operator(TopoLE *le, int o) {
    Operator &op = le->ops[o];
    cudaStream_t s = le->stream;
    for (int l = 0; l < le->nlev; l++) {
        Level &lv = le->L[l];
        const double *kfp = (op.sK != 0.0) ? lv.kfd : nullptr;
        count_launch();
        k_dinv<<<ew_blocks(lv.g.nn()), EW, 0, s>>>(lv.g, lv.fixed, kfp, lv.mfd, op.sK, op.sM, lv.dK[0], lv.dK[1],
                                                   lv.dK[2], lv.dM, op.lv[l].dinvd, op.lv[l].dinvf);
        count_launch();
        k_bounds_init<<<1, 1, 0, s>>>(le->bbits);
        count_launch();
        k_bounds<<<ew_blocks(lv.g.nel()), EW, 0, s>>>(lv.g.nel(), kfp, lv.mfd, op.sK, op.sM, lv.dK[0], lv.dK[1],
                                                      lv.dK[2], lv.dM, lv.lamK, 0.125, 3.375, le->bbits);
        count_launch();
        k_bounds_final<<<1, 1, 0, s>>>(le->bbits, le->p.cheb_ratio, op.lv[l].lohi);
        count_launch();
        k_cheb_table<<<1, 1, 0, s>>>(op.lv[l].lohi, cheb_kmax(le), op.lv[l].cheb);
        count_launch();
        k_cheb_table<<<1, 1, 0, s>>>(op.lv[l].lohi + 2, cheb_kmax(le), op.lv[l].chebf);
    }
    // Kronecker mass preconditioner: node scaling and the stiffness share
    // (sK / sM) max_e(kf_e / mf_e) lambda_max(KE, ME), which bounds the
    // operator against its mass part: u'Au <= (1 + share) sM u'Mu
    {
        Level &l0 = le->L[0];
        count_launch();
        k_kron_scale<double><<<ew_blocks(l0.g.nn()), EW, 0, s>>>(l0.g, l0.fixed, l0.mfd, op.sM, op.kscale_d);
        count_launch();
        k_kron_scale<float><<<ew_blocks(l0.g.nn()), EW, 0, s>>>(l0.g, l0.fixed, l0.mfd, op.sM, op.kscale_f);
        op.share = 0.0;
        if (op.sK != 0.0) {
            unsigned long long hb = 0ull;
            CK(cudaMemsetAsync(le->bbits + 2, 0, sizeof(unsigned long long), s));
            count_launch();
            k_ratio_max<<<red_blocks(l0.g.nel()), EW, 0, s>>>(l0.g.nel(), l0.kfd, l0.mfd, le->bbits + 2);
            CK(cudaMemcpyAsync(&hb, le->bbits + 2, sizeof(hb), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            double ratio;
            memcpy(&ratio, &hb, sizeof(ratio));
            op.share = op.sK / op.sM * ratio * le->mu_KM;
        }
        // the line-staging passes hold whole grid lines in shared memory (FP64: 8 bytes a value)
        const size_t stage = std::max(std::max(kron_x_smem(l0.g, 8), kron_yz_smem(l0.g, 1, 8)),
                                      std::max(kron_yz_smem(l0.g, 2, 8), kron_yz_smem(l0.g, 2, 4, true)));
        op.kron = stage <= KRON_SMEM_MAX && op.sM > 0.0 && op.sK >= 0.0 &&
                  (le->p.mass_precond == 1 || (le->p.mass_precond == 2 && op.share <= le->p.mass_precond_share));
    }
    // adaptive depth: stop at the first level whose Jacobi-scaled operator is
    // well conditioned (bound hi/lo <= adaptive_kappa); a full-spectrum
    // Chebyshev polynomial solves it, so coarser corrections add nothing
    op.depth = le->nlev;
    if (le->p.adaptive_kappa > 0.0) {
        for (int l = 0; l < le->nlev; l++) {
            CK(cudaMemcpyAsync(op.lv[l].hlohi, op.lv[l].lohi, 5 * sizeof(double), cudaMemcpyDeviceToHost, s));
        }
        CK(cudaStreamSynchronize(s));
        for (int l = 0; l < le->nlev - 1; l++) {
            const double *hb = op.lv[l].hlohi;
            if (hb[4] > 0.0 && hb[3] / hb[2] <= le->p.adaptive_kappa) {
                op.depth = l + 1;
                break;
            }
        }
    }
    // dense coarsest operator and its inverse (FP64 Cholesky); not needed
    // when the V-cycle of this operator stops above the coarsest level
    if (!le->coarse_dense || op.depth < le->nlev) {
        CK(cudaGetLastError());
        return TOPO_OK;
    }
    Level &lc = le->L[le->nlev - 1];
    int n = le->ncoarse;
    const double *kfp = (op.sK != 0.0) ? lc.kfd : nullptr;
    count_launch();
    k_coarse_assemble<<<ew_blocks((long long)n * n), EW, 0, s>>>(lc.g, lc.fixed, kfp, lc.mfd, op.sK, op.sM, le->KEc,
                                                                 le->MEc, op.Ainv_d);
    // FP64 Cholesky factor of the coarsest operator, then its inverse from the
    // factor (k_chol_*): A^-1 = L^-T L^-1
    for (int k = 0; k < n; k++) {
        count_launch();
        k_chol_save<<<(n + EW - 1) / EW, EW, 0, s>>>(op.Ainv_d, n, k, le->chol_col);
        count_launch();
        k_chol_update<<<ew_blocks((long long)(n - k) * (n - k)), EW, 0, s>>>(op.Ainv_d, n, k, le->chol_col);
    }
    count_launch();
    k_chol_identity<<<ew_blocks((long long)n * n), EW, 0, s>>>(le->chol_w, n);
    for (int i = 0; i < n; i++) {
        count_launch();
        k_chol_trsv_scale<<<(i + EW) / EW, EW, 0, s>>>(op.Ainv_d, le->chol_w, n, i);
        if (i + 1 < n) {
            count_launch();
            k_chol_trsv_update<<<ew_blocks((long long)(n - i - 1) * (i + 1)), EW, 0, s>>>(op.Ainv_d, le->chol_w,
                                                                                           n, i);
        }
    }
    count_launch();
    k_chol_gram<<<ew_blocks((long long)n * n), EW, 0, s>>>(le->chol_w, n, op.Ainv_d);
    count_launch();
    k_d2f<<<ew_blocks((long long)n * n), EW, 0, s>>>((long long)n * n, op.Ainv_d, op.Ainv_f);
    CK(cudaGetLastError());
    return TOPO_OK;
}

// ---------------------------------------------------------------------------
// V-cycle (returns the buffer holding the level solution)
// ---------------------------------------------------------------------------
template <class T>
struct VW {
    T *b, *xa, *xb, *d, *r;
    const T *dinv;
    const T *kf, *mf;
    const ElemConst<T> *C;
};
template <class T>
static VW<T> vw(TopoLE *le, int o, int l);
template <>
VW<float> vw<float>(TopoLE *le, int o, int l) {
    Level &lv = le->L[l];
    return VW<float>{lv.fb, lv.fxa, lv.fxb, lv.fd, lv.fr, le->ops[o].lv[l].dinvf, lv.kff, lv.mff, &lv.Cf};
}
template <>
VW<double> vw<double>(TopoLE *le, int o, int l) {
    Level &lv = le->L[l];
    return VW<double>{lv.db, lv.dxa, lv.dxb, lv.dd, lv.dr, le->ops[o].lv[l].dinvd, lv.kfd, lv.mfd, &lv.Cd};
}
template <class T>
static const T *kron_fac(TopoLE *le);
template <>
const float *kron_fac<float>(TopoLE *le) { return le->kron_f; }
template <>
const double *kron_fac<double>(TopoLE *le) { return le->kron_d; }
template <class T>
static const T *kron_scale(const Operator &op);
template <>
const float *kron_scale<float>(const Operator &op) { return op.kscale_f; }
template <>
const double *kron_scale<double>(const Operator &op) { return op.kscale_d; }
template <class T>
static const T *ainv(TopoLE *le, int o);
template <>
const float *ainv<float>(TopoLE *le, int o) { return le->ops[o].Ainv_f; }
template <>
const double *ainv<double>(TopoLE *le, int o) { return le->ops[o].Ainv_d; }

// Work of the mixed FCG fused into the fine level of its FP32 V-cycle: the
// first smoothing step re-forms r32 = sigma r after a residual replacement
// (k_mfcg_scale), and the last one computes the FCG dot products of its
// output (k_mfcg_dot).
struct VFuse {
    const double *r64;
    SolveScalars *S;
    const float *q32;
    Partials<2> part;
    bool scaled = false, dotted = false;
};

template <class T>
static T *vcycle(TopoLE *le, int o, int l, const T *b, VFuse *fz = nullptr) {
    cudaStream_t s = le->stream;
    Level &lv = le->L[l];
    VW<T> w = vw<T>(le, o, l);
    Operator &op = le->ops[o];
    long long nd = 3 * lv.g.nn();
    Weights<T> wt{op.sK != 0.0 ? w.kf : nullptr, w.mf, nullptr, (T)op.sK, (T)op.sM};
    const double *lohi = op.lv[l].cheb;
    T *x = w.xa, *xo = w.xb;
    const bool fuse = fz && l == 0 && std::is_same<T, float>::value;
    // first step from zero: x = d = c2 Dinv b
    auto first = [&](const double *tab) {
        if constexpr (std::is_same<T, float>::value) {
            if (fuse) {
                count_launch();
                k_cheb0_rescale<<<ew_blocks(nd), EW, 0, s>>>(nd, fz->r64, const_cast<float *>(b), w.dinv, tab, x, w.d,
                                                             fz->S);
                fz->scaled = true;
                return;
            }
        }
        count_launch();
        k_cheb0<T><<<ew_blocks(nd), EW, 0, s>>>(nd, b, w.dinv, tab, x, w.d);
    };
    // smoothing step k (one operator application); `last`: this level's
    // final step, whose output is the V-cycle result at the fine level
    auto step = [&](const double *tab, int k, bool last) {
        bool done = false;
        if constexpr (std::is_same<T, float>::value) {
            if (fuse && last) {
                PolChebDot pc{lv.fixed, wt, x, b, w.dinv, xo, w.d, tab, k, fz->q32, fz->S, fz->part};
                launch_tile<float>(lv.g, *w.C, pc, s);
                fz->dotted = true;
                done = true;
            }
        }
        if (!done) {
            PolCheb<T> pc{lv.fixed, wt, x, b, w.dinv, xo, w.d, tab, k, {}};
            launch_tile<T>(lv.g, *w.C, pc, s);
        }
        T *t = x;
        x = xo;
        xo = t;
    };
    if (l == op.depth - 1 && op.depth < le->nlev) {
        // well-conditioned level: full-spectrum Chebyshev-Jacobi solve from zero
        const double *full = op.lv[l].chebf;
        first(full);
        for (int k = 1; k < le->p.coarse_smooth; k++) step(full, k, k == le->p.coarse_smooth - 1);
        return x;
    }
    if (l == le->nlev - 1) {
        if (le->coarse_dense) {
            int n = le->ncoarse;
            count_launch();
            k_gemv<T><<<(n * 32 + 255) / 256, 256, 0, s>>>(n, ainv<T>(le, o), b, w.xa);
            return w.xa;
        }
        // iterative coarse solve: Chebyshev-Jacobi polynomial from zero
        first(lohi);
        for (int k = 1; k < le->p.coarse_smooth; k++) step(lohi, k, k == le->p.coarse_smooth - 1);
        return x;
    }
    const int nu = le->p.smooth;
    first(lohi);
    for (int k = 1; k < nu; k++) step(lohi, k, false);
    PolResid<T> pr{lv.fixed, wt, x, b, w.r, {}};
    launch_tile<T>(lv.g, *w.C, pr, s);
    Level &lc = le->L[l + 1];
    VW<T> wc = vw<T>(le, o, l + 1);
    count_launch();
    k_restrict<T><<<ew_blocks(lc.g.nn()), EW, 0, s>>>(lv.g, lc.g, lc.fixed, w.r, wc.b);
    T *xc = vcycle<T>(le, o, l + 1, wc.b);
    count_launch();
    k_prolong<T><<<ew_blocks(lv.g.nn()), EW, 0, s>>>(lv.g, lc.g, lv.fixed, xc, x);
    for (int k = 0; k < nu; k++) step(lohi, k, k == nu - 1);
    return x;
}

// Kronecker mass preconditioner applied to the fine-level residual r;
// returns the buffer holding z = P^-1 r
template <class T>
static T *kron_apply(TopoLE *le, int o, T *r, VFuse *fz = nullptr) {
    cudaStream_t s = le->stream;
    Level &l0 = le->L[0];
    VW<T> w = vw<T>(le, o, 0);
    const GridDesc &g = l0.g;
    KronBand<T> B{kron_fac<T>(le), le->kron_nmax};
    const T *sc = kron_scale<T>(le->ops[o]);
    const bool mixed = fz && std::is_same<T, float>::value;
    const long long nlines = (long long)g.ny * g.nz;
    static int nsm_dev[MAX_DEVICES] = {};
    int &nsm = nsm_dev[device_slot()];
    if (!nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        nsm = std::max(nsm, 1);
    }
    const int kx = kx_lines_launch(g, sizeof(T), 4LL * nsm);  // 4 resident CTAs of the x pass per SM
    const size_t smx = kron_x_smem(g, sizeof(T), kx), smy = kron_yz_smem(g, 1, sizeof(T));
    static bool attr_dev[MAX_DEVICES] = {};
    bool &attr = attr_dev[device_slot()];
    if (!attr) {  // staged lines: the selection keeps every pass within KRON_SMEM_MAX
        cudaFuncSetAttribute(k_kron_x<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KRON_SMEM_MAX);
        cudaFuncSetAttribute(k_kron_yz<T, T, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KRON_SMEM_MAX);
        cudaFuncSetAttribute(k_kron_yz<T, T, 2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KRON_SMEM_MAX);
        cudaFuncSetAttribute(k_kron_yz<T, T, 2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)KRON_SMEM_MAX);
        attr = true;
    }
    bool t;
    count_launch();
    t = timer_begin(TOPO_KT_KRON, g.nn(), s);
    k_kron_x<T, T><<<(unsigned)((nlines + kx - 1) / kx), KRON_THREADS, smx, s>>>(
        g, kx, r, mixed ? fz->r64 : nullptr, mixed ? fz->S : nullptr, sc, B, w.xa);
    timer_end(t, s);
    count_launch();
    t = timer_begin(TOPO_KT_KRON, g.nn(), s);
    k_kron_yz<T, T, 1, false><<<kron_yz_blocks(g, 1), KRON_THREADS, smy, s>>>(g, r, sc, B, w.xa, w.xb, KronDot{});
    timer_end(t, s);
    count_launch();
    t = timer_begin(TOPO_KT_KRON, g.nn(), s);
    if (mixed && le->p.mass_precond_smooth <= 0) {
        k_kron_yz<T, T, 2, true><<<kron_yz_blocks(g, 2), KRON_THREADS, kron_yz_smem(g, 2, sizeof(T), true), s>>>(
            g, r, sc, B, w.xb, w.xa, KronDot{fz->q32, fz->S, fz->part});
        fz->dotted = true;
    } else {
        k_kron_yz<T, T, 2, false><<<kron_yz_blocks(g, 2), KRON_THREADS, kron_yz_smem(g, 2, sizeof(T)), s>>>(
            g, r, sc, B, w.xb, w.xa, KronDot{});
    }
    timer_end(t, s);
    if (mixed) fz->scaled = true;
    return w.xa;
}

// Chebyshev-Jacobi steps over the full spectrum of Dinv A after the
// Kronecker solve z0: z <- z + d, d = c1 d + c2 Dinv (r - A z); with `fz`
// (mixed FCG) the last step also forms the FCG dot products
template <class T>
static T *kron_smooth(TopoLE *le, int o, const T *r, T *z0, VFuse *fz) {
    const int ns = le->p.mass_precond_smooth;
    if (ns <= 0) return z0;
    cudaStream_t s = le->stream;
    Level &l0 = le->L[0];
    VW<T> w = vw<T>(le, o, 0);
    Operator &op = le->ops[o];
    Weights<T> wt{op.sK != 0.0 ? w.kf : nullptr, w.mf, nullptr, (T)op.sK, (T)op.sM};
    const double *tab = op.lv[0].chebf;
    T *x = z0, *xo = (z0 == w.xa) ? w.xb : w.xa;
    for (int k = 0; k < ns; k++) {
        bool done = false;
        if constexpr (std::is_same<T, float>::value) {
            if (fz && k == ns - 1) {
                PolChebDot pc{l0.fixed, wt, x, r, w.dinv, xo, w.d, tab, k, fz->q32, fz->S, fz->part};
                launch_tile<float>(l0.g, *w.C, pc, s);
                fz->dotted = true;
                done = true;
            }
        }
        if (!done) {
            PolCheb<T> pc{l0.fixed, wt, x, r, w.dinv, xo, w.d, tab, k, {}};
            launch_tile<T>(l0.g, *w.C, pc, s);
        }
        T *t = x;
        x = xo;
        xo = t;
    }
    return x;
}

// ---------------------------------------------------------------------------
// flexible CG:  (N A N + I - N) x = b for operator o; sx holds the initial guess
// ---------------------------------------------------------------------------
__global__ void k_solve_prime(SolveScalars *S, double tol2, int maxit, double tau2, int kmax, double ndof) {
    S->ndof = ndof;
    S->tol2 = tol2;
    S->maxit = maxit;
    S->tau2 = tau2;
    S->kmax = kmax;
    S->done = 0;
    S->status = 0;
    S->it = 0;
}
__global__ void k_solve_check(const SolveScalars *S, int *err) {
    if (S->status != 0 && *err == 0) *err = S->status;
}

static const double *&cur_b(TopoLE *le);
// mixed path: tracked operator products (A u of the forward states, A lambda of
// the adjoint iterates) in place of mass products
static bool al_mode(const TopoLE *le) { return le->AUt != nullptr; }
// mixed-precision FCG for this solve (FP64 FCG for the plain path and for
// solves that set fp64_solves)
static bool mixed_fcg(const TopoLE *le) { return le->p.mixed && !le->fp64_solves; }
template <class A>
static void solve_init_t(TopoLE *le, int o, const double *b, cudaGraphConditionalHandle cond, int has_cond) {
    Level &l0 = le->L[0];
    Operator &op = le->ops[o];
    Weights<A> wt = fine_weights<A>(le, op.sK != 0.0, true, nullptr, op.sK, op.sM);
    PolInitResid<A> pi{l0.fixed, wt, le->sx, b, le->sr, mixed_fcg(le) ? le->sr32 : nullptr, le->S, cond, has_cond, P2(le)};
    launch_tile<A>(l0.g, fine_const<A>(le), pi, le->stream);
}
static void fwd_rhs_init(TopoLE *le, cudaGraphConditionalHandle cond, int has_cond);
static void solve_init(TopoLE *le, int o, const double *b, cudaGraphConditionalHandle cond, int has_cond) {
    cur_b(le) = b;
    if (le->fwd_init_pending) {  // right-hand side, initial guess and residual in one pass
        le->fwd_init_pending = false;
        fwd_rhs_init(le, cond, has_cond);
        return;
    }
    if (le->ax0_pending) {  // the caller formed (N A N + I - N) x0 in sq
        le->ax0_pending = false;
        count_launch();
        // AL mode: x0 is accepted only on a true residual, which keeps
        // A lambda = b - r exact for the stored lambda
        k_init_pointwise<<<red_blocks(le->ndof), EW, 0, le->stream>>>(le->ndof, b, le->sq, le->sr, le->S,
                                                                       mixed_fcg(le) ? 1 : 0, al_mode(le) ? 0 : 1,
                                                                       cond, has_cond, P2(le));
        return;
    }
    if (mixed_fcg(le))
        solve_init_t<df>(le, o, b, cond, has_cond);
    else
        solve_init_t<double>(le, o, b, cond, has_cond);
}

// right-hand side of the solve in flight (set by solve_init)
static const double *&cur_b(TopoLE *le) {
    static thread_local const double *b = nullptr;
    (void)le;
    return b;
}

static void solve_iteration(TopoLE *le, int o, cudaGraphConditionalHandle cond, int has_cond) {
    cudaStream_t s = le->stream;
    Level &l0 = le->L[0];
    Operator &op = le->ops[o];
    long long nd = le->ndof;
    unsigned nb = ew_blocks(nd);
    if (mixed_fcg(le)) {
        // reliable-update mixed precision: FP32 recurrence, FP64 replacements.
        // The rescaling of r32 and the dot products ride on the first and
        // last fine-level smoothing steps, the direction update on PolPQ32.
        VFuse fz{le->sr, le->S, le->sq32, P2(le)};
        float *z = nullptr;
        if (op.kron) {
            z = kron_apply<float>(le, o, le->sr32, &fz);
            z = kron_smooth<float>(le, o, le->sr32, z, &fz);
        } else {
            if (le->ops[o].depth == 1 && le->nlev == 1 && le->coarse_dense) {
                count_launch();  // the dense coarse solve has no smoothing step to carry the rescaling
                k_mfcg_scale<<<red_blocks(nd), EW, 0, s>>>(nd, le->sr, le->sr32, le->S);
            }
            z = vcycle<float>(le, o, 0, le->sr32, &fz);
        }
        if (!fz.dotted) {
            count_launch();
            k_mfcg_dot<<<red_blocks(nd), EW, 0, s>>>(nd, z, le->sr32, le->sq32, le->S, P2(le));
        }
        Weights<float> wf{op.sK != 0.0 ? l0.kff : nullptr, l0.mff, nullptr, (float)op.sK, (float)op.sM};
        PolPQ32 pq32{l0.fixed, wf, z, {le->sp32, le->sp32b}, le->sq32, le->S, P1(le)};
        launch_tile<float>(l0.g, l0.Cf, pq32, s);
        count_launch();
        k_mfcg_update<<<red_blocks(nd), EW, 0, s>>>(nd, le->sx, le->sr32, le->sp32, le->sp32b, le->sq32, le->S,
                                                    P1(le));
        Weights<df> wd = fine_weights<df>(le, op.sK != 0.0, true, nullptr, op.sK, op.sM);
        PolReplace<df> rp{l0.fixed, wd, le->sx, cur_b(le), le->sr, le->S, cond, has_cond, P1(le)};
        launch_tile<df>(l0.g, le->Cx, rp, s);
        return;
    } else {
        double *z = op.kron ? kron_smooth<double>(le, o, le->sr, kron_apply<double>(le, o, le->sr), nullptr)
                            : vcycle<double>(le, o, 0, le->sr);
        count_launch();
        k_fcg_dot<double><<<red_blocks(nd), EW, 0, s>>>(nd, z, le->sr, le->sq, le->S, P2(le));
        count_launch();
        k_fcg_p<double><<<nb, EW, 0, s>>>(nd, z, le->sp, le->S);
    }
    Weights<double> wt{op.sK != 0.0 ? l0.kfd : nullptr, l0.mfd, nullptr, op.sK, op.sM};
    PolPQ<double> pq{l0.fixed, wt, le->sp, le->sq, le->S, P1(le)};
    launch_tile<double>(l0.g, l0.Cd, pq, s);
    count_launch();
    k_fcg_update<<<red_blocks(nd), EW, 0, s>>>(nd, le->sx, le->sr, mixed_fcg(le) ? le->sr32 : nullptr, le->sp, le->sq, le->S,
                                   P1(le), cond, has_cond);
}

// direct launches, host checks convergence after every iteration
static int solve_direct(TopoLE *le, int o, const double *b) {
    count_launch();
    k_solve_prime<<<1, 1, 0, le->stream>>>(le->S, le->p.rtol * le->p.rtol, le->p.maxit,
                                              le->p.inner_tol * le->p.inner_tol, le->p.inner_maxit,
                                              (double)le->ndof);
    solve_init(le, o, b, 0, 0);
    SolveScalars h;
    for (;;) {
        CK(cudaMemcpyAsync(&h, le->S, sizeof(h), cudaMemcpyDeviceToHost, le->stream));
        CK(cudaStreamSynchronize(le->stream));
        if (h.done) break;
        solve_iteration(le, o, 0, 0);
        le->direct_iters++;
    }
    count_launch();
    k_fcg_zero_x<<<red_blocks(le->ndof), EW, 0, le->stream>>>(le->ndof, le->sx, le->S);
    count_launch();
    k_solve_check<<<1, 1, 0, le->stream>>>(le->S, le->err);
    le->nsolves++;
    if (!le->ops[o].kron) le->mg_solves++;
    CK(cudaGetLastError());
    return TOPO_OK;
}

// inside stream capture: the FCG loop becomes a conditional WHILE node whose
// body is the iteration; the device sets the condition after each iteration
static int solve_captured(TopoLE *le, int o, const double *b) {
    cudaStream_t s = le->stream;
    count_launch();
    k_solve_prime<<<1, 1, 0, s>>>(le->S, le->p.rtol * le->p.rtol, le->p.maxit, le->p.inner_tol * le->p.inner_tol,
                                  le->p.inner_maxit, (double)le->ndof);
    cudaStreamCaptureStatus cs;
    cudaGraph_t graph;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edata = nullptr;
    size_t ndeps = 0;
    CK(cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, &edata, &ndeps));
    cudaGraphConditionalHandle h;
    CK(cudaGraphConditionalHandleCreate(&h, graph, 0, 0));
    solve_init(le, o, b, h, 1);
    CK(cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, &edata, &ndeps));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode;
    CK(cudaGraphAddNode(&cnode, graph, deps, edata, ndeps, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    CK(cudaStreamUpdateCaptureDependencies(s, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaStream_t bs;
    CK(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking));
    CK(cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    le->stream = bs;
    long long c0 = launch_counter();
    solve_iteration(le, o, h, 1);
    le->body_kernels = launch_counter() - c0;
    le->stream = s;
    cudaGraph_t outg;
    cudaError_t e1 = cudaStreamEndCapture(bs, &outg);
    cudaStreamDestroy(bs);
    CK(e1);
    count_launch();
    k_fcg_zero_x<<<red_blocks(le->ndof), EW, 0, s>>>(le->ndof, le->sx, le->S);
    count_launch();
    k_solve_check<<<1, 1, 0, s>>>(le->S, le->err);
    return TOPO_OK;
}

static int solve(TopoLE *le, int o, const double *b, bool capturing) {
    return capturing ? solve_captured(le, o, b) : solve_direct(le, o, b);
}

// ---------------------------------------------------------------------------
// forward step j of block c (SolveStateBlock, LinearElasticity.cc:1317-1385)
// ---------------------------------------------------------------------------
template <class A>
static void fwd_rhs_t(TopoLE *le) {
    const LEParams &p = le->p;
    Level &l0 = le->L[0];
    const double *a = le->a;
    PolRhsFwd<A> pr;
    memset(&pr, 0, sizeof(pr));
    pr.fixed = l0.fixed;
    pr.w = fine_weights<A>(le, true, true, nullptr, 1.0, 1.0);
    pr.cp = le->cp;
    pr.Uh = le->Uh;
    pr.DUh = le->DUh;
    pr.DDUh = le->DDUh;
    pr.ndof = le->ndof;
    pr.rhs0 = le->rhs0;
    pr.sig = le->sigtab;
    pr.sig2 = le->sigtab + le->Ts;
    pr.load2_dof = p.load2_node >= 0 ? 3LL * p.load2_node + 2 : -1;
    // B1 u- + B2 du- + B3 ddu- = M (cM . s-) + K (cK . s-)  (LinearElasticity.cc:1028-1044)
    pr.cM[0] = a[5] + a[2] * p.dalpha;
    pr.cM[1] = a[3] - a[0] * p.dalpha;
    pr.cM[2] = a[4] - a[1] * p.dalpha;
    pr.cK[0] = a[2] * p.dbeta;
    pr.cK[1] = -a[0] * p.dbeta;
    pr.cK[2] = -a[1] * p.dbeta;
    // Newmark predictor u- + dt du- + (1/2 - 1/4) dt^2 ddu- as initial guess
    double dt = le->dt;
    pr.pred[0] = 1.0;
    pr.pred[1] = (p.ti == 0) ? 0.0 : dt;
    // (second-order guess: the same with the acceleration held over the step,
    // u- + dt du- + dt^2/2 ddu-, the Newmark update with ddu+ = ddu-)
    pr.pred[2] = (p.ti == 0) ? 0.0 : (p.extrapolate ? 0.5 : 0.25) * dt * dt;
    // third-order guess: the Newmark update with ddu+ extrapolated linearly,
    // u- + dt du- + dt^2/4 (ddu- + 2 ddu- - ddu--)
    pr.use_pred2 = (p.ti != 0 && p.extrapolate >= 2) ? 1 : 0;
    pr.pred2[0] = 0.75 * dt * dt;
    pr.pred2[1] = -0.25 * dt * dt;
    pr.st = le->st;
    pr.b = le->sb;
    pr.x0 = le->sx;
    launch_tile<A>(l0.g, fine_const<A>(le), pr, le->stream);
}
static void fwd_rhs(TopoLE *le) {
    if (le->p.mixed)
        fwd_rhs_t<df>(le);
    else
        fwd_rhs_t<double>(le);
}

// coefficients of the next-step preparation (k_newmark_track, k_fwd_prep)
static FwdPrep fwd_prep_args(TopoLE *le) {
    const LEParams &p = le->p;
    const double *a = le->a;
    const Operator &op = le->ops[0];
    FwdPrep P;
    memset(&P, 0, sizeof(P));
    // B_i = cM_i M + cK_i K of (u-, du-, ddu-) (LinearElasticity.cc:1028-1044)
    const double cM[3] = {a[5] + a[2] * p.dalpha, a[3] - a[0] * p.dalpha, a[4] - a[1] * p.dalpha};
    const double cK[3] = {a[2] * p.dbeta, -a[0] * p.dbeta, -a[1] * p.dbeta};
    for (int i = 0; i < 3; i++) {
        P.cA[i] = cM[i] / op.sM;
        P.ck[i] = cK[i] - cM[i] * op.sK / op.sM;
    }
    // initial guess: the Newmark predictor u- + dt du- + (1/2 - 1/4) dt^2 ddu-,
    // or (extrapolate >= 1) with ddu+ = ddu- held over the step,
    // u- + dt du- + dt^2/2 ddu-; third order (extrapolate = 2): ddu+
    // extrapolated linearly, u- + dt du- + dt^2/4 (3 ddu- - ddu--)
    const double dt = le->dt;
    P.pred[0] = 1.0;
    P.pred[1] = (p.ti == 0) ? 0.0 : dt;
    P.pred[2] = (p.ti == 0) ? 0.0 : (p.extrapolate ? 0.5 : 0.25) * dt * dt;
    P.use_pred2 = (p.ti != 0 && p.extrapolate >= 2) ? 1 : 0;
    P.pred2[0] = 0.75 * dt * dt;
    P.pred2[1] = -0.25 * dt * dt;
    P.KS = le->KSt;
    P.X0 = le->sx;
    P.BT = le->sb;
    P.AX = le->sr;
    for (int i = 0; i < 3; i++) {
        P.dck[i] = f64_to_df(P.ck[i]);
        P.dcA[i] = f64_to_df(P.cA[i]);
        P.dpred[i] = f64_to_df(P.pred[i]);
    }
    for (int i = 0; i < 2; i++) P.dpred2[i] = f64_to_df(P.pred2[i]);
    return P;
}

template <bool HK, bool HM>
static void product(TopoLE *le, const double *x, double *y, const double *P, double sK, double sM);
template <class A, bool HK, bool HM>
static void product_t(TopoLE *le, const double *x, double *y, const double *P, double sK, double sM);

// Mixed path only (tracked products exist only there): y = K KS in one K-only
// double-float pass (FP32 rounding of K applied to the near-rigid local motion
// of the state would put noise into b above the solve tolerance: measured 4.3
// instead of 2.8 Krylov iterations per solve on the 96x48x48 cantilever), then
// b, r0 and the FCG set-up in a streaming kernel
static void fwd_rhs_init(TopoLE *le, cudaGraphConditionalHandle cond, int has_cond) {
    const LEParams &p = le->p;
    product_t<df, true, false>(le, le->KSt, le->sq, nullptr, 1.0, 0.0);
    RhsLoad L{le->rhs0, le->sigtab, le->sigtab + le->Ts, p.load2_node >= 0 ? 3LL * p.load2_node + 2 : -1};
    count_launch();
    k_rhs_finish<<<red_blocks(le->ndof), EW, 0, le->stream>>>(le->ndof, le->L[0].fixed, le->sq, L, le->st, le->sb,
                                                               le->sr, le->S, cond, has_cond, P2(le));
}


// tracked products A u, A du, A ddu of a block's start state (checkpoint c),
// then the first step's preparation
static void track_block_start(TopoLE *le, int c) {
    const long long nd = le->ndof;
    const double *base = le->cp + (size_t)c * 3 * nd;
    const Operator &op = le->ops[0];
    product<true, true>(le, base, le->AUt, nullptr, op.sK, op.sM);
    product<true, true>(le, base + nd, le->AVt, nullptr, op.sK, op.sM);
    product<true, true>(le, base + 2 * nd, le->AAt, nullptr, op.sK, op.sM);
    count_launch();
    k_fwd_prep<<<ew_blocks(nd), EW, 0, le->stream>>>(nd, base, base + nd, base + 2 * nd, nullptr, le->AUt, le->AVt,
                                                      le->AAt, nullptr, fwd_prep_args(le));
}

// Re-anchoring of the tracked A du, A ddu before step j of block c (and the
// step's preparation).  Given the states u, the corrector
// du+ = -du + (2/dt) (u+ - u), ddu+ = (4/dt^2) (u+ - u) - (4/dt) du - ddu has
// a double eigenvalue -1, so rounding in the tracked A u (about 1e-14
// relative) grows like n^1.5 in A ddu; over 200 steps it reaches the 1e-10
// solve tolerance and costs extra Krylov iterations.  Exact products every
// TRACK_ANCHOR steps bound n.
constexpr int TRACK_ANCHOR = 32;
static void track_anchor(TopoLE *le, int c, int j) {
    const long long nd = le->ndof;
    const Operator &op = le->ops[0];
    const double *u = le->Uh + (size_t)(j - 1) * nd, *du = le->DUh + (size_t)(j - 1) * nd,
                 *ddu = le->DDUh + (size_t)(j - 1) * nd;
    const double *ddu2 = (j >= 2) ? le->DDUh + (size_t)(j - 2) * nd : le->cp + (size_t)c * 3 * nd + 2 * nd;
    product<true, true>(le, du, le->AVt, nullptr, op.sK, op.sM);
    product<true, true>(le, ddu, le->AAt, nullptr, op.sK, op.sM);
    product<true, true>(le, ddu2, le->AApt, nullptr, op.sK, op.sM);
    count_launch();
    k_fwd_prep<<<ew_blocks(nd), EW, 0, le->stream>>>(nd, u, du, ddu, ddu2, le->AUt, le->AVt, le->AAt, le->AApt,
                                                      fwd_prep_args(le));
}

// Mixed path: right-hand side and initial residual from one K-only pass and a
// streaming kernel (fwd_rhs_init) on what the previous corrector prepared; the corrector
// tracks the products of the new state and prepares the next step
// (k_newmark_track).  Plain FP64 path: right-hand side from the stored
// states, the initial residual b - A x0, the corrector.
static int fwd_step(TopoLE *le, bool capturing) {
    cudaStream_t s = le->stream;
    const bool track = le->AUt != nullptr;
    if (track)
        le->fwd_init_pending = true;
    else
        fwd_rhs(le);
    int rc = solve(le, 0, le->sb, capturing);
    le->fwd_init_pending = false;
    if (rc) return rc;
    Newmark nm;
    memcpy(nm.a, le->a, sizeof(nm.a));
    for (int i = 0; i < 6; i++) nm.da[i] = f64_to_df(nm.a[i]);
    count_launch();
    if (track && le->a[0] == -1.0 && le->a[1] == 0.0)
        k_newmark_track<true><<<ew_blocks(le->ndof), EW, 0, s>>>(le->ndof, le->sx, le->st, le->cp, le->Uh, le->DUh,
                                                                 le->DDUh, nm, le->sb, le->sr, le->S, le->AUt,
                                                                 le->AVt, le->AAt, fwd_prep_args(le));
    else if (track)
        k_newmark_track<false><<<ew_blocks(le->ndof), EW, 0, s>>>(le->ndof, le->sx, le->st, le->cp, le->Uh,
                                                                  le->DUh, le->DDUh, nm, le->sb, le->sr, le->S,
                                                                  le->AUt, le->AVt, le->AAt, fwd_prep_args(le));
    else
        k_newmark<<<ew_blocks(le->ndof), EW, 0, s>>>(le->ndof, le->sx, le->st, le->cp, le->Uh, le->DUh, le->DDUh,
                                                     nm);
    count_launch();
    k_step_add<<<1, 1, 0, s>>>(le->st, +1);
    return TOPO_OK;
}

// ---------------------------------------------------------------------------
// adjoint step j (SolveLagrangen body) and the t = 0 pass (SolveLagrange0)
// ---------------------------------------------------------------------------
template <class A, bool HK, bool HM>
static void product_t(TopoLE *le, const double *x, double *y, const double *P, double sK, double sM) {
    Level &l0 = le->L[0];
    PolProduct<A, HK, HM> pp{fine_weights<A>(le, HK, HM, P, sK, sM), x, y, {}};
    launch_tile<A>(l0.g, fine_const<A>(le), pp, le->stream);
}
template <bool HK, bool HM>
static void product(TopoLE *le, const double *x, double *y, const double *P, double sK, double sM) {
    if (le->p.mixed)
        product_t<df, HK, HM>(le, x, y, P, sK, sM);
    else
        product_t<double, HK, HM>(le, x, y, P, sK, sM);
}

// objective gradient products h (objectives 3-6) of the state `state_base`
// (U/DU base pointers resolved by the step index, or the t = 0 state)
__global__ void k_select_state(long long ndof, const StepCtx *st, const double *Uh, const double *DUh, int t0mode,
                               const double *cp, double *outU, double *outDU) {
    const double *u, *du;
    if (t0mode) {
        u = cp;
        du = cp + ndof;
    } else {
        u = Uh + (long long)st->j * ndof;
        du = DUh + (long long)st->j * ndof;
    }
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x) {
        if (outU) outU[i] = u[i];
        if (outDU) outDU[i] = du[i];
    }
}

static void objective_products(TopoLE *le, int t0mode) {
    int obj = le->p.objective;
    if (obj < 3 || obj == 7) return;
    double dt = le->dt;
    // stage the needed state vectors into the solver scratch (sp, sq are free here)
    bool needU = (obj == 3 || obj == 5), needDU = (obj >= 4);
    count_launch();
    k_select_state<<<ew_blocks(le->ndof), EW, 0, le->stream>>>(le->ndof, le->st, le->Uh, le->DUh, t0mode, le->cp,
                                                                 needU ? le->sp : nullptr, needDU ? le->sq : nullptr);
    if (obj == 3) product<true, false>(le, le->sp, le->hK, le->P, dt, 0.0);
    if (obj == 4) product<false, true>(le, le->sq, le->hM, le->P, 0.0, dt);
    if (obj == 5) {
        product<true, false>(le, le->sp, le->hK, le->P, dt, 0.0);
        product<false, true>(le, le->sq, le->hM, le->P, 0.0, dt);
    }
    if (obj == 6) product<true, true>(le, le->sq, le->hK, le->P, dt * le->p.dbeta, dt * le->p.dalpha);
}

static AdjCombine adj_args(TopoLE *le, int t0mode) {
    const LEParams &p = le->p;
    const double *a = le->a;
    AdjCombine A;
    memset(&A, 0, sizeof(A));
    A.fixed = le->L[0].fixed;
    A.KL = le->KL;
    A.ML = le->ML;
    A.Lp1 = le->Lp1;
    A.DLp1 = le->DLp1;
    A.DDLp1 = le->DDLp1;
    A.Lp2 = le->Lp2;
    A.Lp3 = le->Lp3;
    A.extrapolate = le->p.extrapolate;
    A.hK = le->hK;
    A.hM = le->hM;
    A.cntP = le->cntP;
    A.Ustate = le->Uh;
    A.DUstate = le->DUh;
    A.DDUstate = le->DDUh;
    A.cp = le->cp;
    A.ndof = le->ndof;
    A.objective = p.objective;
    A.out_dof = le->out_dof;
    A.fx = &le->st->fx;
    A.t0mode = t0mode;
    A.dt = le->dt;
    memcpy(A.a, a, sizeof(A.a));
    A.cM[0] = a[5] + a[2] * p.dalpha;
    A.cM[1] = a[3] - a[0] * p.dalpha;
    A.cM[2] = a[4] - a[1] * p.dalpha;
    A.cK[0] = a[2] * p.dbeta;
    A.cK[1] = -a[0] * p.dbeta;
    A.cK[2] = -a[1] * p.dbeta;
    A.st = le->st;
    A.DL = le->DLc;
    A.DDL = le->DDLc;
    A.b = le->sb;
    A.x0 = le->sx;
    if (le->KLh1) {
        A.ax0 = le->sq;
        A.KLh1 = le->KLh1;
        A.MLh1 = le->MLh1;
        A.KLh2 = le->KLh2;
        A.MLh2 = le->MLh2;
        A.sK = t0mode ? le->ops[1].sK : le->ops[0].sK;
        A.sM = t0mode ? le->ops[1].sM : le->ops[0].sM;
    }
    if (al_mode(le)) {
        // the ML slots hold A L (A = sK K + sM M of the step operator):
        // B_i L = cM_i M L + cK_i K L = (cM_i / sM) A L + (cK_i - cM_i sK / sM) K L,
        // and (N A N + I - N) x0 = sum_w w A L directly
        const double sK = le->ops[0].sK, sM = le->ops[0].sM;
        for (int i = 0; i < 3; i++) {
            A.cK[i] -= A.cM[i] * sK / sM;
            A.cM[i] /= sM;
        }
        A.sK = 0.0;
        A.sM = 1.0;
    }
    for (int i = 0; i < 6; i++) A.da[i] = f64_to_df(A.a[i]);
    for (int i = 0; i < 3; i++) {
        A.dcM[i] = f64_to_df(A.cM[i]);
        A.dcK[i] = f64_to_df(A.cK[i]);
    }
    A.ddt = f64_to_df(A.dt);
    A.dsK = f64_to_df(A.sK);
    A.dsM = f64_to_df(A.sM);
    return A;
}

static SensArgs sens_args(TopoLE *le, int t0mode) {
    const LEParams &p = le->p;
    const double *a = le->a;
    SensArgs S;
    memset(&S, 0, sizeof(S));
    S.g = le->g;
    S.lam = le->sx;
    S.Uh = le->Uh;
    S.DUh = le->DUh;
    S.DDUh = le->DDUh;
    S.cp = le->cp;
    S.kf = le->kf;
    S.dkf = le->dkf;
    S.mf = le->mf;
    S.dmf = le->dmf;
    S.P = le->P;
    double al = p.dalpha, be = p.dbeta;
    if (t0mode) {
        // DDL0' (dK u0 + dC du0 + dM ddu0), dC = alpha dM + beta dK (LinearElasticity.cc:2154-2162)
        S.aK[0] = 1.0;
        S.aK[1] = be;
        S.aK[2] = 0.0;
        S.aM[0] = 0.0;
        S.aM[1] = al;
        S.aM[2] = 1.0;
    } else {
        // lambda' (dA/dx u + dB1/dx u- + dB2/dx du- + dB3/dx ddu-) (LinearElasticity.cc:1996-2016)
        S.aK[0] = -(1.0 + a[2] * be);
        S.bK[0] = a[2] * be;
        S.bK[1] = -a[0] * be;
        S.bK[2] = -a[1] * be;
        S.aM[0] = -(a[5] + a[2] * al);
        S.bM[0] = a[5] + a[2] * al;
        S.bM[1] = a[3] - a[0] * al;
        S.bM[2] = a[4] - a[1] * al;
    }
    S.dt = le->dt;
    S.dalpha = al;
    S.dbeta = be;
    S.t0mode = t0mode;
    S.with_objective = 1;
    S.st = le->st;
    S.df = le->df;
    S.fx = &le->st->fx;
    S.part = P1(le);
    for (int i = 0; i < 3; i++) {
        S.daK[i] = f64_to_df(S.aK[i]);
        S.dbK[i] = f64_to_df(S.bK[i]);
        S.daM[i] = f64_to_df(S.aM[i]);
        S.dbM[i] = f64_to_df(S.bM[i]);
    }
    return S;
}

static bool sens_in_fp32(const TopoLE *le) { return le->p.mixed && le->p.sens_fp32; }

template <int OBJ>
static void launch_sens_obj(TopoLE *le, const SensArgs &S) {
    count_launch();
    if (sens_in_fp32(le))
        k_sens<OBJ, float><<<red_blocks(le->nel), EW, 0, le->stream>>>(S, le->L[0].Cf);
    else
        k_sens<OBJ, double><<<red_blocks(le->nel), EW, 0, le->stream>>>(S, le->L[0].Cd);
}
static void launch_sens(TopoLE *le, int t0mode) {
    SensArgs S = sens_args(le, t0mode);
    long long nd = le->ndof;
    if (sens_in_fp32(le)) {
        const int ob = le->p.objective;
        S.wKf = le->sw32;
        S.wMf = le->sw32 + nd;
        S.lamf = le->sw32 + 2 * nd;
        S.uf = (ob == 3 || ob == 5) ? le->sw32 + 3 * nd : nullptr;
        S.duf = (ob == 4 || ob == 5 || ob == 6) ? le->sw32 + 4 * nd : nullptr;
    } else {
        S.wKd = le->sw64;
        S.wMd = le->sw64 + nd;
    }
    count_launch();
    k_sens_nodal<<<ew_blocks(nd), EW, 0, le->stream>>>(S);
    switch (le->p.objective) {
    case 0: launch_sens_obj<0>(le, S); break;
    case 1: launch_sens_obj<1>(le, S); break;
    case 2: launch_sens_obj<2>(le, S); break;
    case 3: launch_sens_obj<3>(le, S); break;
    case 4: launch_sens_obj<4>(le, S); break;
    case 5: launch_sens_obj<5>(le, S); break;
    case 7: launch_sens_obj<7>(le, S); break;
    default: launch_sens_obj<6>(le, S); break;
    }
}

// K L+: its part in the B terms and in A x0 is scaled by the stiffness share
// of the operator, so when that share is tiny an FP32 product is accurate to
// well below the solver tolerance (share 1e-4: FP32 rounding 6e-8 x 1e-4)
static void adj_kl(TopoLE *le) {
    if (le->p.mixed && le->ops[0].share <= 1e-4)
        product_t<float, true, false>(le, le->Lp1, le->KL, nullptr, 1.0, 0.0);
    else
        product<true, false>(le, le->Lp1, le->KL, nullptr, 1.0, 0.0);
}

// the mixed path forms the adjoint right-hand side in double-float arithmetic
static void launch_adj_combine(TopoLE *le, const AdjCombine &A) {
    if (le->p.mixed)
        k_adj_combine<df><<<ew_blocks(le->ndof), EW, 0, le->stream>>>(A);
    else
        k_adj_combine<double><<<ew_blocks(le->ndof), EW, 0, le->stream>>>(A);
}

static int adj_step(TopoLE *le, bool capturing) {
    cudaStream_t s = le->stream;
    // K L+ and M L+ (the B1..B3 products of LinearElasticity.cc:897-899)
    adj_kl(le);
    if (!al_mode(le)) product<false, true>(le, le->Lp1, le->ML, nullptr, 0.0, 1.0);
    objective_products(le, 0);
    count_launch();
    launch_adj_combine(le, adj_args(le, 0));
    le->ax0_pending = le->KLh1 != nullptr;
    int rc = solve(le, 0, le->sb, capturing);
    le->ax0_pending = false;
    if (rc) return rc;
    launch_sens(le, 0);
    count_launch();
    k_adj_advance<<<ew_blocks(le->ndof), EW, 0, s>>>(le->ndof, le->sx, le->DLc, le->DDLc, le->Lp1, le->DLp1, le->DDLp1,
                                                      le->Lp2, le->Lp3,
                                                      KMHist{le->KL, le->ML, le->KLh1, le->MLh1, le->KLh2, le->MLh2,
                                                             al_mode(le) ? le->sb : nullptr, le->sr, le->S});
    count_launch();
    k_step_add<<<1, 1, 0, s>>>(le->st, -1);
    return TOPO_OK;
}

static int lagrange0(TopoLE *le) {
    cudaStream_t s = le->stream;
    adj_kl(le);
    if (!al_mode(le)) product<false, true>(le, le->Lp1, le->ML, nullptr, 0.0, 1.0);
    objective_products(le, 1);
    count_launch();
    launch_adj_combine(le, adj_args(le, 1));
    le->ax0_pending = le->KLh1 != nullptr;
    int rc = solve(le, 1, le->sb, false);
    le->ax0_pending = false;
    if (rc) return rc;
    launch_sens(le, 1);
    count_launch();
    k_copy<<<ew_blocks(le->ndof), EW, 0, s>>>(le->ndof, le->sx, le->DDL0);
    return TOPO_OK;
}

// graph of one step, captured on first use and replayed for every step
static int get_graph(TopoLE *le, int adjoint, cudaGraphExec_t *out) {
    if (le->captured_depth != le->ops[0].depth) {
        if (le->gx_fwd) cudaGraphExecDestroy(le->gx_fwd);
        if (le->gx_adj) cudaGraphExecDestroy(le->gx_adj);
        le->gx_fwd = le->gx_adj = nullptr;
        le->captured_depth = le->ops[0].depth;
    }
    cudaGraphExec_t &gx = adjoint ? le->gx_adj : le->gx_fwd;
    if (!gx) {
        CK(cudaStreamBeginCapture(le->stream, cudaStreamCaptureModeRelaxed));
        long long c0 = launch_counter();
        int rc = adjoint ? adj_step(le, true) : fwd_step(le, true);
        long long captured = launch_counter() - c0;
        launch_counter() -= captured;  // capturing is not launching: counted per replay
        le->step_kernels[adjoint] = captured - le->body_kernels;
        cudaGraph_t g;
        cudaError_t e = cudaStreamEndCapture(le->stream, &g);
        if (rc) return rc;
        CK(e);
        cudaError_t e2 = cudaGraphInstantiate(&gx, g, 0);
        cudaGraphDestroy(g);
        CK(e2);
    }
    *out = gx;
    return TOPO_OK;
}

static int run_block(TopoLE *le, int c, int adjoint) {
    const int tsc = le->p.tsc;
    count_launch();
    k_step_set<<<1, 1, 0, le->stream>>>(le->st, c, adjoint ? tsc - 1 : 0);
    const bool track = !adjoint && le->AUt;
    if (track) track_block_start(le, c);
    cudaGraphExec_t gx = nullptr;
    if (le->p.use_graphs) {
        int rc = get_graph(le, adjoint, &gx);
        if (rc) return rc;
    }
    for (int j = 0; j < tsc; j++) {
        if (track && j > 0 && j % TRACK_ANCHOR == 0) track_anchor(le, c, j);
        if (gx) {
            CK(cudaGraphLaunch(gx, le->stream));
            le->nsolves++;
            if (!le->ops[0].kron) le->mg_solves++;
            count_launch(le->step_kernels[adjoint]);
        } else {
            int rc = adjoint ? adj_step(le, false) : fwd_step(le, false);
            if (rc) return rc;
        }
        if (adjoint && j == 0 && c == le->p.ncp - 1) {  // the terminal adjoint L(T) (LT, LinearElasticity.cc:882-888)
            count_launch();
            k_copy<<<ew_blocks(le->ndof), EW, 0, le->stream>>>(le->ndof, le->Lp1, le->LT);
        }
    }
    CK(cudaGetLastError());
    return TOPO_OK;
}

static int check_err(TopoLE *le) {
    int h = 0;
    CK(cudaMemcpyAsync(&h, le->err, sizeof(int), cudaMemcpyDeviceToHost, le->stream));
    CK(cudaStreamSynchronize(le->stream));
    if (h) {
        set_error(std::string("linear solve failed with status ") + std::to_string(h));
        int z = 0;
        cudaMemcpy(le->err, &z, sizeof(int), cudaMemcpyHostToDevice);
        return h;
    }
    return TOPO_OK;
}

__global__ void k_init_accel_rhs(long long nn, const uint8_t *fixed, const double *rhs0, double s, long long load2_dof,
                                 double s2, const double *Ku, const double *Cdu, double *b) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        uint8_t f = fixed[n];
        for (int c = 0; c < 3; c++) {
            long long i = 3 * n + c;
            b[i] = ((f >> c) & 1) ? 0.0 : (rhs0[i] * s + (i == load2_dof ? s2 : 0.0) - Cdu[i] - Ku[i]);
        }
    }
}

// ---------------------------------------------------------------------------
// public operations
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// SOMMG reduced path (SOMMG.cc:40-265, reduction branches of
// LinearElasticity.cc): basis, reduced system, reduced sweeps
// ---------------------------------------------------------------------------
// out[b * ostride] = Q_b . y for b < kb (Q_b = Qbase + b qs)
template <class QT>
static void multidot(TopoLE *le, const QT *Qbase, long long qs, int kb, const double *y, double *out, int ostride) {
    cudaStream_t s = le->stream;
    count_launch();
    k_md_partial<QT><<<dim3(MD_CHUNKS, kb), 256, 0, s>>>(le->ndof, Qbase, qs, kb, y, le->mdpart);
    count_launch();
    k_md_final<<<1, 32, 0, s>>>(kb, MD_CHUNKS, le->mdpart, out, ostride);
}

enum { RED_KR = 0, RED_MR = 1, RED_KP = 2, RED_MP = 3, RED_GC = 4, RED_UT = 5 };
static double *red_mat(TopoLE *le, int which) { return le->red + (size_t)which * le->kb * le->kb; }
static double *red_pr(TopoLE *le) { return le->red + (size_t)6 * le->kb * le->kb; }
static double *red_fx(TopoLE *le) { return red_pr(le) + le->kb; }

// ConstructBasis (SOMMG.cc:40-210): Qb_0 = P0^-1 N P; Qb_j = P0^-1 N 2 om M Q_{j-1}
// (the moment-matching correction of :113-176 is scaled by the comma
// expression (-1,0) == 0 at :176 and so contributes nothing); modified
// Gram-Schmidt against the accepted vectors and normalisation.  The basis
// solves run the FP64 FCG on both paths: P0 = K - om^2 M with a small om is a
// nearly singular static operator whose FP32 curvature p'P0 p loses its sign
// to rounding (the mixed recurrence breaks down).  The plain path keeps the
// basis in FP64; the mixed path orthonormalises each row in FP64 against the
// stored rows and stores it rounded to FP32, so every later product sees the
// same basis
static int sommg_basis(TopoLE *le) {
    cudaStream_t s = le->stream;
    const long long nd = le->ndof, nn = le->nn;
    const int kb = le->kb;
    const bool b32 = le->basis32;
    const uint8_t *fixed = le->L[0].fixed;
    double *Ut = red_mat(le, RED_UT), *Pv = le->hM;
    struct Fp64Solves {  // FP64 FCG for the basis solves, restored on every exit
        TopoLE *le;
        explicit Fp64Solves(TopoLE *l) : le(l) { le->fp64_solves = true; }
        ~Fp64Solves() { le->fp64_solves = false; }
    } fp64(le);
    count_launch();
    k_mask_scale<<<ew_blocks(nn), EW, 0, s>>>(nn, fixed, le->rhs0, 1.0, Pv);  // VecPointwiseMult(P, P, N), :75
    for (int j = 0; j < kb; j++) {
        double *q = b32 ? le->qd : le->Q + (size_t)j * nd;  // the FP64 working row
        if (j == 0) {
            CK(cudaMemcpyAsync(le->sb, Pv, sizeof(double) * nd, cudaMemcpyDeviceToDevice, s));
        } else {
            const double *prev = le->Q + (size_t)(j - 1) * nd;
            if (b32) {
                count_launch();
                k_f2d_row<<<ew_blocks(nd), EW, 0, s>>>(nd, le->Q32 + (size_t)(j - 1) * le->qld, le->KL);
                prev = le->KL;
            }
            product<false, true>(le, prev, le->ML, nullptr, 0.0, 1.0);
            count_launch();
            k_mask_scale<<<ew_blocks(nn), EW, 0, s>>>(nn, fixed, le->ML, 2.0 * le->p.omega0, le->sb);  // :109-111, :181
        }
        CK(cudaMemsetAsync(le->sx, 0, sizeof(double) * nd, s));
        int rc = solve(le, 2, le->sb, false);  // :78-80, :185
        if (rc) return rc;
        CK(cudaMemcpyAsync(q, le->sx, sizeof(double) * nd, cudaMemcpyDeviceToDevice, s));
        for (int i = 0; i < j; i++) {  // :195-202
            double *coef = Ut + (size_t)i * kb + j;
            count_launch();
            if (b32) {
                const float *Qi = le->Q32 + (size_t)i * le->qld;
                multidot<float>(le, Qi, le->qld, 1, q, coef, 1);
                k_axpy_dev<float><<<ew_blocks(nd), EW, 0, s>>>(nd, q, Qi, coef);
            } else {
                const double *Qi = le->Q + (size_t)i * nd;
                multidot<double>(le, Qi, nd, 1, q, coef, 1);
                k_axpy_dev<double><<<ew_blocks(nd), EW, 0, s>>>(nd, q, Qi, coef);
            }
        }
        multidot<double>(le, q, nd, 1, q, Ut + (size_t)j * kb + j, 1);  // :92, :206
        count_launch();
        k_normalise<<<ew_blocks(nd), EW, 0, s>>>(nd, q, Ut + (size_t)j * kb + j);
        count_launch();
        k_sqrt1<<<1, 1, 0, s>>>(Ut + (size_t)j * kb + j);
        if (b32) {
            count_launch();
            k_d2f_row<<<ew_blocks(nd), EW, 0, s>>>(nd, q, le->Q32 + (size_t)j * le->qld);
        }
    }
    CK(cudaGetLastError());
    return TOPO_OK;
}

// one tensor-core Gram product (gram.cuh): out[a kb + b] = Q_a . W_b with
// W_b = Wh_b + Wl_b, deterministic
static int gram_tc(TopoLE *le, double *out) {
    cudaStream_t s = le->stream;
    static bool attr_dev[MAX_DEVICES] = {};
    bool &attr = attr_dev[device_slot()];
    if (!attr) {
        CK(cudaFuncSetAttribute(k_gram_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, GR_SMEM));
        attr = true;
    }
    const GramArgs g{le->Q32, le->Wh, le->Wl, le->qld, le->kb, le->gpart, le->err, TOPO_ERR_SYNC_TIMEOUT};
    count_launch();
    k_gram_tc<<<le->gram_blocks, GR_THREADS, GR_SMEM, s>>>(g);
    count_launch();
    k_gram_final<<<(le->kb * le->kb + 255) / 256, 256, 0, s>>>(le->gram_blocks, le->gpart, le->kb, out);
    CK(cudaGetLastError());
    return TOPO_OK;
}

// reduced matrices (SOMMG.cc:228-252) and the objective projections of the
// reduced state gradients (LinearElasticity.cc:2318-2336): column j of each is
// Q' (A Q_j); Q vanishes on clamped DOFs, so masked and unmasked products agree.
// Plain path: FP64 dot products per column.  Mixed path: the products of all
// columns first (FP64 products of the FP32 rows, stored as FP32 pairs), then
// one tensor-core Gram per matrix.
static int sommg_reduce(TopoLE *le) {
    cudaStream_t s = le->stream;
    const long long nd = le->ndof, nn = le->nn;
    const int kb = le->kb, ob = le->p.objective;
    const uint8_t *fixed = le->L[0].fixed;
    double *tmp = le->sp;
    const bool useK = ob == 3 || ob == 5 || ob == 6, useM = ob == 4 || ob == 5 || ob == 6, useG = ob <= 2;
    if (!le->basis32) {
        for (int j = 0; j < kb; j++) {
            const double *Qj = le->Q + (size_t)j * nd;
            product<true, false>(le, Qj, le->KL, nullptr, 1.0, 0.0);
            multidot<double>(le, le->Q, nd, kb, le->KL, red_mat(le, RED_KR) + j, kb);
            product<false, true>(le, Qj, le->ML, nullptr, 0.0, 1.0);
            count_launch();
            k_mask_scale<<<ew_blocks(nn), EW, 0, s>>>(nn, fixed, le->ML, 1.0, tmp);
            multidot<double>(le, le->Q, nd, kb, tmp, red_mat(le, RED_MR) + j, kb);
            if (useK) {
                product<true, false>(le, Qj, le->KL, le->P, 1.0, 0.0);
                multidot<double>(le, le->Q, nd, kb, le->KL, red_mat(le, RED_KP) + j, kb);
            }
            if (useM) {
                product<false, true>(le, Qj, le->ML, le->P, 0.0, 1.0);
                multidot<double>(le, le->Q, nd, kb, le->ML, red_mat(le, RED_MP) + j, kb);
            }
            if (useG) {
                count_launch();
                k_cnt_mul<<<ew_blocks(nn), EW, 0, s>>>(nn, le->cntP, Qj, tmp);
                multidot<double>(le, le->Q, nd, kb, tmp, red_mat(le, RED_GC) + j, kb);
            }
        }
        multidot<double>(le, le->Q, nd, kb, le->hM, red_pr(le), 1);  // Pr = Q' N P
        CK(cudaGetLastError());
        return TOPO_OK;
    }
    enum { OP_K, OP_M, OP_KP, OP_MP, OP_GC };
    auto project = [&](int op, int which) -> int {
        for (int j = 0; j < kb; j++) {
            count_launch();
            k_f2d_row<<<ew_blocks(nd), EW, 0, s>>>(nd, le->Q32 + (size_t)j * le->qld, le->qd);
            const double *w = tmp;
            switch (op) {
            case OP_K:
                product<true, false>(le, le->qd, le->KL, nullptr, 1.0, 0.0);
                w = le->KL;
                break;
            case OP_M:
                product<false, true>(le, le->qd, le->ML, nullptr, 0.0, 1.0);
                count_launch();
                k_mask_scale<<<ew_blocks(nn), EW, 0, s>>>(nn, fixed, le->ML, 1.0, tmp);
                break;
            case OP_KP:
                product<true, false>(le, le->qd, le->KL, le->P, 1.0, 0.0);
                w = le->KL;
                break;
            case OP_MP:
                product<false, true>(le, le->qd, le->ML, le->P, 0.0, 1.0);
                w = le->ML;
                break;
            default:
                count_launch();
                k_cnt_mul<<<ew_blocks(nn), EW, 0, s>>>(nn, le->cntP, le->qd, tmp);
            }
            count_launch();
            k_split_f32<<<ew_blocks(nd), EW, 0, s>>>(nd, w, le->Wh + (size_t)j * le->qld, le->Wl + (size_t)j * le->qld);
        }
        return gram_tc(le, red_mat(le, which));
    };
    int rc = project(OP_K, RED_KR);
    if (!rc) rc = project(OP_M, RED_MR);
    if (!rc && useK) rc = project(OP_KP, RED_KP);
    if (!rc && useM) rc = project(OP_MP, RED_MP);
    if (!rc && useG) rc = project(OP_GC, RED_GC);
    if (rc) return rc;
    multidot<float>(le, le->Q32, le->qld, kb, le->hM, red_pr(le), 1);  // Pr = Q' N P
    CK(cudaGetLastError());
    return TOPO_OK;
}

static RedSys red_sys(TopoLE *le) {
    const LEParams &p = le->p;
    const int ob = p.objective;
    RedSys R;
    memset(&R, 0, sizeof(R));
    R.kb = le->kb;
    R.Ts = le->Ts;
    R.objective = ob;
    R.loadsignal = p.loadsignal;
    memcpy(R.a, le->a, sizeof(R.a));
    R.dt = le->dt;
    R.alpha = p.dalpha;
    R.beta = p.dbeta;
    R.load_scale = 1.0 / (p.ny - 1);
    R.Kr = red_mat(le, RED_KR);
    R.Mr = red_mat(le, RED_MR);
    R.Kp = (ob == 3 || ob == 5 || ob == 6) ? red_mat(le, RED_KP) : nullptr;
    R.Mp = (ob == 4 || ob == 5 || ob == 6) ? red_mat(le, RED_MP) : nullptr;
    R.Gc = ob <= 2 ? red_mat(le, RED_GC) : nullptr;
    R.Pr = red_pr(le);
    R.hist = le->rhist;
    R.S = le->Sacc;
    R.fx = red_fx(le);
    R.status = le->rstatus;
    return R;
}

static int red_status(TopoLE *le) {
    int h = 0;
    CK(cudaMemcpyAsync(&h, le->rstatus, sizeof(int), cudaMemcpyDeviceToHost, le->stream));
    CK(cudaStreamSynchronize(le->stream));
    if (h) {
        set_error("SOMMG: singular reduced matrix (basis vectors linearly dependent?)");
        return h;
    }
    return TOPO_OK;
}

static void red_attributes() {
    static bool attr_dev[MAX_DEVICES] = {};
    bool &attr = attr_dev[device_slot()];
    if (!attr) {
        cudaFuncSetAttribute(k_red_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)red_smem_bytes(KB_MAX));
        cudaFuncSetAttribute(k_red_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)red_smem_bytes(KB_MAX));
        attr = true;
    }
}

// CompleteInitialState of the reduced path (LinearElasticity.cc:993-1078)
static int sommg_initial_state(TopoLE *le) {
    cudaStream_t s = le->stream;
    int rc = setup_operator(le, 2);
    if (rc) return rc;
    CK(cudaMemsetAsync(le->red, 0, sizeof(double) * (6 * le->kb * le->kb + le->kb + 1), s));
    CK(cudaMemsetAsync(le->rstatus, 0, sizeof(int), s));
    rc = sommg_basis(le);
    if (rc) return rc;
    rc = sommg_reduce(le);
    if (rc) return rc;
    red_attributes();
    count_launch();
    k_red_forward<<<1, 256, red_smem_bytes(le->kb), s>>>(red_sys(le));
    CK(cudaGetLastError());
    rc = check_err(le);
    if (rc) return rc;
    return red_status(le);
}

// ComputeObjectiveSensitivities of the reduced path: reduced adjoint sweep,
// then one element pass over the accumulated S matrices
static int sommg_objective_sensitivities(TopoLE *le, double *fx, double *dfdx_dev) {
    cudaStream_t s = le->stream;
    const long long nd = le->ndof;
    const int kb = le->kb, ob = le->p.objective;
    red_attributes();
    count_launch();
    k_red_adjoint<<<1, 256, red_smem_bytes(kb), s>>>(red_sys(le));
    CK(cudaGetLastError());
    // Phi_s = Q S_s' for S_K, S_M and the objective terms in use
    const bool useoK = ob == 3 || ob == 5 || ob == 6, useoM = ob >= 4;
    const int ns = (useoK || useoM) ? 4 : 2;
    auto sens = [&](auto *Q, long long qs, auto *Phi) {
        using QT = std::remove_const_t<std::remove_pointer_t<decltype(Q)>>;
        count_launch();
        k_red_phi<QT><<<ew_blocks(nd), 256, 0, s>>>(nd, kb, Q, qs, le->Sacc, ns, Phi);
        RedSens<QT> A;
        A.g = le->g;
        A.kb = kb;
        A.qs = qs;
        A.Q = Q;
        A.phiK = Phi;
        A.phiM = Phi + (size_t)kb * nd;
        A.phioK = useoK ? Phi + (size_t)2 * kb * nd : nullptr;
        A.phioM = useoM ? Phi + (size_t)3 * kb * nd : nullptr;
        A.dkf = le->dkf;
        A.dmf = le->dmf;
        A.P = le->P;
        A.df = le->df;
        count_launch();
        k_red_sens<QT><<<red_blocks(le->nel), EW, 0, s>>>(A, le->L[0].Cd);
    };
    if (le->basis32)
        sens(static_cast<const float *>(le->Q32), le->qld, le->Phi32);
    else
        sens(static_cast<const double *>(le->Q), nd, le->Phi);
    CK(cudaGetLastError());
    if (dfdx_dev) CK(cudaMemcpyAsync(dfdx_dev, le->df, sizeof(double) * le->nel, cudaMemcpyDeviceToDevice, s));
    double h = 0.0;
    CK(cudaMemcpyAsync(&h, red_fx(le), sizeof(double), cudaMemcpyDeviceToHost, s));
    int rc = red_status(le);
    if (rc) return rc;
    *fx = h;
    le->stats.last_fx = h;
    return TOPO_OK;
}

// out[a kb + b] = sum_i Q[a][i] W[b][i] on the tensor cores for device rows Q
// (FP32, stride ldq) and W (FP64, stride ldw), n values each: the Gram
// product of the reduced matrices as a stand-alone routine (it allocates its
// padded operands and per-CTA partials)
int le_gram_tc_dev(const float *Q, long long ldq, const double *W, long long ldw, long long n, int kb, double *out) {
    if (!Q || !W || !out || n < 1 || kb < 1 || kb > 32 || ldq < n || ldw < n) {
        set_error("gram: need 1 <= kb <= 32, n >= 1 and row strides >= n");
        return TOPO_ERR_ARG;
    }
    const long long ld = (n + GR_KC - 1) / GR_KC * GR_KC;
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int nblk = 2 * std::max(1, nsm);
    Arena arena;
    float *q = nullptr, *wh = nullptr, *wl = nullptr;
    double *part = nullptr, *o = nullptr;
    int *err = nullptr;
    struct Release {
        Arena &a;
        ~Release() { a.release(); }
    } rel{arena};
    AG(q, (size_t)kb * ld);
    AG(wh, (size_t)kb * ld);
    AG(wl, (size_t)kb * ld);
    AG(part, (size_t)nblk * 1024);
    AG(o, (size_t)kb * kb);
    AG(err, 1);
    CK(cudaMemcpy2D(q, sizeof(float) * ld, Q, sizeof(float) * ldq, sizeof(float) * n, kb, cudaMemcpyDeviceToDevice));
    for (int b = 0; b < kb; b++) {
        count_launch();
        k_split_f32<<<ew_blocks(n), EW>>>(n, W + (size_t)b * ldw, wh + (size_t)b * ld, wl + (size_t)b * ld);
    }
    CK(cudaFuncSetAttribute(k_gram_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, GR_SMEM));
    const GramArgs g{q, wh, wl, ld, kb, part, err, TOPO_ERR_SYNC_TIMEOUT};
    count_launch();
    k_gram_tc<<<nblk, GR_THREADS, GR_SMEM>>>(g);
    count_launch();
    k_gram_final<<<(kb * kb + 255) / 256, 256>>>(nblk, part, kb, o);
    CK(cudaGetLastError());
    int h = 0;
    CK(cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        set_error("gram: an mbarrier wait of the tensor-core kernel gave up");
        return h;
    }
    CK(cudaMemcpy(out, o, sizeof(double) * kb * kb, cudaMemcpyDeviceToHost));
    return TOPO_OK;
}

// SOMMG::ConstructBasis (SOMMG.cc:40-265) with expansion frequency om on the
// operators of the current design, then the reduced forward sweep, so that a
// following ComputeObjectiveSensitivities integrates in the new basis
int le_sommg_construct_basis(TopoLE *le, double om) {
    if (!le->kb || !le->design_ready) {
        set_error("ConstructBasis needs reduction = 1 and CompleteInitialState");
        return TOPO_ERR_STATE;
    }
    if (!(om > 0.0)) {
        set_error("ConstructBasis: om must be > 0 (the basis recursion scales by om)");
        return TOPO_ERR_ARG;
    }
    le->p.omega0 = om;
    le->ops[2].sM = -om * om;
    return sommg_initial_state(le);
}

int le_reduced_system(TopoLE *le, double *Q, double *Kr, double *Mr, double *Pr) {
    if (!le->kb || !le->design_ready) {
        set_error("reduced_system needs reduction = 1 and CompleteInitialState");
        return TOPO_ERR_STATE;
    }
    cudaStream_t s = le->stream;
    const size_t k2 = (size_t)le->kb * le->kb;
    if (Q && le->basis32) {  // the FP32 rows, widened
        std::vector<float> h((size_t)le->kb * le->ndof);
        CK(cudaMemcpy2DAsync(h.data(), sizeof(float) * le->ndof, le->Q32, sizeof(float) * le->qld,
                             sizeof(float) * le->ndof, le->kb, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        for (size_t i = 0; i < h.size(); i++) Q[i] = h[i];
    } else if (Q) {
        CK(cudaMemcpyAsync(Q, le->Q, sizeof(double) * le->kb * le->ndof, cudaMemcpyDeviceToHost, s));
    }
    if (Kr) CK(cudaMemcpyAsync(Kr, red_mat(le, RED_KR), sizeof(double) * k2, cudaMemcpyDeviceToHost, s));
    if (Mr) CK(cudaMemcpyAsync(Mr, red_mat(le, RED_MR), sizeof(double) * k2, cudaMemcpyDeviceToHost, s));
    if (Pr) CK(cudaMemcpyAsync(Pr, red_pr(le), sizeof(double) * le->kb, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return TOPO_OK;
}

// Physics output: the `write, output` arguments of CompleteInitialState,
// GenerateCheckPoints and ComputeObjectiveSensitivities.  Every dataset is the
// displacement of one time step and xPhys (MPIIO::WriteVTK(da, U, xPhys, itr),
// MPIIO.cc:215-268), converted on the device straight into the writer's
// pinned records on this object's stream.
static int out_state(TopoLE *le, unsigned long long itr, const double *u) {
    const double *x = le->xPhys;
    return mpiio_write(le->out, itr, &u, 1, &x, 1, 1, le->stream);
}

// steps tsc*c + 1 .. tsc*(c + 1) of the resident forward block c
// (LinearElasticity.cc:1220-1252, :1736-1742)
static int out_block(TopoLE *le, int c) {
    const int tsc = le->p.tsc;
    for (int j = 0; j < tsc; j++) {
        int rc = out_state(le, (unsigned long long)tsc * c + j + 1, le->Uh + (size_t)j * le->ndof);
        if (rc) return rc;
    }
    return TOPO_OK;
}

// full = sum_k r_k Q_k (the lifts of LinearElasticity.cc:1087-1108, :1225-1243)
static void lift(TopoLE *le, const double *r, double *full) {
    const long long nd = le->ndof;
    count_launch();
    if (le->basis32)
        k_lift<float><<<ew_blocks(nd), EW, 0, le->stream>>>(nd, le->kb, le->Q32, le->qld, r, full);
    else
        k_lift<double><<<ew_blocks(nd), EW, 0, le->stream>>>(nd, le->kb, le->Q, nd, r, full);
}

// reduced path: steps t0..t1 of the reduced history lifted to the full space,
// U = sum_k u_k Q_k (LinearElasticity.cc:1087-1108, :1225-1243)
static int out_reduced(TopoLE *le, int t0, int t1) {
    for (int t = t0; t <= t1; t++) {
        lift(le, le->rhist + (size_t)t * 3 * le->kb, le->sp);
        int rc = out_state(le, (unsigned long long)t, le->sp);
        if (rc) return rc;
    }
    CK(cudaGetLastError());
    return TOPO_OK;
}

int le_set_output(TopoLE *le, topo_mpiio *io) {
    if (io && (mpiio_point_fields(io) != 3 || mpiio_cell_fields(io) != 1 || mpiio_points(io) != le->nn ||
               mpiio_cells(io) != le->nel)) {
        set_error("physics output needs a writer of this mesh (" + std::to_string(le->nn) + " nodes, " +
                  std::to_string(le->nel) + " cells) with 3 point fields (ux, uy, uz) and 1 cell field (xPhys)");
        return TOPO_ERR_ARG;
    }
    le->out = io;
    return TOPO_OK;
}

int le_complete_initial_state(TopoLE *le, const double *xPhys_dev, double Emin, double Emax, double Rmin, double Rmax,
                              double penalK, double penalM) {
    cudaStream_t s = le->stream;
    const LEParams &p = le->p;
    CK(cudaMemcpyAsync(le->xPhys, xPhys_dev, sizeof(double) * le->nel, cudaMemcpyDeviceToDevice, s));
    MatParams mp{p.sInt, p.mInt, Emin, Emax, penalK, Rmin, Rmax, penalM};
    count_launch();
    k_interp<<<ew_blocks(le->nel), EW, 0, s>>>(le->nel, le->xPhys, mp, le->kf, le->dkf, le->mf, le->dmf, le->L[0].kff,
                                               le->L[0].mff, le->kfx, le->mfx);
    for (int l = 1; l < le->nlev; l++) {
        count_launch();
        k_coarsen<<<ew_blocks(le->L[l].g.nel()), EW, 0, s>>>(le->L[l - 1].g, le->L[l].g, le->L[l - 1].kfd,
                                                             le->L[l - 1].mfd, le->L[l].kfd, le->L[l].mfd,
                                                             le->L[l].kff, le->L[l].mff);
    }
    if (le->kb) {
        int rc = sommg_initial_state(le);
        if (rc) return rc;
        le->design_ready = 1;
        le->last_block_resident = le->p.ncp - 1;
        return le->out ? out_reduced(le, 0, 0) : TOPO_OK;
    }
    int rc = setup_operator(le, 0);
    if (rc) return rc;
    rc = setup_operator(le, 1);
    if (rc) return rc;
    // initial acceleration: (N M N + I - N) ddu0 = N (f(0) - C du0 - K u0)
    // (LinearElasticity.cc:1046-1078); u0 = du0 = 0 (LinearElasticity.cc:521-587)
    long long nd = le->ndof;
    CK(cudaMemsetAsync(le->cp, 0, sizeof(double) * 3 * nd, s));
    if (le->u0init)  // LoadSolutionAsU0 (LinearElasticity.cc:2621-2677)
        CK(cudaMemcpyAsync(le->cp, le->u0init, sizeof(double) * nd, cudaMemcpyDeviceToDevice, s));
    product<true, false>(le, le->cp, le->KL, nullptr, 1.0, 0.0);
    product<true, true>(le, le->cp + nd, le->ML, nullptr, p.dbeta, p.dalpha);
    double s0 = 0.0;
    {
        // host evaluation of the load signal at t = 0 (same formula as the device)
        if (p.loadsignal == 1)
            s0 = 0.0;
        else {
            double t = 0.0 - 8.0, c = 1.1;
            s0 = exp(-(t * t) / ((2 * c) * (2 * c))) * cos(4.0 * t) * cos(5.0 * t) * cos(6.0 * t) * cos(7.0 * t);
        }
        s0 /= (p.ny - 1);
    }
    count_launch();
    // second point load at t = 0 (workload extension)
    const long long l2 = p.load2_node >= 0 ? 3LL * p.load2_node + 2 : -1;
    const double s2 = l2 >= 0 ? sin(p.load2_phase) / (p.ny - 1) : 0.0;
    k_init_accel_rhs<<<ew_blocks(le->nn), EW, 0, s>>>(le->nn, le->L[0].fixed, le->rhs0, s0, l2, s2, le->KL, le->ML,
                                                      le->sb);
    CK(cudaMemsetAsync(le->sx, 0, sizeof(double) * nd, s));
    rc = solve(le, 1, le->sb, false);
    if (rc) return rc;
    count_launch();
    k_copy<<<ew_blocks(nd), EW, 0, s>>>(nd, le->sx, le->cp + 2 * nd);
    rc = check_err(le);
    if (rc) return rc;
    le->design_ready = 1;
    le->checkpoints_ready = le->p.ncp <= 1;
    le->last_block_resident = -1;
    return le->out ? out_state(le, 0, le->cp) : TOPO_OK;  // U0 (LinearElasticity.cc:1087-1114)
}

int le_generate_checkpoints(TopoLE *le) {
    if (!le->design_ready) {
        set_error("GenerateCheckPoints called before CompleteInitialState");
        return TOPO_ERR_STATE;
    }
    if (le->p.ncp <= 1) return TOPO_OK;
    if (le->kb)  // the reduced history is complete after CompleteInitialState
        return le->out ? out_reduced(le, 1, le->p.ncp * le->p.tsc) : TOPO_OK;
    long long nd = le->ndof;
    int tsc = le->p.tsc;
    for (int c = 0; c < le->p.ncp; c++) {
        int rc = run_block(le, c, 0);
        if (rc) return rc;
        if (le->out) {
            rc = out_block(le, c);
            if (rc) return rc;
        }
        double *dst = le->cp + (size_t)(c + 1) * 3 * nd;
        CK(cudaMemcpyAsync(dst, le->Uh + (size_t)(tsc - 1) * nd, sizeof(double) * nd, cudaMemcpyDeviceToDevice, le->stream));
        CK(cudaMemcpyAsync(dst + nd, le->DUh + (size_t)(tsc - 1) * nd, sizeof(double) * nd, cudaMemcpyDeviceToDevice,
                           le->stream));
        CK(cudaMemcpyAsync(dst + 2 * nd, le->DDUh + (size_t)(tsc - 1) * nd, sizeof(double) * nd,
                           cudaMemcpyDeviceToDevice, le->stream));
    }
    le->last_block_resident = le->p.ncp - 1;
    le->checkpoints_ready = 1;
    return check_err(le);
}

int le_compute_objective_sensitivities(TopoLE *le, double *fx, double *dfdx_dev) {
    if (!le->design_ready) {
        set_error("ComputeObjectiveSensitivities called before CompleteInitialState");
        return TOPO_ERR_STATE;
    }
    if (le->kb) {
        if (le->out && le->p.ncp == 1) {
            int rc = out_reduced(le, 1, le->p.tsc);
            if (rc) return rc;
        }
        return sommg_objective_sensitivities(le, fx, dfdx_dev);
    }
    if (!le->checkpoints_ready) {  // the reverse sweep restarts blocks from checkpoints 1..ncp-1
        set_error("ComputeObjectiveSensitivities with ncp > 1 needs GenerateCheckPoints after CompleteInitialState");
        return TOPO_ERR_STATE;
    }
    cudaStream_t s = le->stream;
    long long nd = le->ndof;
    CK(cudaMemsetAsync(le->df, 0, sizeof(double) * le->nel, s));
    CK(cudaMemsetAsync(le->Lp1, 0, sizeof(double) * nd, s));
    CK(cudaMemsetAsync(le->DLp1, 0, sizeof(double) * nd, s));
    CK(cudaMemsetAsync(le->DDLp1, 0, sizeof(double) * nd, s));
    CK(cudaMemsetAsync(le->Lp2, 0, sizeof(double) * nd, s));
    CK(cudaMemsetAsync(le->Lp3, 0, sizeof(double) * nd, s));
    if (al_mode(le)) CK(cudaMemsetAsync(le->ML, 0, sizeof(double) * nd, s));  // A L+ of L+ = 0
    CK(cudaMemsetAsync(&le->st->nadj, 0, sizeof(int), s));
    CK(cudaMemsetAsync(&le->st->fx, 0, sizeof(double), s));
    for (int c = le->p.ncp - 1; c >= 0; c--) {
        if (le->last_block_resident != c) {
            int rc = run_block(le, c, 0);
            if (rc) return rc;
            le->last_block_resident = c;
        }
        if (le->out && le->p.ncp == 1) {  // the forward history of the single block is resident
            int rc = out_block(le, c);
            if (rc) return rc;
        }
        int rc = run_block(le, c, 1);
        if (rc) return rc;
        if (c == 0) {
            rc = lagrange0(le);
            if (rc) return rc;
        }
    }
    if (dfdx_dev) CK(cudaMemcpyAsync(dfdx_dev, le->df, sizeof(double) * le->nel, cudaMemcpyDeviceToDevice, s));
    double h = 0.0;
    CK(cudaMemcpyAsync(&h, &le->st->fx, sizeof(double), cudaMemcpyDeviceToHost, s));
    int rc = check_err(le);
    if (rc) return rc;
    *fx = h;
    le->stats.last_fx = h;
    return TOPO_OK;
}

int le_get_checkpoint(TopoLE *le, int c, double *U, double *DU, double *DDU) {
    if (c < 0 || c >= le->p.ncp || le->kb) {
        set_error("checkpoint index outside 0..ncp-1 (or the reduced path, which keeps no checkpoints)");
        return TOPO_ERR_ARG;
    }
    if (!le->design_ready || (c > 0 && !le->checkpoints_ready)) {
        set_error("checkpoint requested before CompleteInitialState / GenerateCheckPoints");
        return TOPO_ERR_STATE;
    }
    const long long nd = le->ndof;
    const double *base = le->cp + (size_t)c * 3 * nd;
    CK(cudaMemcpyAsync(U, base, sizeof(double) * nd, cudaMemcpyDeviceToHost, le->stream));
    CK(cudaMemcpyAsync(DU, base + nd, sizeof(double) * nd, cudaMemcpyDeviceToHost, le->stream));
    CK(cudaMemcpyAsync(DDU, base + 2 * nd, sizeof(double) * nd, cudaMemcpyDeviceToHost, le->stream));
    CK(cudaStreamSynchronize(le->stream));
    return TOPO_OK;
}

int le_set_initial_displacement(TopoLE *le, const double *U0, int on_device) {
    if (le->kb) {
        set_error("an initial displacement needs the full path: the reduced path starts from rest");
        return TOPO_ERR_ARG;
    }
    const long long nd = le->ndof;
    if (!U0) {
        if (le->u0init) cudaFree(le->u0init);
        le->u0init = nullptr;
        le->design_ready = 0;
        return TOPO_OK;
    }
    if (!le->u0init) {
        cudaError_t e = cudaMalloc(&le->u0init, sizeof(double) * nd);
        if (e != cudaSuccess) {
            le->u0init = nullptr;
            set_error(std::string("initial displacement: ") + cudaGetErrorString(e));
            return TOPO_ERR_OOM;
        }
    }
    CK(cudaMemcpyAsync(le->u0init, U0, sizeof(double) * nd, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                       le->stream));
    CK(cudaStreamSynchronize(le->stream));
    le->design_ready = 0;  // CompleteInitialState must run again
    return TOPO_OK;
}

int le_get_restart_state(TopoLE *le, double *DDU0, double *LT, double *DDL0) {
    if (le->kb) {
        set_error("RestartSol vectors are kept on the full path only");
        return TOPO_ERR_ARG;
    }
    if (!le->design_ready) {
        set_error("restart vectors requested before CompleteInitialState");
        return TOPO_ERR_STATE;
    }
    const long long nd = le->ndof;
    CK(cudaMemcpyAsync(DDU0, le->cp + 2 * nd, sizeof(double) * nd, cudaMemcpyDeviceToHost, le->stream));
    CK(cudaMemcpyAsync(LT, le->LT, sizeof(double) * nd, cudaMemcpyDeviceToHost, le->stream));
    CK(cudaMemcpyAsync(DDL0, le->DDL0, sizeof(double) * nd, cudaMemcpyDeviceToHost, le->stream));
    CK(cudaStreamSynchronize(le->stream));
    return TOPO_OK;
}

int le_get_state(TopoLE *le, int which, int j, double *out) {
    if (which < 0 || which > 2 || j < -1 || j >= le->p.tsc) return TOPO_ERR_ARG;
    long long nd = le->ndof;
    if (le->kb) {  // lift the reduced state (LinearElasticity.cc:1225-1243)
        const int t = le->p.tsc * (le->p.ncp - 1) + j + 1;
        lift(le, le->rhist + ((size_t)t * 3 + which) * le->kb, le->sp);
        CK(cudaMemcpyAsync(out, le->sp, sizeof(double) * nd, cudaMemcpyDeviceToHost, le->stream));
        CK(cudaStreamSynchronize(le->stream));
        return TOPO_OK;
    }
    const double *src;
    if (j < 0) {
        int blk = le->last_block_resident < 0 ? 0 : le->last_block_resident;
        src = le->cp + (size_t)blk * 3 * nd + which * nd;
    } else {
        const double *base = which == 0 ? le->Uh : (which == 1 ? le->DUh : le->DDUh);
        src = base + (size_t)j * nd;
    }
    CK(cudaMemcpyAsync(out, src, sizeof(double) * nd, cudaMemcpyDeviceToHost, le->stream));
    CK(cudaStreamSynchronize(le->stream));
    return TOPO_OK;
}

int le_apply_km(TopoLE *le, const double *x_dev, double *Kx_dev, double *Mx_dev) {
    product<true, false>(le, x_dev, Kx_dev, nullptr, 1.0, 0.0);
    product<false, true>(le, x_dev, Mx_dev, nullptr, 0.0, 1.0);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(le->stream));
    return TOPO_OK;
}

int le_stats(TopoLE *le, LEStats *out) {
    SolveScalars h;
    CK(cudaMemcpyAsync(&h, le->S, sizeof(h), cudaMemcpyDeviceToHost, le->stream));
    CK(cudaStreamSynchronize(le->stream));
    le->stats.cg_iterations = h.total_it;
    le->stats.solves = le->nsolves;
    le->stats.mg_solves = le->mg_solves;
    le->stats.step_precond = le->design_ready ? (le->ops[0].kron ? 1 : 0) : -1;
    le->stats.graph_body_launches = (h.total_it - le->direct_iters) * le->body_kernels;
    le->stats.replacements = h.replacements;
    *out = le->stats;
    return TOPO_OK;
}

long long le_nel(const TopoLE *le) { return le->nel; }
int le_basis(const TopoLE *le) { return le->kb; }
void le_damping(const TopoLE *le, double *alpha, double *beta) {
    *alpha = le->p.dalpha;
    *beta = le->p.dbeta;
}
long long le_ndof(const TopoLE *le) { return le->ndof; }
void *le_stream(TopoLE *le) { return (void *)le->stream; }

}  // namespace topo

namespace topo {
// event-timed operator apply (roofline measurement hook)
__global__ void k_fill(long long n, double *x, double v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = v * (double)((i * 2654435761ull) % 1000) * 1e-3;
}
int le_time_apply(TopoLE *le, int precision, int warmup, int reps, double *ms) {
    if (!le->design_ready) {
        set_error("time_apply needs CompleteInitialState first");
        return TOPO_ERR_STATE;
    }
    cudaStream_t s = le->stream;
    Level &l0 = le->L[0];
    Operator &op = le->ops[0];
    long long nd = le->ndof;
    count_launch();
    k_fill<<<ew_blocks(nd), EW, 0, s>>>(nd, le->sp, 1.0);
    count_launch();
    k_d2f<<<ew_blocks(nd), EW, 0, s>>>(nd, le->sp, l0.fr);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    auto one = [&]() {
        if (precision == 0) {
            Weights<double> wt{l0.kfd, l0.mfd, nullptr, op.sK, op.sM};
            PolResid<double> pr{l0.fixed, wt, le->sp, le->sb, le->sq, {}};
            launch_tile<double>(l0.g, l0.Cd, pr, s);
        } else if (precision == 3) {
            Weights<float> wt{l0.kff, l0.mff, nullptr, (float)op.sK, (float)op.sM};
            PolCheb<float> pc{l0.fixed, wt, l0.fr, l0.fb, op.lv[0].dinvf, l0.fxa, l0.fd, op.lv[0].cheb, 1, {}};
            launch_tile<float>(l0.g, l0.Cf, pc, s);
        } else if (precision == 2) {
            Weights<df> wt = fine_weights<df>(le, true, true, nullptr, op.sK, op.sM);
            PolProduct<df, true, true> pp{wt, le->sp, le->sq, {}};
            launch_tile<df>(l0.g, le->Cx, pp, s);
        } else {
            Weights<float> wt{l0.kff, l0.mff, nullptr, (float)op.sK, (float)op.sM};
            PolResid<float> pr{l0.fixed, wt, l0.fr, l0.fb, l0.fd, {}};
            launch_tile<float>(l0.g, l0.Cf, pr, s);
        }
    };
    for (int i = 0; i < warmup; i++) one();
    CK(cudaEventRecord(e0, s));
    for (int i = 0; i < reps; i++) one();
    CK(cudaEventRecord(e1, s));
    CK(cudaEventSynchronize(e1));
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = (double)t / reps;
    return TOPO_OK;
}
int le_kernel_timing(TopoLE *le, int kclass, int enable, double *ms_total, long long *launches) {
    static LaunchTimer timer;
    if (enable) {
        if (kclass < TOPO_KT_SMOOTH || kclass > TOPO_KT_DFPROD) {
            set_error("unknown kernel class " + std::to_string(kclass));
            return TOPO_ERR_ARG;
        }
        timer.cls = kclass;
        timer.nn = le->L[0].g.nn();
        timer.used = 0;
        g_timer = &timer;
        return TOPO_OK;
    }
    if (g_timer != &timer) {
        set_error("kernel timing was not armed");
        return TOPO_ERR_STATE;
    }
    g_timer = nullptr;
    CK(cudaStreamSynchronize(le->stream));
    double tot = 0.0;
    for (size_t i = 0; i + 1 < timer.used; i += 2) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, timer.ev[i], timer.ev[i + 1]));
        tot += t;
    }
    if (ms_total) *ms_total = tot;
    if (launches) *launches = (long long)(timer.used / 2);
    timer.used = 0;
    return TOPO_OK;
}
}  // namespace topo
