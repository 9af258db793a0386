// sens.cuh -- adjoint right-hand side and element sensitivity kernels.
#pragma once
#include "kernels.cuh"

namespace topo {

// ---------------------------------------------------------------------------
// Adjoint step right-hand side, SolveLagrangen (LinearElasticity.cc:890-926):
//   DL  = -(h_du  + B2 L+ - a0 DL+ + a3 DDL+)
//   DDL = -(h_ddu + B3 L+ + a4 DDL+)
//   R1  = N ( -(h_u + B1 L+ + a2 DL+ + a5 DDL+) + a2 DL + a5 DDL )
// with B_i L+ = N (cMi M + cKi K) N L+.  The terminal step (:864-889) is the
// same formula with L+ = DL+ = DDL+ = 0, which is how the sweep starts.
// h_* (ComputeGradientObjectiveElementLoop, :2206-2356) come either from the
// per-node region count (objectives 0-2: dt * sum_{e ni n} P_e * state) or
// from weighted element products computed beforehand (objectives 3-6).
// Values on clamped DOFs of DL/DDL never reach lambda or the sensitivities.
// ---------------------------------------------------------------------------
struct AdjCombine {
    const uint8_t *fixed;
    const double *KL, *ML;        // K L+ and M L+ (unmasked element sums, masked input)
    const double *Lp1, *DLp1, *DDLp1;
    const double *Lp2, *Lp3;      // lambda two and three steps later (initial-guess extrapolation)
    int extrapolate;
    const double *hK, *hM;        // product-form objective gradients (or null)
    const float *cntP;            // per node sum of P over adjacent elements
    const double *Ustate, *DUstate, *DDUstate;  // state at this step (base of history)
    const double *cp;             // checkpoints (for j < 0: t = 0 state)
    long long ndof;
    int objective;
    long long out_dof;            // objective 7: the output DOF
    double *fx;                   // objective accumulator (objective 7 adds its value here)
    int t0mode;                   // 1: SolveLagrange0 right-hand side R3
    double dt;
    double a[6];
    double cM[3], cK[3];          // B1..B3 coefficients
    const StepCtx *st;
    double *DL, *DDL, *b, *x0;
    // optional: the masked operator applied to the initial guess,
    // (N A N + I - N) x0, from the K and M products of the last adjoint
    // iterates (KL, ML = K L+, M L+; KLh1, MLh1 = K L++, M L++; KLh2, MLh2 =
    // K L+++, M L+++), so that the solve needs no operator pass for its
    // initial residual
    double *ax0;
    const double *KLh1, *MLh1, *KLh2, *MLh2;
    double sK, sM;  // A = sK K + sM M
    // the coefficients as double-float pairs (split on the host) for the
    // double-float form of the mixed path
    df da[6], dcM[3], dcK[3], ddt, dsK, dsM;
};
template <class R>
__device__ __forceinline__ R adj_coef(double d, const df &f);
template <>
__device__ __forceinline__ double adj_coef<double>(double d, const df &) {
    return d;
}
template <>
__device__ __forceinline__ df adj_coef<df>(double, const df &f) {
    return f;
}

// R = double: the plain FP64 path.  R = df: the mixed path, in
// double-float arithmetic on the FP32 pipes with the FP64 inputs split on the
// integer pipes and one FP64 addition per output (about 25 FP64 operations per
// DOF otherwise, which GB300 runs at two per clock and SM).
template <class R>
static __global__ void k_adj_combine(AdjCombine A) {
    long long nn = A.ndof / 3;
    const double *u, *du, *ddu;
    if (A.t0mode) {
        u = A.cp;
        du = A.cp + A.ndof;
        ddu = A.cp + 2 * A.ndof;
    } else {
        long long off = (long long)A.st->j * A.ndof;
        u = A.Ustate + off;
        du = A.DUstate + off;
        ddu = A.DDUstate + off;
    }
    R a[6], cM[3], cK[3];
#pragma unroll
    for (int k = 0; k < 6; k++) a[k] = adj_coef<R>(A.a[k], A.da[k]);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        cM[k] = adj_coef<R>(A.cM[k], A.dcM[k]);
        cK[k] = adj_coef<R>(A.cK[k], A.dcK[k]);
    }
    const R dt = adj_coef<R>(A.dt, A.ddt), sK = adj_coef<R>(A.sK, A.dsK), sM = adj_coef<R>(A.sM, A.dsM);
    const R zero = R(0.0);
    const bool ax_is_mx = A.sK == 0.0 && A.sM == 1.0;  // mixed path: the ML slots hold A L
    const int nadj = A.st->nadj;  // adjoint steps done: lambda+, ++, +++ valid when nadj >= 1, 2, 3
    // x0 = w1 L+ + w2 L++ + w3 L+++
    double w1 = 1.0, w2 = 0.0, w3 = 0.0;
    if (A.extrapolate >= 2 && nadj >= 3) {
        w1 = 3.0;
        w2 = -3.0;
        w3 = 1.0;
    } else if (A.extrapolate >= 1 && nadj >= 2) {
        w1 = 2.0;
        w2 = -1.0;
    }
    const R W1 = R(w1), W2 = R(w2), W3 = R(w3);
    // one DOF per thread: its inputs are all loaded before its stores
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 3 * nn;
         i += (long long)gridDim.x * blockDim.x) {
        const long long n = i / 3;
        const int c = (int)(i - 3 * n);
        uint8_t f = A.fixed[n];
        const R cnt = R((double)A.cntP[n]);
        {
            R hu = zero, hdu = zero, hddu = zero;
            switch (A.objective) {
            case 0: hu = dt * cnt * R(u[i]); break;
            case 1: hdu = dt * cnt * R(du[i]); break;
            case 2: hddu = dt * cnt * R(ddu[i]); break;
            case 3: hu = R(A.hK[i]); break;
            case 4: hdu = R(A.hM[i]); break;
            case 5:
                hu = R(A.hK[i]);
                hdu = R(A.hM[i]);
                break;
            case 7:  // extension: dt/2 u_out^2, gradient dt u_out at the output DOF
                if (i == A.out_dof) {
                    hu = dt * R(u[i]);
                    *A.fx += 0.5 * A.dt * u[i] * u[i];  // the one thread of this DOF
                }
                break;
            default: hdu = R(A.hK[i]); break;
            }
            bool fx = (f >> c) & 1;
            // the inputs of this DOF are loaded before its first store (the
            // outputs may alias them as far as the compiler knows, and a load
            // after a store waits for another memory round trip)
            const double KLi = A.KL[i], MLi = A.ML[i], DLp1i = A.DLp1[i], DDLp1i = A.DDLp1[i];
            double Lp1i = 0.0, Lp2i = 0.0, Lp3i = 0.0, MLh1i = 0.0, MLh2i = 0.0, KLh1i = 0.0, KLh2i = 0.0;
            if (!A.t0mode) {
                Lp1i = A.Lp1[i];
                if (w2 != 0.0) Lp2i = A.Lp2[i];
                if (w3 != 0.0) Lp3i = A.Lp3[i];
                if (A.ax0) {
                    if (w2 != 0.0) MLh1i = A.MLh1[i];
                    if (w3 != 0.0) MLh2i = A.MLh2[i];
                    if (!ax_is_mx && A.sK != 0.0) {
                        if (w2 != 0.0) KLh1i = A.KLh1[i];
                        if (w3 != 0.0) KLh2i = A.KLh2[i];
                    }
                }
            }
            const R kl = fx ? zero : R(KLi), ml = fx ? zero : R(MLi);
            const R B1 = cM[0] * ml + cK[0] * kl;
            const R B2 = cM[1] * ml + cK[1] * kl;
            const R B3 = cM[2] * ml + cK[2] * kl;
            const R dlp = R(DLp1i), ddlp = R(DDLp1i);
            if (A.t0mode) {
                // SolveLagrange0 R3 (LinearElasticity.cc:753-758)
                const R r3 = -(hddu + B3 - a[1] * dlp + a[4] * ddlp);
                A.b[i] = fx ? 0.0 : todbl(r3);
                A.x0[i] = 0.0;
                if (A.ax0) A.ax0[i] = 0.0;
            } else {
                const R DL = -(hdu + B2 - a[0] * dlp + a[3] * ddlp);
                const R DDL = -(hddu + B3 + a[4] * ddlp);
                const R R1 = -(hu + B1 + a[2] * dlp + a[5] * ddlp) + a[2] * DL + a[5] * DDL;
                A.DL[i] = todbl(DL);
                A.DDL[i] = todbl(DDL);
                // the reference solves (N A N + I - N) L = R1 with A = -Keff
                // (LinearElasticity.cc:1022-1026, :924): Keff L = -R1 on free DOFs
                A.b[i] = fx ? 0.0 : todbl(-R1);
                R g = W1 * R(Lp1i);
                if (w2 != 0.0) g += W2 * R(Lp2i);
                if (w3 != 0.0) g += W3 * R(Lp3i);
                A.x0[i] = fx ? 0.0 : todbl(g);
                if (A.ax0) {
                    R mx = W1 * R(MLi);
                    if (w2 != 0.0) mx += W2 * R(MLh1i);
                    if (w3 != 0.0) mx += W3 * R(MLh2i);
                    R ax = mx;
                    if (!ax_is_mx) {
                        R kx = zero;
                        if (A.sK != 0.0) {
                            kx = W1 * R(KLi);
                            if (w2 != 0.0) kx += W2 * R(KLh1i);
                            if (w3 != 0.0) kx += W3 * R(KLh2i);
                        }
                        ax = sK * kx + sM * mx;
                    }
                    A.ax0[i] = fx ? 0.0 : todbl(ax);
                }
            }
        }
    }
}

// per-node count of adjacent elements inside the objective region
static __global__ void k_count_region(GridDesc g, const double *__restrict__ P, float *cnt) {
    long long nn = g.nn();
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        lex3(n, g.nx, g.ny, i, j, k);
        double s = 0.0;
        for (int c = 0; c < 8; c++) {
            int ei = i - (c & 1), ej = j - ((c >> 1) & 1), ek = k - (c >> 2);
            if (ei < 0 || ej < 0 || ek < 0 || ei >= g.ex || ej >= g.ey || ek >= g.ez) continue;
            s += P[ei + (long long)g.ex * (ej + (long long)g.ey * ek)];
        }
        cnt[n] = (float)s;
    }
}

// after the adjoint solve of step j: L+++ <- L++, L++ <- L+, L+ <- lambda_j,
// DL+ <- DL_j, DDL+ <- DDL_j (k_adj_combine uses the older lambdas only once
// the sweep has produced them)
// Mixed path (AL set): the ML slots hold A L instead of M L (A = sK K + sM M,
// the step operator).  A lambda_j = b - r of the solve just finished (its
// final residual is FP64-accurate), so no mass product is formed; with x zeroed
// by the solve (b = 0) A lambda_j = 0.
struct KMHist {
    const double *KL;
    double *ML;
    double *KLh1, *MLh1, *KLh2, *MLh2;  // null: not kept
    const double *b, *r;                // AL mode: the adjoint solve's b and final r (else null)
    const SolveScalars *S;
};
static __global__ void k_adj_advance(long long ndof, const double *__restrict__ lam, const double *__restrict__ DL,
                              const double *__restrict__ DDL, double *Lp1, double *DLp1, double *DDLp1, double *Lp2,
                              double *Lp3, KMHist H) {
    const bool zx = H.b && H.S->zero_x;
    // every value is loaded before the first store: the slots may alias as
    // far as the compiler knows, and a load after a store would wait for a
    // second memory round trip
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x) {
        const double lp2 = Lp2[i], lp1 = Lp1[i], l = lam[i], dl = DL[i], ddl = DDL[i];
        if (H.b) {  // AL mode: A L++ <- A L+, A L+ <- A lambda_j
            const double m1 = H.MLh1[i], m0 = H.ML[i], bv = H.b[i], rv = H.r[i];
            H.MLh2[i] = m1;
            H.MLh1[i] = m0;
            H.ML[i] = zx ? 0.0 : bv - rv;
        } else if (H.KLh1) {  // K, M products follow their lambdas: K L++ <- K L+, ...
            const double k1 = H.KLh1[i], m1 = H.MLh1[i], k0 = H.KL[i], m0 = H.ML[i];
            H.KLh2[i] = k1;
            H.MLh2[i] = m1;
            H.KLh1[i] = k0;
            H.MLh1[i] = m0;
        }
        Lp3[i] = lp2;
        Lp2[i] = lp1;
        Lp1[i] = l;
        DLp1[i] = dl;
        DDLp1[i] = ddl;
    }
}

// FCG initial residual from a precomputed (N A N + I - N) x0:
// r = b - ax0, reductions b.b and r.r, then the same solver-state set-up as
// the operator-pass initial residual (PolInitResid)
static __global__ void k_init_pointwise(long long ndof, const double *__restrict__ b, const double *__restrict__ ax0,
                                        double *r, SolveScalars *S, int has_r32, int accept_x0,
                                        cudaGraphConditionalHandle cond, int has_cond, Partials<2> part) {
    double red[2] = {0.0, 0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndof; i += (long long)gridDim.x * blockDim.x) {
        const double bv = b[i], rv = bv - ax0[i];
        r[i] = rv;
        red[0] += bv * bv;
        red[1] += rv * rv;
    }
    double tot[2];
    if (grid_reduce<EW, 2>(red, part, tot)) init_finish(S, tot, has_r32, cond, has_cond, accept_x0 != 0);
}

// ---------------------------------------------------------------------------
// Element sensitivities + objective, ComputeSensitivitiesElementLoopn
// (LinearElasticity.cc:1911-2077), ComputeSensitivitiesElementLoop0
// (:2080-2204) and ComputeObjectiveElementLoop (:2359-2452), fused.
//
// The 4 x 576 multiply-adds per element of the reference reduce to
//   df_e += P_e dfx0_e + lam_e' (dkfac_e KE wK_e + dmfac_e ME wM_e)
// with wK = sum aK_i s_i + bK_i p_i and wM likewise over the current state
// s = (u, du, ddu) and the previous state p (formed per node by
// k_sens_nodal); evaluated in the mode basis as
//   Lam' Khat WK  and  sum_m W_m Lam_m WM_m.
// One thread per element; OBJ is the reference objective (EvaluateObjective,
// :1416-1465, EvaluateObjectiveGradient :1469-1514).
// ---------------------------------------------------------------------------
struct SensArgs {
    GridDesc g;
    const double *lam;                       // adjoint (lambda_j, or DDL0)
    const double *Uh, *DUh, *DDUh;           // history base (current = slot j)
    const double *cp;                        // checkpoints (block start / t = 0 state)
    const double *kf, *dkf, *mf, *dmf, *P;
    double aK[3], bK[3], aM[3], bM[3];       // wK, wM combination coefficients
    double dt, dalpha, dbeta;
    int t0mode;                              // 1: state = t = 0, no previous state
    int with_objective;                      // accumulate the objective of the current state
    const StepCtx *st;
    // per-node vectors written by k_sens_nodal: FP64 combinations (element
    // math in FP64) or FP32 combinations plus FP32 copies of lambda and of the
    // states the objective quadratic form reads (element math in FP32)
    double *wKd, *wMd;
    float *wKf, *wMf, *lamf, *uf, *duf;
    double *df;
    double *fx;                              // device accumulator
    Partials<1> part;
    // aK, bK, aM, bM as double-float pairs (split on the host), for the
    // FP32-output form of k_sens_nodal
    topo::df daK[3], dbK[3], daM[3], dbM[3];
};

// current state (t0mode: the t = 0 state) and previous state of the step
__device__ __forceinline__ void sens_states(const SensArgs &A, long long ndof, const double *&u, const double *&du,
                                            const double *&ddu, const double *&up, const double *&dup,
                                            const double *&ddup) {
    up = dup = ddup = nullptr;
    if (A.t0mode) {
        u = A.cp;
        du = A.cp + ndof;
        ddu = A.cp + 2 * ndof;
        return;
    }
    int j = A.st->j;
    u = A.Uh + (long long)j * ndof;
    du = A.DUh + (long long)j * ndof;
    ddu = A.DDUh + (long long)j * ndof;
    if (j == 0) {
        const double *base = A.cp + (long long)A.st->block * 3 * ndof;
        up = base;
        dup = base + ndof;
        ddup = base + 2 * ndof;
    } else {
        up = A.Uh + (long long)(j - 1) * ndof;
        dup = A.DUh + (long long)(j - 1) * ndof;
        ddup = A.DDUh + (long long)(j - 1) * ndof;
    }
}

// c . (v0, v1, v2) evaluated as c0 v0 followed by FMAs, skipping the terms
// whose coefficient is exactly zero (several are for Newmark beta = 1/4,
// gamma = 1/2): the same value with fewer FP64 operations
__device__ __forceinline__ double comb3(const double c[3], double v0, double v1, double v2) {
    double s = c[0] * v0;
    if (c[1] != 0.0) s = fma(c[1], v1, s);
    if (c[2] != 0.0) s = fma(c[2], v2, s);
    return s;
}

// the same in double-float; nz holds the nonzero pattern of c (bit k: c[k])
__device__ __forceinline__ topo::df comb3(const topo::df c[3], int nz, topo::df v0, topo::df v1, topo::df v2) {
    topo::df s = c[0] * v0;
    if (nz & 2) s += c[1] * v1;
    if (nz & 4) s += c[2] * v2;
    return s;
}
__host__ __device__ __forceinline__ int comb3_nz(const double c[3]) {
    return (c[0] != 0.0 ? 1 : 0) | (c[1] != 0.0 ? 2 : 0) | (c[2] != 0.0 ? 4 : 0);
}

// wK = aK . (u, du, ddu) + bK . (u-, du-, ddu-) and wM likewise, once per DOF
// (every node is shared by up to 8 elements, so this is 8x less work than
// forming them inside the element loop).  FP64 element math: FP64
// combinations.  FP32 element math: the combinations in double-float on the
// FP32 pipes from inputs split on the integer pipes, rounded to FP32 (the hi
// part): no FP64 instruction, where the FP64 form was bound by GB300's FP64
// rate.
static __global__ void k_sens_nodal(const SensArgs A) {
    const long long ndof = 3 * A.g.nn();
    const double *u, *du, *ddu, *up, *dup, *ddup;
    sens_states(A, ndof, u, du, ddu, up, dup, ddup);
    if (A.wKd) {
        for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < ndof;
             q += (long long)gridDim.x * blockDim.x) {
            double s0 = u[q], s1 = du[q], s2 = ddu[q];
            double wk = comb3(A.aK, s0, s1, s2);
            double wm = comb3(A.aM, s0, s1, s2);
            if (!A.t0mode) {
                double p0 = up[q], p1 = dup[q], p2 = ddup[q];
                wk += comb3(A.bK, p0, p1, p2);
                wm += comb3(A.bM, p0, p1, p2);
            }
            A.wKd[q] = wk;
            A.wMd[q] = wm;
        }
        return;
    }
    const int nzaK = comb3_nz(A.aK), nzaM = comb3_nz(A.aM), nzbK = comb3_nz(A.bK), nzbM = comb3_nz(A.bM);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < ndof; q += (long long)gridDim.x * blockDim.x) {
        // every input is loaded before the first store (a load behind a
        // possibly aliasing store waits for another memory round trip)
        const double s0 = u[q], s1 = du[q], s2 = ddu[q], lq = A.lam[q];
        double p0v = 0.0, p1v = 0.0, p2v = 0.0;
        if (!A.t0mode) {
            p0v = up[q];
            p1v = dup[q];
            p2v = ddup[q];
        }
        const topo::df d0(s0), d1(s1), d2(s2);
        topo::df wk = comb3(A.daK, nzaK, d0, d1, d2);
        topo::df wm = comb3(A.daM, nzaM, d0, d1, d2);
        if (!A.t0mode) {
            const topo::df p0(p0v), p1(p1v), p2(p2v);
            wk += comb3(A.dbK, nzbK, p0, p1, p2);
            wm += comb3(A.dbM, nzbM, p0, p1, p2);
        }
        A.wKf[q] = wk.hi;
        A.wMf[q] = wm.hi;
        A.lamf[q] = f64_to_f32(lq);
        if (A.uf) A.uf[q] = d0.hi;
        if (A.duf) A.duf[q] = d1.hi;
    }
}

template <class T, class S>
__device__ __forceinline__ void gather8(const S *v, const long long nodes[8], T out[3][8]) {
#pragma unroll
    for (int L = 0; L < 8; L++)
#pragma unroll
        for (int c = 0; c < 3; c++) out[c][L] = (T)v[3 * nodes[L] + c];
}

template <class T>
__device__ __forceinline__ T quad_K(const ElemConst<T> &C, T A[3][8], T B[3][8]) {
    // A, B already in mode space; returns A' Khat B
    T Y[3][8];
    mode_khat(C, B, Y);
    T s = T(0);
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int m = 0; m < 8; m++) s += A[c][m] * Y[c][m];
    return s;
}
template <class T>
__device__ __forceinline__ T quad_M(const ElemConst<T> &C, T A[3][8], T B[3][8]) {
    T s = T(0);
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int m = 0; m < 8; m++) s += C.W[m] * A[c][m] * B[c][m];
    return s;
}

// source of a gathered vector: the FP64 vector for FP64 element math, its
// FP32 copy for FP32 element math
__device__ __forceinline__ const double *sens_src(const double *d, const float *, double) { return d; }
__device__ __forceinline__ const float *sens_src(const double *, const float *f, float) { return f; }

template <int OBJ, class T>
static __global__ void __launch_bounds__(EW) k_sens(const SensArgs A, const ElemConst<T> C) {
    const GridDesc g = A.g;
    const long long nel = g.nel(), ndof = 3 * g.nn();
    const double *u, *du, *ddu, *up, *dup, *ddup;
    sens_states(A, ndof, u, du, ddu, up, dup, ddup);
    const auto lam = sens_src(A.lam, A.lamf, T());
    const auto wK = sens_src(A.wKd, A.wKf, T());
    const auto wM = sens_src(A.wMd, A.wMf, T());
    const auto su = sens_src(u, A.uf, T());
    const auto sdu = sens_src(du, A.duf, T());
    double fxv[1] = {0.0};
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nel; e += (long long)gridDim.x * blockDim.x) {
        int i, jj, k;
        lex3(e, g.ex, g.ey, i, jj, k);
        long long nodes[8];
#pragma unroll
        for (int L = 0; L < 8; L++)
            nodes[L] = (i + (L & 1)) + (long long)g.nx * ((jj + ((L >> 1) & 1)) + (long long)g.ny * (k + (L >> 2)));
        // lam' KE wK = (Khat Lam)' WK in mode space (Khat symmetric): only
        // Khat Lam and W Lam stay live while WK and WM stream in per component
        T KL[3][8], ML[3][8];
        {
            T Lm[3][8];
            gather8<T>(lam, nodes, Lm);
#pragma unroll
            for (int c = 0; c < 3; c++) mode_fwd(Lm[c]);
            mode_khat(C, Lm, KL);
#pragma unroll
            for (int c = 0; c < 3; c++)
#pragma unroll
                for (int m = 0; m < 8; m++) ML[c][m] = C.W[m] * Lm[c][m];
        }
        T sK = T(0), sM = T(0);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            T wk8[8], wm8[8];
#pragma unroll
            for (int L = 0; L < 8; L++) {
                wk8[L] = (T)wK[3 * nodes[L] + c];
                wm8[L] = (T)wM[3 * nodes[L] + c];
            }
            mode_fwd(wk8);
            mode_fwd(wm8);
#pragma unroll
            for (int m = 0; m < 8; m++) {
                sK += KL[c][m] * wk8[m];
                sM += ML[c][m] * wm8[m];
            }
        }
        double dkfe = A.dkf[e], dmfe = A.dmf[e], kfe = A.kf[e], mfe = A.mf[e], Pe = A.P[e];
        double t3 = dkfe * (double)sK + dmfe * (double)sM;
        // objective value h0 and its explicit density derivative dfx0
        double h0 = 0.0, dfx0 = 0.0;
        if (OBJ == 7) {
            // the output-DOF objective has no element part (k_adj_combine adds it)
        } else if (OBJ == 0 || OBJ == 1 || OBJ == 2) {
            if (A.with_objective) {
                const double *s = (OBJ == 0) ? u : (OBJ == 1 ? du : ddu);
                double acc = 0.0;
#pragma unroll
                for (int L = 0; L < 8; L++)
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        double v = s[3 * nodes[L] + c];
                        acc += v * v;
                    }
                h0 = A.dt * 0.5 * acc;
            }
        } else {
            T S0[3][8];
            gather8<T>((OBJ == 3) ? su : sdu, nodes, S0);
#pragma unroll
            for (int c = 0; c < 3; c++) mode_fwd(S0[c]);
            if (OBJ == 3) {
                double uKu = (double)quad_K(C, S0, S0);
                h0 = A.dt * 0.5 * kfe * uKu;
                dfx0 = A.dt * 0.5 * dkfe * uKu;
            } else if (OBJ == 4) {
                double vMv = (double)quad_M(C, S0, S0);
                h0 = A.dt * 0.5 * mfe * vMv;
                dfx0 = A.dt * 0.5 * dmfe * vMv;
            } else if (OBJ == 5) {
                double vMv = (double)quad_M(C, S0, S0);
                T S1[3][8];
                gather8<T>(su, nodes, S1);
#pragma unroll
                for (int c = 0; c < 3; c++) mode_fwd(S1[c]);
                double uKu = (double)quad_K(C, S1, S1);
                h0 = A.dt * 0.5 * (kfe * uKu + mfe * vMv);
                dfx0 = A.dt * 0.5 * (dkfe * uKu + dmfe * vMv);
            } else {  // 6: dissipated energy with interpolated damping
                double vKv = (double)quad_K(C, S0, S0);
                double vMv = (double)quad_M(C, S0, S0);
                h0 = A.dt * 0.5 * (A.dalpha * mfe * vMv + A.dbeta * kfe * vKv);
                dfx0 = A.dt * 0.5 * (A.dalpha * dmfe * vMv + A.dbeta * dkfe * vKv);
            }
        }
        A.df[e] += Pe * dfx0 + t3;
        if (A.with_objective) fxv[0] += Pe * h0;
    }
    double tot[1];
    if (grid_reduce<EW, 1>(fxv, A.part, tot)) *A.fx += tot[0];
}

}  // namespace topo
