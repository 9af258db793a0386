// sommg.cuh -- SOMMG reduced-order path (SOMMG.cc:40-265 and the reduction
// branches of LinearElasticity.cc).
//
// The reference builds a basis Q of kb vectors from solves with
// P0 = K - om^2 M, projects K, M, C and the load onto it, integrates the
// Newmark forward and adjoint recursions with the dense kb x kb matrices, and
// lifts every step's states and adjoints back to the full grid to run the
// element objective and sensitivity loops (LinearElasticity.cc:1683-1868).
//
// Here the lifts are never formed.  Every full-grid quantity the reference
// computes from lifted fields is bilinear in reduced vectors:
//   objective          sum_e P_e h(u_e) = u_r' (Q' K(kf P) Q) u_r, ...
//   state gradients    Q' h_full = dt (Q' K(kf P) Q) u_r, ...
//   sensitivities      sum_t lam_e' KE w_e = sum_{a,b} S[a,b] x_a,e' KE x_b,e,
//                      S = sum_t lam_r w_r'   (x_a = column a of Q)
// so both sweeps run in reduced space in one single-CTA kernel each, and the
// sensitivities need one element pass with Phi = Q S' per accumulated S.
#pragma once
#include "sens.cuh"

namespace topo {

constexpr int KB_MAX = 32;  // basis vectors supported by the reduced kernels

// ---- reductions against the basis: out[b * ostride] = Q_b . y, b < kb ----
// deterministic: per-chunk partials, then a fixed-order sum
// (Q_b = Q + b qs: FP64 rows of the plain path, FP32 rows of the mixed path)
constexpr int MD_CHUNKS = 152;
template <class QT>
static __global__ void __launch_bounds__(256) k_md_partial(long long nd, const QT *__restrict__ Q, long long qs, int kb,
                                                           const double *__restrict__ y, double *part) {
    const int b = blockIdx.y;
    const QT *q = Q + (size_t)b * qs;
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x)
        s += (double)q[i] * y[i];
    __shared__ double sm[8];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sm[w];
        part[(size_t)b * gridDim.x + blockIdx.x] = t;
    }
}
static __global__ void k_md_final(int kb, int nchunk, const double *__restrict__ part, double *out, int ostride) {
    const int b = threadIdx.x;
    if (b >= kb) return;
    double t = 0.0;
    for (int c = 0; c < nchunk; c++) t += part[(size_t)b * nchunk + c];
    out[(size_t)b * ostride] = t;
}

// modified Gram-Schmidt step (SOMMG.cc:195-202): v -= coef * q
template <class QT>
static __global__ void k_axpy_dev(long long nd, double *v, const QT *__restrict__ q, const double *coef) {
    const double c = *coef;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x)
        v[i] -= c * (double)q[i];
}
// basis row j of the FP32 basis from its FP64 solve, and back
static __global__ void k_d2f_row(long long nd, const double *__restrict__ x, float *q) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x)
        q[i] = (float)x[i];
}
static __global__ void k_f2d_row(long long nd, const float *__restrict__ q, double *x) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x)
        x[i] = (double)q[i];
}
// normalisation (SOMMG.cc:92-95, :206-208): v /= sqrt(nrm2)
static __global__ void k_normalise(long long nd, double *v, const double *nrm2) {
    const double n = sqrt(*nrm2);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x)
        v[i] /= n;
}
static __global__ void k_sqrt1(double *v) { *v = sqrt(*v); }
// y = s N x (Dirichlet mask per node byte)
static __global__ void k_mask_scale(long long nn, const uint8_t *__restrict__ fixed, const double *__restrict__ x,
                                    double s, double *y) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        const uint8_t f = fixed[n];
        for (int c = 0; c < 3; c++) y[3 * n + c] = ((f >> c) & 1) ? 0.0 : s * x[3 * n + c];
    }
}
// y = cnt_n x (the per-node region count of objectives 0-2)
static __global__ void k_cnt_mul(long long nn, const float *__restrict__ cnt, const double *__restrict__ x, double *y) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        const double c = cnt[n];
        for (int k = 0; k < 3; k++) y[3 * n + k] = c * x[3 * n + k];
    }
}
// full = sum_b r[b] Q_b (the lift of LinearElasticity.cc:1089-1107), for output
template <class QT>
static __global__ void k_lift(long long nd, int kb, const QT *__restrict__ Q, long long qs,
                              const double *__restrict__ r, double *full) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < kb; b++) s += r[b] * (double)Q[(size_t)b * qs + i];
        full[i] = s;
    }
}

// ---- reduced sweeps ----
// Reduced matrices in device memory, row-major kb x kb: Kr, Mr (basis
// projections of K and of the masked M), Kp, Mp, Gc (objective region
// projections Q' K(kf P) Q, Q' M(mf P) Q, Q' diag(cnt) Q), Pr (load).
struct RedSys {
    int kb, Ts, objective, loadsignal;
    double a[6], dt, alpha, beta, load_scale;
    const double *Kr, *Mr, *Kp, *Mp, *Gc, *Pr;
    double *hist;  // [Ts][3][kb]: u, du, ddu
    double *S;     // [4][kb*kb]: S_K, S_M, S_oK, S_oM
    double *fx;    // objective
    int *status;   // 0 ok, TOPO_ERR_NAN on a singular reduced matrix
};

// Gauss-Jordan inverse of an SPD kb x kb matrix held in shared memory
// (A is destroyed, Ainv receives the inverse); all threads of the CTA
__device__ void red_invert(int kb, double *A, double *Ainv, int *bad) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < kb * kb; i += nt) Ainv[i] = (i / kb == i % kb) ? 1.0 : 0.0;
    __syncthreads();
    for (int c = 0; c < kb; c++) {
        const double piv = A[c * kb + c];
        if (tid == 0 && !(fabs(piv) > 0.0)) *bad = 1;
        __syncthreads();
        for (int j = tid; j < kb; j += nt) {
            A[c * kb + j] /= piv;
            Ainv[c * kb + j] /= piv;
        }
        __syncthreads();
        for (int i = tid; i < kb * kb; i += nt) {
            const int r = i / kb, j = i % kb;
            if (r == c) continue;
            const double f = A[r * kb + c];
            if (j != c) A[r * kb + j] -= f * A[c * kb + j];
            Ainv[r * kb + j] -= f * Ainv[c * kb + j];
        }
        __syncthreads();
        for (int r = tid; r < kb; r += nt)
            if (r != c) A[r * kb + c] = 0.0;
        __syncthreads();
    }
}
// y = A x (kb x kb, row-major in shared memory), threads over rows
__device__ __forceinline__ void red_gemv(int kb, const double *A, const double *x, double *y) {
    for (int i = threadIdx.x; i < kb; i += blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < kb; j++) s += A[i * kb + j] * x[j];
        y[i] = s;
    }
}

// shared-memory layout of the sweeps: matrices [RED_NMAT][kb*kb] then vectors
constexpr int RED_NMAT = 9;  // Kinv, Minv, B1, B2, B3, Kp, Mp, Gc, scratch
constexpr int RED_NVEC = 24;
__host__ inline size_t red_smem_bytes(int kb) {
    return sizeof(double) * ((size_t)RED_NMAT * kb * kb + (size_t)RED_NVEC * kb + 8);
}

// the matrices of the reduced Newmark recursion (N = 1, LinearElasticity.cc:1000-1044):
// Keff = K + a5 M + a2 C, B1 = a5 M + a2 C, B2 = a3 M - a0 C, B3 = a4 M - a1 C,
// C = alpha M + beta K
__device__ void red_setup(const RedSys &R, double *sm, int *bad) {
    const int kb = R.kb, k2 = kb * kb;
    double *Kinv = sm, *Minv = sm + k2, *B1 = sm + 2 * k2, *B2 = sm + 3 * k2, *B3 = sm + 4 * k2;
    double *Kp = sm + 5 * k2, *Mp = sm + 6 * k2, *Gc = sm + 7 * k2, *W = sm + 8 * k2;
    const double *a = R.a;
    for (int i = threadIdx.x; i < k2; i += blockDim.x) {
        const double K = R.Kr[i], M = R.Mr[i], C = R.alpha * M + R.beta * K;
        W[i] = K + a[5] * M + a[2] * C;
        B1[i] = a[5] * M + a[2] * C;
        B2[i] = a[3] * M - a[0] * C;
        B3[i] = a[4] * M - a[1] * C;
        Kp[i] = R.Kp ? R.Kp[i] : 0.0;
        Mp[i] = R.Mp ? R.Mp[i] : 0.0;
        Gc[i] = R.Gc ? R.Gc[i] : 0.0;
    }
    __syncthreads();
    red_invert(kb, W, Kinv, bad);
    for (int i = threadIdx.x; i < k2; i += blockDim.x) W[i] = R.Mr[i];
    __syncthreads();
    red_invert(kb, W, Minv, bad);
}

// forward sweep: CompleteInitialState (u0 = du0 = 0, M ddu0 = f(0),
// LinearElasticity.cc:1049-1078) and every SolveStateBlock step (:1298-1397)
static __global__ void k_red_forward(RedSys R) {
    TOPO_DYNAMIC_SMEM(double, red_sm);
    __shared__ int bad;
    const int kb = R.kb, k2 = kb * kb;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    red_setup(R, red_sm, &bad);
    const double *Kinv = red_sm, *Minv = red_sm + k2, *B1 = red_sm + 2 * k2, *B2 = red_sm + 3 * k2,
                 *B3 = red_sm + 4 * k2;
    double *v = red_sm + RED_NMAT * k2;
    double *rhs = v, *t1 = v + kb, *t2 = v + 2 * kb, *t3 = v + 3 * kb;
    const double *a = R.a;
    const double s0 = load_signal(R.loadsignal, 0.0) * R.load_scale;
    for (int i = threadIdx.x; i < kb; i += blockDim.x) {
        rhs[i] = R.Pr[i] * s0;
        R.hist[i] = 0.0;
        R.hist[kb + i] = 0.0;
    }
    __syncthreads();
    red_gemv(kb, Minv, rhs, R.hist + 2 * kb);
    __syncthreads();
    for (int t = 1; t < R.Ts; t++) {
        const double *u = R.hist + (size_t)(t - 1) * 3 * kb, *du = u + kb, *ddu = u + 2 * kb;
        double *un = R.hist + (size_t)t * 3 * kb;
        red_gemv(kb, B1, u, t1);
        red_gemv(kb, B2, du, t2);
        red_gemv(kb, B3, ddu, t3);
        __syncthreads();
        const double st = load_signal(R.loadsignal, t * R.dt) * R.load_scale;
        for (int i = threadIdx.x; i < kb; i += blockDim.x) rhs[i] = R.Pr[i] * st + t1[i] + t2[i] + t3[i];
        __syncthreads();
        red_gemv(kb, Kinv, rhs, un);
        __syncthreads();
        for (int i = threadIdx.x; i < kb; i += blockDim.x) {
            const double d = un[i] - u[i];
            un[kb + i] = a[0] * du[i] + a[1] * ddu[i] + a[2] * d;
            un[2 * kb + i] = -a[3] * du[i] - a[4] * ddu[i] + a[5] * d;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && bad) *R.status = TOPO_ERR_NAN;
}

// objective value h(t) and state gradients of one state (EvaluateObjective
// :1416-1465 and ComputeGradientObjectiveElementLoop :2206-2356 on the lifted
// state, in reduced form); h1, h2, h3 = d h / d(u, du, ddu)
__device__ void red_objective(const RedSys &R, const double *Kp, const double *Mp, const double *Gc, const double *u,
                              const double *du, const double *ddu, double *h1, double *h2, double *h3, double *tmp,
                              double *hval) {
    const int kb = R.kb;
    const double dt = R.dt;
    for (int i = threadIdx.x; i < kb; i += blockDim.x) h1[i] = h2[i] = h3[i] = 0.0;
    __syncthreads();
    double hv = 0.0;
    if (R.objective <= 2) {
        // dt/2 s' diag(cnt) s of the objective's state s
        const double *s = R.objective == 0 ? u : (R.objective == 1 ? du : ddu);
        double *h = R.objective == 0 ? h1 : (R.objective == 1 ? h2 : h3);
        red_gemv(kb, Gc, s, tmp);
        __syncthreads();
        for (int i = threadIdx.x; i < kb; i += blockDim.x) h[i] = dt * tmp[i];
        if (threadIdx.x == 0) {
            double q = 0.0;
            for (int i = 0; i < kb; i++) q += s[i] * tmp[i];
            hv = 0.5 * dt * q;
        }
    } else {
        const bool useK = R.objective == 3 || R.objective == 5, useM = R.objective >= 4;
        if (useK) {
            red_gemv(kb, Kp, u, tmp);
            __syncthreads();
            for (int i = threadIdx.x; i < kb; i += blockDim.x) h1[i] = dt * tmp[i];
            if (threadIdx.x == 0) {
                double q = 0.0;
                for (int i = 0; i < kb; i++) q += u[i] * tmp[i];
                hv += 0.5 * dt * q;
            }
            __syncthreads();
        }
        if (useM) {
            // objective 6: dt/2 du' (alpha M(mf P) + beta K(kf P)) du
            const double cm = (R.objective == 6) ? R.alpha : 1.0, ck = (R.objective == 6) ? R.beta : 0.0;
            for (int i = threadIdx.x; i < kb; i += blockDim.x) {
                double sm = 0.0, sk = 0.0;
                for (int j = 0; j < kb; j++) {
                    sm += Mp[i * kb + j] * du[j];
                    sk += Kp[i * kb + j] * du[j];
                }
                tmp[i] = cm * sm + ck * sk;
            }
            __syncthreads();
            for (int i = threadIdx.x; i < kb; i += blockDim.x) h2[i] = dt * tmp[i];
            if (threadIdx.x == 0) {
                double q = 0.0;
                for (int i = 0; i < kb; i++) q += du[i] * tmp[i];
                hv += 0.5 * dt * q;
            }
        }
    }
    if (threadIdx.x == 0) *hval = hv;
    __syncthreads();
}

// S[a][b] += c x[a] y[b] for the kb x kb accumulator S
__device__ __forceinline__ void red_outer(int kb, double *S, double c, const double *x, const double *y) {
    for (int i = threadIdx.x; i < kb * kb; i += blockDim.x) S[i] += c * x[i / kb] * y[i % kb];
}

// adjoint sweep: SolveLagrangen (:808-954) backwards over every step, then
// SolveLagrange0 (:678-804), with the objective and the sensitivity
// accumulators S_K, S_M (lambda w' of ComputeSensitivitiesElementLoopn /
// Loop0 :1911-2204) and S_oK, S_oM (the explicit dfx0 terms)
static __global__ void k_red_adjoint(RedSys R) {
    TOPO_DYNAMIC_SMEM(double, red_sm);
    __shared__ int bad;
    __shared__ double hval;
    const int kb = R.kb, k2 = kb * kb;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    red_setup(R, red_sm, &bad);
    const double *Kinv = red_sm, *Minv = red_sm + k2, *B1 = red_sm + 2 * k2, *B2 = red_sm + 3 * k2,
                 *B3 = red_sm + 4 * k2, *Kp = red_sm + 5 * k2, *Mp = red_sm + 6 * k2, *Gc = red_sm + 7 * k2;
    double *v = red_sm + RED_NMAT * k2;
    double *h1 = v, *h2 = v + kb, *h3 = v + 2 * kb, *tmp = v + 3 * kb, *L = v + 4 * kb, *DL = v + 5 * kb,
           *DDL = v + 6 * kb, *Lp = v + 7 * kb, *DLp = v + 8 * kb, *DDLp = v + 9 * kb, *t1 = v + 10 * kb,
           *t2 = v + 11 * kb, *t3 = v + 12 * kb, *rr = v + 13 * kb, *wK = v + 14 * kb, *wM = v + 15 * kb;
    // the S accumulators live in global memory (4 kb^2), zeroed here
    double *SK = R.S, *SM = R.S + k2, *SoK = R.S + 2 * k2, *SoM = R.S + 3 * k2;
    for (int i = threadIdx.x; i < 4 * k2; i += blockDim.x) R.S[i] = 0.0;
    for (int i = threadIdx.x; i < kb; i += blockDim.x) Lp[i] = DLp[i] = DDLp[i] = 0.0;
    __syncthreads();
    const double *a = R.a, al = R.alpha, be = R.beta, dt = R.dt;
    // explicit density derivative of the objective (EvaluateObjectiveGradient :1469-1514)
    const double oK = (R.objective == 3 || R.objective == 5) ? 0.5 * dt : (R.objective == 6 ? 0.5 * dt * be : 0.0);
    const double oM = (R.objective == 4 || R.objective == 5) ? 0.5 * dt : (R.objective == 6 ? 0.5 * dt * al : 0.0);
    double fx = 0.0;
    for (int t = R.Ts - 1; t >= 1; t--) {
        const double *u = R.hist + (size_t)t * 3 * kb, *du = u + kb, *ddu = u + 2 * kb;
        const double *ub = R.hist + (size_t)(t - 1) * 3 * kb, *dub = ub + kb, *ddub = ub + 2 * kb;
        red_objective(R, Kp, Mp, Gc, u, du, ddu, h1, h2, h3, tmp, &hval);
        fx += hval;
        if (t == R.Ts - 1) {
            for (int i = threadIdx.x; i < kb; i += blockDim.x) {
                DL[i] = -h2[i];
                DDL[i] = -h3[i];
                rr[i] = h1[i] - a[2] * DL[i] - a[5] * DDL[i];  // -R1: Keff L = -R1
            }
        } else {
            red_gemv(kb, B1, Lp, t1);
            red_gemv(kb, B2, Lp, t2);
            red_gemv(kb, B3, Lp, t3);
            __syncthreads();
            for (int i = threadIdx.x; i < kb; i += blockDim.x) {
                DL[i] = -(h2[i] + t2[i] - a[0] * DLp[i] + a[3] * DDLp[i]);
                DDL[i] = -(h3[i] + t3[i] + a[4] * DDLp[i]);
                const double r1 = -(h1[i] + t1[i] + a[2] * DLp[i] + a[5] * DDLp[i]) + a[2] * DL[i] + a[5] * DDL[i];
                rr[i] = -r1;
            }
        }
        __syncthreads();
        red_gemv(kb, Kinv, rr, L);
        __syncthreads();
        // sensitivity combinations of this step (ComputeSensitivitiesElementLoopn)
        for (int i = threadIdx.x; i < kb; i += blockDim.x) {
            wK[i] = -(1.0 + a[2] * be) * u[i] + a[2] * be * ub[i] - a[0] * be * dub[i] - a[1] * be * ddub[i];
            wM[i] = -(a[5] + a[2] * al) * u[i] + (a[5] + a[2] * al) * ub[i] + (a[3] - a[0] * al) * dub[i] +
                    (a[4] - a[1] * al) * ddub[i];
        }
        __syncthreads();
        red_outer(kb, SK, 1.0, L, wK);
        red_outer(kb, SM, 1.0, L, wM);
        if (oK != 0.0) red_outer(kb, SoK, oK, (R.objective == 6) ? du : u, (R.objective == 6) ? du : u);
        if (oM != 0.0) red_outer(kb, SoM, oM, du, du);
        __syncthreads();
        for (int i = threadIdx.x; i < kb; i += blockDim.x) {
            Lp[i] = L[i];
            DLp[i] = DL[i];
            DDLp[i] = DDL[i];
        }
        __syncthreads();
    }
    // t = 0: objective of the initial state, SolveLagrange0 and Loop0
    {
        const double *u = R.hist, *du = u + kb, *ddu = u + 2 * kb;
        red_objective(R, Kp, Mp, Gc, u, du, ddu, h1, h2, h3, tmp, &hval);
        fx += hval;
        red_gemv(kb, B3, Lp, t3);
        __syncthreads();
        for (int i = threadIdx.x; i < kb; i += blockDim.x) rr[i] = -(h3[i] + t3[i] - a[1] * DLp[i] + a[4] * DDLp[i]);
        __syncthreads();
        red_gemv(kb, Minv, rr, L);  // DDL0
        __syncthreads();
        for (int i = threadIdx.x; i < kb; i += blockDim.x) {
            wK[i] = u[i] + be * du[i];
            wM[i] = al * du[i] + ddu[i];
        }
        __syncthreads();
        red_outer(kb, SK, 1.0, L, wK);
        red_outer(kb, SM, 1.0, L, wM);
        if (oK != 0.0) red_outer(kb, SoK, oK, (R.objective == 6) ? du : u, (R.objective == 6) ? du : u);
        if (oM != 0.0) red_outer(kb, SoM, oM, du, du);
    }
    if (threadIdx.x == 0) {
        *R.fx = fx;
        if (bad) *R.status = TOPO_ERR_NAN;
    }
}

// Phi_s = Q S_s' for the accumulators in use: Phi_s[a] = sum_b S_s[a][b] Q_b
// (FP64 sums; Phi stored in the basis type, rows of nd values)
template <class QT>
static __global__ void __launch_bounds__(256) k_red_phi(long long nd, int kb, const QT *__restrict__ Q, long long qs,
                                                        const double *__restrict__ S, int ns, QT *Phi) {
    __shared__ double sS[4 * KB_MAX * KB_MAX];
    for (int i = threadIdx.x; i < ns * kb * kb; i += blockDim.x) sS[i] = S[i];
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nd; i += (long long)gridDim.x * blockDim.x) {
        double q[KB_MAX];
#pragma unroll
        for (int b = 0; b < KB_MAX; b++) q[b] = b < kb ? (double)Q[(size_t)b * qs + i] : 0.0;
        for (int s = 0; s < ns; s++)
            for (int a = 0; a < kb; a++) {
                double acc = 0.0;
#pragma unroll
                for (int b = 0; b < KB_MAX; b++)
                    if (b < kb) acc += sS[(s * kb + a) * kb + b] * q[b];
                Phi[((size_t)s * kb + a) * nd + i] = (QT)acc;
            }
    }
}

// element sensitivities of the reduced path (the sum over every step of
// ComputeSensitivitiesElementLoopn / Loop0, in mode space):
//   df_e = dkf_e sum_a x_a' KE (phiK_a + P_e phioK_a) + dmf_e sum_a x_a' ME (phiM_a + P_e phioM_a)
template <class QT>
struct RedSens {
    GridDesc g;
    int kb;
    long long qs;                                // row stride of Q
    const QT *Q, *phiK, *phiM, *phioK, *phioM;  // phio* may be null; Phi rows of nd values
    const double *dkf, *dmf, *P;
    double *df;
};
template <class QT>
static __global__ void __launch_bounds__(EW) k_red_sens(const RedSens<QT> A, const ElemConst<double> C) {
    const GridDesc g = A.g;
    const long long nel = g.nel(), nd = 3 * g.nn();
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nel; e += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        lex3(e, g.ex, g.ey, i, j, k);
        long long nodes[8];
#pragma unroll
        for (int L = 0; L < 8; L++)
            nodes[L] = (i + (L & 1)) + (long long)g.nx * ((j + ((L >> 1) & 1)) + (long long)g.ny * (k + (L >> 2)));
        const double Pe = A.P[e];
        double sK = 0.0, sM = 0.0;
        for (int a = 0; a < A.kb; a++) {
            const size_t off = (size_t)a * nd;
            double X[3][8], Y[3][8], KX[3][8];
            gather8<double>(A.Q + (size_t)a * A.qs, nodes, X);
#pragma unroll
            for (int c = 0; c < 3; c++) mode_fwd(X[c]);
            mode_khat(C, X, KX);
#pragma unroll
            for (int L = 0; L < 8; L++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const long long q = 3 * nodes[L] + c;
                    Y[c][L] = (double)A.phiK[off + q] + (A.phioK ? Pe * (double)A.phioK[off + q] : 0.0);
                }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                mode_fwd(Y[c]);
#pragma unroll
                for (int m = 0; m < 8; m++) sK += KX[c][m] * Y[c][m];
            }
#pragma unroll
            for (int L = 0; L < 8; L++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const long long q = 3 * nodes[L] + c;
                    Y[c][L] = (double)A.phiM[off + q] + (A.phioM ? Pe * (double)A.phioM[off + q] : 0.0);
                }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                mode_fwd(Y[c]);
#pragma unroll
                for (int m = 0; m < 8; m++) sM += C.W[m] * X[c][m] * Y[c][m];
            }
        }
        A.df[e] = A.dkf[e] * sK + A.dmf[e] * sM;
    }
}

}  // namespace topo
