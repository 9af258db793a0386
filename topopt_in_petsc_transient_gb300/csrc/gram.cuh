// gram.cuh -- tall-skinny Gram products of the SOMMG reduction on the
// fifth-generation tensor cores (tcgen05, TMEM accumulators).
//
//   out[a * kb + b] = sum_k Q[a][k] W[b][k]      a, b < kb <= 32
//
// for a basis Q stored in FP32 and products W = A Q given as an FP32 pair
// (W = Wh + Wl, the FP64 value to about 2^-48), over ld values per vector
// (ld a multiple of GR_KC; the padding of every row is zero).  This is the
// contraction of the reduced matrices Kr = Q'KQ, Mr = Q'MQ and the objective
// projections (SOMMG.cc:226-251).
//
// Precision.  Every FP32 operand is split into TF32 pieces with
// round-to-nearest, v = h + m + l (h = rna(v), m = rna(v - h), l = v - h - m;
// the split is exact).  The A operand (M = 128 rows, K-major) holds the rows
// [Wh.h | Wh.m | Wh.l | rna(Wl)] of the 32 basis slots, the B operand
// (N = 96 rows, K-major) [Q.h | Q.m | Q.l], so one tcgen05.mma.kind::tf32
// of shape 128 x 96 x 8 forms every piece product, each exact in FP32 (two
// 11-bit significands).  D accumulates in TMEM in FP32 over GR_RD chunks of
// GR_KC values (four MMAs a chunk); the warps then read their lanes (row = A
// row) and add the values into double-float (FP32 pair) register
// accumulators with an error-free two-sum, the small pieces going straight
// into the low word.  The FP32 sums in TMEM are the one rounded step: on
// GB300 a same-signed sum (a diagonal entry) loses about 6e-8 of its size per
// accumulated MMA, so the error grows with the MMAs per readout; one chunk
// per readout keeps it near 2e-7 of sum |q w| (measured 2.5e-7 with two).  A
// CTA's four row groups are summed in FP64 at the end and the per-CTA
// partials are added in a fixed order by k_gram_final (deterministic).
//
// Data path.  Each thread keeps two chunks of loads in flight (6 float4 per
// chunk: W rows, Wl rows and Q rows of 128 bytes), converts a chunk into the
// 128-byte-swizzled K-major layout of the UMMA shared-memory descriptor
// (8-row atoms of 1024 bytes, 16-byte granule g of row r at g ^ (r & 7)), one
// thread issues the four MMAs of the chunk and commits them to an mbarrier.
// Two stages alternate, so the conversion of chunk c overlaps the MMAs of
// chunk c - 1.  Waits on the mbarrier are bounded: a wait that gives up sets
// *err, and the CTA frees its TMEM and returns.
#pragma once
#include <cstdint>

namespace topo {

constexpr int GR_KC = 32;                           // values per chunk: one 128-byte row per vector
constexpr int GR_THREADS = 128;                     // warp w reads TMEM lanes 32w .. 32w + 31
constexpr int GR_RD = 1;                            // chunks accumulated in TMEM between readouts
constexpr int GR_A_BYTES = 128 * 128;               // A: 128 rows of 128 bytes
constexpr int GR_B_BYTES = 96 * 128;                // B: 96 rows of 128 bytes
constexpr int GR_STAGE = GR_A_BYTES + GR_B_BYTES;   // 28 KB, a multiple of the 1024-byte atom
constexpr int GR_SMEM = 2 * GR_STAGE + 1024 + 64;   // two stages, alignment slack, mbarrier and TMEM address
constexpr int GR_TMEM_COLS = 128;                   // D: 96 FP32 columns, allocated as a power of two
constexpr int GR_SPIN = 1 << 20;                    // bound on the polls of one mbarrier wait
// instruction descriptor of kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32
// (bits 7-9 and 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28
constexpr uint32_t GR_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((96u >> 3) << 17) | ((128u >> 4) << 24);

struct GramArgs {
    const float *Q, *Wh, *Wl;  // [kb][ld]
    long long ld;              // values per row, a multiple of GR_KC
    int kb;
    double *part;              // [gridDim.x][32][32]: sum_k W_i Q_j of each CTA
    int *err;                  // receives err_code when an mbarrier wait gave up
    int err_code;
};

__device__ __forceinline__ uint32_t gr_smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ float gr_rna(float v) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
    return __uint_as_float(r);
}

// shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading
// byte offset 1 (unused by swizzled K-major operands, bits 16-29), stride
// byte offset 1024 >> 4 between 8-row atoms (bits 32-45), descriptor version
// 1 (bits 46-47), 128-byte swizzle (layout 2, bits 61-63)
__device__ __forceinline__ uint64_t gr_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void gr_st(uint8_t *tile, int row, int g, float4 v) {
    *reinterpret_cast<float4 *>(tile + row * 128 + ((g ^ (row & 7)) << 4)) = v;
}

__device__ __forceinline__ void gr_split3(float v, float &h, float &m, float &l) {
    h = gr_rna(v);
    const float r = v - h;
    m = gr_rna(r);
    l = r - m;
}

__device__ __forceinline__ bool gr_wait(uint32_t mbar, uint32_t parity) {
    for (int i = 0; i < GR_SPIN; i++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void gr_tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

// loads of chunk c: t = 0, 1 rows of Wh; 2, 3 rows of Wl; 4, 5 rows of Q
// (thread tid, slot t: index tid + 128 t = 256 array + 8 row + granule)
__device__ __forceinline__ void gr_load(const GramArgs &A, long long c, long long c1, float4 (&v)[6]) {
#pragma unroll
    for (int t = 0; t < 6; t++) {
        const int idx = threadIdx.x + GR_THREADS * t, row = (idx >> 3) & 31, g = idx & 7;
        const float *arr = t < 2 ? A.Wh : (t < 4 ? A.Wl : A.Q);
        v[t] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (row < A.kb && c < c1)
            v[t] = __ldcs(reinterpret_cast<const float4 *>(arr + (size_t)row * A.ld + c * GR_KC + 4 * g));
    }
}

__device__ __forceinline__ void gr_store(const GramArgs &A, const float4 (&v)[6], uint8_t *stage) {
    uint8_t *ta = stage, *tb = stage + GR_A_BYTES;
#pragma unroll
    for (int t = 0; t < 6; t++) {
        const int idx = threadIdx.x + GR_THREADS * t, row = (idx >> 3) & 31, g = idx & 7;
        if (row >= A.kb) continue;
        const float4 x = v[t];
        if (t >= 2 && t < 4) {
            gr_st(ta, 96 + row, g, make_float4(gr_rna(x.x), gr_rna(x.y), gr_rna(x.z), gr_rna(x.w)));
        } else {
            float4 h, m, l;
            gr_split3(x.x, h.x, m.x, l.x);
            gr_split3(x.y, h.y, m.y, l.y);
            gr_split3(x.z, h.z, m.z, l.z);
            gr_split3(x.w, h.w, m.w, l.w);
            uint8_t *tile = t < 2 ? ta : tb;
            gr_st(tile, row, g, h);
            gr_st(tile, 32 + row, g, m);
            gr_st(tile, 64 + row, g, l);
        }
    }
}

// double-float accumulation of one TMEM readout: this thread's lane is A
// row 32 w + lane; columns j (Q.h), 32 + j (Q.m), 64 + j (Q.l)
__device__ __forceinline__ void gr_readout(uint32_t tmem, float (&hi)[32], float (&lo)[32]) {
    const uint32_t row = tmem + ((uint32_t)(32 * (threadIdx.x >> 5)) << 16);
#pragma unroll
    for (int j0 = 0; j0 < 32; j0 += 16) {
        uint32_t rh[16], rm[16], rl[16];
        gr_tmem_ld16(row + j0, rh);
        gr_tmem_ld16(row + 32 + j0, rm);
        gr_tmem_ld16(row + 64 + j0, rl);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const float b = __uint_as_float(rh[j]);
            const float s = hi[j0 + j] + b, bb = s - hi[j0 + j];
            const float e = (hi[j0 + j] - (s - bb)) + (b - bb);
            hi[j0 + j] = s;
            lo[j0 + j] += e + (__uint_as_float(rm[j]) + __uint_as_float(rl[j]));
        }
    }
}

static __global__ void __launch_bounds__(GR_THREADS, 2) k_gram_tc(const GramArgs A) {
    extern __shared__ uint8_t gr_raw[];
    uint8_t *base = gr_raw + ((1024u - (gr_smem_addr(gr_raw) & 1023u)) & 1023u);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(base + 2 * GR_STAGE);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(base + 2 * GR_STAGE + 8);
    int *abort_flag = reinterpret_cast<int *>(base + 2 * GR_STAGE + 16);
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t mb = gr_smem_addr(mbar);

    for (int i = tid; i < 2 * GR_STAGE / 16; i += GR_THREADS)
        reinterpret_cast<float4 *>(base)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(gr_smem_addr(tslot)),
                     "r"(GR_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    const long long nch = A.ld / GR_KC;
    const long long per = nch / gridDim.x, rem = nch % gridDim.x;
    const long long c0 = blockIdx.x * per + (blockIdx.x < rem ? blockIdx.x : rem);
    const long long c1 = c0 + per + (blockIdx.x < rem ? 1 : 0);

    float hi[32], lo[32];
#pragma unroll
    for (int j = 0; j < 32; j++) hi[j] = lo[j] = 0.f;
    float4 va[6], vb[6];
    gr_load(A, c0, c1, va);
    gr_load(A, c0 + 1, c1, vb);
    uint32_t parity = 0;
    bool failed = false;

    // one chunk: store, retire the previous chunk's MMAs (readout at the end
    // of a group), issue this chunk's MMAs, prefetch chunk c + 2
    auto step = [&](long long c, float4(&cur)[6]) {
        uint8_t *stage = base + (size_t)((c - c0) & 1) * GR_STAGE;
        gr_store(A, cur, stage);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (c > c0) {
            const bool ok = gr_wait(mb, parity);
            if (__syncthreads_or(!ok)) {
                failed = true;
                return;
            }
            parity ^= 1u;
            if ((c - c0) % GR_RD == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                gr_readout(tmem, hi, lo);
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = gr_smem_addr(stage);
            const uint64_t da = gr_desc(sa), db = gr_desc(sa + GR_A_BYTES);
            const bool first = (c - c0) % GR_RD == 0;
#pragma unroll
            for (int k = 0; k < GR_KC / 8; k++) {  // K = 8 TF32 values (32 bytes) per MMA
                const uint32_t accum = (first && k == 0) ? 0u : 1u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(da + (uint64_t)(2 * k)), "l"(db + (uint64_t)(2 * k)), "r"(GR_IDESC), "r"(accum)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                         : "memory");
        }
        gr_load(A, c + 2, c1, cur);
    };

    long long c = c0;
    for (; c + 1 < c1 && !failed; c += 2) {
        step(c, va);
        if (!failed) step(c + 1, vb);
    }
    if (c < c1 && !failed) step(c, va);
    if (c1 > c0 && !failed) {  // retire the last chunk
        const bool ok = gr_wait(mb, parity);
        if (__syncthreads_or(!ok)) {
            failed = true;
        } else {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            gr_readout(tmem, hi, lo);
        }
    }
    if (failed) {
        // an MMA may still be in flight: give it one more bounded wait before
        // the columns are freed, and report
        gr_wait(mb, parity);
        if (tid == 0) atomicExch(A.err, A.err_code);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(GR_TMEM_COLS)
                     : "memory");

    // the four row groups of slot i: sum in FP64 (stage memory is free now)
    double *red = reinterpret_cast<double *>(base);  // [4][32][32]
#pragma unroll
    for (int j = 0; j < 32; j++) red[(size_t)tid * 32 + j] = failed ? 0.0 : (double)hi[j] + (double)lo[j];
    __syncthreads();
    double *out = A.part + (size_t)blockIdx.x * 1024;
    for (int q = tid; q < 1024; q += GR_THREADS)
        out[q] = ((red[q] + red[1024 + q]) + red[2048 + q]) + red[3072 + q];
}

// out[a * kb + b] = sum over CTAs of part[cta][b][a]: Q_a . W_b
static __global__ void k_gram_final(int nblk, const double *__restrict__ part, int kb, double *out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= kb * kb) return;
    const int a = q / kb, b = q % kb;
    double s = 0.0;
    for (int k = 0; k < nblk; k++) s += part[(size_t)k * 1024 + b * 32 + a];
    out[q] = s;
}

// W = Wh + Wl of an FP64 vector, rows of the basis layout
static __global__ void k_split_f32(long long n, const double *__restrict__ w, float *wh, float *wl) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = w[i];
        const float h = (float)v;
        wh[i] = h;
        wl[i] = (float)(v - (double)h);
    }
}

}  // namespace topo
