// Split-precision complex64 form on the tcgen05 tensor cores, d = 64.
//
// Same polynomial and the same chunked running product as k_split_steps
// (split.cu): U_j = I + E_j with the reference's Chebyshev-Bessel polynomial
// regrouped by powers of X_j, each CTA multiplying its chunk of consecutive
// steps into E^P in double-float, the chunk products combined by the
// double-float tree (split.cu).  What changes is where the products run: every d^3 product is a
// sliced bf16 product on the tensor cores (ozaki.cuh) whose levels accumulate
// exactly in tensor memory.
//
//   * The polynomial terms are small: |mu_2 X^2| ~ (h ||X||)^2 and below.  X^2
//     and X Q take three slices per operand (24 bits, six slice products),
//     X^4 and X^6 two (three slice products).
//   * The running product E E^P carries the whole propagator and is where
//     FP32 rounding used to dominate the error (an emulation of the FP32
//     kernel attributes over 99 % of its error to this one product); it takes
//     four slices of each operand (ten slice products), exact to about 2^-29
//     of the row and column scales.  Three slices of E^P measured 1.4e-6 at
//     65536 steps, no better than FP32.
//
// The coefficients of the polynomial are real for even powers and imaginary
// for odd ones (mu_n = m_n / Hnorm^n, m_n from J_0 + 2 sum (-i)^k J_k T_k),
// so with Q = i N, N = sum nu_(2k+1) X^(2k), nu real, every update works on
// one real plane at a time: the accumulators of the real-stacked product put
// Re C in tensor-memory lanes 0..63 and Im C in lanes 64..127, and each thread
// keeps the plane of its own lane for 32 columns.  X Q = i X N comes from the
// same A slices of X as X^2 (kept in shared memory, row scales included) with
// the A blocks swapped (ozaki.cuh).  Only the first-order term mu_1 X =
// i nu_1 X couples the planes: X_j arrives in double-float (k_split_assemble
// forms it for every step) and each thread forms its plane of mu_1 X from the
// other plane there.
//
// When X_j is exactly Hermitian (Hermitian inputs and real control samples;
// k_split_assemble flags each step), so is the computed X^2 (exact integer
// level sums, symmetric scales), and the products X X, X^2 X^2 and
// X^(2k-2) X^2 take their B operand from the A slices of X or X^2:
// B^T = conj(A), copies of the [A_r] and [-A_i] blocks written as stacks
// along N while A is sliced (ozaki.cuh, herm_stacks), with the row scales as
// column scales.  The slices are the same numbers the B slicing would
// produce, so the result is bit-identical; such a step just skips the B
// slicing of X and X^2 with their column maxima, and forms E from the planes
// while the tensor core runs X^2.
//
// Layout of one CTA (512 threads, one per SM): shared memory holds the A
// slices (4 x 24 KB), the B slices (4 x 16 KB) and a third buffer (2 x 24 KB)
// for the A slices of X^4, X^6 (Hermitian steps: of X^2) and then the B
// slices of N; at the start of a step the B and third buffers receive the
// planes that hand X_j to the lane layout (Hermitian steps put the A slices
// of X^4, X^6 in the B buffer).  Tensor memory holds the product levels (columns 0..255), E^P in
// double-float (256..383) and E of the current step (384..511) while the
// polynomial products run.  Sixteen warps hide the latency of the elementwise
// work (slicing, epilogues) that surrounds each product; each thread owns one
// plane of 16 columns of one row.  While the tensor core runs X Q, the threads
// slice E^P, the B operand of the running product.  Every wait on the tensor core is bounded: a wait that
// runs out stops the CTA, adds one to the calling context's fault counter and
// frees tensor memory.
#include <math.h>
#include <stdlib.h>

#include <algorithm>

#include "ctx.h"
#include "kernels.h"
#include "ozaki.cuh"
#include "split_common.cuh"
#include "tc_slice.cuh"

namespace pgb {

constexpr int kTcdMaxKe = 64;
// Slices per operand.  X^2 and X Q carry terms up to (h ||X||)^2 and need
// three slices (24 bits); X^4, X^6 are two orders smaller and take two; the
// running product takes four slices of each operand.
constexpr int kTcdHi = 4;
constexpr int kTcdX2 = 3;
constexpr int kTcdG = 2;
constexpr size_t kTcdSA = (size_t)kTcdHi * oz::kASlice;
constexpr size_t kTcdSB = (size_t)kTcdHi * oz::kBSlice;
// A third slice buffer takes the A slices of X^4, X^6 (two each) and then the
// B slices of N (three), so that the A slices of X from the X^2 product stay
// for the odd part X Q and the B buffer is free for E^P while X Q runs.
constexpr size_t kTcdSG = (size_t)kTcdG * oz::kASlice;
constexpr size_t kTcdSmem = kTcdSA + kTcdSB + kTcdSG + 1024;
// Hermitian steps also keep the B^T blocks of X (three slices) and of X^2
// (two) as stacks that the tensor core reads along N: the [A_r] stack in the
// tail of the A slice buffer (free while the polynomial runs), the [-A_i]
// stack in the tail of the B slice buffer, past the lo planes of X (during
// X^2) and past the A slices of X^4, X^6 (during those products).
constexpr uint32_t kTcdStk0 = (uint32_t)kTcdX2 * oz::kASlice;  // in SA
constexpr uint32_t kTcdStkX1 = 40960;                           // in SB
constexpr uint32_t kTcdStkG1 = (uint32_t)kTcdG * oz::kASlice;   // in SB
static_assert(kTcdStk0 + kTcdX2 * oz::kBlk <= kTcdSA, "[A_r] stack of X exceeds the A slice buffer");
static_assert(kTcdStkX1 + kTcdX2 * oz::kBlk <= kTcdSB, "[-A_i] stack of X exceeds the B slice buffer");
static_assert(kTcdStkG1 + kTcdG * oz::kBlk <= kTcdSB, "[-A_i] stack of X^2 exceeds the B slice buffer");
// X_j reaches the lane layout through four planes (re hi, im hi, re lo, im
// lo) of 64 rows padded to 68 floats (conflict-free 16-byte reads of a column
// block by 32 consecutive rows).  k_split_assemble writes them for every step
// in that layout.  The hi pair and the lo pair travel by separate bulk copies
// of kTcdPairBytes each: the hi pair into the third slice buffer, free from
// the end of a step's X Q product to the next step's X^2 epilogue (a whole
// step ahead), the lo pair into the B slice buffer, free from the end of the
// running product to the next step's X^2 slicing.
constexpr int kTcdPlaneLd = 68;
constexpr int kTcdPlane = 64 * kTcdPlaneLd;
constexpr uint32_t kTcdPairBytes = 2 * kTcdPlane * sizeof(float);
static_assert(kTcdPairBytes <= kTcdSG && kTcdPairBytes <= kTcdSB && kTcdPairBytes % 16 == 0,
              "plane pairs exceed their slice buffers");
static_assert(kTcdPairBytes <= kTcdStkX1, "the [-A_i] stack of X overlaps the lo planes");
// Float index, within the planes of a step, of the flag that k_split_assemble
// leaves in the row padding (plane 0, row 0, column 64): nonzero when X_j is
// exactly Hermitian (Hermitian inputs, anti-Hermitian commutators, real
// control weights and imaginary commutator weights).
constexpr int kTcdHermFlag = 64;
static_assert(kTcdPlane * 4 == kSplitXStride, "plane layout of k_split_assemble");

// Bounded waits that gave up, for launches without a context's counter.
__device__ int g_split_tc_faults;

// The running product's four levels combined in double-float and added, with
// E, to E^P (tensor memory): E^P <- E^P + E + 2^(e_r - 7) 2^(e_c - 7) sum_L 2^(-8 L) D_L.
__device__ __forceinline__ void epilogue_running(const TcdShared &sh, const TcdThread &t, const float (&eh)[16],
                                                 const float (&el)[16]) {
    const float rm = sh.rowmul[t.r];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        float d0[8], d1[8], d2[8], d3[8], ph[8], pl[8];
        tmem_ld8_nowait(t.tm_acc + 8 * h, d0);
        tmem_ld8_nowait(t.tm_acc + 64 + 8 * h, d1);
        tmem_ld8_nowait(t.tm_acc + 128 + 8 * h, d2);
        tmem_ld8_nowait(t.tm_acc + 192 + 8 * h, d3);
        tmem_ld8_nowait(t.tm_ep + 8 * h, ph);
        tmem_ld8_nowait(t.tm_ep + 16 + 8 * h, pl);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            float s, e;
            two_sum(d0[j], d1[j] * 0.00390625f, s, e);
            e = __fadd_rn(e, __fmaf_rn(d3[j], 5.9604644775390625e-8f, d2[j] * 1.52587890625e-5f));
            df v = df_norm(s, e);
            const float sc = rm * sh.colmul_p[t.c0 + 8 * h + j];
            v.hi *= sc;
            v.lo *= sc;
            df w = df_add(df{ph[j], pl[j]}, df{eh[8 * h + j], el[8 * h + j]});
            w = df_add(w, v);
            ph[j] = w.hi;
            pl[j] = w.lo;
        }
        uint32_t rh[8], rl[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            rh[j] = __float_as_uint(ph[j]);
            rl[j] = __float_as_uint(pl[j]);
        }
        asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(t.tm_ep + 8 * h),
                     "r"(rh[0]), "r"(rh[1]), "r"(rh[2]), "r"(rh[3]), "r"(rh[4]), "r"(rh[5]), "r"(rh[6]), "r"(rh[7])
                     : "memory");
        asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(
                         t.tm_ep + 16 + 8 * h),
                     "r"(rl[0]), "r"(rl[1]), "r"(rl[2]), "r"(rl[3]), "r"(rl[4]), "r"(rl[5]), "r"(rl[6]), "r"(rl[7])
                     : "memory");
    }
    tc::tmem_wait_st();
}

// (c_r, c_i) += w (h_r, h_i) with one paired FMA (each half rounds as fmaf).
__device__ __forceinline__ void fma2(float &cr, float &ci, float w, float hr, float hi) {
    asm("{\n\t"
        ".reg .b64 C, W, H;\n\t"
        "mov.b64 C, {%0, %1};\n\t"
        "mov.b64 W, {%2, %2};\n\t"
        "mov.b64 H, {%3, %4};\n\t"
        "fma.rn.f32x2 C, W, H, C;\n\t"
        "mov.b64 {%0, %1}, C;\n\t"
        "}"
        : "+f"(cr), "+f"(ci)
        : "f"(w), "f"(hr), "f"(hi));
}

// acc += w h for a double-float real w and a float h; the compensation term
// collects the rounding of the sum and the product without renormalising.
__device__ __forceinline__ void df_mac_lazy(float &hi, float &lo, float wh, float wl, float h) {
    const float p = __fmul_rn(wh, h);
    float e = __fmaf_rn(wh, h, -p);
    e = __fmaf_rn(wl, h, e);
    float s, t;
    two_sum(hi, p, s, t);
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(t, e));
}

// The same on two values at once with the paired FP32 instructions of
// sm_100-family GPUs (add/mul/fma.rn.f32x2: each half rounds exactly as the
// scalar instruction): (hi, lo)[k] += w h[k], k = 0, 1 (the real and
// imaginary parts of one element, which share the weight).
__device__ __forceinline__ void df_mac_lazy2(float &hi0, float &hi1, float &lo0, float &lo1, float wh, float wl,
                                             float h0, float h1) {
    asm("{\n\t"
        ".reg .b64 H, L, W, N, V, X, P, E, S, B, T, U;\n\t"
        "mov.b64 H, {%0, %1};\n\t"
        "mov.b64 L, {%2, %3};\n\t"
        "mov.b64 W, {%4, %4};\n\t"
        "mov.b64 N, {%8, %8};\n\t"
        "mov.b64 V, {%5, %5};\n\t"
        "mov.b64 X, {%6, %7};\n\t"
        "mul.rn.f32x2 P, W, X;\n\t"       // p = wh h
        "mul.rn.f32x2 E, N, X;\n\t"       // -p
        "fma.rn.f32x2 E, W, X, E;\n\t"    // e = wh h - p (exact)
        "fma.rn.f32x2 E, V, X, E;\n\t"    // e += wl h
        "add.rn.f32x2 S, H, P;\n\t"       // two_sum(hi, p): s
        "sub.rn.f32x2 B, S, H;\n\t"       // bb = s - hi
        "sub.rn.f32x2 T, S, B;\n\t"
        "sub.rn.f32x2 T, H, T;\n\t"       // hi - (s - bb)
        "sub.rn.f32x2 U, P, B;\n\t"       // p - bb
        "add.rn.f32x2 T, T, U;\n\t"       // t
        "add.rn.f32x2 T, T, E;\n\t"
        "add.rn.f32x2 L, L, T;\n\t"       // lo += t + e
        "mov.b64 {%0, %1}, S;\n\t"
        "mov.b64 {%2, %3}, L;\n\t"
        "}"
        : "+f"(hi0), "+f"(hi1), "+f"(lo0), "+f"(lo1)
        : "f"(wh), "f"(wl), "f"(h0), "f"(h1), "f"(-wh));
}

__global__ void __launch_bounds__(kTcdThreads, 1) k_split_tc(const __grid_constant__ SplitArgs a) {
    extern __shared__ unsigned char smem_raw[];
    // 1024-byte alignment by pointer arithmetic on the shared array, so that the
    // compiler keeps every access derived from it in the shared state space.
    unsigned char *smem = smem_raw + ((1024u - (tc::smem_addr(smem_raw) & 1023u)) & 1023u);
    unsigned char *SA = smem;
    unsigned char *SB = smem + kTcdSA;
    unsigned char *SG = SB + kTcdSB;
    __shared__ TcdShared sh;

    const int warp = threadIdx.x >> 5;
    TcdThread t;
    t.tid = threadIdx.x;
    t.lane = threadIdx.x & 31;
    const int q4 = warp & 3;
    t.cb = warp >> 2;
    t.p = q4 >> 1;
    t.r = 32 * (q4 & 1) + t.lane;
    t.c0 = kTcdCols * t.cb;
    const long long s0 = a.P * blockIdx.x / a.nchunks;
    const long long s1 = a.P * (blockIdx.x + 1) / a.nchunks;
    const int M = a.M;

    if (warp == 0) {
        tc::tmem_alloc(&sh.tmem_base, 512);
        tc::tmem_relinquish();
    }
    if (t.tid == 0) {
        tc::mbar_init(&sh.bar, 1);
        tc::mbar_init(&sh.hbar, 1);
        tc::mbar_init(&sh.lbar, 1);
        tc::fence_mbar_init();
    }
    if (t.tid < 64) {
        sh.amax[0][t.tid] = sh.amax[1][t.tid] = 0;
        sh.bmax[0][t.tid] = sh.bmax[1][t.tid] = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t lane_base = (uint32_t)(32 * q4) << 16;
    t.tm_acc = sh.tmem_base + lane_base + (uint32_t)t.c0;
    t.tm_ep = sh.tmem_base + lane_base + 256u + 32u * (uint32_t)t.cb;
    t.tm_e = sh.tmem_base + lane_base + 384u + 32u * (uint32_t)t.cb;

    // Coefficients: c0 = m_0 - 1 and even mu real, odd mu = i nu.
    const df nu1 = df_from(a.mu[1].y);
    const df mu2 = df_from(a.mu[2].x);
    const df c0d = df_from(a.c0.x);

    uint32_t ncommit = 0;
    int nb = 0;  // max-buffer parity
    bool ok = true;
    // The X planes of step st reach shared memory by two bulk copies: the hi
    // pair (what a step reads first) into the third slice buffer SG as soon as
    // the previous step's X Q product is done with it, the lo pair into the B
    // slice buffer SB once the previous step's running product is.
    uint32_t hphase = 0, hissued = 0, lphase = 0, lissued = 0;  // copies waited for / issued (same in every thread)
    auto issue_hi = [&](long long st) {
        ++hissued;
        if (t.tid == 0) {
            mbar_expect_tx(&sh.hbar, kTcdPairBytes);
            bulk_g2s(SG, a.xplanes + (size_t)st * kSplitXStride, kTcdPairBytes, &sh.hbar);
        }
    };
    auto issue_lo = [&](long long st) {
        ++lissued;
        if (t.tid == 0) {
            mbar_expect_tx(&sh.lbar, kTcdPairBytes);
            bulk_g2s(SB, a.xplanes + (size_t)st * kSplitXStride + 2 * kTcdPlane, kTcdPairBytes, &sh.lbar);
        }
    };
    const float *XH = reinterpret_cast<const float *>(SG);
    const float *XL = reinterpret_cast<const float *>(SB);
    // E = c0 I + i nu_1 X in this thread's plane (E_re = c0 d - nu_1 X_im,
    // E_im = nu_1 X_re), from the other plane's double-float X; E waits in
    // tensor memory while the polynomial products run.
    auto form_e = [&]() {
        ok = tc::mbar_wait(&sh.lbar, lphase & 1, kTcdWait) && ok;
        ++lphase;
        float Eh[16], El[16];
        const float4 *oh = reinterpret_cast<const float4 *>(XH + (1 - t.p) * kTcdPlane + t.r * kTcdPlaneLd + t.c0);
        const float4 *ol = reinterpret_cast<const float4 *>(XL + (1 - t.p) * kTcdPlane + t.r * kTcdPlaneLd + t.c0);
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            const float4 h = oh[g], l = ol[g];
            const float hs[4] = {h.x, h.y, h.z, h.w}, ls[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int j = 4 * g + i;
                df e = df_mul(nu1, df{hs[i], ls[i]});
                if (t.p == 0) {
                    e = df_neg(e);
                    if (t.c0 + j == t.r) e = df_add(e, c0d);
                }
                Eh[j] = e.hi;
                El[j] = e.lo;
            }
        }
        store_ep(t.tm_e, Eh, El);
    };
    if (s1 > s0) {
        issue_hi(s0);
        issue_lo(s0);
    }
    for (long long st = s0; st < s1; ++st) {
        ok = tc::mbar_wait(&sh.hbar, hphase & 1, kTcdWait) && ok;
        ++hphase;
        // Hermitian step (flag in the planes' row padding, k_split_assemble):
        // the products of X and X^2 take their B operands from the A slices,
        // and E is formed while the tensor core runs X^2.
        const bool herm = XH[kTcdHermFlag] != 0.0f;
        float X[16];
        {
            const float4 *own = reinterpret_cast<const float4 *>(XH + t.p * kTcdPlane + t.r * kTcdPlaneLd + t.c0);
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                const float4 x = own[g];
                X[4 * g] = x.x;
                X[4 * g + 1] = x.y;
                X[4 * g + 2] = x.z;
                X[4 * g + 3] = x.w;
            }
        }
        // ---- X^2
        if (herm) {
            reduce_max<true, false>(sh, t, nb, X, X);
            store_a<kTcdX2, false, true, true>(sh, SA, t, nb, X, X, SA + kTcdStk0, SB + kTcdStkX1);
            nb ^= 1;
            if (!issue_sliced(sh, t, SA, SA + kTcdStk0, kTcdX2, kTcdX2, kTcdX2 - 1, false, ok,
                              oz::herm_stacks((uint32_t)kTcdSA - kTcdStk0 + kTcdStkX1)))
                break;
            form_e();
            wait_sliced(sh, ncommit, ok);
        } else {
            form_e();  // before the B slices of X overwrite the planes
            reduce_max<true, true>(sh, t, nb, X, X);
            store_a<kTcdX2, false>(sh, SA, t, nb, X, X);
            store_b<kTcdX2, false>(SB, t, sh.bmax[nb], X, X, sh.colmul);
            nb ^= 1;
            if (!run_product(sh, t, SA, SB, kTcdX2, kTcdX2, kTcdX2 - 1, false, ncommit, ok)) break;
        }
        if (t.tid < 64) sh.rowmul_x[t.tid] = sh.rowmul[t.tid];
        float N[16], G[16];
        epilogue_f<kTcdX2 - 1>(sh, t, G);
        {
            const float nu3 = (float)a.mu[3].y;
            float Eh[16], El[16];
            load_ep(t.tm_e, Eh, El);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const df v = df_add(df{Eh[j], El[j]}, df_mul_f(mu2, G[j]));
                Eh[j] = v.hi;
                El[j] = v.lo;
                N[j] = nu3 * G[j];
            }
            store_ep(t.tm_e, Eh, El);
        }
        // ---- higher even powers X^(2k) = X^(2k-2) X^2.  Their terms mu_(2k) X^(2k)
        // are of order (h ||X||)^4 and below: they collect in FP32 (Se) and
        // reach E together with the odd part.  Hermitian steps keep the A
        // slices of X^2 in SG (they are also the B operand of every X^(2k)
        // product) and put those of X^(2k-2), k > 2, in SB.
        float Se[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) Se[j] = 0.0f;
        bool live = true;
        for (int k = 2; 2 * k <= M; ++k) {
            if (herm) {
                reduce_max<true, false>(sh, t, nb, G, G);
                unsigned char *dst = k == 2 ? SG : SB;
                if (k == 2)
                    store_a<kTcdG, false, true, true>(sh, dst, t, nb, G, G, SA + kTcdStk0, SB + kTcdStkG1);
                else
                    store_a<kTcdG, false>(sh, dst, t, nb, G, G);
                nb ^= 1;
                if (!(live = run_product(sh, t, dst, SA + kTcdStk0, kTcdG, kTcdG, kTcdG - 1, false, ncommit, ok,
                                         oz::herm_stacks((uint32_t)kTcdSA - kTcdStk0 + kTcdStkG1))))
                    break;
            } else {
                if (k == 2)
                    reduce_max<true, true>(sh, t, nb, G, G);
                else
                    reduce_max<true, false>(sh, t, nb, G, G);
                store_a<kTcdG, false>(sh, SG, t, nb, G, G);
                if (k == 2) store_b<kTcdG, false>(SB, t, sh.bmax[nb], G, G, sh.colmul);
                nb ^= 1;
                if (!(live = run_product(sh, t, SG, SB, kTcdG, kTcdG, kTcdG - 1, false, ncommit, ok))) break;
            }
            epilogue_f<kTcdG - 1>(sh, t, G);
            const float me = (float)a.mu[2 * k].x;
            const float no = (2 * k + 1 <= M) ? (float)a.mu[2 * k + 1].y : 0.0f;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                Se[j] = fmaf(me, G[j], Se[j]);
                N[j] = fmaf(no, G[j], N[j]);
            }
        }
        if (!live) break;
        // ---- odd part X Q = i X N: the A slices of X are still in SA; the B
        // slices of N go to SG (free after the last even power).  N is sliced
        // with its own column maxima on every step: X^6 = X^4 X^2 from
        // truncated slices is Hermitian only to their precision, and so is N.
        reduce_max<false, true>(sh, t, nb, X, N);
        if (t.tid < 64) sh.rowmul[t.tid] = sh.rowmul_x[t.tid];
        store_b<kTcdX2, false>(SG, t, sh.bmax[nb], N, N, sh.colmul);
        nb ^= 1;
        if (!issue_sliced(sh, t, SA, SG, kTcdX2, kTcdX2, kTcdX2 - 1, true, ok)) break;
        if (st > s0) {
            // While the tensor core runs X Q: the B operand of the running
            // product, E^P of the previous steps, sliced into SB (its column
            // scales in colmul_p, apart from those of N).
            float Ph[16], Pl[16];
            load_ep(t.tm_ep, Ph, Pl);
            reduce_max<false, true>(sh, t, nb, Ph, Ph);
            store_b<kTcdHi, true>(SB, t, sh.bmax[nb], Ph, Pl, sh.colmul_p);
        }
        wait_sliced(sh, ncommit, ok);
        if (st + 1 < s1) issue_hi(st + 1);  // SG is free again
        epilogue_f<kTcdX2 - 1>(sh, t, G);
        float Eh[16], El[16];
        load_ep(t.tm_e, Eh, El);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const df v = df_add_f(df_add_f(df{Eh[j], El[j]}, G[j]), Se[j]);
            Eh[j] = v.hi;
            El[j] = v.lo;
        }
        // ---- running product E^P <- E^P + E + E E^P
        if (st == s0) {
            if (st + 1 < s1) issue_lo(st + 1);  // SB is free again
            store_ep(t.tm_ep, Eh, El);
        } else {
            reduce_max<true, false>(sh, t, nb, Eh, Eh);
            store_a<kTcdHi, true>(sh, SA, t, nb, Eh, El);
            nb ^= 1;
            if (!run_product(sh, t, SA, SB, kTcdHi, kTcdHi, kTcdHi - 1, false, ncommit, ok)) break;
            if (st + 1 < s1) issue_lo(st + 1);  // SB is free again
            epilogue_running(sh, t, Eh, El);
        }
    }
    // The last product's wait, combined over the CTA.
    ok = __syncthreads_and(ok) != 0;
    if (ok && s1 > s0) {
        // Chunk product I + E^P in complex128: plane p of row r, 16 columns.
        float Ph[16], Pl[16];
        load_ep(t.tm_ep, Ph, Pl);
        double *dst = reinterpret_cast<double *>(a.chunks + (size_t)blockIdx.x * 4096);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int c = t.c0 + j;
            double v = (double)Ph[j] + (double)Pl[j];
            if (t.p == 0 && c == t.r) v += 1.0;
            dst[2 * (t.r * 64 + c) + t.p] = v;
        }
    }
    if (!ok) {
        if (t.tid == 0) atomicAdd(a.fault ? a.fault : &g_split_tc_faults, 1);
        // Let any product or copy still in flight finish before tensor memory
        // and shared memory are released.
        if (ncommit > 0) tc::mbar_wait(&sh.bar, (ncommit - 1) & 1, kTcdWait);
    }
    for (; hphase < hissued; ++hphase) tc::mbar_wait(&sh.hbar, hphase & 1, kTcdWait);
    for (; lphase < lissued; ++lphase) tc::mbar_wait(&sh.lbar, lphase & 1, kTcdWait);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(sh.tmem_base, 512);
    }
}

// X_j of steps s_off .. s_off + n - 1 of the split form, in double-float, for
// the tensor-core step kernel: X_j = H_0 + sum_m w_jm H_m with the weights of
// k_split_weights.  Thread f of the CTA row blockIdx.x owns float4 f of every
// expansion matrix (complex elements 2f, 2f + 1), keeps that slice of the
// stack in registers (RK > 0: up to RK + 1 matrices, loops unrolled) or in
// shared memory (RK = 0), stages the weights of the CTA's kAsmSteps steps
// blockIdx.y kAsmSteps, ... in shared memory and walks those steps.  Each
// element takes the same operations in the same order as an assembly inside
// the step kernel would (real weights: paired double-float multiply-add;
// complex weights: complex double-float; commutator slots: FP32 sums added at
// the end).  Output: four planes (re hi, im hi, re lo, im lo) of 64 rows x 68
// floats per step, kSplitXStride floats apart.
constexpr int kAsmSteps = 32;
// Shared memory of k_split_assemble at the largest Ke: its stack slice and the
// weights of its steps.
static_assert(sizeof(float4) * (128 * (kTcdMaxKe + 1) + kAsmSteps * kTcdMaxKe) + 16 <= 232448,
              "k_split_assemble exceeds 227 KB of shared memory");
constexpr int kAsmRegKe = 15;  // largest Ke with the stack slice in registers

template <int RK>
__global__ void __launch_bounds__(128) k_split_assemble(const __grid_constant__ SplitArgs a, float *xp,
                                                        long long s_off, long long n) {
    extern __shared__ float4 hs[];  // RK = 0: (1 + Ke) x 128 float4 of the stack; then kAsmSteps x Ke weights
    const int Ke = RK > 0 ? min(a.Ke, RK) : a.Ke;
    float4 *wsa = hs + (RK > 0 ? 0 : (Ke + 1) * 128);
    const int f = blockIdx.x * 128 + threadIdx.x;
    const long long sb = (long long)blockIdx.y * kAsmSteps;
    const int ns = (int)(n - sb < kAsmSteps ? n - sb : kAsmSteps);
    const float4 *stack4 = reinterpret_cast<const float4 *>(a.stack);
    float4 hr[RK + 1];
    if constexpr (RK > 0) {
#pragma unroll
        for (int m = 0; m <= RK; ++m) hr[m] = m <= Ke ? stack4[(size_t)m * 2048 + f] : make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        for (int m = 0; m <= Ke; ++m) hs[m * 128 + threadIdx.x] = stack4[(size_t)m * 2048 + f];
    }
    // Per step: does any weight leave the usual pattern (real control
    // weights, imaginary commutator weights)?  Steps that keep it take the
    // branch-free loops below.
    __shared__ int odd_step[kAsmSteps];
    if (threadIdx.x < kAsmSteps) odd_step[threadIdx.x] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < ns * Ke; i += 128) {
        const float4 w = a.wts[(size_t)(s_off + sb) * Ke + i];
        wsa[i] = w;
        const int m = i % Ke;
        if (m < a.K ? (w.z != 0.0f || w.w != 0.0f) : (w.x != 0.0f || w.y != 0.0f)) odd_step[i / Ke] = 1;
    }
    __syncthreads();
    const int row = f >> 5, col = 2 * (f & 31);
    for (int k = 0; k < ns; ++k) {
        const long long s = sb + k;
        const float4 *ws = wsa + k * Ke;
        float4 h0;
        if constexpr (RK > 0) h0 = hr[0]; else h0 = hs[threadIdx.x];
        float xrh[2] = {h0.x, h0.z}, xih[2] = {h0.y, h0.w};
        float xrl[2] = {0.f, 0.f}, xil[2] = {0.f, 0.f}, sr[2] = {0.f, 0.f}, si[2] = {0.f, 0.f};
        if (!odd_step[k]) {
            // Real control weights: paired double-float multiply-adds.
#pragma unroll
            for (int m = 0; m < (RK > 0 ? RK : 1 << 30); ++m) {
                if (m >= a.K || m >= Ke) break;
                float4 v;
                if constexpr (RK > 0) v = hr[m + 1]; else v = hs[(m + 1) * 128 + threadIdx.x];
                const float4 w = ws[m];
                df_mac_lazy2(xrh[0], xih[0], xrl[0], xil[0], w.x, w.y, v.x, v.y);
                df_mac_lazy2(xrh[1], xih[1], xrl[1], xil[1], w.x, w.y, v.z, v.w);
            }
            // Imaginary commutator weights i v: w h = -v h_i + i v h_r, summed
            // as c += v h with paired FMAs (sr = -Im c, si = Re c: the same
            // roundings as the scalar sums of the general branch).
            float c0r = 0.f, c0i = 0.f, c1r = 0.f, c1i = 0.f;
#pragma unroll
            for (int m = 0; m < (RK > 0 ? RK : 1 << 30); ++m) {
                if (m >= Ke) break;
                if (m < a.K) continue;
                float4 v;
                if constexpr (RK > 0) v = hr[m + 1]; else v = hs[(m + 1) * 128 + threadIdx.x];
                const float wz = ws[m].z;
                fma2(c0r, c0i, wz, v.x, v.y);
                fma2(c1r, c1i, wz, v.z, v.w);
            }
            sr[0] = -c0i;
            si[0] = c0r;
            sr[1] = -c1i;
            si[1] = c1r;
        } else
#pragma unroll
        for (int m = 0; m < (RK > 0 ? RK : 1 << 30); ++m) {
            if (m >= Ke) break;
            float4 v;
            if constexpr (RK > 0) v = hr[m + 1]; else v = hs[(m + 1) * 128 + threadIdx.x];
            const float gr[2] = {v.x, v.z}, gi[2] = {v.y, v.w};
            const float4 w = ws[m];
            // The branches depend on the slot's weight only: uniform over the CTA.
            if (m < a.K) {
                if (w.z == 0.0f && w.w == 0.0f) {  // real weight (real control samples)
#pragma unroll
                    for (int j = 0; j < 2; ++j) df_mac_lazy2(xrh[j], xih[j], xrl[j], xil[j], w.x, w.y, gr[j], gi[j]);
                } else {
                    const cdf wd = {{w.x, w.y}, {w.z, w.w}};
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        const cdf x = cdf_add(cdf{df_norm(xrh[j], xrl[j]), df_norm(xih[j], xil[j])},
                                              cdf_mul_c(wd, make_float2(gr[j], gi[j])));
                        xrh[j] = x.re.hi;
                        xrl[j] = x.re.lo;
                        xih[j] = x.im.hi;
                        xil[j] = x.im.lo;
                    }
                }
            } else if (w.x == 0.0f) {
                // commutator slot with an imaginary weight i v: w h = -v h_i + i v h_r
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    sr[j] = fmaf(-w.z, gi[j], sr[j]);
                    si[j] = fmaf(w.z, gr[j], si[j]);
                }
            } else {
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    sr[j] = fmaf(w.x, gr[j], fmaf(-w.z, gi[j], sr[j]));
                    si[j] = fmaf(w.x, gi[j], fmaf(w.z, gr[j], si[j]));
                }
            }
        }
        const df r0 = df_add_f(df_norm(xrh[0], xrl[0]), sr[0]);
        const df r1 = df_add_f(df_norm(xrh[1], xrl[1]), sr[1]);
        const df i0 = df_add_f(df_norm(xih[0], xil[0]), si[0]);
        const df i1 = df_add_f(df_norm(xih[1], xil[1]), si[1]);
        float *o = xp + (size_t)s * kSplitXStride + row * kTcdPlaneLd + col;
        *reinterpret_cast<float2 *>(o) = make_float2(r0.hi, r1.hi);
        *reinterpret_cast<float2 *>(o + kTcdPlane) = make_float2(i0.hi, i1.hi);
        *reinterpret_cast<float2 *>(o + 2 * kTcdPlane) = make_float2(r0.lo, r1.lo);
        *reinterpret_cast<float2 *>(o + 3 * kTcdPlane) = make_float2(i0.lo, i1.lo);
        if (col == 62) {
            // The row padding too, so that every 32-byte sector of the planes
            // is written whole (no read of a partly written sector); row 0 of
            // plane 0 carries the step's Hermitian flag.
            float flag = 0.0f;
            if (row == 0 && a.herm_stack) {
                bool herm = true;
                for (int m = 0; m < Ke; ++m) {
                    const float4 w = ws[m];
                    herm = herm && (m < a.K ? (w.z == 0.0f && w.w == 0.0f) : (w.x == 0.0f && w.y == 0.0f));
                }
                flag = herm ? 1.0f : 0.0f;
            }
#pragma unroll
            for (int pl = 0; pl < 4; ++pl)
                *reinterpret_cast<float4 *>(o + pl * kTcdPlane + 2) =
                    make_float4(pl == 0 ? flag : 0.f, 0.f, 0.f, 0.f);
        }
    }
}

// Step weights of the split form in double-float for all steps (the step
// kernel reads them one step ahead): weight m of step s at wts[s Ke + m].
__global__ void k_split_weights(const __grid_constant__ SplitArgs a, float4 *wts) {
    const long long n = a.P * a.Ke;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long st = i / a.Ke;
        const int m = (int)(i - st * a.Ke);
        const double2 w = split_weight(a, m, st);
        const df re = df_from(w.x), im = df_from(w.y);
        wts[i] = make_float4(re.hi, re.lo, im.hi, im.lo);
    }
}

static bool split_tc_disabled() {
    static const bool off = [] {
        const char *v = getenv("PARAMENT_DISABLE_TENSOR_CORES");
        return v && v[0] && v[0] != '0';
    }();
    return off;
}

bool split_tc_applies(int d, int Ke, int M) {
    return d == 64 && Ke <= kTcdMaxKe && M >= 3 && M <= kSplitMaxOrder && !split_tc_disabled();
}

cudaError_t launch_split_tc(const SplitArgs &a, int num_sms, float *xplanes, int *nchunks, cudaStream_t stream,
                            cudaEvent_t ev0, cudaEvent_t ev1) {
    cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void *>(&k_split_tc),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcdSmem);
    if (e != cudaSuccess) return e;
    // The stack slice of an assemble thread sits in registers up to Ke = kAsmRegKe.
    const bool asm_reg = a.Ke <= kAsmRegKe;
    const void *asm_fn = asm_reg ? reinterpret_cast<const void *>(&k_split_assemble<kAsmRegKe>)
                                 : reinterpret_cast<const void *>(&k_split_assemble<0>);
    const size_t hs_bytes = sizeof(float4) * ((asm_reg ? 0 : 128 * (size_t)(a.Ke + 1)) + (size_t)kAsmSteps * a.Ke) + 16;
    e = cudaFuncSetAttribute(asm_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hs_bytes);
    if (e != cudaSuccess) return e;
    if (a.Ke > 0) {
        const long long n = a.P * a.Ke;
        const int blocks = (int)std::min<long long>((n + 255) / 256, 8L * num_sms);
        k_split_weights<<<blocks, 256, 0, stream>>>(a, const_cast<float4 *>(a.wts));
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    // Batches of up to kSplitXBatch steps: the X planes of the batch, then the
    // step kernel over it; the chunks of successive batches follow each other.
    int total = 0;
    for (long long b0 = 0; b0 < a.P; b0 += kSplitXBatch) {
        const long long nb = std::min<long long>(kSplitXBatch, a.P - b0);
        const int gy = (int)((nb + kAsmSteps - 1) / kAsmSteps);
        long long off = b0, cnt = nb;
        void *args[] = {const_cast<SplitArgs *>(&a), &xplanes, &off, &cnt};
        e = cudaLaunchKernel(asm_fn, dim3(16, gy), dim3(128), args, hs_bytes, stream);
        if (e != cudaSuccess) return e;
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        SplitArgs b = a;
        b.P = nb;
        b.xplanes = xplanes;
        b.nchunks = (int)std::max<long long>(1, std::min<long long>((long long)num_sms, nb));
        b.chunks = a.chunks + (size_t)total * 4096;
        if (ev0 && b0 == 0) cudaEventRecord(ev0, stream);
        k_split_tc<<<b.nchunks, kTcdThreads, kTcdSmem, stream>>>(b);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        total += b.nchunks;
    }
    if (ev1) cudaEventRecord(ev1, stream);
    *nchunks = total;
    return cudaSuccess;
}

}  // namespace pgb
