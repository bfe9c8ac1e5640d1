// Plain complex64 form at d = 64 on the tcgen05 tensor cores.
//
// The reference's scheme in complex64 arithmetic, as k_small_steps<float>
// (step_small.cu) runs it on the FP32 pipe: X_j = H_0 + sum_m w_jm H_m with the
// complex64 step weights, the Clenshaw recurrence
//     b_M = J_M I,  b_(M-1) = s J_M X + J_(M-1) I,
//     b_k = s X b_(k+1) + beta_k b_(k+2) + J_k I   (beta = -1, and -2 at k = 0),
// U_j = b_0 (src/cuda/parament.cpp:569-652, src/cuda/diagonal_add.cu:21-51),
// and the running product of a chunk of consecutive steps as P + (U_j - I) P
// (the lower levels of the tree, src/cuda/parament.cpp:657-718).  The d^3
// products run on the tensor cores as exact sliced bf16 products (ozaki.cuh):
// four 8-bit slices per operand, levels s + t <= 3 accumulated exactly in
// tensor memory, so a product carries about 2^-32 of its row and column
// scales and is rounded once, in the FP32 epilogue.  Three slices (2^-24 of
// the row and column maxima, coarser than FP32 for the smaller entries)
// measured 6.0e-5 against the oracle's complex64 arithmetic over the 65536
// steps of the d = 64 Magnus workload, where the FP32 products give 7.4e-6.
//
//   * k_plain_assemble forms X_j of every step of a batch (the same operations
//     in the same order as the SIMT kernel's assembly, so X_j is bit-identical)
//     as two planes (re, im) of 64 rows padded to 68 floats.
//   * k_small_tc: one CTA of 512 threads per SM walks a chunk of steps.  Per
//     step it slices X once (the A operand of every Clenshaw product, row
//     scales), then per order slices b_(k+1) as the B operand (column scales),
//     hands the product to the tensor core and forms b_k from its levels in
//     FP32.  U_j - I and P then make the chunk product; P stays in tensor
//     memory.  The planes of step j + 1 arrive by bulk copy while step j runs.
// Each thread keeps one plane of 16 columns of one row (tc_slice.cuh), so the
// Clenshaw updates work plane by plane: s is real and J_k I touches the
// diagonal only.  Every wait is bounded; a wait that runs out stops the CTA and
// adds one to the context's fault counter.
#include <stdlib.h>

#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "tc_slice.cuh"

namespace pgb {

constexpr int kStcSlices = 4;
constexpr size_t kStcSA = (size_t)kStcSlices * oz::kASlice;  // 96 KB
constexpr size_t kStcSB = (size_t)kStcSlices * oz::kBSlice;  // 64 KB
constexpr int kStcPlaneLd = 68;
constexpr int kStcPlane = 64 * kStcPlaneLd;
constexpr int kSmallXStride = 2 * kStcPlane;                  // floats per step: planes re, im
constexpr uint32_t kStcXBytes = kSmallXStride * sizeof(float);  // 34,816
constexpr size_t kStcSmem = kStcSA + kStcSB + (size_t)kStcXBytes + 1024;
constexpr long long kSmallXBatch = 65536;
constexpr int kStcMaxKe = 64;
static_assert(kStcSmem + sizeof(TcdShared) + 64 <= 232448, "k_small_tc exceeds 227 KB of shared memory");
static_assert(kStcXBytes % 16 == 0 && (kStcSA + kStcSB) % 1024 == 0, "plane buffers must stay 16-byte aligned");

struct SmallTcArgs {
    float2 J[kMaxOrder + 1];  // (-i)^k J_k(x) in complex64
    const float *xplanes;     // planes of the batch's steps, kSmallXStride floats apart
    float2 *chunks;           // nchunks products, row-major complex64
    long long P;              // steps of the batch
    int nchunks, M;
    float s;                  // 2 / Hnorm
    int *fault;
};

__device__ int g_small_tc_faults;

// X planes of steps s_off .. s_off + n - 1.  Thread f of CTA row blockIdx.x
// owns float4 f of every expansion matrix (complex elements 2f, 2f + 1) and
// keeps that slice of the stack in registers (RK > 0: up to RK + 1 matrices,
// loops unrolled) or in shared memory (RK = 0); the CTA forms the complex64
// weights of its kPlainAsmSteps steps in shared memory and walks them.
// X = H_0 + sum_m w_m H_m by complex fused multiply-adds in slot order, as in
// k_small_steps.
constexpr int kPlainAsmSteps = 32;
constexpr int kPlainAsmRegKe = 15;  // largest Ke with the stack slice in registers
template <int RK>
__global__ void __launch_bounds__(128) k_plain_assemble(const float2 *__restrict__ stack, const float2 *__restrict__ carr,
                                                        WeightSpec w, int Ke, float *xp, long long s_off,
                                                        long long n) {
    extern __shared__ float4 hs[];  // RK = 0: (1 + Ke) x 128 float4 of the stack
    __shared__ float2 ws[kPlainAsmSteps * kStcMaxKe];
    const int f = blockIdx.x * 128 + threadIdx.x;
    const long long sb = (long long)blockIdx.y * kPlainAsmSteps;
    const int ns = (int)(n - sb < kPlainAsmSteps ? n - sb : kPlainAsmSteps);
    const float4 *stack4 = reinterpret_cast<const float4 *>(stack);
    float4 hr[RK + 1];
    if constexpr (RK > 0) {
#pragma unroll
        for (int m = 0; m <= RK; ++m) hr[m] = m <= Ke ? stack4[(size_t)m * 2048 + f] : make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
        for (int m = 0; m <= Ke; ++m) hs[m * 128 + threadIdx.x] = stack4[(size_t)m * 2048 + f];
    }
    for (int i = threadIdx.x; i < ns * Ke; i += 128) ws[i] = step_weight(carr, w, i % Ke, s_off + sb + i / Ke);
    __syncthreads();
    const int row = f >> 5, col = 2 * (f & 31);
    for (int k = 0; k < ns; ++k) {
        float4 h0;
        if constexpr (RK > 0) h0 = hr[0]; else h0 = hs[threadIdx.x];
        float2 v0 = make_float2(h0.x, h0.y), v1 = make_float2(h0.z, h0.w);
#pragma unroll
        for (int m = 0; m < (RK > 0 ? RK : 1 << 30); ++m) {
            if (m >= Ke) break;
            float4 h;
            if constexpr (RK > 0) h = hr[m + 1]; else h = hs[(m + 1) * 128 + threadIdx.x];
            const float2 wm = ws[k * Ke + m];
            cfma(v0, wm, make_float2(h.x, h.y));
            cfma(v1, wm, make_float2(h.z, h.w));
        }
        float *o = xp + (size_t)(sb + k) * kSmallXStride + row * kStcPlaneLd + col;
        *reinterpret_cast<float2 *>(o) = make_float2(v0.x, v1.x);
        *reinterpret_cast<float2 *>(o + kStcPlane) = make_float2(v0.y, v1.y);
        if (col == 62) {
            // The row padding too, so that every 32-byte sector is written whole.
            *reinterpret_cast<float2 *>(o + 2) = make_float2(0.f, 0.f);
            *reinterpret_cast<float2 *>(o + 4) = make_float2(0.f, 0.f);
            *reinterpret_cast<float2 *>(o + kStcPlane + 2) = make_float2(0.f, 0.f);
            *reinterpret_cast<float2 *>(o + kStcPlane + 4) = make_float2(0.f, 0.f);
        }
    }
}

__global__ void __launch_bounds__(kTcdThreads, 1) k_small_tc(const __grid_constant__ SmallTcArgs a) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((1024u - (tc::smem_addr(smem_raw) & 1023u)) & 1023u);
    unsigned char *SA = smem;
    unsigned char *SB = smem + kStcSA;
    unsigned char *XB = SB + kStcSB;  // the planes of one step
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
    const long long n = s1 - s0;
    const int M = a.M;
    const float s = a.s;

    if (warp == 0) {
        tc::tmem_alloc(&sh.tmem_base, 512);
        tc::tmem_relinquish();
    }
    if (t.tid == 0) {
        tc::mbar_init(&sh.bar, 1);
        tc::mbar_init(&sh.hbar, 1);  // plane copies
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
    t.tm_ep = sh.tmem_base + lane_base + 256u + 16u * (uint32_t)t.cb;  // P of this thread
    t.tm_e = 0;

    // The planes of step i + 1 are copied as soon as every thread has read
    // those of step i, early in step i.  Copies are issued and waited for in
    // step order.
    long long nissued = 0, nwaited = 0;
    auto issue_x = [&](long long i) {
        ++nissued;
        if (t.tid == 0) {
            mbar_expect_tx(&sh.hbar, kStcXBytes);
            bulk_g2s(XB, a.xplanes + (size_t)(s0 + i) * kSmallXStride, kStcXBytes, &sh.hbar);
        }
    };
    if (n > 0) issue_x(0);

    uint32_t ncommit = 0;
    int nb = 0;
    bool ok = true;
    const int sgn = t.p == 0 ? -1 : 1;  // plane p of J X: J_re X_p + sgn J_im X_(1-p)
    auto jp = [&](int k) { return t.p == 0 ? a.J[k].x : a.J[k].y; };
    for (long long i = 0; i < n; ++i) {
        ok = tc::mbar_wait(&sh.hbar, (uint32_t)i & 1, kTcdWait) && ok;
        ++nwaited;
        const float *XP = reinterpret_cast<const float *>(XB);
        float X[16], b1[16], b2[16];
        {
            const float4 *own = reinterpret_cast<const float4 *>(XP + t.p * kStcPlane + t.r * kStcPlaneLd + t.c0);
            const float4 *oth = reinterpret_cast<const float4 *>(XP + (1 - t.p) * kStcPlane + t.r * kStcPlaneLd + t.c0);
            const float2 JM = a.J[M];
            const float jm1 = jp(M - 1), jm = jp(M);
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                const float4 x = own[g], y = oth[g];
                const float xs[4] = {x.x, x.y, x.z, x.w}, ys[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int j = 4 * g + q;
                    const bool dg = t.c0 + j == t.r;
                    X[j] = xs[q];
                    b1[j] = (JM.x * xs[q] + sgn * JM.y * ys[q]) * s + (dg ? jm1 : 0.0f);
                    b2[j] = dg ? jm : 0.0f;
                }
            }
        }
        // Every thread has read the planes (the barrier in reduce_max), so the
        // copy of step i + 1 may overwrite them.
        tc::fence_proxy_async();
        reduce_max<true, false>(sh, t, nb, X, X);
        if (i + 1 < n) issue_x(i + 1);
        store_a<kStcSlices, false>(sh, SA, t, nb, X, X);
        nb ^= 1;
        bool live = true;
        for (int k = M - 2; k >= 0; --k) {
            reduce_max<false, true>(sh, t, nb, X, b1);
            store_b<kStcSlices, false>(SB, t, sh.bmax[nb], b1, b1, sh.colmul);
            nb ^= 1;
            if (!(live = run_product(sh, t, SA, SB, kStcSlices, kStcSlices, kStcSlices - 1, false, ncommit, ok)))
                break;
            float D[16];
            epilogue_f<kStcSlices - 1>(sh, t, D);
            const float beta = k == 0 ? -2.0f : -1.0f, jk = jp(k);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                float v = D[j] * s;
                v += beta * b2[j];
                if (t.c0 + j == t.r) v += jk;
                b2[j] = b1[j];
                b1[j] = v;  // k = 0: U_j
            }
        }
        if (!live) break;
        // Chunk product P <- U P = P + (U - I) P (later step on the left).
        if (i == 0) {
            tc::tmem_st16(t.tm_ep, b1);
            tc::tmem_wait_st();
        } else {
            float Pv[16];
            tc::tmem_ld16(t.tm_ep, Pv);
#pragma unroll
            for (int j = 0; j < 16; ++j)
                if (t.p == 0 && t.c0 + j == t.r) b1[j] -= 1.0f;
            reduce_max<true, true>(sh, t, nb, b1, Pv);
            store_a<kStcSlices, false>(sh, SA, t, nb, b1, b1);
            store_b<kStcSlices, false>(SB, t, sh.bmax[nb], Pv, Pv, sh.colmul);
            nb ^= 1;
            if (!run_product(sh, t, SA, SB, kStcSlices, kStcSlices, kStcSlices - 1, false, ncommit, ok)) break;
            float D[16];
            epilogue_f<kStcSlices - 1>(sh, t, D);
#pragma unroll
            for (int j = 0; j < 16; ++j) Pv[j] += D[j];
            tc::tmem_st16(t.tm_ep, Pv);
            tc::tmem_wait_st();
        }
    }
    ok = __syncthreads_and(ok) != 0;
    if (ok && n > 0) {
        float Pv[16];
        tc::tmem_ld16(t.tm_ep, Pv);
        float *dst = reinterpret_cast<float *>(a.chunks + (size_t)blockIdx.x * 4096);
#pragma unroll
        for (int j = 0; j < 16; ++j) dst[2 * (t.r * 64 + t.c0 + j) + t.p] = Pv[j];
    }
    if (!ok) {
        if (t.tid == 0) atomicAdd(a.fault ? a.fault : &g_small_tc_faults, 1);
        if (ncommit > 0) tc::mbar_wait(&sh.bar, (ncommit - 1) & 1, kTcdWait);
    }
    for (; nwaited < nissued; ++nwaited) tc::mbar_wait(&sh.hbar, (uint32_t)nwaited & 1, kTcdWait);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(sh.tmem_base, 512);
    }
}

static bool small_tc_disabled() {
    static const bool off = [] {
        const char *v = getenv("PARAMENT_DISABLE_TENSOR_CORES");
        return v && v[0] && v[0] != '0';
    }();
    return off;
}

bool small_tc_applies(bool fp64, int d, int Ke, int M) {
    return !fp64 && d == 64 && Ke <= kStcMaxKe && M >= 1 && M <= kMaxOrder && !small_tc_disabled();
}

size_t small_tc_xplane_bytes(long long P) {
    return sizeof(float) * kSmallXStride * (size_t)std::min<long long>(P, kSmallXBatch);
}

int small_tc_max_chunks(long long P, int num_sms) {
    const long long batches = (P + kSmallXBatch - 1) / kSmallXBatch;
    return (int)std::max<long long>(1, std::min<long long>((long long)num_sms * batches, P));
}

cudaError_t launch_small_tc(const StepLaunch &l, int num_sms, float *xplanes, int *fault, int *nchunks,
                            cudaEvent_t ev0, cudaEvent_t ev1) {
    if (l.fp64 || l.d != 64 || l.Ke > kStcMaxKe || l.M < 1 || l.M > kMaxOrder) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void *>(&k_small_tc),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStcSmem);
    if (e != cudaSuccess) return e;
    SmallTcArgs a;
    for (int k = 0; k <= l.M; ++k) a.J[k] = make_float2((float)l.J[2 * k], (float)l.J[2 * k + 1]);
    a.xplanes = xplanes;
    a.M = l.M;
    a.s = (float)l.s;
    a.fault = fault;
    const WeightSpec w{l.w.pts, l.w.K, l.w.amps, l.w.mode, l.w.magnus, l.w.hfac};
    const float2 *stack = static_cast<const float2 *>(l.stack);
    const float2 *carr = static_cast<const float2 *>(l.carr);
    const bool asm_reg = l.Ke <= kPlainAsmRegKe;
    const void *asm_fn = asm_reg ? reinterpret_cast<const void *>(&k_plain_assemble<kPlainAsmRegKe>)
                                 : reinterpret_cast<const void *>(&k_plain_assemble<0>);
    const size_t hs_bytes = asm_reg ? 0 : sizeof(float4) * 128 * (size_t)(l.Ke + 1);
    if ((e = cudaFuncSetAttribute(asm_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hs_bytes)) != cudaSuccess)
        return e;
    int total = 0;
    for (long long b0 = 0; b0 < l.P; b0 += kSmallXBatch) {
        const long long nb = std::min<long long>(kSmallXBatch, l.P - b0);
        const dim3 ag(16, (unsigned)((nb + kPlainAsmSteps - 1) / kPlainAsmSteps));
        int ke = l.Ke;
        long long off = b0, cnt = nb;
        float *xpp = xplanes;
        WeightSpec wv = w;
        void *args[] = {const_cast<float2 **>(&stack), const_cast<float2 **>(&carr), &wv, &ke, &xpp, &off, &cnt};
        if ((e = cudaLaunchKernel(asm_fn, ag, dim3(128), args, hs_bytes, l.stream)) != cudaSuccess) return e;
        a.P = nb;
        a.nchunks = (int)std::max<long long>(1, std::min<long long>((long long)num_sms, nb));
        a.chunks = static_cast<float2 *>(l.chunks) + (size_t)total * 4096;
        if (ev0 && b0 == 0) cudaEventRecord(ev0, l.stream);
        k_small_tc<<<a.nchunks, kTcdThreads, kStcSmem, l.stream>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        total += a.nchunks;
    }
    if (ev1) cudaEventRecord(ev1, l.stream);
    *nchunks = total;
    return cudaSuccess;
}

}  // namespace pgb
