// Complex64 batched GEMM on the tcgen05 tensor cores, 3xTF32 split products.
//
//   C_b = alpha * A_b B_b + beta * Cin_b + diag * I       (d x d, row-major)
//
// Used for the large-d plain path (d >= 256, d % 128 == 0) in place of the
// SIMT k_gemm: the reference's cublasCgemmStridedBatched calls of the Clenshaw
// recurrence and the tree (src/cuda/parament.cpp:596-636, :681-690).
//
// Real formulation per CTA tile (128 rows x 64 complex columns), per K slab of
// 16 complex columns of A / rows of B:
//   D[128 x 128] += A' [128 x 32] * B'' [32 x 128]
//   A'  = [A_r | A_i],   B'' = [[B_r, B_i], [-B_i, B_r]]
// so D = [C_r | C_i].  Each FP32 operand is split x = hi + lo with hi, lo TF32
// and D accumulates hi*hi + hi*lo + lo*hi in FP32 (TMEM), which keeps the
// products near FP32 accuracy.  Operands are staged by all 256 threads into
// 128-byte-swizzled K-major shared-memory tiles (two stages); one thread
// issues the tcgen05.mma instructions and commits them to the stage's
// mbarrier; the epilogue reads the accumulators with tcgen05.ld.
#include <stdlib.h>

#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "tc.cuh"

namespace pgb {

constexpr int kTcStages = 2;
constexpr int kTcTileBytes = 128 * 128;  // 128 rows x 32 FP32 = 16 KB
constexpr int kTcStageBytes = 4 * kTcTileBytes;
constexpr uint32_t kTcWaitLimit = 1u << 22;

__device__ int g_tc_faults;  // bounded waits that gave up (0 in normal operation)

struct TcArgs {
    const float2 *A, *B, *Cin;
    float2 *Cout;
    long long sA, sB, sCin, sCout;
    float2 alpha, diag;
    float beta;
    int d, batch, tiles_n, a_minus_identity;
};

__device__ __forceinline__ void put_split(unsigned char *hi, unsigned char *lo, uint32_t off, float x) {
    const float h = tc::to_tf32(x);
    *reinterpret_cast<float *>(hi + off) = h;
    *reinterpret_cast<float *>(lo + off) = tc::to_tf32(x - h);
}

__global__ void __launch_bounds__(256, 1) k_tc_cgemm(const __grid_constant__ TcArgs g) {
    extern __shared__ unsigned char smem_dyn[];
    __shared__ uint64_t mbar[kTcStages];
    __shared__ uint32_t tmem_base;
    unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int d = g.d;
    const int tile = blockIdx.x;
    const int r0 = (tile / g.tiles_n) * 128, c0 = (tile % g.tiles_n) * 64;
    const uint32_t idesc = tc::idesc_tf32(128, 128);

    if (warp == 0) {
        tc::tmem_alloc(&tmem_base, 128);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s) tc::mbar_init(&mbar[s], 1);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tmem_base;
    bool ok = true;

    // Commits issued to each stage's mbarrier so far (every thread keeps the
    // same count): the n-th completion of a barrier has phase parity n & 1.
    uint32_t issued[kTcStages] = {0, 0};
    for (int b = blockIdx.y; b < g.batch; b += gridDim.y) {
        const float2 *A = g.A + (size_t)b * g.sA;
        const float2 *B = g.B + (size_t)b * g.sB;
        const int nk = d / 16;
        // Slab kc + 1 is loaded into registers while slab kc is converted and
        // multiplied, so global latency overlaps the tensor-core work.
        float2 ra[8], rb[4];
        auto load_slab = [&](int kc) {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int e = tid + 256 * i, row = e >> 4, kk = e & 15;
                ra[i] = A[(size_t)(r0 + row) * d + 16 * kc + kk];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int e = tid + 256 * i, kk = e >> 6, nn = e & 63;
                rb[i] = B[(size_t)(16 * kc + kk) * d + c0 + nn];
            }
        };
        load_slab(0);
        for (int kc = 0; kc < nk; ++kc) {
            const int s = kc & 1;
            unsigned char *Ah = smem + s * kTcStageBytes, *Al = Ah + kTcTileBytes;
            unsigned char *Bh = Al + kTcTileBytes, *Bl = Bh + kTcTileBytes;
            if (issued[s] > 0) {
                // The MMAs that last read this stage must be complete.
                if (!tc::mbar_wait(&mbar[s], (issued[s] - 1) & 1, kTcWaitLimit)) ok = false;
            }
            // A' slab: rows r0..r0+127, complex columns 16 kc .. 16 kc + 15.
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int e = tid + 256 * i, row = e >> 4, kk = e & 15;
                float2 a = ra[i];
                if (g.a_minus_identity && r0 + row == 16 * kc + kk) a.x -= 1.0f;
                put_split(Ah, Al, tc::sw128_offset(row, kk), a.x);
                put_split(Ah, Al, tc::sw128_offset(row, 16 + kk), a.y);
            }
            // B''^T slab: rows n (0..63: real part of C, 64..127: imaginary), K = 32.
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int e = tid + 256 * i, kk = e >> 6, nn = e & 63;
                const float2 v = rb[i];
                put_split(Bh, Bl, tc::sw128_offset(nn, kk), v.x);
                put_split(Bh, Bl, tc::sw128_offset(nn, 16 + kk), -v.y);
                put_split(Bh, Bl, tc::sw128_offset(64 + nn, kk), v.y);
                put_split(Bh, Bl, tc::sw128_offset(64 + nn, 16 + kk), v.x);
            }
            if (kc + 1 < nk) load_slab(kc + 1);
            tc::fence_proxy_async();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                const uint32_t ah = tc::smem_addr(Ah), al = tc::smem_addr(Al);
                const uint32_t bh = tc::smem_addr(Bh), bl = tc::smem_addr(Bl);
#pragma unroll
                for (int k8 = 0; k8 < 4; ++k8) {
                    const uint32_t o = 32 * k8;  // 8 TF32 = 32 bytes along K
                    tc::mma_tf32(taddr, tc::desc_k_sw128(ah + o), tc::desc_k_sw128(bh + o), idesc,
                                 (kc > 0 || k8 > 0) ? 1u : 0u);
                    tc::mma_tf32(taddr, tc::desc_k_sw128(ah + o), tc::desc_k_sw128(bl + o), idesc, 1u);
                    tc::mma_tf32(taddr, tc::desc_k_sw128(al + o), tc::desc_k_sw128(bh + o), idesc, 1u);
                }
                tc::mma_commit(&mbar[s]);
            }
            ++issued[s];
        }
        // Wait for the last commit (it covers every MMA issued before it).
        {
            const int s = (nk - 1) & 1;
            if (!tc::mbar_wait(&mbar[s], (issued[s] - 1) & 1, kTcWaitLimit)) ok = false;
            const int so = s ^ 1;
            if (issued[so] > 0 && !tc::mbar_wait(&mbar[so], (issued[so] - 1) & 1, kTcWaitLimit)) ok = false;
        }
        tc::fence_after_sync();
        // Epilogue: warps 0-3 own TMEM lanes 32 (warp % 4) .. +31 (rows of the
        // tile); warps w and w + 4 split the 64 complex columns in halves.
        const int q = warp & 3, half = warp >> 2;
        const int row = r0 + 32 * q + lane;
        const float2 *Cin = g.Cin ? g.Cin + (size_t)b * g.sCin : nullptr;
        float2 *Co = g.Cout + (size_t)b * g.sCout;
        for (int cc = 0; cc < 2; ++cc) {
            const int col0 = 32 * half + 16 * cc;  // complex column within the tile
            float re[16], im[16];
            const uint32_t lane_base = (uint32_t)(32 * q) << 16;
            tc::tmem_ld16(taddr + lane_base + col0, re);
            tc::tmem_ld16(taddr + lane_base + 64 + col0, im);
            if (!ok) continue;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int col = c0 + col0 + j;
                const size_t e = (size_t)row * d + col;
                float2 v = make_float2(g.alpha.x * re[j] - g.alpha.y * im[j], g.alpha.x * im[j] + g.alpha.y * re[j]);
                if (Cin) {
                    const float2 o = Cin[e];
                    v.x += g.beta * o.x;
                    v.y += g.beta * o.y;
                }
                if (row == col) {
                    v.x += g.diag.x;
                    v.y += g.diag.y;
                }
                Co[e] = v;
            }
        }
        tc::fence_before_sync();
        __syncthreads();
    }
    if (!ok && lane == 0) atomicAdd(&g_tc_faults, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(taddr, 128);
    }
}

static bool tc_disabled() {
    static const bool off = [] {
        const char *v = getenv("PARAMENT_DISABLE_TENSOR_CORES");
        return v && v[0] && v[0] != '0';
    }();
    return off;
}

bool tc_gemm_applies(const GemmLaunch &l) { return !l.fp64 && l.d >= 256 && l.d % 128 == 0 && !tc_disabled(); }

cudaError_t launch_tc_gemm(const GemmLaunch &l) {
    TcArgs g;
    g.A = static_cast<const float2 *>(l.A);
    g.B = static_cast<const float2 *>(l.B);
    g.Cin = static_cast<const float2 *>(l.Cin);
    g.Cout = static_cast<float2 *>(l.Cout);
    g.sA = l.strideA;
    g.sB = l.strideB;
    g.sCin = l.strideCin;
    g.sCout = l.strideCout;
    g.alpha = make_float2((float)l.alpha_re, (float)l.alpha_im);
    g.diag = make_float2((float)l.diag_re, (float)l.diag_im);
    g.beta = (float)l.beta;
    g.d = l.d;
    g.batch = l.batch;
    g.tiles_n = l.d / 64;
    g.a_minus_identity = l.a_minus_identity ? 1 : 0;
    const size_t smem = (size_t)kTcStages * kTcStageBytes + 1024;
    cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void *>(&k_tc_cgemm),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((l.d / 128) * (l.d / 64), std::min(l.batch, 65535));
    k_tc_cgemm<<<grid, 256, smem, l.stream>>>(g);
    return cudaGetLastError();
}

int tc_take_faults() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_tc_faults, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (v) {
        int z = 0;
        cudaMemcpyToSymbol(g_tc_faults, &z, sizeof(int));
    }
    return v;
}

}  // namespace pgb
