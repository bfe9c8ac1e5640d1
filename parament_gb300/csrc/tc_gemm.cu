// Complex64 batched GEMM on the tcgen05 tensor cores, 3xTF32 split products.
//
//   C_b = alpha * A_b B_b + beta * Cin_b + diag * I       (d x d, row-major)
//
// Used for the large-d plain path (d >= 256, d % 128 == 0) in place of the
// SIMT k_gemm: the reference's cublasCgemmStridedBatched calls of the Clenshaw
// recurrence and the tree (src/cuda/parament.cpp:596-636, :681-690).
//
// Real formulation per CTA tile (128 rows x 64 complex columns), per K slab of
// 16 complex columns of A / rows of B, with K ordered as (re, im) pairs:
//   D[128 x 128] += A' [128 x 32] * B'' [32 x 128]
//   A'[m][2k + p] = (A_r, A_i)[p][m][k]     (the row-major complex data as is)
//   B''[2k][n]    = B_r[k][n],  B''[2k + 1][n]      = -B_i[k][n]    (n < 64)
//   B''[2k][64+n] = B_i[k][n],  B''[2k + 1][64 + n] =  B_r[k][n]
// so D = [C_r | C_i].  Each FP32 operand is split x = hi + lo with hi, lo TF32
// and D accumulates hi*hi + hi*lo + lo*hi in FP32 (TMEM), which keeps the
// products near FP32 accuracy.
//
// Warp roles.  Warp 8 (one thread) issues the tiled TMA copies of the A and B
// slabs into a four-deep raw ring (A lands already in the 128-byte-swizzled
// K-major operand layout) and the tcgen05.mma instructions of each converted
// stage, committing them to the stage's "empty" mbarrier.  Warps 0-7 split
// each raw slab into the hi / lo operand tiles of one of two stages with
// 16-byte shared-memory accesses and arrive on the stage's "full" mbarrier;
// at the end of a batch item they read the accumulators with tcgen05.ld into
// a padded staging tile and write the item's rows with coalesced 16-byte
// accesses.
#include <cuda.h>
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
// Raw complex64 slabs arrive by tiled TMA copies into a ring of kTcRaw
// stages: A rows r0..r0+127 x 16 complex columns (128 bytes per row), then B
// rows 16 kc .. 16 kc + 15 x 64 complex columns (512 bytes per row).
constexpr int kTcRaw = 4;
constexpr int kTcRawA = 128 * 128;
constexpr int kTcRawB = 16 * 512;
constexpr int kTcRawStage = kTcRawA + kTcRawB;
constexpr size_t kTcSmem = (size_t)kTcStages * kTcStageBytes + (size_t)kTcRaw * kTcRawStage + 1024;
static_assert(kTcSmem <= 232448, "shared memory of k_tc_cgemm exceeds 227 KB");

__device__ __forceinline__ void tc_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// One box of a 3-D tensor map (FP32 elements; x, y, z = float column, row,
// batch item) into shared memory.
__device__ __forceinline__ void tc_tma_load3(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(tc::smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(tc::smem_addr(bar))
        : "memory");
}

__device__ int g_tc_faults;  // bounded waits that gave up (0 in normal operation)

struct TcArgs {
    // A and B as 3-D FP32 tensors (2 d floats per row, d rows, batch items);
    // an operand shared by every item has one item (batched* = 0).
    CUtensorMap tmA, tmB;
    int batchedA, batchedB;
    const float2 *A, *B, *Cin;
    float2 *Cout;
    long long sA, sB, sCin, sCout;
    float2 alpha, diag;
    float beta;
    int d, batch, tiles_n, a_minus_identity;
};

__device__ __forceinline__ float4 lds128(uint32_t a) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
    return v;
}
__device__ __forceinline__ float2 lds64(uint32_t a) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
    return v;
}
__device__ __forceinline__ void sts128(uint32_t a, float4 v) {
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}
// Round to TF32 (10 explicit mantissa bits), nearest with ties away from zero,
// by integer operations on the bits: half an ulp of TF32 is added to the
// magnitude and the 13 low bits are cleared (a carry moves into the exponent).
__device__ __forceinline__ float tf32_rna(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}
// x = hi + lo with hi, lo TF32; stores hi at hi_addr and lo at lo_addr.
__device__ __forceinline__ void put_split4(uint32_t hi_addr, uint32_t lo_addr, float4 x) {
    const float4 h = make_float4(tf32_rna(x.x), tf32_rna(x.y), tf32_rna(x.z), tf32_rna(x.w));
    sts128(hi_addr, h);
    sts128(lo_addr, make_float4(tf32_rna(x.x - h.x), tf32_rna(x.y - h.y), tf32_rna(x.z - h.z), tf32_rna(x.w - h.w)));
}

__device__ __forceinline__ void tc_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_addr(bar)) : "memory");
}
// Barrier 1 among the 256 converter threads (the issuer warp does not take part).
__device__ __forceinline__ void conv_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

constexpr int kTcThreads = 288;     // warps 0-7 convert, warp 8 issues copies and MMAs
constexpr int kTcStagePitch = 528;  // bytes per row of the epilogue's staging tile (64 complex + 16)

__global__ void __launch_bounds__(kTcThreads, 1) k_tc_cgemm(const __grid_constant__ TcArgs g) {
    extern __shared__ unsigned char smem_dyn[];
    __shared__ uint64_t empty[kTcStages];  // MMAs that read a converted stage completed
    __shared__ uint64_t full[kTcStages];   // the 256 converter threads filled a stage
    __shared__ uint64_t rawbar[kTcRaw];    // the TMA copies of a raw stage landed
    __shared__ uint32_t tmem_base;
    unsigned char *smem = smem_dyn + ((1024u - (tc::smem_addr(smem_dyn) & 1023u)) & 1023u);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int d = g.d;
    const int tile = blockIdx.x;
    const int r0 = (tile / g.tiles_n) * 128, c0 = (tile % g.tiles_n) * 64;
    const uint32_t idesc = tc::idesc_tf32(128, 128);

    if (warp == 8) {
        tc::tmem_alloc(&tmem_base, 128);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            tc::mbar_init(&empty[s], 1);
            tc::mbar_init(&full[s], 256);
        }
        for (int s = 0; s < kTcRaw; ++s) tc::mbar_init(&rawbar[s], 1);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tmem_base;
    bool ok = true;

    // The CTA's slabs q = j nk + kc run over its batch items b = blockIdx.y +
    // j gridDim.y and their K slabs kc.  Slab q is converted into stage q % 2;
    // its raw data sits in raw stage q % kTcRaw.  The n-th completion of a
    // barrier has phase parity n & 1.
    const int nk = d / 16;
    const int nitems = (g.batch - (int)blockIdx.y + (int)gridDim.y - 1) / (int)gridDim.y;
    const int nslab = nitems * nk;
    unsigned char *raw0 = smem + (size_t)kTcStages * kTcStageBytes;

    if (warp == 8) {
        if (lane == 0) {
            int jn = 0, kn = 0;  // item and slab of the next raw copy
            auto issue_raw = [&](int q) {
                const int st = q % kTcRaw;
                unsigned char *ra = raw0 + st * kTcRawStage, *rb = ra + kTcRawA;
                const int b = (int)blockIdx.y + jn * (int)gridDim.y;
                tc_expect_tx(&rawbar[st], kTcRawA + kTcRawB);
                tc_tma_load3(ra, &g.tmA, 32 * kn, r0, g.batchedA ? b : 0, &rawbar[st]);
                tc_tma_load3(rb, &g.tmB, 2 * c0, 16 * kn, g.batchedB ? b : 0, &rawbar[st]);
                if (++kn == nk) kn = 0, ++jn;
            };
            for (int q = 0; q < kTcRaw && q < nslab; ++q) issue_raw(q);
            int kc = 0;
            for (int q = 0; q < nslab; ++q) {
                const int s = q & 1;
                if (!tc::mbar_wait(&full[s], (uint32_t)(q >> 1) & 1, kTcWaitLimit)) ok = false;
                tc::fence_after_sync();
                const uint32_t ah = tc::smem_addr(smem + s * kTcStageBytes), al = ah + kTcTileBytes;
                const uint32_t bh = al + kTcTileBytes, bl = bh + kTcTileBytes;
#pragma unroll
                for (int k8 = 0; k8 < 4; ++k8) {
                    const uint32_t o = 32 * k8;  // 8 TF32 = 32 bytes along K
                    tc::mma_tf32(taddr, tc::desc_k_sw128(ah + o), tc::desc_k_sw128(bh + o), idesc,
                                 (kc > 0 || k8 > 0) ? 1u : 0u);
                    tc::mma_tf32(taddr, tc::desc_k_sw128(ah + o), tc::desc_k_sw128(bl + o), idesc, 1u);
                    tc::mma_tf32(taddr, tc::desc_k_sw128(al + o), tc::desc_k_sw128(bh + o), idesc, 1u);
                }
                tc::mma_commit(&empty[s]);
                // The converters read raw stage q % kTcRaw before they arrived on full[s].
                if (q + kTcRaw < nslab) issue_raw(q + kTcRaw);
                if (++kc == nk) kc = 0;
            }
        }
        __syncwarp();
    } else {
        unsigned char *stg = smem;  // epilogue staging tile: 128 rows x kTcStagePitch bytes
        const uint32_t stg_a = tc::smem_addr(stg);
        int j = 0, kc = 0;
        for (int q = 0; q < nslab; ++q) {
            const int s = q & 1, rs = q % kTcRaw;
            // The MMAs of slab q - 2 read stage s.
            if (q >= 2 && !tc::mbar_wait(&empty[s], (uint32_t)((q - 2) >> 1) & 1, kTcWaitLimit)) ok = false;
            if (!tc::mbar_wait(&rawbar[rs], (uint32_t)(q / kTcRaw) & 1, kTcWaitLimit)) ok = false;
            const uint32_t ra = tc::smem_addr(raw0 + rs * kTcRawStage), rb = ra + kTcRawA;
            const uint32_t ah = tc::smem_addr(smem + s * kTcStageBytes), al = ah + kTcTileBytes;
            const uint32_t bh = al + kTcTileBytes, bl = bh + kTcTileBytes;
            // A' slab (rows r0..r0+127, complex columns 16 kc .. 16 kc + 15): the
            // TMA copy left it in the operand layout, so hi and lo go to the same
            // offsets.  Chunk f holds complex columns 2 ch, 2 ch + 1 of row f / 8.
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int f = tid + 256 * i;
                float4 x = lds128(ra + 16 * f);
                if (g.a_minus_identity) {
                    const int row = f >> 3, ch = (f & 7) ^ (row & 7);
                    const int dk = r0 + row - 16 * kc - 2 * ch;
                    if (dk == 0) x.x -= 1.0f;
                    if (dk == 1) x.z -= 1.0f;
                }
                put_split4(ah + 16 * f, al + 16 * f, x);
            }
            // B''^T slab (rows n, 32 K values): task (n, c) writes K = 4c .. 4c + 3
            // of rows n and 64 + n from B rows 2c, 2c + 1 (raw rows of 512 bytes).
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int t = tid + 256 * i, n = t & 63, c = t >> 6;
                const float2 v0 = lds64(rb + (uint32_t)((2 * c) * 64 + n) * 8);
                const float2 v1 = lds64(rb + (uint32_t)((2 * c + 1) * 64 + n) * 8);
                const uint32_t o_re = tc::sw128_offset(n, 4 * c), o_im = tc::sw128_offset(64 + n, 4 * c);
                put_split4(bh + o_re, bl + o_re, make_float4(v0.x, -v0.y, v1.x, -v1.y));
                put_split4(bh + o_im, bl + o_im, make_float4(v0.y, v0.x, v1.y, v1.x));
            }
            tc::fence_proxy_async();
            tc_arrive(&full[s]);
            if (++kc < nk) continue;
            kc = 0;
            // Last slab of item b: its commit covers every MMA of the item.
            const int b = (int)blockIdx.y + j * (int)gridDim.y;
            ++j;
            if (!tc::mbar_wait(&empty[s], (uint32_t)(q >> 1) & 1, kTcWaitLimit)) ok = false;
            tc::fence_after_sync();
            // Epilogue, first half: warp w reads TMEM lanes 32 (w % 4) .. +31
            // (rows of the tile), complex columns 32 (w / 4) .. +31, into the
            // staging tile (both stages are idle until the next item).
            {
                const int wq = warp & 3, half = warp >> 2, rl = 32 * wq + lane;
                const uint32_t lane_base = (uint32_t)(32 * wq) << 16;
#pragma unroll
                for (int cc = 0; cc < 2; ++cc) {
                    const int col0 = 32 * half + 16 * cc;
                    float re[16], im[16];
                    tc::tmem_ld16(taddr + lane_base + col0, re);
                    tc::tmem_ld16(taddr + lane_base + 64 + col0, im);
#pragma unroll
                    for (int jj = 0; jj < 8; ++jj)
                        sts128(stg_a + rl * kTcStagePitch + (col0 + 2 * jj) * 8,
                               make_float4(re[2 * jj], im[2 * jj], re[2 * jj + 1], im[2 * jj + 1]));
                }
            }
            tc::fence_before_sync();
            conv_sync();
            // Second half: rows of the tile, 16 bytes (two complex) per thread;
            // the sixteen Cin loads are all in flight before the first use.
            {
                const float2 *Cin = g.Cin ? g.Cin + (size_t)b * g.sCin : nullptr;
                float2 *Co = g.Cout + (size_t)b * g.sCout;
                float4 ci[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int idx = tid + 256 * i, rl = idx >> 5, c4 = idx & 31;
                    ci[i] = Cin ? *reinterpret_cast<const float4 *>(Cin + (size_t)(r0 + rl) * d + c0 + 2 * c4)
                                : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int idx = tid + 256 * i, rl = idx >> 5, c4 = idx & 31;
                    const float4 v = lds128(stg_a + rl * kTcStagePitch + 16 * c4);
                    const int row = r0 + rl, col = c0 + 2 * c4;
                    const size_t e = (size_t)row * d + col;
                    float4 o = make_float4(g.alpha.x * v.x - g.alpha.y * v.y, g.alpha.x * v.y + g.alpha.y * v.x,
                                           g.alpha.x * v.z - g.alpha.y * v.w, g.alpha.x * v.w + g.alpha.y * v.z);
                    if (Cin) {
                        o.x += g.beta * ci[i].x;
                        o.y += g.beta * ci[i].y;
                        o.z += g.beta * ci[i].z;
                        o.w += g.beta * ci[i].w;
                    }
                    if (row == col) o.x += g.diag.x, o.y += g.diag.y;
                    if (row == col + 1) o.z += g.diag.x, o.w += g.diag.y;
                    if (ok) *reinterpret_cast<float4 *>(Co + e) = o;
                }
            }
            // The staging tile is read before the next item's slabs overwrite it.
            conv_sync();
        }
        // Every raw copy was waited for in the loop; a wait that gave up is
        // tried once more so that no copy lands after the CTA has exited.
        if (!ok)
            for (int q = (nslab > kTcRaw ? nslab - kTcRaw : 0); q < nslab; ++q)
                tc::mbar_wait(&rawbar[q % kTcRaw], (uint32_t)(q / kTcRaw) & 1, kTcWaitLimit);
    }
    if (!ok) atomicAdd(&g_tc_faults, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 8) {
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

// The raw slabs arrive by TMA copies and the epilogue moves 16 bytes per
// access: base addresses and batch strides must be multiples of 16 bytes.
static bool aligned16(const void *p, long long stride) {
    return p == nullptr || ((reinterpret_cast<uintptr_t>(p) & 15) == 0 && (stride & 1) == 0 && stride >= 0);
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiled encode_tiled() {
    static EncodeTiled fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

// Tensor map of one operand: FP32 view (2 d, d, items) with the given box.
static bool make_map(CUtensorMap *m, const void *base, int d, long long stride, int batch, uint32_t box_x,
                     uint32_t box_y, CUtensorMapSwizzle swz, int *batched) {
    EncodeTiled enc = encode_tiled();
    if (!enc) return false;
    *batched = (stride > 0 && batch > 1) ? 1 : 0;
    const cuuint64_t dims[3] = {(cuuint64_t)2 * d, (cuuint64_t)d, (cuuint64_t)(*batched ? batch : 1)};
    const cuuint64_t strides[2] = {(cuuint64_t)d * 8, (cuuint64_t)(*batched ? stride : (long long)d * d) * 8};
    const cuuint32_t box[3] = {box_x, box_y, 1}, estr[3] = {1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void *>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool tc_gemm_applies(const GemmLaunch &l) {
    return !l.fp64 && l.d >= 256 && l.d % 128 == 0 && !tc_disabled() && aligned16(l.A, l.strideA) &&
           aligned16(l.B, l.strideB) && aligned16(l.Cin, l.strideCin) && aligned16(l.Cout, l.strideCout);
}

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
    if (!make_map(&g.tmA, l.A, l.d, l.strideA, l.batch, 32, 128, CU_TENSOR_MAP_SWIZZLE_128B, &g.batchedA) ||
        !make_map(&g.tmB, l.B, l.d, l.strideB, l.batch, 128, 16, CU_TENSOR_MAP_SWIZZLE_NONE, &g.batchedB))
        return cudaErrorInvalidValue;
    const size_t smem = kTcSmem;
    cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void *>(&k_tc_cgemm),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((l.d / 128) * (l.d / 64), std::min(l.batch, 65535));
    k_tc_cgemm<<<grid, kTcThreads, smem, l.stream>>>(g);
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
