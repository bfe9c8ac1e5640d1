// Complex64 batched GEMM on the tcgen05 tensor cores, 3xTF32 split products.
//
//   C_b = alpha * A_b B_b + beta * Cin_b + diag * I       (d x d, row-major)
//
// Used for the large-d plain path (d >= 256, d % 128 == 0) in place of the
// SIMT k_gemm: the reference's cublasCgemmStridedBatched calls of the Clenshaw
// recurrence and the tree (src/cuda/parament.cpp:596-636, :681-690).
//
// Real formulation per unit (a tile of 128 rows x 128 complex columns of one
// batch item), per K slab of 16 complex columns of A / rows of B, with K
// ordered as (re, im) pairs:
//   D[128 x 256] += A' [128 x 32] * B'' [32 x 256]
//   A'[m][2k + p] = (A_r, A_i)[p][m][k]     (the row-major complex data as is)
//   B''[2k][n]     = B_r[k][n],  B''[2k + 1][n]       = -B_i[k][n]    (n < 128)
//   B''[2k][128+n] = B_i[k][n],  B''[2k + 1][128 + n] =  B_r[k][n]
// so D = [C_r | C_i].  Each FP32 operand is split x = hi + lo with hi, lo TF32
// and D accumulates hi*hi + hi*lo + lo*hi in FP32 (TMEM), which keeps the
// products near FP32 accuracy.
//
// The grid is persistent: one CTA per SM walks the units.  Warp roles:
//  - warp 8 (one thread) issues the tiled TMA copies of the raw A and B slabs
//    into a three-deep ring (A lands 128-byte swizzled, so that a warp reading
//    one row per lane meets no bank conflicts) and, per converted stage, 12
//    tcgen05.mma (M = 128, N = 256, K = 8, A from tensor memory), committed to
//    the stage's "empty" mbarrier and, at the end of a unit, to "accf";
//  - warps 0-7 split each raw slab into the hi / lo operands of one of two
//    stages - A' into tensor memory (tcgen05.st, one row per lane), B'' into
//    128-byte-swizzled K-major shared memory with 16-byte stores - and arrive
//    on the stage's "full" mbarrier;
//  - warps 9-16 wait for "accf", read the accumulator with tcgen05.ld (one row
//    per lane, 64 complex columns per warp), arrive on "acce" after the last
//    load (the issuer waits for it before the next unit's first MMA) and write
//    C with 16-byte accesses.
//
// Tensor memory (512 columns): accumulator D in columns 0-255; stage s keeps
// A' hi in columns 256 + 64 s .. +31 and A' lo in the next 32.
#include <cuda.h>
#include <stdlib.h>

#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "tc.cuh"

namespace pgb {

constexpr int kTcStages = 2;
constexpr int kTcTileBytes = 256 * 128;  // B'' slab: 256 rows x 32 FP32 = 32 KB
constexpr int kTcStageBytes = 2 * kTcTileBytes;  // B'' hi and lo (A lives in tensor memory)
constexpr uint32_t kTcWaitLimit = 1u << 22;
// Raw complex64 slabs arrive by tiled TMA copies into a ring of kTcRaw
// stages: A rows r0..r0+127 x 16 complex columns (128 bytes per row), then B
// rows 16 kc .. 16 kc + 15 x 128 complex columns (1024 bytes per row).
constexpr int kTcRaw = 3;
constexpr int kTcRawA = 128 * 128;
constexpr int kTcRawB = 16 * 1024;
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

// Bounded waits that gave up, for launches without a context's counter.
__device__ int g_tc_faults;

struct TcArgs {
    // A and B as 3-D FP32 tensors (2 d floats per row, d rows, batch items);
    // an operand shared by every item has one item (batched* = 0).
    CUtensorMap tmA, tmB;
    int batchedA, batchedB;
    const float2 *A, *B, *Cin;
    float2 *Cout;
    long long sA, sB, sCin, sCout;
    float2 alpha, diag;
    float beta, beta_im;
    int d, batch, tiles_n, a_minus_identity;
    int *fault;  // the calling context's counter of CTAs whose waits gave up
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
constexpr int kTcConv = 256;       // converter threads: warps 0-7
constexpr int kTcIssuer = 8;       // warp 8 issues the copies and the MMAs
constexpr int kTcEpi = 9;          // warps 9-16 drain the accumulator
constexpr int kTcEpiThreads = 256;
constexpr int kTcThreads = kTcEpi * 32 + kTcEpiThreads;
constexpr int kTcTmemCols = 512;   // accumulator D in columns 0-255
constexpr int kTcAcol = 256;       // stage s: A' hi in columns 256 + 64 s .. +31, lo in the next 32

// Work unit k of a CTA: tile (128 rows x 128 complex columns) of batch item b.
struct TcWork {
    int b, r0, c0;
};
__device__ __forceinline__ TcWork tc_work(const TcArgs &g, int k) {
    const long long w = (long long)blockIdx.x + (long long)k * gridDim.x;
    const int ntiles = (g.d / 128) * g.tiles_n;
    const int tile = (int)(w % ntiles);
    return TcWork{(int)(w / ntiles), (tile / g.tiles_n) * 128, (tile % g.tiles_n) * 128};
}

__global__ void __launch_bounds__(kTcThreads, 1) k_tc_cgemm(const __grid_constant__ TcArgs g) {
    extern __shared__ unsigned char smem_dyn[];
    __shared__ uint64_t empty[kTcStages];  // MMAs that read a converted stage completed
    __shared__ uint64_t full[kTcStages];   // the converter threads filled a stage
    __shared__ uint64_t rawbar[kTcRaw];    // the TMA copies of a raw stage landed
    __shared__ uint64_t accf;              // every MMA of the unit completed
    __shared__ uint64_t acce;              // the epilogue warps read the accumulator
    __shared__ uint32_t tmem_base;
    unsigned char *smem = smem_dyn + ((1024u - (tc::smem_addr(smem_dyn) & 1023u)) & 1023u);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int d = g.d;
    const uint32_t idesc = tc::idesc_tf32(128, 256);

    if (warp == kTcIssuer) {
        tc::tmem_alloc(&tmem_base, kTcTmemCols);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            tc::mbar_init(&empty[s], 1);
            tc::mbar_init(&full[s], kTcConv);
        }
        for (int s = 0; s < kTcRaw; ++s) tc::mbar_init(&rawbar[s], 1);
        tc::mbar_init(&accf, 1);
        tc::mbar_init(&acce, kTcEpiThreads);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tmem_base;
    bool ok = true;

    // The CTA's work units k = 0, 1, ... (tc_work) each run over the K slabs
    // kc of their tile: slab q = k nk + kc is converted into stage q % kTcStages
    // from raw stage q % kTcRaw.  The n-th completion of a barrier has phase
    // parity n & 1.
    const int nk = d / 16;
    const long long total = (long long)((d / 128) * g.tiles_n) * g.batch;
    const int nunits = (int)((total - (long long)blockIdx.x + gridDim.x - 1) / gridDim.x);
    const int nslab = nunits * nk;
    unsigned char *raw0 = smem + (size_t)kTcStages * kTcStageBytes;

    if (warp == kTcIssuer) {
        if (lane == 0) {
            int kn = 0, kcn = 0;  // unit and slab of the next raw copy
            TcWork wn = tc_work(g, 0);
            auto issue_raw = [&](int q) {
                const int st = q % kTcRaw;
                unsigned char *ra = raw0 + st * kTcRawStage, *rb = ra + kTcRawA;
                tc_expect_tx(&rawbar[st], kTcRawA + kTcRawB);
                tc_tma_load3(ra, &g.tmA, 32 * kcn, wn.r0, g.batchedA ? wn.b : 0, &rawbar[st]);
                tc_tma_load3(rb, &g.tmB, 2 * wn.c0, 16 * kcn, g.batchedB ? wn.b : 0, &rawbar[st]);
                if (++kcn == nk) kcn = 0, wn = tc_work(g, ++kn);
            };
            asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&g.tmA)) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&g.tmB)) : "memory");
            for (int q = 0; q < kTcRaw && q < nslab; ++q) issue_raw(q);
            int kc = 0, k = 0;
            for (int q = 0; q < nslab; ++q) {
                const int s = q % kTcStages;
                if (kc == 0 && k >= 1) {
                    // The epilogue warps read the accumulator of unit k - 1.
                    if (!tc::mbar_wait(&acce, (uint32_t)(k - 1) & 1, kTcWaitLimit)) ok = false;
                }
                if (!tc::mbar_wait(&full[s], (uint32_t)(q / kTcStages) & 1, kTcWaitLimit)) ok = false;
                tc::fence_after_sync();
                const uint32_t acc = taddr;
                const uint32_t ah = taddr + kTcAcol + 64 * s, al = ah + 32;
                const uint32_t bh = tc::smem_addr(smem + s * kTcStageBytes), bl = bh + kTcTileBytes;
#pragma unroll
                for (int k8 = 0; k8 < 4; ++k8) {
                    const uint32_t o = 32 * k8;  // 8 TF32 = 32 bytes along a K-major row
                    tc::mma_tf32_ta(acc, ah + 8 * k8, tc::desc_k_sw128(bh + o), idesc, (kc > 0 || k8 > 0) ? 1u : 0u);
                    tc::mma_tf32_ta(acc, ah + 8 * k8, tc::desc_k_sw128(bl + o), idesc, 1u);
                    tc::mma_tf32_ta(acc, al + 8 * k8, tc::desc_k_sw128(bh + o), idesc, 1u);
                }
                tc::mma_commit(&empty[s]);
                if (kc == nk - 1) tc::mma_commit(&accf);
                // The converters read raw stage q % kTcRaw before they arrived on full[s].
                if (q + kTcRaw < nslab) issue_raw(q + kTcRaw);
                if (++kc == nk) kc = 0, ++k;
            }
        }
        __syncwarp();
    } else if (warp < kTcIssuer) {
        int k = 0, kc = 0;
        TcWork wk = tc_work(g, 0);
        for (int q = 0; q < nslab; ++q) {
            const int s = q % kTcStages, rs = q % kTcRaw;
            // The MMAs of slab q - kTcStages read stage s.
            if (q >= kTcStages &&
                !tc::mbar_wait(&empty[s], (uint32_t)((q - kTcStages) / kTcStages) & 1, kTcWaitLimit))
                ok = false;
            if (!tc::mbar_wait(&rawbar[rs], (uint32_t)(q / kTcRaw) & 1, kTcWaitLimit)) ok = false;
            tc::fence_after_sync();
            const uint32_t ra = tc::smem_addr(raw0 + rs * kTcRawStage), rb = ra + kTcRawA;
            const uint32_t bh = tc::smem_addr(smem + s * kTcStageBytes), bl = bh + kTcTileBytes;
            // A' slab (rows r0..r0+127, complex columns 16 kc .. 16 kc + 15) into
            // tensor memory: warp w writes lanes 32 (w % 4) .. +31, K values
            // 16 (w / 4) .. +15 of one row per lane.  Logical 16-byte chunk c of
            // the row (complex columns 2c, 2c + 1) sits at chunk c ^ (row % 8).
            {
                const int wq = warp & 3, h = warp >> 2, rl = 32 * wq + lane;
                float hi[16], lo[16];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int c = 4 * h + i;
                    float4 x = lds128(ra + rl * 128 + 16 * (c ^ (rl & 7)));
                    if (g.a_minus_identity) {
                        const int dk = wk.r0 + rl - 16 * kc - 2 * c;
                        if (dk == 0) x.x -= 1.0f;
                        if (dk == 1) x.z -= 1.0f;
                    }
                    const float v[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        hi[4 * i + e] = tf32_rna(v[e]);
                        lo[4 * i + e] = tf32_rna(v[e] - hi[4 * i + e]);
                    }
                }
                const uint32_t ta = taddr + ((uint32_t)(32 * wq) << 16) + kTcAcol + 64 * s + 16 * h;
                tc::tmem_st16(ta, hi);
                tc::tmem_st16(ta + 32, lo);
            }
            // B''^T slab (rows n, 32 K values): task (n, c) writes K = 4c .. 4c + 3
            // of rows n and 128 + n from B rows 2c, 2c + 1 (raw rows of 1024 bytes).
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int t = tid + kTcConv * i, n = t & 127, c = t >> 7;
                const float2 v0 = lds64(rb + (uint32_t)((2 * c) * 128 + n) * 8);
                const float2 v1 = lds64(rb + (uint32_t)((2 * c + 1) * 128 + n) * 8);
                const uint32_t o_re = tc::sw128_offset(n, 4 * c), o_im = tc::sw128_offset(128 + n, 4 * c);
                put_split4(bh + o_re, bl + o_re, make_float4(v0.x, -v0.y, v1.x, -v1.y));
                put_split4(bh + o_im, bl + o_im, make_float4(v0.y, v0.x, v1.y, v1.x));
            }
            tc::tmem_wait_st();
            tc::fence_proxy_async();
            tc::fence_before_sync();
            tc_arrive(&full[s]);
            if (++kc == nk) kc = 0, wk = tc_work(g, ++k);
        }
        // Every raw copy was waited for in the loop; a wait that gave up is
        // tried once more so that no copy lands after the CTA has exited.
        if (!ok)
            for (int q = (nslab > kTcRaw ? nslab - kTcRaw : 0); q < nslab; ++q)
                tc::mbar_wait(&rawbar[q % kTcRaw], (uint32_t)(q / kTcRaw) & 1, kTcWaitLimit);
    } else {
        // Epilogue warps: warp w reads TMEM lanes 32 (w % 4) .. +31, one row of
        // the tile per lane, complex columns 64 h .. 64 h + 63 (h = (w - 9) / 4)
        // 16 at a time, and writes  C = alpha D + beta Cin + diag I  for its row
        // with 16-byte accesses.  The accumulator is released after the last
        // tensor-memory load, before the last stores.
        const int wq = warp & 3, h = (warp - kTcEpi) >> 2, rl = 32 * wq + lane;
        for (int k = 0; k < nunits; ++k) {
            const TcWork wk = tc_work(g, k);
            const int row = wk.r0 + rl, cb = wk.c0 + 64 * h;
            const float2 *Cin = g.Cin ? g.Cin + (size_t)wk.b * g.sCin + (size_t)row * d + cb : nullptr;
            float2 *Co = g.Cout + (size_t)wk.b * g.sCout + (size_t)row * d + cb;
            // This thread's 512 bytes of Cin move to L2 while the unit's MMAs run,
            // so that the loads between the accumulator's arrival and release hit L2.
            if (Cin)
#pragma unroll
                for (int i = 0; i < 4; ++i) asm volatile("prefetch.global.L2 [%0];" ::"l"(Cin + 16 * i));
            if (!tc::mbar_wait(&accf, (uint32_t)k & 1, kTcWaitLimit)) ok = false;
            tc::fence_after_sync();
            const uint32_t acc = taddr + ((uint32_t)(32 * wq) << 16) + 64 * h;
#pragma unroll 1
            for (int cc = 0; cc < 4; ++cc) {
                float4 ci[8];
#pragma unroll
                for (int jj = 0; jj < 8; ++jj)
                    ci[jj] = Cin ? *reinterpret_cast<const float4 *>(Cin + 16 * cc + 2 * jj)
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
                float re[16], im[16];
                tc::tmem_ld16(acc + 16 * cc, re);
                tc::tmem_ld16(acc + 128 + 16 * cc, im);
                if (cc == 3) {
                    tc::fence_before_sync();
                    tc_arrive(&acce);
                }
#pragma unroll
                for (int jj = 0; jj < 8; ++jj) {
                    const int col = cb + 16 * cc + 2 * jj;
                    const float xr = re[2 * jj], xi = im[2 * jj], yr = re[2 * jj + 1], yi = im[2 * jj + 1];
                    float4 o = make_float4(g.alpha.x * xr - g.alpha.y * xi, g.alpha.x * xi + g.alpha.y * xr,
                                           g.alpha.x * yr - g.alpha.y * yi, g.alpha.x * yi + g.alpha.y * yr);
                    o.x = fmaf(g.beta, ci[jj].x, o.x);
                    o.y = fmaf(g.beta, ci[jj].y, o.y);
                    o.z = fmaf(g.beta, ci[jj].z, o.z);
                    o.w = fmaf(g.beta, ci[jj].w, o.w);
                    o.x = fmaf(-g.beta_im, ci[jj].y, o.x);
                    o.y = fmaf(g.beta_im, ci[jj].x, o.y);
                    o.z = fmaf(-g.beta_im, ci[jj].w, o.z);
                    o.w = fmaf(g.beta_im, ci[jj].z, o.w);
                    if (row == col) o.x += g.diag.x, o.y += g.diag.y;
                    if (row == col + 1) o.z += g.diag.x, o.w += g.diag.y;
                    if (ok) *reinterpret_cast<float4 *>(Co + 16 * cc + 2 * jj) = o;
                }
            }
        }
    }
    if (!ok) atomicAdd(g.fault ? g.fault : &g_tc_faults, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == kTcIssuer) {
        tc::fence_after_sync();
        tc::tmem_dealloc(taddr, kTcTmemCols);
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
    return !l.fp64 && !l.simt_only && l.d >= 256 && l.d % 128 == 0 && !tc_disabled() && aligned16(l.A, l.strideA) &&
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
    g.beta_im = (float)l.beta_im;
    g.d = l.d;
    g.batch = l.batch;
    g.tiles_n = l.d / 128;
    g.a_minus_identity = l.a_minus_identity ? 1 : 0;
    g.fault = l.fault;
    if (!make_map(&g.tmA, l.A, l.d, l.strideA, l.batch, 32, 128, CU_TENSOR_MAP_SWIZZLE_128B, &g.batchedA) ||
        !make_map(&g.tmB, l.B, l.d, l.strideB, l.batch, 256, 16, CU_TENSOR_MAP_SWIZZLE_NONE, &g.batchedB))
        return cudaErrorInvalidValue;
    const size_t smem = kTcSmem;
    cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void *>(&k_tc_cgemm),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    // Persistent grid: one CTA per SM walks the (tile, item) units.
    const long long units = (long long)(l.d / 128) * (l.d / 128) * l.batch;
    const int sms = l.num_sms > 0 ? l.num_sms : 148;
    const int grid = (int)std::min<long long>(units, sms);
    k_tc_cgemm<<<grid, kTcThreads, smem, l.stream>>>(g);
    return cudaGetLastError();
}

}  // namespace pgb
