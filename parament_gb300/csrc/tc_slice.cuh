// Shared pieces of the kernels that run 64 x 64 complex products as exact
// sliced bf16 products on the tcgen05 tensor cores inside one CTA (the split
// form, split_tc.cu; the plain complex64 form, small_tc.cu): the lane layout
// of the accumulators, row / column maxima, slicing into the A and B
// operands (ozaki.cuh), the hand-over of a product to the tensor core, the
// wait for it and the epilogue that combines its levels; bulk copies from
// global memory on an mbarrier.
//
// Thread (warp w, lane l) of the 512: tensor-memory lane rho = 32 (w % 4) + l,
// plane p = rho / 64 (0: real, 1: imaginary), matrix row r = rho % 64, columns
// c0 .. c0 + 15 with c0 = 16 (w / 4).  Warps w and w ^ 2 hold the two planes
// of the same elements.
#pragma once

#include "ozaki.cuh"
#include "split_common.cuh"

namespace pgb {

constexpr int kTcdThreads = 512;
constexpr int kTcdCols = 16;  // columns per thread
constexpr uint32_t kTcdWait = 1u << 24;

// Bulk copy global -> shared memory completing on an mbarrier (transaction
// count), and the arrival that announces the bytes to expect.
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     tc::smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(tc::smem_addr(bar))
                 : "memory");
}


// Column maxima of a warp: v[j] holds this lane's value of column j; on
// return v[0] holds the maximum over the 32 lanes of column lane % 16.
__device__ __forceinline__ void warp_column_max(float (&v)[16], int lane) {
#pragma unroll
    for (int o = 8; o >= 1; o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < o; ++i) {
            const float send = upper ? v[i] : v[i + o];
            const float keep = upper ? v[i + o] : v[i];
            v[i] = fmaxf(keep, __shfl_xor_sync(0xffffffffu, send, o));
        }
    }
    v[0] = fmaxf(v[0], __shfl_xor_sync(0xffffffffu, v[0], 16));
}

// Peels scaled double-float values t = hi + lo (|t| < 128) into S slices.
template <int S>
__device__ __forceinline__ void peel8_df(const float (&hi)[8], const float (&lo)[8], float (&q)[S][8]) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float r0 = rintf(hi[j]);
        q[0][j] = r0;
        float t = ((hi[j] - r0) + lo[j]) * 256.0f;
#pragma unroll
        for (int s = 1; s < S; ++s) {
            const float r = rintf(t);
            q[s][j] = r;
            t = __fmaf_rn(t, 256.0f, -256.0f * r);
        }
    }
}

struct TcdShared {
    int amax[2][64], bmax[2][64];
    float rowmul[64], colmul[64];  // 2^(e - 7) of the last A rows / B columns
    float rowmul_x[64];            // the same for the A slices of X (X^2 and X Q)
    float colmul_p[64];            // column scales of the running product's B (E^P)
    uint64_t bar;                  // tensor-core products
    uint64_t hbar, lbar;           // bulk copies of the X planes (hi pair, lo pair)
    uint32_t tmem_base;
};

// Per-thread view of the CTA: the lane layout above, and the tensor-memory
// addresses of this thread's columns (product levels, E^P / P, E).
struct TcdThread {
    int tid, lane, p, r, c0, cb;
    uint32_t tm_acc, tm_ep, tm_e;
};

// Operand slicing.  reduce_max() posts this thread's row maximum of the A
// values and (HAS_B) column maxima of the B values; after one barrier,
// store_a() / store_b() write the slices.  `b` selects the max
// buffer; the other buffer is cleared for the next product.
template <bool HAS_A, bool HAS_B>
__device__ __forceinline__ void reduce_max(TcdShared &sh, const TcdThread &t, int b, const float (&a)[16],
                                           const float (&bv)[16]) {
    if (HAS_A) {
        float m = 0.0f;
#pragma unroll
        for (int j = 0; j < 16; ++j) m = fmaxf(m, fabsf(a[j]));
        atomicMax(&sh.amax[b][t.r], __float_as_int(m));
    }
    if (HAS_B) {
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = fabsf(bv[j]);
        warp_column_max(v, t.lane);
        if (t.lane < 16) atomicMax(&sh.bmax[b][t.c0 + t.lane], __float_as_int(v[0]));
    }
    __syncthreads();
    if (t.tid < 64) {
        sh.amax[b ^ 1][t.tid] = 0;
        sh.bmax[b ^ 1][t.tid] = 0;
    }
}

// Scale that brings values of magnitude below the maximum m (float bits) under
// 128: 2^(7 - e) with m < 2^e, from the exponent field alone (maxima below
// 2^-100, zero included, are treated as 2^-100).
__device__ __forceinline__ float scale_of(int mbits) {
    return __int_as_float((260 << 23) - (max(mbits, 27 << 23) & 0x7F800000));
}
// Its inverse 2^(e - 7), the factor the epilogue applies.
__device__ __forceinline__ float unscale_of(int mbits) {
    return __int_as_float((max(mbits, 27 << 23) & 0x7F800000) - (6 << 23));
}

// With SETCOL the row scales also become the column scales (colmul): the
// product's B is this A's conjugate transpose, read from the same slices.
// With BSTACK the [A_r] and [-A_i] blocks are also written as two stacks,
// slice after slice, at bt0 and bt1: the K-major B^T of a Hermitian operand
// in the layout that stacks along N (ozaki.cuh, herm_stacks).
template <int S, bool DF, bool SETCOL = false, bool BSTACK = false>
__device__ __forceinline__ void store_a(TcdShared &sh, unsigned char *SA, const TcdThread &t, int b,
                                        const float (&hi)[16], const float (&lo)[16], unsigned char *bt0 = nullptr,
                                        unsigned char *bt1 = nullptr) {
    const int mb = sh.amax[b][t.r];
    if (t.p == 0 && t.cb == 0) {
        sh.rowmul[t.r] = unscale_of(mb);
        if (SETCOL) sh.colmul[t.r] = unscale_of(mb);
    }
    const float sc = scale_of(mb);
#pragma unroll
    for (int g = 0; g < 2; ++g) {
        float q[S][8];
        float th[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) th[j] = hi[8 * g + j] * sc;
        if (DF) {
            float tl[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) tl[j] = lo[8 * g + j] * sc;
            peel8_df<S>(th, tl, q);
        } else {
            oz::peel8<S>(th, q);
        }
        if (BSTACK) {
            const uint32_t off = oz::sw(t.r, t.c0 + 8 * g);
#pragma unroll
            for (int s = 0; s < S; ++s) {
                const uint4 v = oz::pack8(q[s]);
                unsigned char *base = SA + s * oz::kASlice;
                if (t.p == 0) {
                    *reinterpret_cast<uint4 *>(base + oz::kBlk + off) = v;
                    *reinterpret_cast<uint4 *>(bt0 + s * oz::kBlk + off) = v;
                } else {
                    const uint4 nv = oz::neg8(v);
                    *reinterpret_cast<uint4 *>(base + 2 * oz::kBlk + off) = v;
                    *reinterpret_cast<uint4 *>(base + off) = nv;
                    *reinterpret_cast<uint4 *>(bt1 + s * oz::kBlk + off) = nv;
                }
            }
        } else {
            oz::store_a8<S>(SA, t.r, t.c0 + 8 * g, t.p, q);
        }
    }
}

// B slices, MN-major: row r of plane p is K row 64 p + r of [B_r; B_i], the
// thread's 16 columns are contiguous within it.
// `cmax` holds the column maxima (float bits): sh.bmax of the product, or,
// for a Hermitian B, sh.amax (its row maxima, the same numbers).
template <int S, bool DF>
__device__ __forceinline__ void store_b(unsigned char *SB, const TcdThread &t, const int *cmax,
                                        const float (&hi)[16], const float (&lo)[16], float *colmul) {
    if (t.p == 0 && t.r < 16) colmul[t.c0 + t.lane] = unscale_of(cmax[t.c0 + t.lane]);
    const int k = 64 * t.p + t.r;
    const int4 *cm = reinterpret_cast<const int4 *>(cmax + t.c0);
#pragma unroll
    for (int g = 0; g < 2; ++g) {
        const int4 m0 = cm[2 * g], m1 = cm[2 * g + 1];
        const float sc[8] = {scale_of(m0.x), scale_of(m0.y), scale_of(m0.z), scale_of(m0.w),
                             scale_of(m1.x), scale_of(m1.y), scale_of(m1.z), scale_of(m1.w)};
        float th[8], q[S][8];
#pragma unroll
        for (int j = 0; j < 8; ++j) th[j] = hi[8 * g + j] * sc[j];
        if (DF) {
            float tl[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) tl[j] = lo[8 * g + j] * sc[j];
            peel8_df<S>(th, tl, q);
        } else {
            oz::peel8<S>(th, q);
        }
        const uint32_t off = oz::sw(k, t.c0 + 8 * g);
#pragma unroll
        for (int s = 0; s < S; ++s) *reinterpret_cast<uint4 *>(SB + s * oz::kBSlice + off) = oz::pack8(q[s]);
    }
}

// Makes the slices visible to the tensor core and issues one sliced product.
// `ok` carries this thread's result of the previous wait; the barrier before
// the issue combines it over the CTA, and a product is issued only if every
// earlier wait succeeded (returns false otherwise, in every thread).
__device__ __forceinline__ bool issue_sliced(TcdShared &sh, const TcdThread &t, unsigned char *SA, unsigned char *SB,
                                             int sa_n, int sb_n, int lmax, bool imag, bool ok,
                                             oz::BLayout bl = oz::kBSlicesMn) {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    const bool all_ok = __syncthreads_and(ok) != 0;
    tc::fence_after_sync();
    if (!all_ok) return false;
    if (t.tid == 0) {
        oz::issue_product_stacked(sh.tmem_base, tc::smem_addr(SA), tc::smem_addr(SB), sa_n, sb_n, lmax, imag, true,
                                  bl);
        tc::mma_commit(&sh.bar);
    }
    return true;
}
// Waits for the product issued last.
__device__ __forceinline__ void wait_sliced(TcdShared &sh, uint32_t &ncommit, bool &ok) {
    ok = tc::mbar_wait(&sh.bar, ncommit & 1, kTcdWait);
    ++ncommit;
    tc::fence_after_sync();
}
__device__ __forceinline__ bool run_product(TcdShared &sh, const TcdThread &t, unsigned char *SA, unsigned char *SB,
                                            int sa_n, int sb_n, int lmax, bool imag, uint32_t &ncommit, bool &ok,
                                            oz::BLayout bl = oz::kBSlicesMn) {
    if (!issue_sliced(sh, t, SA, SB, sa_n, sb_n, lmax, imag, ok, bl)) return false;
    wait_sliced(sh, ncommit, ok);
    return true;
}

// TMEM -> registers, 32 lanes x 16 columns (no wait).
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Loads the levels of the last product for this thread's 16 columns and
// combines them in FP32: v_j = 2^(e_r - 7) 2^(e_c - 7) sum_L 2^(-8 L) D_L.
template <int LMAX>
__device__ __forceinline__ void epilogue_f(const TcdShared &sh, const TcdThread &t, float (&out)[16]) {
    float lv[LMAX + 1][16];
#pragma unroll
    for (int L = 0; L <= LMAX; ++L) tmem_ld16_nowait(t.tm_acc + 64 * L, lv[L]);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    const float rm = sh.rowmul[t.r];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        float v = lv[LMAX][j];
#pragma unroll
        for (int L = LMAX - 1; L >= 0; --L) v = fmaf(v, 0.00390625f, lv[L][j]);
        out[j] = v * (rm * sh.colmul[t.c0 + j]);
    }
}

// TMEM -> registers, 32 lanes x 8 columns (no wait).
__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// E^P of this thread (16 columns, double-float) from / to tensor memory.
__device__ __forceinline__ void load_ep(uint32_t taddr, float (&hi)[16], float (&lo)[16]) {
    tc::tmem_ld16(taddr, hi);
    tc::tmem_ld16(taddr + 16, lo);
}
__device__ __forceinline__ void store_ep(uint32_t taddr, const float (&hi)[16], const float (&lo)[16]) {
    tc::tmem_st16(taddr, hi);
    tc::tmem_st16(taddr + 16, lo);
    tc::tmem_wait_st();
}

}  // namespace pgb
