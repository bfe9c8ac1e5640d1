// Sliced complex products with exact accumulation on the tcgen05 tensor cores.
//
// A product C = A B of two 64 x 64 complex matrices is computed from bf16
// slices of integers: every row r of A is scaled by 2^(7 - ea_r) and every
// column n of B by 2^(7 - eb_n) (ea, eb the exponents of the row / column
// maxima), and the scaled values are peeled into slices
//     t = sum_s q_s 2^(-8 s),   q_s integers in [-128, 128]
// (round to nearest at every peel, so the truncation is unbiased).  Products
// of slices are integers of at most 2^14; K = 128 of them sum to at most 2^21,
// and the products of one level L = s + t (at most four) to at most 2^23, so
// the FP32 accumulators in tensor memory hold every level exactly.  The
// epilogue forms C = 2^(ea_r + eb_n - 14) sum_L 2^(-8 L) D_L.  With S slices
// and levels up to S - 1, C is exact up to about 2^(-8 S) of the row / column
// scales; S = 4 goes well beyond FP32, S = 2 is enough for small terms.
//
// Real formulation (M = 128 rows, N = 64 columns, K = 128):
//     [C_r; C_i] = [[A_r, -A_i], [A_i, A_r]] [B_r; B_i]
// The A operand of one slice is stored as three 64-row blocks [-A_i][A_r][A_i]
// so that the first K half reads [A_r; A_i] and the second [-A_i; A_r] as one
// contiguous 128-row operand each.  B is stored K-major as [B_r^T | B_i^T].
// All blocks are 64 rows x 64 bf16 (128 bytes) with the 128-byte swizzle.
// Swapping the two K halves' A blocks and negating the second gives i*C.
// B may instead be stored MN-major: rows k of [B_r; B_i] (128 of them) with
// the 64 columns contiguous, the natural row-major layout, so that a thread
// holding 8 consecutive columns of one row writes them with one 16-byte store.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "tc.cuh"

namespace pgb {
namespace oz {

constexpr int kBlk = 8192;            // one 64 x 64 bf16 block
constexpr int kASlice = 3 * kBlk;     // [-A_i][A_r][A_i]
constexpr int kBSlice = 2 * kBlk;     // [B_r^T][B_i^T]
constexpr int kMaxSlices = 4;

// Byte offset of bf16 element (row, k) in a 128-byte-swizzled K-major block.
__device__ __forceinline__ uint32_t sw(int row, int k) {
    return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((((k >> 3) ^ row) & 7) << 4) + ((k & 7) << 1));
}

// kind::f16 instruction descriptor: BF16 x BF16 -> FP32, A K-major, M = 128,
// N columns (a multiple of 16 up to 256); bit 13 negates A, bit 16 selects an
// MN-major B.
__host__ __device__ constexpr uint32_t idesc_bf16(bool negate_a, bool b_mn = false, int N = 64) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((negate_a ? 1u : 0u) << 13) | ((b_mn ? 1u : 0u) << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

// Shared-memory descriptor of an MN-major operand with the 128-byte swizzle:
// 64 bf16 of N per swizzle atom, 1024 bytes between groups of eight K rows
// (stride byte offset), and `atom_stride` bytes from one atom of 64 N columns
// to the next (leading byte offset; unused when N = 64).
__device__ __forceinline__ uint64_t desc_mn_sw128(uint32_t saddr, uint32_t atom_stride = 16u) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((atom_stride >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Where the B slices of a product sit: slice t at sb + t * stride, its K half
// 0 (rows 0..63 of [B_r; B_i]) at + h0 and K half 1 at + h1, each a 64 x 64
// block stored K-major ([B^T] rows) or MN-major ([B] rows).
struct BLayout {
    uint32_t stride, h0, h1;
    bool mn;
};
// B slices of their own: [B_r][B_i] blocks per slice, MN-major or K-major.
constexpr BLayout kBSlicesMn = {(uint32_t)kBSlice, 0u, (uint32_t)kBlk, true};
constexpr BLayout kBSlicesK = {(uint32_t)kBSlice, 0u, (uint32_t)kBlk, false};
// B = A^H for a Hermitian operand A: B^T = conj(A), so the K-major blocks
// B_r^T = A_r and B_i^T = -A_i are copies of A's [A_r] and [-A_i] blocks, and
// A's row scales are B's column scales.  The copies are written as two
// stacks, slice after slice: the [A_r] blocks from sb on and the [-A_i]
// blocks from sb + h1 (stackable along N).
__host__ __device__ constexpr BLayout herm_stacks(uint32_t h1) { return {(uint32_t)kBlk, 0u, h1, false}; }

// Issues the MMAs of one sliced product (one thread).  Slices s < sa_n of A
// at sa (kASlice bytes each) and t < sb_n of B at sb (laid out as bl says);
// level L = s + t <= lmax accumulates at tmem column d_tmem + 64 L.  With
// imag set the product is i * A * B.
__device__ __forceinline__ void issue_product(uint32_t d_tmem, uint32_t sa, uint32_t sb, int sa_n, int sb_n,
                                              int lmax, bool imag, BLayout bl = kBSlicesK) {
    const bool b_mn = bl.mn;
    const uint32_t id_pos = idesc_bf16(false, b_mn), id_neg = idesc_bf16(true, b_mn);
    // B address of K chunk kk (16 K values) within one K half: 32 bytes along
    // a K-major row, or 16 rows of 128 bytes MN-major.
    const uint32_t b_step = b_mn ? 2048u : 32u;
    uint32_t started = 0;
    for (int s = 0; s < sa_n; ++s) {
        for (int t = 0; t < sb_n; ++t) {
            const int L = s + t;
            if (L > lmax) continue;
            const uint32_t d = d_tmem + 64u * (uint32_t)L;
            const uint32_t a = sa + (uint32_t)s * kASlice, b = sb + (uint32_t)t * bl.stride;
            // K half 0: A' columns 0..63 = [A_r; A_i] (i*A: [-A_i; A_r]), B rows 0..63 = B_r.
            const uint32_t a0 = imag ? a : a + kBlk;
            // K half 1: [-A_i; A_r] (i*A: -[A_r; A_i]), B rows 64..127 = B_i.
            const uint32_t a1 = imag ? a + kBlk : a;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const uint32_t bb = b + bl.h0 + b_step * kk;
                mma_bf16(d, tc::desc_k_sw128(a0 + 32u * kk), b_mn ? desc_mn_sw128(bb) : tc::desc_k_sw128(bb), id_pos,
                         ((started >> L) & 1u) | (kk > 0 ? 1u : 0u));
            }
            started |= 1u << L;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const uint32_t bb = b + bl.h1 + b_step * kk;
                mma_bf16(d, tc::desc_k_sw128(a1 + 32u * kk), b_mn ? desc_mn_sw128(bb) : tc::desc_k_sw128(bb),
                         imag ? id_neg : id_pos, 1u);
            }
        }
    }
}

// Whether issue_product_stacked can stack the B slices of layout bl along N:
// MN-major slices (one swizzle atom of N each, bl.stride apart: the leading
// byte offset), or K-major slices whose 64-row blocks follow each other
// (stride kBlk: the 8-row groups stay 1024 bytes apart across slices).
__host__ __device__ constexpr bool stackable(BLayout bl) { return bl.mn || bl.stride == (uint32_t)kBlk; }

// The same product with the B slices stacked along N: for A slice s, chains
// of MMAs with N = 64 n (n <= 4 B slices, N <= 256) cover B slices
// t = 0 .. n_t - 1, n_t = min(sb_n, lmax - s + 1), and write levels s + t at
// their tensor-memory columns d_tmem + 64 (s + t), which are contiguous.  A is
// read once per chain instead of once per slice pair: the N = 64 products are
// bound by the shared-memory operand reads (6 KB per MMA).  With lmax < sb_n
// the chains of slice s = 0 cover every level; with `fresh` they start them
// (first MMA of each without accumulate), otherwise they add to what the
// levels hold.  Per level the sums are those of issue_product, in the same
// order; other shapes and layouts go to issue_product.
__device__ __forceinline__ void issue_product_stacked(uint32_t d_tmem, uint32_t sa, uint32_t sb, int sa_n, int sb_n,
                                                      int lmax, bool imag, bool fresh = true,
                                                      BLayout bl = kBSlicesMn) {
    if ((lmax >= sb_n && fresh) || !stackable(bl)) {
        issue_product(d_tmem, sa, sb, sa_n, sb_n, lmax, imag, bl);
        return;
    }
    const uint32_t b_step = bl.mn ? 2048u : 32u;
    for (int s = 0; s < sa_n; ++s) {
        const int nt = min(sb_n, lmax - s + 1);
        const uint32_t a = sa + (uint32_t)s * kASlice;
        const uint32_t a0 = imag ? a : a + kBlk;
        const uint32_t a1 = imag ? a + kBlk : a;
        for (int t0 = 0; t0 < nt; t0 += 4) {
            const int n = min(4, nt - t0);
            const uint32_t id_pos = idesc_bf16(false, bl.mn, 64 * n), id_neg = idesc_bf16(true, bl.mn, 64 * n);
            const uint32_t d = d_tmem + 64u * (uint32_t)(s + t0);
            const uint32_t b = sb + (uint32_t)t0 * bl.stride;
            const uint32_t first = (s == 0 && fresh) ? 0u : 1u;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const uint32_t bb = b + bl.h0 + b_step * kk;
                mma_bf16(d, tc::desc_k_sw128(a0 + 32u * kk), bl.mn ? desc_mn_sw128(bb, bl.stride) : tc::desc_k_sw128(bb),
                         id_pos, kk > 0 ? 1u : first);
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const uint32_t bb = b + bl.h1 + b_step * kk;
                mma_bf16(d, tc::desc_k_sw128(a1 + 32u * kk), bl.mn ? desc_mn_sw128(bb, bl.stride) : tc::desc_k_sw128(bb),
                         imag ? id_neg : id_pos, 1u);
            }
        }
    }
}

// Exponent e with |v| < 2^e for every |v| <= m (0 for m == 0).
__device__ __forceinline__ int scale_exp(float m) {
    int e = 0;
    if (m > 0.0f) frexpf(m, &e);
    return e;
}

// Peels 8 scaled values (already multiplied by 2^(7 - e)) into up to S
// slices; q[s][j] receives slice s of value j.  (t - r) * 256 is exact, so one
// fused multiply-add forms it.
template <int S>
__device__ __forceinline__ void peel8(float (&t)[8], float (&q)[S][8]) {
#pragma unroll
    for (int s = 0; s < S; ++s)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float r = rintf(t[j]);
            q[s][j] = r;
            t[j] = __fmaf_rn(t[j], 256.0f, -256.0f * r);
        }
}

__device__ __forceinline__ uint4 pack8(const float (&v)[8]) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
        w[i] = *reinterpret_cast<uint32_t *>(&h);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// The same eight bf16 values negated (sign bits flipped).
__device__ __forceinline__ uint4 neg8(uint4 v) {
    return make_uint4(v.x ^ 0x80008000u, v.y ^ 0x80008000u, v.z ^ 0x80008000u, v.w ^ 0x80008000u);
}

// Stores slices of 8 consecutive elements (row, k0..k0+7) of a real plane into
// the A operand: plane 0 -> block A_r, plane 1 -> blocks A_i and -A_i.
// k0 must be a multiple of 8.
template <int S>
__device__ __forceinline__ void store_a8(unsigned char *sa, int row, int k0, int plane, const float (&q)[S][8]) {
    const uint32_t off = sw(row, k0);
#pragma unroll
    for (int s = 0; s < S; ++s) {
        unsigned char *base = sa + s * kASlice;
        const uint4 v = pack8(q[s]);
        if (plane == 0) {
            *reinterpret_cast<uint4 *>(base + kBlk + off) = v;
        } else {
            *reinterpret_cast<uint4 *>(base + 2 * kBlk + off) = v;
            *reinterpret_cast<uint4 *>(base + off) = neg8(v);
        }
    }
}

// Stores slices of 8 consecutive rows k0..k0+7 of column n of plane `plane`
// of B into B^T (row n, K index 64 * plane + k).
template <int S>
__device__ __forceinline__ void store_b8(unsigned char *sb, int n, int k0, int plane, const float (&q)[S][8]) {
    const uint32_t off = sw(n, k0) + (uint32_t)plane * kBlk;
#pragma unroll
    for (int s = 0; s < S; ++s) *reinterpret_cast<uint4 *>(sb + s * kBSlice + off) = pack8(q[s]);
}

}  // namespace oz
}  // namespace pgb
