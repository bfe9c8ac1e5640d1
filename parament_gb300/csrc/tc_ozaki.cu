// Exact sliced complex64 GEMM for large d on the tcgen05 tensor cores.
//
//   C_b = alpha * A_b B_b + beta * Cin_b + diag * I       (d x d, row-major)
//
// For the products that must not carry a rounding bias (the split form for
// d > 64, split_large.cu).  The 3xTF32 kernel (tc_gemm.cu) accumulates in the
// tensor core's FP32 adder, whose rounding we measured to bias the split form
// past its 1e-6 bar; here every partial sum the tensor core forms is an
// integer below 2^24, so it is exact whatever the adder's rounding:
//
//   * Every row of A and every column of B is scaled by a power of two into
//     (-32, 32) (pre-pass k_oz_scales: the row / column maxima over the whole
//     K), and peeled into five 6-bit integer slices (round to nearest at every
//     peel): x 2^(5 - e) = sum_s q_s 64^(-s), |q_s| <= 32.
//   * Slice products of level L = s + t <= 4 accumulate in their own FP32
//     accumulator (tensor memory columns 64 L .. 64 L + 63).  One product
//     term is at most 2^10; a level holds at most five slice products over
//     K = 128 real terms per 64-column block of K and d / 64 blocks, so its
//     sums stay below 5 * 2^17 d / 64 <= 2^24 for d <= 1536.
//   * The epilogue forms 2^(e_r + e_c - 10) sum_L 64^(-L) D_L in FP32 (round
//     to nearest) and C = alpha D + beta Cin + diag I.
// The slices carry 30 bits of each operand relative to its row / column
// maximum, and the levels dropped (s + t >= 5) are below 2^-30 of the row and
// column scales: the product is FP32-rounded once, in the epilogue.  With
// four slices and levels <= 3 (2^-24, dropped cross terms that repeat from
// one step to the next) the split form measured 5.7e-6 after 8192 steps at
// d = 512, against 6.5e-7 on the FP32 SIMT kernel.
//
// Layout (ozaki.cuh): the complex product of one 64 x 64 output block over a
// K block of 64 complex columns is the real-stacked M = 128, N = 64, K = 128
// product [[A_r, -A_i], [A_i, A_r]] [B_r; B_i]: the A slices as the K-major
// blocks [-A_i][A_r][A_i], the B slices MN-major (rows k of [B_r; B_i]).  Re C
// lands in tensor-memory lanes 0..63, Im C in 64..127.
//
// One CTA of 512 threads per SM walks the (item, block row, block column)
// units; per K block every thread loads 8 complex values of A and of B (one
// row, 8 columns), slices them into shared memory, and one thread issues the
// 15 slice products as 6 chains of 8 MMAs (the B slices of one A slice stacked
// along N, ozaki.cuh); the next K block's values are loaded while those run.
// Every wait on the tensor core is bounded.
#include <stdlib.h>

#include <algorithm>

#include "kernels.h"
#include "ozaki.cuh"

namespace pgb {

constexpr int kOzThreads = 512;
constexpr int kOzSlices = 5;
constexpr uint32_t kOzWait = 1u << 24;
constexpr size_t kOzSA = (size_t)kOzSlices * oz::kASlice;  // 120 KB
constexpr size_t kOzSB = (size_t)kOzSlices * oz::kBSlice;  // 80 KB
constexpr size_t kOzSmem = kOzSA + kOzSB + 1024;
constexpr int kOzMaxDim = 1536;
static_assert(kOzSmem + 64 <= 232448, "shared memory of k_oz_cgemm exceeds 227 KB");
// The epilogue stages the 64 x 64 complex block in the A slice buffer.
static_assert(64 * 65 * 8 <= kOzSA, "staging exceeds the A slice buffer");

// Bounded waits that gave up, for launches without a context's counter.
__device__ int g_oz_faults;

struct OzArgs {
    const float2 *A, *B, *Cin;
    float2 *Cout;
    long long sA, sB, sCin, sCout;
    const int *ea, *eb;  // exponents of the row maxima of A / column maxima of B (per operand item)
    float2 alpha, diag;
    float beta, beta_im;
    int d, batch, nblk;
    int *fault;
};

// Exponent e with |v| < 2^e for every |v| <= m; maxima below 2^-100
// (zero included) count as 2^-100.
__device__ __forceinline__ int oz_exp(float m) {
    int e = -100;
    if (m >= 7.8886e-31f) frexpf(m, &e);
    return e;
}

// Row maxima of A (over all columns, both planes) and column maxima of B,
// as exponents, for every operand item.  Block (x, item): one warp per row of
// A; then the block's threads over the columns of B.
__global__ void k_oz_scales(const float2 *A, long long sA, int nA, const float2 *B, long long sB, int nB, int d,
                            int *ea, int *eb) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int item = blockIdx.y;
    if (item < nA) {
        const float2 *a = A + (size_t)item * sA;
        for (int r = blockIdx.x * nw + warp; r < d; r += gridDim.x * nw) {
            float m = 0.0f;
            for (int c = lane; c < d; c += 32) {
                const float2 v = a[(size_t)r * d + c];
                m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) ea[(size_t)item * d + r] = oz_exp(m);
        }
    }
    if (item < nB) {
        const float2 *b = B + (size_t)item * sB;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < d; c += gridDim.x * blockDim.x) {
            float m = 0.0f;
            for (int k = 0; k < d; ++k) {
                const float2 v = b[(size_t)k * d + c];
                m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
            }
            eb[(size_t)item * d + c] = oz_exp(m);
        }
    }
}

// 2^n for an integer n in the normal range.
__device__ __forceinline__ float oz_pow2(int n) { return __int_as_float((n + 127) << 23); }

// Peels 8 scaled values (|t| < 32) into kOzSlices 6-bit slices.
__device__ __forceinline__ void oz_peel(float (&t)[8], float (&q)[kOzSlices][8]) {
#pragma unroll
    for (int s = 0; s < kOzSlices; ++s)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float r = rintf(t[j]);
            q[s][j] = r;
            t[j] = __fmaf_rn(t[j], 64.0f, -64.0f * r);
        }
}

// Eight complex values of a row-major matrix: row `row`, columns col0 ..
// col0 + 7 (64 contiguous bytes; eight threads cover a row of a K block, so a
// warp reads four rows of 512 bytes), split into the two planes.
__device__ __forceinline__ void oz_load8(const float2 *m, int d, int row, int col0, float (&re)[8], float (&im)[8]) {
    const float4 *p = reinterpret_cast<const float4 *>(m + (size_t)row * d + col0);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float4 x = __ldg(p + i);
        re[2 * i] = x.x;
        im[2 * i] = x.y;
        re[2 * i + 1] = x.z;
        im[2 * i + 1] = x.w;
    }
}

__device__ __forceinline__ void oz_ld16(uint32_t taddr, float (&v)[16]) {
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

__global__ void __launch_bounds__(kOzThreads, 1) k_oz_cgemm(const __grid_constant__ OzArgs g) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((1024u - (tc::smem_addr(smem_raw) & 1023u)) & 1023u);
    unsigned char *SA = smem;
    unsigned char *SB = smem + kOzSA;
    float2 *stage = reinterpret_cast<float2 *>(SA);  // 64 x 65 complex, after the last MMA of a unit
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_base;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int q4 = warp & 3, cb = warp >> 2;
    const int p = q4 >> 1;                   // plane: 0 real, 1 imaginary
    const int r = 32 * (q4 & 1) + lane;      // row of the 64 x 64 block
    const int c0 = 16 * cb;                  // first of this thread's 16 columns
    const int d = g.d, nblk = g.nblk;

    if (warp == 0) {
        tc::tmem_alloc(&tmem_base, 512);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tm = tmem_base + ((uint32_t)(32 * q4) << 16) + (uint32_t)c0;

    bool ok = true;
    uint32_t ncommit = 0;
    const long long nunits = (long long)g.batch * nblk * nblk;
    for (long long u = blockIdx.x; u < nunits && ok; u += gridDim.x) {
        const int b = (int)(u / ((long long)nblk * nblk));
        const int rem = (int)(u % ((long long)nblk * nblk));
        const int I = rem / nblk, J = rem % nblk;
        const int ia = g.sA > 0 ? b : 0, ib = g.sB > 0 ? b : 0;
        const float2 *A = g.A + (size_t)ia * g.sA;
        const float2 *B = g.B + (size_t)ib * g.sB;
        // Slicing: thread (lr, lg) takes row lr of the K block of A (and of B),
        // complex columns 8 lg .. 8 lg + 7, both planes.
        const int lr = tid >> 3, lg = tid & 7;
        const float sa = oz_pow2(5 - g.ea[(size_t)ia * d + I * 64 + lr]);
        float sb[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) sb[j] = oz_pow2(5 - g.eb[(size_t)ib * d + J * 64 + 8 * lg + j]);
        float ar[8], ai[8], br[8], bi[8];
        oz_load8(A, d, I * 64 + lr, 8 * lg, ar, ai);
        oz_load8(B, d, lr, J * 64 + 8 * lg, br, bi);
        for (int kb = 0; kb < nblk; ++kb) {
            // Slices of this K block into shared memory.
            {
                float t[8], q[kOzSlices][8];
#pragma unroll
                for (int j = 0; j < 8; ++j) t[j] = ar[j] * sa;
                oz_peel(t, q);
                oz::store_a8<kOzSlices>(SA, lr, 8 * lg, 0, q);
#pragma unroll
                for (int j = 0; j < 8; ++j) t[j] = ai[j] * sa;
                oz_peel(t, q);
                oz::store_a8<kOzSlices>(SA, lr, 8 * lg, 1, q);
#pragma unroll
                for (int j = 0; j < 8; ++j) t[j] = br[j] * sb[j];
                oz_peel(t, q);
                uint32_t off = oz::sw(lr, 8 * lg);
#pragma unroll
                for (int s = 0; s < kOzSlices; ++s)
                    *reinterpret_cast<uint4 *>(SB + s * oz::kBSlice + off) = oz::pack8(q[s]);
#pragma unroll
                for (int j = 0; j < 8; ++j) t[j] = bi[j] * sb[j];
                oz_peel(t, q);
                off = oz::sw(64 + lr, 8 * lg);
#pragma unroll
                for (int s = 0; s < kOzSlices; ++s)
                    *reinterpret_cast<uint4 *>(SB + s * oz::kBSlice + off) = oz::pack8(q[s]);
            }
            tc::fence_proxy_async();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
            if (tid == 0) {
                // Levels s + t <= 4, the B slices of each A slice stacked along
                // N; the first K block starts every level.
                oz::issue_product_stacked(tmem_base, tc::smem_addr(SA), tc::smem_addr(SB), kOzSlices, kOzSlices,
                                          kOzSlices - 1, false, kb == 0);
                tc::mma_commit(&bar);
            }
            // The next K block's values load while the tensor core runs.
            if (kb + 1 < nblk) {
                oz_load8(A, d, I * 64 + lr, (kb + 1) * 64 + 8 * lg, ar, ai);
                oz_load8(B, d, (kb + 1) * 64 + lr, J * 64 + 8 * lg, br, bi);
            }
            ok = tc::mbar_wait(&bar, ncommit & 1, kOzWait);
            ++ncommit;
            tc::fence_after_sync();
            ok = __syncthreads_and(ok) != 0;
            if (!ok) break;
        }
        if (!ok) break;
        // Epilogue: levels combined, unscaled, staged as a complex block.
        {
            float lv[kOzSlices][16];
#pragma unroll
            for (int L = 0; L < kOzSlices; ++L) oz_ld16(tm + 64u * L, lv[L]);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const int era = g.ea[(size_t)ia * d + I * 64 + r];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                float v = lv[kOzSlices - 1][j];
#pragma unroll
                for (int L = kOzSlices - 2; L >= 0; --L) v = __fmaf_rn(v, 0.015625f, lv[L][j]);
                const int e = era + g.eb[(size_t)ib * d + J * 64 + c0 + j] - 10;
                // 2^e in two factors, so that neither leaves the normal range.
                v = v * oz_pow2(e / 2) * oz_pow2(e - e / 2);
                float *sp = reinterpret_cast<float *>(stage + r * 65 + c0 + j);
                sp[p] = v;
            }
        }
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        {
            const float2 *Cin = g.Cin ? g.Cin + (size_t)b * g.sCin : nullptr;
            float2 *Co = g.Cout + (size_t)b * g.sCout;
            for (int e = tid; e < 64 * 64; e += kOzThreads) {
                const int rr = e >> 6, cc = e & 63;
                const float2 dv = stage[rr * 65 + cc];
                const size_t gi = (size_t)(I * 64 + rr) * d + J * 64 + cc;
                float2 o = make_float2(g.alpha.x * dv.x - g.alpha.y * dv.y, g.alpha.x * dv.y + g.alpha.y * dv.x);
                if (Cin) {
                    const float2 ci = Cin[gi];
                    o.x = fmaf(g.beta, ci.x, o.x);
                    o.y = fmaf(g.beta, ci.y, o.y);
                    o.x = fmaf(-g.beta_im, ci.y, o.x);
                    o.y = fmaf(g.beta_im, ci.x, o.y);
                }
                if (I * 64 + rr == J * 64 + cc) o.x += g.diag.x, o.y += g.diag.y;
                Co[gi] = o;
            }
        }
        __syncthreads();  // the staging buffer is the next unit's A slice buffer
    }
    if (!ok) {
        if (tid == 0) atomicAdd(g.fault ? g.fault : &g_oz_faults, 1);
        // Let the MMAs still in flight finish before tensor memory is freed.
        if (ncommit > 0) tc::mbar_wait(&bar, (ncommit - 1) & 1, kOzWait);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem_base, 512);
    }
}

static bool oz_disabled() {
    static const bool off = [] {
        const char *v = getenv("PARAMENT_DISABLE_TENSOR_CORES");
        return v && v[0] && v[0] != '0';
    }();
    return off;
}

bool oz_gemm_applies(const GemmLaunch &l) {
    auto al = [](const void *ptr, long long stride) {
        return ptr == nullptr || ((reinterpret_cast<uintptr_t>(ptr) & 15) == 0 && (stride & 1) == 0 && stride >= 0);
    };
    return !l.fp64 && !l.a_minus_identity && !oz_disabled() && l.d >= 128 && l.d % 64 == 0 && l.d <= kOzMaxDim &&
           al(l.A, l.strideA) && al(l.B, l.strideB) && al(l.Cin, l.strideCin) && al(l.Cout, l.strideCout);
}

cudaError_t launch_oz_gemm(const GemmLaunch &l, int *scales) {
    OzArgs g;
    g.A = static_cast<const float2 *>(l.A);
    g.B = static_cast<const float2 *>(l.B);
    g.Cin = static_cast<const float2 *>(l.Cin);
    g.Cout = static_cast<float2 *>(l.Cout);
    g.sA = l.batch > 1 ? l.strideA : 0;
    g.sB = l.batch > 1 ? l.strideB : 0;
    g.sCin = l.strideCin;
    g.sCout = l.strideCout;
    g.alpha = make_float2((float)l.alpha_re, (float)l.alpha_im);
    g.diag = make_float2((float)l.diag_re, (float)l.diag_im);
    g.beta = (float)l.beta;
    g.beta_im = (float)l.beta_im;
    g.d = l.d;
    g.batch = l.batch;
    g.nblk = l.d / 64;
    g.fault = l.fault;
    const int nA = g.sA > 0 ? l.batch : 1, nB = g.sB > 0 ? l.batch : 1;
    g.ea = scales;
    g.eb = scales + (size_t)nA * l.d;
    k_oz_scales<<<dim3((unsigned)std::max(1, std::min(l.d / 8, 64)), (unsigned)std::max(nA, nB)), 256, 0, l.stream>>>(
        g.A, g.sA, nA, g.B, g.sB, nB, l.d, scales, scales + (size_t)nA * l.d);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(reinterpret_cast<const void *>(&k_oz_cgemm), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kOzSmem);
    if (e != cudaSuccess) return e;
    const long long units = (long long)l.batch * g.nblk * g.nblk;
    const int grid = (int)std::min<long long>(units, l.num_sms > 0 ? l.num_sms : 148);
    k_oz_cgemm<<<grid, kOzThreads, kOzSmem, l.stream>>>(g);
    return cudaGetLastError();
}

size_t oz_scale_ints(const GemmLaunch &l) {
    const size_t nA = l.batch > 1 && l.strideA > 0 ? l.batch : 1, nB = l.batch > 1 && l.strideB > 0 ? l.batch : 1;
    return (nA + nB) * (size_t)l.d;
}

}  // namespace pgb
