// Split-precision form of the equiprop path for complex64 contexts, d <= 64.
//
// Why: over tens of thousands of steps, any rounding that repeats identically
// at every step (the float copies of H0, of 2/Hnorm, of the Bessel
// coefficients) adds up coherently; in plain complex64 that alone costs ~1e-4
// relative error.  Here the step exponential is written U_j = I + E_j and the
// Chebyshev-Bessel polynomial of the reference (the same coefficients
// (-i)^k J_k(x), src/cuda/mathhelper.cpp:69-80) is regrouped by powers of X_j:
//
//   E_j = (m_0 - 1) I + mu_1 X + mu_2 X^2 + X (mu_3 X^2 + mu_5 X^4 + ...) + mu_4 X^4 + ...
//
// with mu_n = m_n / Hnorm^n and m_n the monomial coefficients of
// J_0 + 2 sum_k (-i)^k J_k(x) T_k(t).  The first- and second-order terms
// (|mu_1 X| ~ Hnorm dt, |mu_2 X^2| ~ (Hnorm dt)^2) are formed in double-float
// (pairs of floats), X itself accumulated in double-float from FP64 weights
// and the complex64 expansion stack; X^2 uses
// the three products hi*hi + hi*lo + lo*hi; the higher orders, whose size is
// below 1e-5 of the result, stay in FP32.  Each CTA multiplies its chunk of
// consecutive steps into E^P (P = I + E^P) held in double-float, adding the
// FP32 product E_j E^P; the chunk products are then combined by the FP64 tree.
//
// The Chebyshev order is the smallest odd M >= 3 whose truncation, summed over
// all P steps (2 P |J_(M+1)(x)|), stays below 1e-9; x = Hnorm * dt_eff must
// not exceed 0.5 so that the regrouped polynomial has no cancellation.
#include <math.h>
#include <stdlib.h>

#include <algorithm>
#include <vector>

#include "ctx.h"
#include "kernels.h"
#include "split_common.cuh"

namespace pgb {

// acc = A * B (+ A2 * B2 when TWO) over the thread's micro-tile.
template <int TM, bool TWO>
__device__ __forceinline__ void tile_gemm_f(float2 (&acc)[TM][TM], const float2 *__restrict__ A,
                                            const float2 *__restrict__ B, const float2 *__restrict__ A2,
                                            const float2 *__restrict__ B2, int d, int ld, int ty, int tx) {
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TM; ++j) acc[i][j] = make_float2(0.f, 0.f);
    int ro[TM], co[TM];
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        ro[i] = min(ty + 16 * i, d - 1) * ld;
        co[i] = min(tx + 16 * i, d - 1);
    }
#pragma unroll 4
    for (int k = 0; k < d; ++k) {
        float2 av[TM], bv[TM];
#pragma unroll
        for (int i = 0; i < TM; ++i) av[i] = A[ro[i] + k];
#pragma unroll
        for (int j = 0; j < TM; ++j) bv[j] = B[k * ld + co[j]];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j) cfma(acc[i][j], av[i], bv[j]);
        if (TWO) {
#pragma unroll
            for (int i = 0; i < TM; ++i) av[i] = A2[ro[i] + k];
#pragma unroll
            for (int j = 0; j < TM; ++j) bv[j] = B2[k * ld + co[j]];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) cfma(acc[i][j], av[i], bv[j]);
        }
    }
}


template <int TM>
__global__ void __launch_bounds__(256, 1) k_split_steps(const __grid_constant__ SplitArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // Shared-memory matrices use row stride ld = d + 1 (bank-conflict free A reads).
    const int d = a.d, dd = d * d, ld = d + 1, sz = d * ld;
    float2 *Xh = reinterpret_cast<float2 *>(smem_raw);  // X hi
    float2 *Xl = Xh + sz;                               // X lo, later Q (odd part)
    float2 *G2 = Xl + sz;                               // X^2, later E hi
    float2 *Gc = G2 + sz;                               // X^(2k)
    float2 *Ph = Gc + sz;                               // E^P hi
    float2 *Pl = Ph + sz;                               // E^P lo
    float4 *ws = reinterpret_cast<float4 *>(Pl + sz);   // step weights (re_hi, re_lo, im_hi, im_lo)
    __shared__ float2 muf[kSplitMaxOrder + 1];          // mu_n rounded to float (orders >= 3)
    if (threadIdx.x <= kSplitMaxOrder) muf[threadIdx.x] = make_float2((float)a.mu[threadIdx.x].x, (float)a.mu[threadIdx.x].y);
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const long long s0 = a.P * blockIdx.x / a.nchunks;
    const long long s1 = a.P * (blockIdx.x + 1) / a.nchunks;
    const int M = a.M;

    int eo[TM][TM];
    bool own[TM][TM], dg[TM][TM];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TM; ++j) {
            int r = ty + 16 * i, c = tx + 16 * j;
            own[i][j] = r < d && c < d;
            eo[i][j] = r * ld + c;
            dg[i][j] = r == c;
        }
    const cdf mu1 = {df_from(a.mu[1].x), df_from(a.mu[1].y)};
    const cdf mu2 = {df_from(a.mu[2].x), df_from(a.mu[2].y)};
    const cdf c0 = {df_from(a.c0.x), df_from(a.c0.y)};

    cdf E[TM][TM];
    float2 acc[TM][TM], Q[TM][TM];
    for (long long st = s0; st < s1; ++st) {
        for (int m = tid; m < a.Ke; m += blockDim.x) {
            double2 w = split_weight(a, m, st);
            df re = df_from(w.x), im = df_from(w.y);
            ws[m] = make_float4(re.hi, re.lo, im.hi, im.lo);
        }
        __syncthreads();
        // X = H0 + sum_m w_m H_m in double-float; E starts as (m_0-1) I + mu_1 X.
        // X = H0 + sum_m w_m H_m.  The matrices are complex64 (H0 and H_k are
        // the caller's complex64 inputs, exact; the Magnus commutators are
        // formed in FP64 and rounded).  Control slots (< K) carry FP64 weights
        // as float pairs and accumulate in double-float; the commutator slots
        // carry weights of order dt |du| and accumulate in FP32 -- their
        // rounding is far below the error bar even when it repeats at every
        // step.  The loop runs matrix by matrix so that a thread's loads of
        // one matrix are independent and in flight together.
        {
            cdf xa[TM][TM];
            float2 sa[TM][TM];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) {
                    float2 h = own[i][j] ? a.stack[(ty + 16 * i) * d + tx + 16 * j] : make_float2(0.f, 0.f);
                    xa[i][j] = cdf{{h.x, 0.f}, {h.y, 0.f}};
                    sa[i][j] = make_float2(0.f, 0.f);
                }
            for (int m = 0; m < a.Ke; ++m) {
                const float2 *Hm = a.stack + (size_t)(m + 1) * dd;
                const float4 w = ws[m];
                float2 g[TM][TM];
#pragma unroll
                for (int i = 0; i < TM; ++i)
#pragma unroll
                    for (int j = 0; j < TM; ++j)
                        g[i][j] = own[i][j] ? Hm[(ty + 16 * i) * d + tx + 16 * j] : make_float2(0.f, 0.f);
                if (m < a.K) {
                    const cdf wd = {{w.x, w.y}, {w.z, w.w}};
#pragma unroll
                    for (int i = 0; i < TM; ++i)
#pragma unroll
                        for (int j = 0; j < TM; ++j) xa[i][j] = cdf_add(xa[i][j], cdf_mul_c(wd, g[i][j]));
                } else {
                    const float2 wf = make_float2(w.x, w.z);
#pragma unroll
                    for (int i = 0; i < TM; ++i)
#pragma unroll
                        for (int j = 0; j < TM; ++j) cfma(sa[i][j], wf, g[i][j]);
                }
            }
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) {
                    if (!own[i][j]) continue;
                    const int e = eo[i][j];
                    const cdf x = cdf_add_c(xa[i][j], sa[i][j]);
                    Xh[e] = cdf_hi(x);
                    Xl[e] = cdf_lo(x);
                    cdf v = cdf_mul(mu1, x);
                    if (dg[i][j]) v = cdf_add(v, c0);
                    E[i][j] = v;
                }
        }
        __syncthreads();
        // G2 = X^2 = Xh Xh + (Xh Xl + Xl Xh).
        tile_gemm_f<TM, false>(acc, Xh, Xh, nullptr, nullptr, d, ld, ty, tx);
        {
            float2 cr[TM][TM];
            tile_gemm_f<TM, true>(cr, Xh, Xl, Xl, Xh, d, ld, ty, tx);
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) acc[i][j] = make_float2(acc[i][j].x + cr[i][j].x, acc[i][j].y + cr[i][j].y);
        }
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j) {
                if (!own[i][j]) continue;
                E[i][j] = cdf_add(E[i][j], cdf_mul_c(mu2, acc[i][j]));
                Q[i][j] = (M >= 3) ? cmul(muf[3], acc[i][j]) : make_float2(0.f, 0.f);
                G2[eo[i][j]] = acc[i][j];
                Gc[eo[i][j]] = acc[i][j];
            }
        __syncthreads();
        // Higher even powers X^(2k) = X^(2k-2) X^2 in FP32.
        for (int k = 2; 2 * k <= M; ++k) {
            tile_gemm_f<TM, false>(acc, Gc, G2, nullptr, nullptr, d, ld, ty, tx);
            __syncthreads();
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) {
                    if (!own[i][j]) continue;
                    E[i][j] = cdf_add_c(E[i][j], cmul(muf[2 * k], acc[i][j]));
                    if (2 * k + 1 <= M) {
                        float2 q = cmul(muf[2 * k + 1], acc[i][j]);
                        Q[i][j] = make_float2(Q[i][j].x + q.x, Q[i][j].y + q.y);
                    }
                    Gc[eo[i][j]] = acc[i][j];
                }
            __syncthreads();
        }
        // Odd part X * Q.
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j)
                if (own[i][j]) Xl[eo[i][j]] = Q[i][j];
        __syncthreads();
        tile_gemm_f<TM, false>(acc, Xh, Xl, nullptr, nullptr, d, ld, ty, tx);
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j) {
                if (!own[i][j]) continue;
                E[i][j] = cdf_add_c(E[i][j], acc[i][j]);
            }
        // Running product: E^P <- E^P + E + E E^P.
        if (st == s0) {
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j)
                    if (own[i][j]) {
                        Ph[eo[i][j]] = cdf_hi(E[i][j]);
                        Pl[eo[i][j]] = cdf_lo(E[i][j]);
                    }
            __syncthreads();
        } else {
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j)
                    if (own[i][j]) G2[eo[i][j]] = cdf_hi(E[i][j]);
            __syncthreads();
            tile_gemm_f<TM, false>(acc, G2, Ph, nullptr, nullptr, d, ld, ty, tx);
            __syncthreads();
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) {
                    if (!own[i][j]) continue;
                    const int e = eo[i][j];
                    float2 ph = Ph[e], pl = Pl[e];
                    cdf p = {{ph.x, pl.x}, {ph.y, pl.y}};
                    p = cdf_add(p, E[i][j]);
                    p = cdf_add_c(p, acc[i][j]);
                    Ph[e] = cdf_hi(p);
                    Pl[e] = cdf_lo(p);
                }
            __syncthreads();
        }
    }
    if (s1 > s0) {
        double2 *dst = a.chunks + (size_t)blockIdx.x * dd;
        for (int e = tid; e < dd; e += blockDim.x) {
            const int se = (e / d) * ld + e % d;
            float2 ph = Ph[se], pl = Pl[se];
            double re = (double)ph.x + (double)pl.x, im = (double)ph.y + (double)pl.y;
            if (e / d == e % d) re += 1.0;
            dst[e] = make_double2(re, im);
        }
    }
}

__global__ void k_c128_to_c64(const double2 *src, float2 *dst, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = make_float2((float)src[i].x, (float)src[i].y);
}

// The chunk products of the split form multiplied in order, in double-float.
// Each product keeps about 2^-44 relative.  FP64 runs at 1/64 of the FP32 rate
// on this GPU, and double-float is far more than the form's 1e-6 needs.
//
// Level: W_i = U_(2i) + (U_(2i+1) - I) U_(2i), with the later factor on the
// left (the pairing of src/cuda/parament.cpp:657-718).  An odd leftover moves
// to the end unchanged.  One CTA forms one 16 x 16 tile of one W_i; the CTAs
// of index `pairs` copy the leftover.  Elements are float4 (re hi, re lo,
// im hi, im lo); IN = double2 reads the complex128 chunk products of the step
// kernels.
__device__ __forceinline__ float4 to_df4(double2 v) {
    const df r = df_from(v.x), i = df_from(v.y);
    return make_float4(r.hi, r.lo, i.hi, i.lo);
}
__device__ __forceinline__ float4 to_df4(float4 v) { return v; }

// (hi, lo) += x y for double-float x, y, without renormalising: the product's
// rounding error joins lo with the rounding of the sum.
__device__ __forceinline__ void df_mac_dd(float &hi, float &lo, float xh, float xl, float yh, float yl) {
    const float p = __fmul_rn(xh, yh);
    float e = __fmaf_rn(xh, yh, -p);
    e = __fmaf_rn(xh, yl, e);
    e = __fmaf_rn(xl, yh, e);
    float s, t;
    two_sum(hi, p, s, t);
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(t, e));
}

template <class IN>
__global__ void __launch_bounds__(256) k_tree_df(const IN *__restrict__ in, float4 *__restrict__ out, int d,
                                                 long long pairs) {
    __shared__ float4 As[16][kSmallMaxDim + 1];  // rows r0..r0+15 of A - I
    __shared__ float4 Bs[kSmallMaxDim][17];      // columns c0..c0+15 of B
    const int tiles = (d + 15) / 16;
    const int r0 = (blockIdx.x / tiles) * 16, c0 = (blockIdx.x % tiles) * 16;
    const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15, r = r0 + ty, c = c0 + tx;
    const long long pr = blockIdx.y;
    const size_t dd = (size_t)d * d;
    if (pr == pairs) {  // the odd leftover
        if (r < d && c < d) out[pr * dd + (size_t)r * d + c] = to_df4(in[2 * pr * dd + (size_t)r * d + c]);
        return;
    }
    const IN *A = in + (2 * pr + 1) * dd, *B = in + 2 * pr * dd;
    for (int i = threadIdx.x; i < 16 * d; i += 256) {
        const int rr = r0 + i / d, k = i % d;
        float4 v = rr < d ? to_df4(A[(size_t)rr * d + k]) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (rr == k) {
            // A - I: the hi part of a diagonal entry near 1 loses the 1 exactly.
            const df t = df_add_f(df{v.x, v.y}, -1.0f);
            v.x = t.hi;
            v.y = t.lo;
        }
        As[i / d][k] = v;
    }
    for (int i = threadIdx.x; i < 16 * d; i += 256) {
        const int k = i / 16, cc = c0 + i % 16;
        Bs[k][i % 16] = cc < d ? to_df4(B[(size_t)k * d + cc]) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    if (r >= d || c >= d) return;
    const float4 b0 = to_df4(B[(size_t)r * d + c]);
    float rh = b0.x, rl = b0.y, ih = b0.z, il = b0.w;
    for (int k = 0; k < d; ++k) {
        const float4 a = As[ty][k], b = Bs[k][tx];
        df_mac_dd(rh, rl, a.x, a.y, b.x, b.y);
        df_mac_dd(rh, rl, -a.z, -a.w, b.z, b.w);
        df_mac_dd(ih, il, a.x, a.y, b.z, b.w);
        df_mac_dd(ih, il, a.z, a.w, b.x, b.y);
    }
    const df re = df_norm(rh, rl), im = df_norm(ih, il);
    out[pr * dd + (size_t)r * d + c] = make_float4(re.hi, re.lo, im.hi, im.lo);
}

__global__ void k_df_to_c64(const float4 *src, float2 *dst, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = make_float2(__fadd_rn(src[i].x, src[i].y), __fadd_rn(src[i].z, src[i].w));
}

// Product of n chunk products (complex128, in order of time) into the complex64
// output; bufa, bufb hold at least ceil(n / 2) d x d double-float matrices
// (bufa may be the chunk buffer itself).
static cudaError_t tree_df(int d, const double2 *chunks, long long n, float4 *bufa, float4 *bufb, float2 *out,
                           cudaStream_t stream, int *levels) {
    *levels = 0;
    const int dd = d * d, tiles = (d + 15) / 16;
    if (n == 1) {
        k_c128_to_c64<<<(dd + 255) / 256, 256, 0, stream>>>(chunks, out, dd);
        return cudaGetLastError();
    }
    long long remain = n;
    const float4 *cur = nullptr;
    float4 *dst = bufb;
    while (remain > 1) {
        const long long pairs = remain / 2;
        dim3 grid(tiles * tiles, (unsigned)(pairs + remain % 2));
        if (cur == nullptr)
            k_tree_df<double2><<<grid, 256, 0, stream>>>(chunks, dst, d, pairs);
        else
            k_tree_df<float4><<<grid, 256, 0, stream>>>(cur, dst, d, pairs);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        ++*levels;
        remain = pairs + remain % 2;
        cur = dst;
        dst = (dst == bufb) ? bufa : bufb;
    }
    k_df_to_c64<<<(dd + 255) / 256, 256, 0, stream>>>(cur, out, dd);
    return cudaGetLastError();
}

__global__ void k_c64_to_c128_chunks(const float2 *src, double2 *dst, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = make_double2(src[i].x, src[i].y);
}

cudaError_t tree_df_c64(int d, const float2 *chunks, long long n, void *buf128, void *bufb, float2 *out,
                        cudaStream_t stream, int *levels) {
    const long long m = (long long)d * d * n;
    k_c64_to_c128_chunks<<<(int)std::min<long long>(4096, (m + 255) / 256), 256, 0, stream>>>(
        chunks, static_cast<double2 *>(buf128), m);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = tree_df(d, static_cast<const double2 *>(buf128), n, static_cast<float4 *>(buf128), static_cast<float4 *>(bufb),
                out, stream, levels);
    *levels += 2;  // the conversions in and out
    return e;
}

// Complex64 stack from the FP64 stack (round to nearest).
__global__ void k_split_stack(const double2 *src, float2 *dst, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = make_float2((float)src[i].x, (float)src[i].y);
}
__global__ void k_c64_to_c128(const float2 *src, double2 *dst, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = make_double2(src[i].x, src[i].y);
}

static size_t split_smem(int d, int Ke) { return 6 * (size_t)d * (d + 1) * sizeof(float2) + (size_t)std::max(Ke, 1) * 16; }

template <int TM>
static const void *split_kernel_ptr() {
    return reinterpret_cast<const void *>(&k_split_steps<TM>);
}
static const void *pick_split(int d) {
    switch ((d + 15) / 16) {
        case 1: return split_kernel_ptr<1>();
        case 2: return split_kernel_ptr<2>();
        case 3: return split_kernel_ptr<3>();
        default: return split_kernel_ptr<4>();
    }
}

// ---------------------------------------------------------------- host side

int split_order(double hnorm, double h, long long P) {
    const double x = hnorm * h;
    if (!(x <= kSplitMaxX)) return -1;
    for (int M = 3; M <= kSplitMaxOrder; M += 2)
        if (2.0 * (double)P * fabs(jn(M + 1, x)) <= 1e-9) return M;
    return kSplitMaxOrder;
}

// Monomial coefficients m_n of J_0(x) + 2 sum_(k=1..M) (-i)^k J_k(x) T_k(t);
// returns mu_n = m_n / Hnorm^n (n >= 1) and c0 = m_0 - 1.
static void split_coefficients(int M, double x, double hnorm, double *c0, std::vector<double> &mu) {
    std::vector<double> J(2 * (M + 1));
    bessel_coeffs(M, x, J.data());
    std::vector<double> re(M + 1, 0.0), im(M + 1, 0.0);
    std::vector<double> tkm1(M + 1, 0.0), tk(M + 1, 0.0), tkp1(M + 1, 0.0);
    tkm1[0] = 1.0;  // T_0
    if (M >= 1) tk[1] = 1.0;  // T_1
    // m_0 - 1 computed without forming 1 + small - 1.
    double c0r = jn(0, x) - 1.0, c0i = 0.0;
    for (int k = 1; k <= M; ++k) {
        for (int n = 0; n <= M; ++n) {
            double t = 2.0 * tk[n];  // tk holds the monomial coefficients of T_k
            if (t == 0.0) continue;
            if (n == 0) {
                c0r += t * J[2 * k];
                c0i += t * J[2 * k + 1];
            } else {
                re[n] += t * J[2 * k];
                im[n] += t * J[2 * k + 1];
            }
        }
        // T_(k+1) = 2 t T_k - T_(k-1)
        for (int n = 0; n <= M; ++n) tkp1[n] = (n > 0 ? 2.0 * tk[n - 1] : 0.0) - tkm1[n];
        tkm1 = tk;
        tk = tkp1;
    }
    c0[0] = c0r;
    c0[1] = c0i;
    mu.assign(2 * (M + 1), 0.0);
    double scale = 1.0;
    for (int n = 1; n <= M; ++n) {
        scale /= hnorm;
        mu[2 * n] = re[n] * scale;
        mu[2 * n + 1] = im[n] * scale;
    }
}

// Builds the split form's stack: the complex64 inputs (exact), and the Magnus
// commutators recomputed in FP64 from them and rounded to complex64.
static Parament_ErrorCode prepare_split_stack(Ctx *c) {
    if (c->split_ready) return PARAMENT_STATUS_SUCCESS;
    const size_t dd = (size_t)c->dim * c->dim, n = dd * (1 + c->Ke);
    DevBuf tmp;
    if (tmp.ensure(n * sizeof(double2)) != cudaSuccess || c->split_stack.ensure(n * sizeof(float2)) != cudaSuccess) {
        tmp.release();
        return PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
    }
    double2 *s64 = static_cast<double2 *>(tmp.ptr);
    const float2 *s32 = static_cast<const float2 *>(c->stack.ptr);
    const unsigned K = c->K;
    const size_t base = c->magnus ? dd * (1 + K) : n;  // inputs: H0 and H_1..H_K
    k_c64_to_c128<<<256, 256, 0, c->stream>>>(s32, s64, (long long)base);
    cudaError_t e = cudaGetLastError();
    auto commutator = [&](size_t x, size_t y, size_t dst) -> cudaError_t {
        GemmLaunch g{};
        g.fp64 = true;
        g.d = (int)c->dim;
        g.batch = 1;
        g.A = s64 + dd * x;
        g.B = s64 + dd * y;
        g.Cout = s64 + dd * dst;
        g.alpha_re = 1.0;
        g.stream = c->stream;
        g.num_sms = c->num_sms;
        cudaError_t r = launch_gemm(g);
        if (r != cudaSuccess) return r;
        g.A = s64 + dd * y;
        g.B = s64 + dd * x;
        g.Cin = s64 + dd * dst;
        g.alpha_re = -1.0;
        g.beta = 1.0;
        return launch_gemm(g);
    };
    if (c->magnus) {
        for (unsigned k = 0; k < K && e == cudaSuccess; ++k) e = commutator(0, 1 + k, 1 + K + k);
        for (unsigned i = 1; i < K && e == cudaSuccess; ++i)
            for (unsigned j = 0; j < i && e == cudaSuccess; ++j)
                e = commutator(1 + j, 1 + i, 1 + 2 * K + i * (i - 1) / 2 + j);
    }
    if (e == cudaSuccess) {
        k_split_stack<<<512, 256, 0, c->stream>>>(s64, static_cast<float2 *>(c->split_stack.ptr), (long long)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    tmp.release();
    // Exact (anti-)Hermitian symmetry of the complex64 stack: H_0 and H_k
    // Hermitian, the commutator slots anti-Hermitian.  With real control
    // weights and imaginary commutator weights every X_j is then exactly
    // Hermitian, which the tensor-core kernel exploits.
    bool herm = true;
    if (e == cudaSuccess) {
        std::vector<float2> h(n);
        e = cudaMemcpy(h.data(), c->split_stack.ptr, n * sizeof(float2), cudaMemcpyDeviceToHost);
        const unsigned d = c->dim;
        for (size_t m = 0; e == cudaSuccess && herm && m < 1 + (size_t)c->Ke; ++m) {
            const float sg = m <= K ? 1.0f : -1.0f;  // +: Hermitian, -: anti-Hermitian
            const float2 *x = h.data() + m * dd;
            for (unsigned i = 0; herm && i < d; ++i)
                for (unsigned j = 0; j <= i; ++j) {
                    const float2 u = x[(size_t)i * d + j], v = x[(size_t)j * d + i];
                    if (!(u.x == sg * v.x && u.y == -sg * v.y)) {
                        herm = false;
                        break;
                    }
                }
        }
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return PARAMENT_STATUS_CUBLAS_FAILED;
    }
    c->split_herm = herm;
    c->split_ready = true;
    return PARAMENT_STATUS_SUCCESS;
}

Parament_ErrorCode run_split(Ctx *c, const void *d_carr, unsigned pts, unsigned amps, double h, int M, long long P,
                             void *d_out, cudaStream_t stream) {
    const int d = (int)c->dim;
    if (M > kSplitMaxOrder || c->hnorm * h > kSplitMaxX) return PARAMENT_STATUS_SELECT_SMALLER_DT;
    Parament_ErrorCode r = prepare_split_stack(c);
    if (r != PARAMENT_STATUS_SUCCESS) return r;
    SplitArgs a;
    double c0[2];
    std::vector<double> mu;
    split_coefficients(M, h * c->hnorm, c->hnorm, c0, mu);
    a.c0 = make_double2(c0[0], c0[1]);
    for (int n = 0; n <= kSplitMaxOrder; ++n)
        a.mu[n] = (n >= 1 && n <= M) ? make_double2(mu[2 * n], mu[2 * n + 1]) : make_double2(0, 0);
    a.stack = static_cast<const float2 *>(c->split_stack.ptr);
    a.carr = static_cast<const float2 *>(d_carr);
    a.P = P;
    a.d = d;
    a.Ke = (int)c->Ke;
    a.M = M;
    a.pts = pts;
    a.K = (int)c->K;
    a.amps = (int)amps;
    a.mode = c->quad;
    a.magnus = c->magnus ? 1 : 0;
    a.hfac = h / 12.0;
    a.fault = c->d_fault;
    // PARAMENT_SPLIT_HERMITIAN=0 turns the Hermitian-step shortcut of the
    // tensor-core kernel off (a test hook: the results are bit-identical).
    const char *hv = getenv("PARAMENT_SPLIT_HERMITIAN");
    a.herm_stack = (c->split_herm && !(hv && hv[0] == '0')) ? 1 : 0;
    a.wts = nullptr;
    a.xplanes = nullptr;
    a.chunks = nullptr;
    a.nchunks = 0;
    if (d > kSmallMaxDim) return run_split_large(c, a, h, d_out, stream);
    const size_t dd = (size_t)d * d;
    const bool tensor = split_tc_applies(d, (int)c->Ke, M);
    const void *fn = pick_split(d);
    const size_t smem = split_smem(d, (int)c->Ke);
    cudaError_t e = cudaSuccess;
    a.wts = nullptr;
    a.xplanes = nullptr;
    if (tensor) {
        // One CTA per SM (tensor-core kernel) per batch of steps; the step
        // weights go to a buffer of P x Ke double-float values first and the X
        // planes of a batch to a buffer of kSplitXBatch steps.
        const long long batches = (P + kSplitXBatch - 1) / kSplitXBatch;
        a.nchunks = (int)std::max<long long>(1, std::min<long long>((long long)c->num_sms * batches, P));
        if (c->wts.ensure(std::max<size_t>(16, sizeof(float4) * (size_t)P * c->Ke)) != cudaSuccess ||
            c->xplanes.ensure(sizeof(float) * kSplitXStride * (size_t)std::min<long long>(P, kSplitXBatch)) !=
                cudaSuccess)
            return PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
        a.wts = static_cast<const float4 *>(c->wts.ptr);
    } else {
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = 0;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, smem);
        if (e != cudaSuccess || per_sm < 1) {
            cudaGetLastError();
            return PARAMENT_STATUS_CUBLAS_FAILED;
        }
        a.nchunks = (int)std::max<long long>(1, std::min<long long>((long long)per_sm * c->num_sms, P));
    }
    if (c->chunks.ensure(sizeof(double2) * dd * a.nchunks) != cudaSuccess ||
        c->work.ensure(sizeof(double2) * dd * a.nchunks) != cudaSuccess ||
        c->aux.ensure(sizeof(double2) * dd) != cudaSuccess)
        return PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
    a.chunks = static_cast<double2 *>(c->chunks.ptr);
    if (tensor) {
        int nch = 0;
        e = launch_split_tc(a, c->num_sms, static_cast<float *>(c->xplanes.ptr), &nch, stream,
                            c->timing ? c->ev_start : nullptr, c->timing ? c->ev_stop : nullptr);
        a.nchunks = nch;
    } else {
        void *args[] = {&a};
        if (c->timing) cudaEventRecord(c->ev_start, stream);
        e = cudaLaunchKernel(fn, dim3(a.nchunks), dim3(256), args, smem, stream);
        if (c->timing) cudaEventRecord(c->ev_stop, stream);
    }
    int levels = 0;
    if (e == cudaSuccess)
        e = tree_df(d, static_cast<const double2 *>(c->chunks.ptr), a.nchunks, static_cast<float4 *>(c->chunks.ptr),
                    static_cast<float4 *>(c->work.ptr), static_cast<float2 *>(d_out), stream, &levels);
    // Step kernels (tensor form: step weights, then X planes and step kernel
    // per batch), the tree levels and the final conversion.
    const long long batches = (P + kSplitXBatch - 1) / kSplitXBatch;
    c->launches = (tensor ? (c->Ke > 0 ? 1 : 0) + 2 * (int)batches : 1) + levels + 1;
    if (e != cudaSuccess) {
        cudaGetLastError();
        return PARAMENT_STATUS_CUBLAS_FAILED;
    }
    return PARAMENT_STATUS_SUCCESS;
}

}  // namespace pgb
