// Batched complex GEMM with a fused Clenshaw epilogue, the pairwise tree
// product, and the large-d plain path built on them.
//
// C_b = alpha * A_b B_b + beta * Cin_b + diag * I  (row-major d x d)
//
// Replaces the reference's cublasGgemmStridedBatched calls plus the separate
// diagonal-add kernels (src/cuda/parament.cpp:596-643, src/cuda/diagonal_add.cu:21-51)
// and its tree product (src/cuda/parament.cpp:657-718).  Tiles of BT x BT
// outputs per CTA (BT = 64, 32 or 16, picked so the grid covers the SMs),
// 16-deep k slabs staged in shared memory, 256 threads with (BT/16)^2
// accumulators each.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace pgb {

template <class R>
struct GemmArgs {
    const cplx_t<R> *A, *B, *Cin;
    cplx_t<R> *Cout;
    long long sA, sB, sCin, sCout;
    cplx_t<R> alpha, diag;
    R beta, beta_im;
    int d, batch, tiles_per_row;
    int a_minus_identity;  // load A - I instead of A
};

template <class R, int BT>
__global__ void __launch_bounds__(256) k_gemm(const __grid_constant__ GemmArgs<R> g) {
    using C = cplx_t<R>;
    constexpr int TMi = BT / 16;
    constexpr int BK = 16;
    __shared__ C As[BT][BK + 1];
    __shared__ C Bs[BK][BT];
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const int d = g.d;
    const int tile = blockIdx.x;
    const int r0 = (tile / g.tiles_per_row) * BT, c0 = (tile % g.tiles_per_row) * BT;
    for (int b = blockIdx.y; b < g.batch; b += gridDim.y) {
        const C *A = g.A + (size_t)b * g.sA;
        const C *B = g.B + (size_t)b * g.sB;
        C acc[TMi][TMi];
#pragma unroll
        for (int i = 0; i < TMi; ++i)
#pragma unroll
            for (int j = 0; j < TMi; ++j) acc[i][j] = mk<C>(0.0, 0.0);
        for (int k0 = 0; k0 < d; k0 += BK) {
            for (int t = tid; t < BT * BK; t += 256) {
                int i = t / BK, kk = t % BK;
                int r = r0 + i, k = k0 + kk;
                C v = (r < d && k < d) ? A[(size_t)r * d + k] : mk<C>(0.0, 0.0);
                if (g.a_minus_identity && r == k && r < d) v.x -= (R)1;
                As[i][kk] = v;
            }
            for (int t = tid; t < BT * BK; t += 256) {
                int kk = t / BT, j = t % BT;
                int k = k0 + kk, c = c0 + j;
                Bs[kk][j] = (k < d && c < d) ? B[(size_t)k * d + c] : mk<C>(0.0, 0.0);
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < BK; ++kk) {
                C a[TMi], bb[TMi];
#pragma unroll
                for (int i = 0; i < TMi; ++i) a[i] = As[ty + 16 * i][kk];
#pragma unroll
                for (int j = 0; j < TMi; ++j) bb[j] = Bs[kk][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < TMi; ++i)
#pragma unroll
                    for (int j = 0; j < TMi; ++j) cfma(acc[i][j], a[i], bb[j]);
            }
            __syncthreads();
        }
        const C *Cin = g.Cin ? g.Cin + (size_t)b * g.sCin : nullptr;
        C *Co = g.Cout + (size_t)b * g.sCout;
#pragma unroll
        for (int i = 0; i < TMi; ++i)
#pragma unroll
            for (int j = 0; j < TMi; ++j) {
                int r = r0 + ty + 16 * i, c = c0 + tx + 16 * j;
                if (r >= d || c >= d) continue;
                size_t e = (size_t)r * d + c;
                C v = cmul(g.alpha, acc[i][j]);
                if (Cin) {
                    C o = Cin[e];
                    v.x = fma(g.beta, o.x, v.x);
                    v.y = fma(g.beta, o.y, v.y);
                    v.x = fma(-g.beta_im, o.y, v.x);
                    v.y = fma(g.beta_im, o.x, v.y);
                }
                if (r == c) v = cadd(v, g.diag);
                Co[e] = v;
            }
    }
}

template <class R, int BT>
static cudaError_t run_gemm(const GemmLaunch &l) {
    using C = cplx_t<R>;
    GemmArgs<R> g;
    g.A = static_cast<const C *>(l.A);
    g.B = static_cast<const C *>(l.B);
    g.Cin = static_cast<const C *>(l.Cin);
    g.Cout = static_cast<C *>(l.Cout);
    g.sA = l.strideA;
    g.sB = l.strideB;
    g.sCin = l.strideCin;
    g.sCout = l.strideCout;
    g.alpha = mk<C>(l.alpha_re, l.alpha_im);
    g.diag = mk<C>(l.diag_re, l.diag_im);
    g.beta = (R)l.beta;
    g.beta_im = (R)l.beta_im;
    g.d = l.d;
    g.batch = l.batch;
    g.tiles_per_row = (l.d + BT - 1) / BT;
    g.a_minus_identity = l.a_minus_identity ? 1 : 0;
    dim3 grid(g.tiles_per_row * g.tiles_per_row, std::min(l.batch, 65535));
    k_gemm<R, BT><<<grid, 256, 0, l.stream>>>(g);
    return cudaGetLastError();
}

cudaError_t launch_gemm(const GemmLaunch &l) {
    if (l.batch <= 0) return cudaSuccess;
    if (l.d < 1) return cudaErrorInvalidValue;
    if (l.exact && l.scales && oz_gemm_applies(l)) return launch_oz_gemm(l, l.scales);
    if (!l.exact && tc_gemm_applies(l)) return launch_tc_gemm(l);
    // Largest tile that still gives two CTAs per SM; small products get small tiles.
    auto tiles = [&](int bt) { long long t = (l.d + bt - 1) / bt; return t * t * (long long)l.batch; };
    int bt = 16;
    if (tiles(64) >= 2LL * l.num_sms) bt = 64;
    else if (tiles(32) >= 2LL * l.num_sms) bt = 32;
    if (l.fp64) {
        if (bt == 64) return run_gemm<double, 64>(l);
        if (bt == 32) return run_gemm<double, 32>(l);
        return run_gemm<double, 16>(l);
    }
    if (bt == 64) return run_gemm<float, 64>(l);
    if (bt == 32) return run_gemm<float, 32>(l);
    return run_gemm<float, 16>(l);
}

cudaError_t tree_product(bool fp64, int d, void *in, long long n, void *work, void *out, cudaStream_t stream,
                         int num_sms, int *levels, int *fault) {
    if (levels) *levels = 0;
    const size_t es = fp64 ? 16 : 8;
    const long long dd = (long long)d * d;
    char *cur = static_cast<char *>(in), *nxt = static_cast<char *>(work);
    long long remain = n;
    while (remain > 1) {
        long long pairs = remain / 2;
        GemmLaunch g{};
        g.fp64 = fp64;
        g.d = d;
        g.batch = (int)pairs;
        // W_i = U_(2i+1) U_(2i) (the later factor on the left), formed as
        // U_(2i) + (U_(2i+1) - I) U_(2i) so that near-identity factors do not
        // round their small terms against the unit diagonal.
        g.A = cur + dd * es;
        g.strideA = 2 * dd;
        g.a_minus_identity = true;
        g.B = cur;
        g.strideB = 2 * dd;
        g.Cin = cur;
        g.strideCin = 2 * dd;
        g.beta = 1.0;
        g.Cout = nxt;
        g.strideCout = dd;
        g.alpha_re = 1.0;
        g.stream = stream;
        g.num_sms = num_sms;
        g.fault = fault;
        cudaError_t e = launch_gemm(g);
        if (e != cudaSuccess) return e;
        if (levels) ++*levels;
        if (remain % 2) {
            e = cudaMemcpyAsync(nxt + pairs * dd * es, cur + 2 * pairs * dd * es, dd * es, cudaMemcpyDeviceToDevice,
                                stream);
            if (e != cudaSuccess) return e;
        }
        remain = pairs + remain % 2;
        std::swap(cur, nxt);
    }
    if (out != cur) return cudaMemcpyAsync(out, cur, dd * es, cudaMemcpyDeviceToDevice, stream);
    return cudaSuccess;
}

// ---------------------------------------------------------------- large-d path

template <class R>
struct AssembleArgs {
    cplx_t<R> JM, JM1;
    const cplx_t<R> *stack, *carr;
    cplx_t<R> *X, *B1, *B2;
    long long s0;
    int count, d, Ke, M;
    R s;
    WeightSpec w;
};

// X_g = H0 + sum_m w_m(s0+g) H_m, and the first Clenshaw terms
// B2 = b_M = J[M] I, B1 = b_(M-1) = s J[M] X + J[M-1] I (or U for M = 1).
template <class R>
__global__ void __launch_bounds__(256) k_assemble(const __grid_constant__ AssembleArgs<R> a) {
    using C = cplx_t<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *ws = reinterpret_cast<C *>(smem_raw);
    const int g = blockIdx.y;
    const long long st = a.s0 + g;
    for (int m = threadIdx.x; m < a.Ke; m += blockDim.x) ws[m] = step_weight(a.carr, a.w, m, st);
    __syncthreads();
    const long long dd = (long long)a.d * a.d;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < dd; e += (long long)gridDim.x * blockDim.x) {
        C v = a.stack[e];
        for (int m = 0; m < a.Ke; ++m) cfma(v, ws[m], a.stack[(size_t)(m + 1) * dd + e]);
        const bool dg = (e / a.d) == (e % a.d);
        a.X[g * dd + e] = v;
        C b1 = cscale(cmul(a.JM, v), a.s);
        if (dg) b1 = cadd(b1, a.JM1);
        a.B1[g * dd + e] = b1;
        if (a.M > 1) a.B2[g * dd + e] = dg ? a.JM : mk<C>(0.0, 0.0);
    }
}

template <class R>
static cudaError_t run_large(const LargeLaunch &l, int *launches) {
    using C = cplx_t<R>;
    const size_t es = sizeof(C);
    const long long dd = (long long)l.d * l.d;
    long long nb = 0;
    for (long long b0 = l.s0; b0 < l.s1; b0 += l.batch, ++nb) {
        const int cnt = (int)std::min<long long>(l.batch, l.s1 - b0);
        AssembleArgs<R> a;
        a.JM = mk<C>(l.J[2 * l.M], l.J[2 * l.M + 1]);
        a.JM1 = mk<C>(l.J[2 * (l.M - 1)], l.J[2 * (l.M - 1) + 1]);
        a.stack = static_cast<const C *>(l.stack);
        a.carr = static_cast<const C *>(l.carr);
        a.X = static_cast<C *>(l.X);
        a.B1 = static_cast<C *>(l.B1);
        a.B2 = static_cast<C *>(l.B2);
        a.s0 = b0;
        a.count = cnt;
        a.d = l.d;
        a.Ke = l.Ke;
        a.M = l.M;
        a.s = (R)l.s;
        a.w = WeightSpec{l.w.pts, l.w.K, l.w.amps, l.w.mode, l.w.magnus, l.w.hfac};
        int bx = (int)std::min<long long>((dd + 255) / 256, 1024);
        k_assemble<R><<<dim3(bx, cnt), 256, es * std::max(1, l.Ke), l.stream>>>(a);
        cudaError_t e = cudaGetLastError();
        if (launches) *launches += 1;
        if (e != cudaSuccess) return e;
        void *b1 = l.B1, *b2 = l.B2;
        for (int k = l.M - 2; k >= 0; --k) {
            GemmLaunch g{};
            g.fp64 = l.fp64;
            g.d = l.d;
            g.batch = cnt;
            g.A = b1;
            g.strideA = dd;
            g.B = l.X;
            g.strideB = dd;
            g.Cin = b2;
            g.strideCin = dd;
            g.Cout = b2;
            g.strideCout = dd;
            g.alpha_re = l.s;
            g.beta = (k == 0) ? -2.0 : -1.0;
            g.diag_re = l.J[2 * k];
            g.diag_im = l.J[2 * k + 1];
            g.stream = l.stream;
            g.num_sms = l.num_sms;
            g.fault = l.fault;
            e = launch_gemm(g);
            if (e != cudaSuccess) return e;
            if (launches) *launches += 1;
            std::swap(b1, b2);
        }
        // b1 now holds the step exponentials of this batch.
        int lv = 0;
        e = tree_product(l.fp64, l.d, b1, cnt, b2, static_cast<char *>(l.out) + nb * dd * es, l.stream, l.num_sms,
                         &lv, l.fault);
        if (e != cudaSuccess) return e;
        if (launches) *launches += lv;
    }
    return cudaSuccess;
}

cudaError_t launch_large_range(const LargeLaunch &l, int *launches) {
    if (launches) *launches = 0;
    if (l.M < 1 || l.batch < 1) return cudaErrorInvalidValue;
    return l.fp64 ? run_large<double>(l, launches) : run_large<float>(l, launches);
}

template <class S, class D>
__global__ void k_convert(const S *src, D *dst, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        D v;
        v.x = src[i].x;
        v.y = src[i].y;
        dst[i] = v;
    }
}

cudaError_t convert_complex(bool to_fp64, const void *src, void *dst, long long n, cudaStream_t stream) {
    const int blocks = (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4096));
    if (to_fp64)
        k_convert<float2, double2><<<blocks, 256, 0, stream>>>(static_cast<const float2 *>(src),
                                                               static_cast<double2 *>(dst), n);
    else
        k_convert<double2, float2><<<blocks, 256, 0, stream>>>(static_cast<const double2 *>(src),
                                                               static_cast<float2 *>(dst), n);
    return cudaGetLastError();
}

template <class R>
__global__ void k_fill_identity(cplx_t<R> *dst, int d, long long count, cplx_t<R> v) {
    const long long dd = (long long)d * d, n = dd * count;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        long long e = i % dd;
        dst[i] = ((e / d) == (e % d)) ? v : mk<cplx_t<R>>(0.0, 0.0);
    }
}

cudaError_t fill_identity(bool fp64, void *dst, int d, long long count, double re, double im, cudaStream_t stream) {
    long long n = (long long)d * d * count;
    int blocks = (int)std::min<long long>((n + 255) / 256, 4096);
    if (blocks < 1) return cudaSuccess;
    if (fp64)
        k_fill_identity<double><<<blocks, 256, 0, stream>>>(static_cast<double2 *>(dst), d, count, make_double2(re, im));
    else
        k_fill_identity<float><<<blocks, 256, 0, stream>>>(static_cast<float2 *>(dst), d, count,
                                                           make_float2((float)re, (float)im));
    return cudaGetLastError();
}

}  // namespace pgb
