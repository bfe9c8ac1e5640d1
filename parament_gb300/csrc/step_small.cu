// Fused plain-path kernel for d <= 64: Hamiltonian assembly, Chebyshev
// (Clenshaw) exponential and the running product of a chunk of consecutive
// steps, all resident in shared memory.  One CTA owns one chunk; nothing but
// the samples is read from HBM per step (the expansion stack stays in L2) and
// one d x d product per chunk is written back.
//
// Replaces, for small d, the reference's expansion GEMMs and quadrature kernels
// (src/cuda/parament.cpp:486-563, src/cuda/control_expansion.cu:27-170), the
// batched Clenshaw GEMMs plus diagonal adds (src/cuda/parament.cpp:569-652,
// src/cuda/diagonal_add.cu:21-51) and the lower levels of the tree product
// (src/cuda/parament.cpp:657-718).
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace pgb {

template <class R>
struct SmallArgs {
    cplx_t<R> J[kMaxOrder + 1];
    const cplx_t<R> *stack;
    const cplx_t<R> *carr;
    cplx_t<R> *chunks;
    long long P;
    int nchunks;
    int d, Ke, M;
    R s;
    WeightSpec w;
};

// Complex64 instances keep to 128 registers so that two CTAs share an SM.
template <class R, int TM>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 2 : 1) k_small_steps(const __grid_constant__ SmallArgs<R> a) {
    using C = cplx_t<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int d = a.d, dd = d * d, ld = d + 1, sz = d * ld;
    C *Xs = reinterpret_cast<C *>(smem_raw);
    C *Bs = Xs + sz;
    C *Ps = Bs + sz;
    C *ws = Ps + sz;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const long long s0 = a.P * blockIdx.x / a.nchunks;
    const long long s1 = a.P * (blockIdx.x + 1) / a.nchunks;
    const int M = a.M;
    const R s = a.s;

    bool own[TM][TM];
    int eo[TM][TM];  // shared-memory index (stride ld); the global index is r*d+c
    bool diag[TM][TM];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TM; ++j) {
            int r = ty + 16 * i, c = tx + 16 * j;
            own[i][j] = (r < d) && (c < d);
            eo[i][j] = r * ld + c;
            diag[i][j] = (r == c);
        }

    C b2[TM][TM], acc[TM][TM];
    for (long long st = s0; st < s1; ++st) {
        for (int m = tid; m < a.Ke; m += blockDim.x) ws[m] = step_weight(a.carr, a.w, m, st);
        __syncthreads();
        // X = H0 + sum_m w_m H_m (own elements), straight from the L2-resident
        // stack; b_M = J[M] I and b_(M-1) = s J[M] X + J[M-1] I need only the
        // thread's own elements, so they are formed in the same pass.
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j) {
                if (!own[i][j]) continue;
                const int e = eo[i][j];
                const int ge = (ty + 16 * i) * d + tx + 16 * j;
                C v = a.stack[ge];
                for (int m = 0; m < a.Ke; ++m) cfma(v, ws[m], a.stack[(size_t)(m + 1) * dd + ge]);
                Xs[e] = v;
                C bm1 = cscale(cmul(a.J[M], v), s);
                if (diag[i][j]) bm1 = cadd(bm1, a.J[M - 1]);
                if (M == 1) {
                    acc[i][j] = bm1;  // U = s J[1] X + J[0] I, since b_2 = 0
                } else {
                    b2[i][j] = diag[i][j] ? a.J[M] : mk<C>(0.0, 0.0);
                    Bs[e] = bm1;
                }
            }
        if (M > 1) {
            __syncthreads();
            for (int k = M - 2; k >= 0; --k) {
                tile_gemm<C, TM>(acc, Bs, Xs, d, ld, ty, tx);
                __syncthreads();
                const R beta = (k == 0) ? (R)-2 : (R)-1;
#pragma unroll
                for (int i = 0; i < TM; ++i)
#pragma unroll
                    for (int j = 0; j < TM; ++j) {
                        if (!own[i][j]) continue;
                        C v = cscale(acc[i][j], s);
                        v.x += beta * b2[i][j].x;
                        v.y += beta * b2[i][j].y;
                        if (diag[i][j]) v = cadd(v, a.J[k]);
                        if (k > 0) {
                            b2[i][j] = Bs[eo[i][j]];
                            Bs[eo[i][j]] = v;
                        } else {
                            acc[i][j] = v;  // U_j
                        }
                    }
                if (k > 0) __syncthreads();
            }
        }
        // Chunk product P <- U_j P (later step on the left).
        if (st == s0) {
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j)
                    if (own[i][j]) Ps[eo[i][j]] = acc[i][j];
            __syncthreads();
        } else {
            // U P = P + (U - I) P: the near-identity factor enters the sums
            // without its unit diagonal, so sequential accumulation does not
            // round small contributions against 1 (that bias adds up
            // coherently over thousands of steps in FP32).
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j)
                    if (own[i][j]) {
                        C u = acc[i][j];
                        if (diag[i][j]) u.x -= (R)1;
                        Bs[eo[i][j]] = u;
                    }
            __syncthreads();
            tile_gemm<C, TM>(acc, Bs, Ps, d, ld, ty, tx);
            __syncthreads();
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j)
                    if (own[i][j]) Ps[eo[i][j]] = cadd(Ps[eo[i][j]], acc[i][j]);
            __syncthreads();
        }
    }
    if (s1 > s0) {
        C *dst = a.chunks + (size_t)blockIdx.x * dd;
        for (int e = tid; e < dd; e += blockDim.x) dst[e] = Ps[(e / d) * ld + e % d];
    }
}

size_t small_smem_bytes(bool fp64, int d, int Ke) {
    size_t c = fp64 ? 16 : 8;
    return c * (3 * (size_t)d * (d + 1) + (size_t)Ke);
}

template <class R, int TM>
static const void *small_kernel_ptr() {
    return reinterpret_cast<const void *>(&k_small_steps<R, TM>);
}

static const void *pick_small(bool fp64, int d) {
    int tm = (d + 15) / 16;
    if (fp64) {
        switch (tm) {
            case 1: return small_kernel_ptr<double, 1>();
            case 2: return small_kernel_ptr<double, 2>();
            case 3: return small_kernel_ptr<double, 3>();
            default: return small_kernel_ptr<double, 4>();
        }
    }
    switch (tm) {
        case 1: return small_kernel_ptr<float, 1>();
        case 2: return small_kernel_ptr<float, 2>();
        case 3: return small_kernel_ptr<float, 3>();
        default: return small_kernel_ptr<float, 4>();
    }
}

int small_chunk_count(bool fp64, int d, int Ke, long long P, int num_sms) {
    const void *fn = pick_small(fp64, d);
    size_t smem = small_smem_bytes(fp64, d, Ke);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, smem) != cudaSuccess || per_sm < 1) per_sm = 1;
    long long n = (long long)per_sm * num_sms;
    return (int)std::max<long long>(1, std::min<long long>(n, P));
}

template <class R>
static cudaError_t launch_small_t(const StepLaunch &l) {
    using C = cplx_t<R>;
    SmallArgs<R> a;
    for (int k = 0; k <= l.M; ++k) a.J[k] = mk<C>(l.J[2 * k], l.J[2 * k + 1]);
    a.stack = static_cast<const C *>(l.stack);
    a.carr = static_cast<const C *>(l.carr);
    a.chunks = static_cast<C *>(l.chunks);
    a.P = l.P;
    a.nchunks = l.nchunks;
    a.d = l.d;
    a.Ke = l.Ke;
    a.M = l.M;
    a.s = (R)l.s;
    a.w = WeightSpec{l.w.pts, l.w.K, l.w.amps, l.w.mode, l.w.magnus, l.w.hfac};
    size_t smem = small_smem_bytes(l.fp64, l.d, l.Ke);
    const void *fn = pick_small(l.fp64, l.d);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void *args[] = {&a};
    return cudaLaunchKernel(fn, dim3(l.nchunks), dim3(256), args, smem, l.stream);
}

cudaError_t launch_small_steps(const StepLaunch &l) {
    if (l.d < 1 || l.d > kSmallMaxDim || l.M < 1 || l.M > kMaxOrder || l.nchunks < 1) return cudaErrorInvalidValue;
    return l.fp64 ? launch_small_t<double>(l) : launch_small_t<float>(l);
}

}  // namespace pgb
