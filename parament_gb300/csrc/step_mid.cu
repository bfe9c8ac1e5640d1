// Fused plain-path kernel for 64 < d <= 128: one cluster of four CTAs per
// chunk of consecutive steps, the whole Clenshaw recurrence and the chunk's
// running product resident in the cluster's shared memory.
//
// Same method as k_small_steps (step_small.cu) and the reference's
// expansion, Clenshaw and tree (src/cuda/parament.cpp:486-718); what changes
// is where the matrices live.  A d x d matrix of d = 128 is 132 KB in
// complex64, too much for three copies in one CTA, so the four CTAs of a
// cluster (rank q) share the work:
//
//   * every CTA assembles the whole X_j of the step (from the L2-resident
//     expansion stack) into its full-matrix buffer F;
//   * CTA q runs the Clenshaw recurrence for rows [q rb, (q + 1) rb) of the
//     b_k (rb = ceil(d / 4)): b_k rows = 2 X' b_(k+1) rows ..., which needs
//     only its own rows of b_(k+1) and the whole X -- no traffic between the
//     CTAs;
//   * its rows of U_j - I go to the F buffers of all four CTAs (stores into
//     the other CTAs' shared memory, between two cluster barriers), where X_j
//     was;
//   * CTA q keeps columns [q rb, (q + 1) rb) of the running product P and
//     updates them as P <- P + (U_j - I) P, which needs the whole U_j - I
//     (now in F) and only its own columns of P.
//
// Shared memory per CTA: F (d x (d + 1)), the b rows (rb x (d + 1)), the P
// columns (d x (rb + 1)) and the step weights: 199 KB for complex64 at
// d = 128, and complex128 up to d = 96.  Nothing is read from other CTAs:
// the only traffic between them is the all-gather of U_j - I.  No thread
// waits on anything but the CTA and cluster barriers.
#include <cooperative_groups.h>

#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace pgb {

constexpr int kMidCluster = 4;
constexpr int kMidMaxDim = 128;

template <class R>
struct MidArgs {
    cplx_t<R> J[kMaxOrder + 1];
    const cplx_t<R> *stack;
    const cplx_t<R> *carr;
    cplx_t<R> *chunks;
    long long P;
    int nchunks;  // clusters
    int d, Ke, M;
    R s;
    WeightSpec w;
};

template <class R>
__global__ void __cluster_dims__(kMidCluster, 1, 1) __launch_bounds__(256, 1)
    k_mid_steps(const __grid_constant__ MidArgs<R> a) {
    using C = cplx_t<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cg::cluster_group cluster = cg::this_cluster();
    const int q = (int)cluster.block_rank();
    const int chunk = blockIdx.x / kMidCluster;
    const int d = a.d, dd = d * d, ld = d + 1;
    const int rb = (d + kMidCluster - 1) / kMidCluster, ldp = rb + 1;
    C *F = reinterpret_cast<C *>(smem_raw);  // X, then U - I
    C *Bs = F + d * ld;                        // rows q rb .. of b_(k+1)
    C *Pc = Bs + rb * ld;                      // columns q rb .. of P
    C *ws = Pc + d * ldp;                      // step weights
    C *Fr[kMidCluster];
#pragma unroll
    for (int k = 0; k < kMidCluster; ++k) Fr[k] = cluster.map_shared_rank(F, k);
    const int tid = threadIdx.x;
    const long long s0 = a.P * chunk / a.nchunks;
    const long long s1 = a.P * (chunk + 1) / a.nchunks;
    const int M = a.M;
    const R s = a.s;
    const int r0 = q * rb, c0 = q * rb;
    const C zero = mk<C>(0.0, 0.0);

    // Row-block products (Clenshaw): 32 rows x 128 columns as 8 x 32 threads,
    // rows ty + 8 i (local), columns tx + 32 j.
    const int ty = tid >> 5, tx = tid & 31;
    bool own[4][4], dg[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int lr = ty + 8 * i, c = tx + 32 * j;
            own[i][j] = lr < rb && r0 + lr < d && c < d;
            dg[i][j] = r0 + lr == c;
        }
    // Column-block products (running product): 128 rows x 32 columns as
    // 32 x 8 threads, rows py + 32 i, local columns px + 8 j.
    const int py = tid >> 3, px = tid & 7;
    bool pown[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) pown[i][j] = py + 32 * i < d && px + 8 * j < rb && c0 + px + 8 * j < d;

    C acc[4][4], b2[4][4];
    for (long long st = s0; st < s1; ++st) {
        for (int m = tid; m < a.Ke; m += blockDim.x) ws[m] = step_weight(a.carr, a.w, m, st);
        __syncthreads();
        // X of the step, whole, into F.
        for (int e = tid; e < dd; e += blockDim.x) {
            C v = a.stack[e];
            for (int m = 0; m < a.Ke; ++m) cfma(v, ws[m], a.stack[(size_t)(m + 1) * dd + e]);
            F[(e / d) * ld + e % d] = v;
        }
        __syncthreads();
        // b_M = J[M] I, b_(M-1) = s J[M] X + J[M-1] I (own rows).
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (!own[i][j]) continue;
                const int lr = ty + 8 * i, c = tx + 32 * j;
                C v = cscale(cmul(a.J[M], F[(r0 + lr) * ld + c]), s);
                if (dg[i][j]) v = cadd(v, a.J[M - 1]);
                if (M == 1) {
                    acc[i][j] = v;
                } else {
                    b2[i][j] = dg[i][j] ? a.J[M] : zero;
                    Bs[lr * ld + c] = v;
                }
            }
        if (M > 1) {
            __syncthreads();
            for (int k = M - 2; k >= 0; --k) {
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = zero;
                int ra[4], cb[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    ra[i] = min(ty + 8 * i, rb - 1) * ld;
                    cb[i] = min(tx + 32 * i, d - 1);
                }
#pragma unroll 4
                for (int kk = 0; kk < d; ++kk) {
                    C av[4], bv[4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) av[i] = Bs[ra[i] + kk];
#pragma unroll
                    for (int j = 0; j < 4; ++j) bv[j] = F[kk * ld + cb[j]];
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) cfma(acc[i][j], av[i], bv[j]);
                }
                __syncthreads();
                const R beta = (k == 0) ? (R)-2 : (R)-1;
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        if (!own[i][j]) continue;
                        const int e = (ty + 8 * i) * ld + tx + 32 * j;
                        C v = cscale(acc[i][j], s);
                        v.x += beta * b2[i][j].x;
                        v.y += beta * b2[i][j].y;
                        if (dg[i][j]) v = cadd(v, a.J[k]);
                        if (k > 0) {
                            b2[i][j] = Bs[e];
                            Bs[e] = v;
                        } else {
                            acc[i][j] = v;  // U_j, own rows
                        }
                    }
                if (k > 0) __syncthreads();
            }
        }
        // Every CTA is done with its X: the rows of U - I go to all four F.
        cluster.sync();
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (!own[i][j]) continue;
                C u = acc[i][j];
                if (dg[i][j]) u.x -= (R)1;
                const int e = (r0 + ty + 8 * i) * ld + tx + 32 * j;
#pragma unroll
                for (int t = 0; t < kMidCluster; ++t) Fr[t][e] = u;
            }
        cluster.sync();
        // Running product, own columns: P <- U P = P + (U - I) P (P = U first).
        if (st == s0) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (!pown[i][j]) continue;
                    const int r = py + 32 * i, lc = px + 8 * j;
                    C u = F[r * ld + c0 + lc];
                    if (r == c0 + lc) u.x += (R)1;
                    Pc[r * ldp + lc] = u;
                }
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = zero;
            int ra[4], cb[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                ra[i] = min(py + 32 * i, d - 1) * ld;
                cb[i] = min(px + 8 * i, rb - 1);
            }
#pragma unroll 4
            for (int kk = 0; kk < d; ++kk) {
                C av[4], bv[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) av[i] = F[ra[i] + kk];
#pragma unroll
                for (int j = 0; j < 4; ++j) bv[j] = Pc[kk * ldp + cb[j]];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) cfma(acc[i][j], av[i], bv[j]);
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (!pown[i][j]) continue;
                    const int e = (py + 32 * i) * ldp + px + 8 * j;
                    Pc[e] = cadd(Pc[e], acc[i][j]);
                }
        }
        __syncthreads();
    }
    if (s1 > s0) {
        C *dst = a.chunks + (size_t)chunk * dd;
        for (int e = tid; e < d * rb; e += blockDim.x) {
            const int r = e / rb, lc = e % rb;
            if (c0 + lc < d) dst[(size_t)r * d + c0 + lc] = Pc[r * ldp + lc];
        }
    }
    // No CTA leaves while another may still store into its shared memory.
    cluster.sync();
}

size_t mid_smem_bytes(bool fp64, int d, int Ke) {
    const size_t c = fp64 ? 16 : 8;
    const size_t rb = (d + kMidCluster - 1) / kMidCluster;
    return c * ((size_t)d * (d + 1) + rb * (d + 1) + (size_t)d * (rb + 1) + (size_t)std::max(Ke, 1));
}

bool mid_applies(bool fp64, int d, int Ke) {
    return d > kSmallMaxDim && d <= kMidMaxDim && mid_smem_bytes(fp64, d, Ke) <= 232448;
}

int mid_chunk_count(int num_sms, long long P) {
    return (int)std::max<long long>(1, std::min<long long>(num_sms / kMidCluster, P));
}

template <class R>
static cudaError_t launch_mid_t(const StepLaunch &l) {
    using C = cplx_t<R>;
    MidArgs<R> a;
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
    const size_t smem = mid_smem_bytes(l.fp64, l.d, l.Ke);
    const void *fn = reinterpret_cast<const void *>(&k_mid_steps<R>);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void *args[] = {&a};
    return cudaLaunchKernel(fn, dim3(kMidCluster * l.nchunks), dim3(256), args, smem, l.stream);
}

cudaError_t launch_mid_steps(const StepLaunch &l) {
    if (!mid_applies(l.fp64, l.d, l.Ke) || l.M < 1 || l.M > kMaxOrder || l.nchunks < 1)
        return cudaErrorInvalidValue;
    return l.fp64 ? launch_mid_t<double>(l) : launch_mid_t<float>(l);
}

}  // namespace pgb
