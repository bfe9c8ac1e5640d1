// Batched ensembles: many independent equiprop problems of uneven dimension,
// step count and control count in one persistent launch.  No counterpart in
// the reference (which runs one problem per call, src/cuda/parament.cpp:791-851);
// each problem follows the reference's scheme (norm bound, order table, Bessel
// coefficients, quadrature weights, Clenshaw, time-ordered product).
//
// Work decomposition: every problem's steps are cut into chunks; chunks of the
// same dimension class (4, 8, 16, 32, 64) are grouped into bundles that fill
// one CTA: sixteen 4x4 chunks (16 threads each, half-warp synchronisation),
// four 8x8 chunks (64 threads, named barriers), or one chunk for the larger
// classes (the whole CTA).  A persistent kernel pulls bundles from an atomic
// counter -- no waiting on other CTAs, so no spin loops -- and writes one
// product per chunk; a second kernel multiplies each problem's chunk products
// in order.  Both, with the counter reset, are captured in a CUDA graph.  The
// chunk length per class comes from an autotuner that times a few candidate
// granularities on the actual ensemble.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "common.cuh"
#include "ctx.h"
#include "kernels.h"

namespace pgb {

constexpr int kEnsMaxK = 16;
constexpr int kEnsRegK = 4;  // controls whose matrices a thread caches in registers
constexpr int kEnsClasses = 5;
static const int kClassDim[kEnsClasses] = {4, 8, 16, 32, 64};
static const int kClassGroups[kEnsClasses] = {16, 4, 1, 1, 1};

struct EnsProblem {
    int d, K, mode, M;
    unsigned pts;
    long long P;
    double s;
    long long stack_off, carr_off, out_off, chunk_off;
    int j_off, nchunks;
};
struct EnsItem {
    int prob, slot;
    long long s0, s1;
};
struct EnsBundle {
    int cls, count, first;
};

template <class R>
struct EnsArgs {
    const EnsProblem *probs;
    const EnsItem *items;
    const EnsBundle *bundles;
    int nbundles;
    int *counter;
    const cplx_t<R> *stack, *carr, *J;
    cplx_t<R> *chunks;
};

template <int D>
__device__ __forceinline__ void group_sync(int g) {
    if (D == 4) {
        __syncwarp(0xFFFFu << (16 * (g & 1)));
    } else if (D == 8) {
        asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(64) : "memory");
    } else {
        __syncthreads();
    }
}

// Product of one chunk of problem p, computed by a group of T*T threads
// (T = D for D <= 16, else 16 with TM x TM elements per thread).
template <class R, int TM, int D>
__device__ void ens_chunk(const EnsArgs<R> &a, const EnsProblem &p, const EnsItem &it, int g, int gt,
                          cplx_t<R> *sm) {
    using C = cplx_t<R>;
    constexpr int T = (D <= 16) ? D : 16;
    const int d = p.d, dd = d * d, ld = d + 1, sz = d * ld;
    C *Xs = sm, *Bs = Xs + sz, *Ps = Bs + sz, *ws = Ps + sz;
    const int ty = gt / T, tx = gt % T;
    const C *stack = a.stack + p.stack_off;
    const C *J = a.J + p.j_off;
    const int M = p.M;
    const R s = (R)p.s;
    WeightSpec w{p.pts, p.K, p.K, p.mode, 0, 0.0};
    const C *carr = a.carr + p.carr_off;
    C b2[TM][TM], acc[TM][TM];
    // The expansion matrices do not change from step to step: for TM <= 2 and
    // up to kEnsRegK controls each thread keeps its own elements of them in
    // registers for the whole chunk instead of re-reading them every step.
    constexpr bool kCache = TM <= 2;
    C hreg[kCache ? TM : 1][kCache ? TM : 1][kCache ? kEnsRegK + 1 : 1];
    const bool cached = kCache && p.K <= kEnsRegK;
    if (kCache && cached) {
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j) {
                const int r = min(ty + T * i, d - 1), c = min(tx + T * j, d - 1);
#pragma unroll
                for (int m = 0; m <= kEnsRegK; ++m)
                    hreg[kCache ? i : 0][kCache ? j : 0][kCache ? m : 0] =
                        (m <= p.K) ? stack[(size_t)m * dd + r * d + c] : mk<C>(0.0, 0.0);
            }
    }
    // Weight of the thread's control for the first step; later steps are
    // fetched one step ahead so the sample load overlaps the step's products.
    C wnext = (gt < p.K) ? step_weight(carr, w, gt, it.s0) : mk<C>(0.0, 0.0);
    for (long long st = it.s0; st < it.s1; ++st) {
        if (gt < p.K) {
            ws[gt] = wnext;
            if (st + 1 < it.s1) wnext = step_weight(carr, w, gt, st + 1);
        }
        for (int m = gt + T * T; m < p.K; m += T * T) ws[m] = step_weight(carr, w, m, st);
        group_sync<D>(g);
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j) {
                const int r = ty + T * i, c = tx + T * j;
                if (r >= d || c >= d) continue;
                C v;
                if (kCache && cached) {
                    v = hreg[kCache ? i : 0][kCache ? j : 0][0];
#pragma unroll
                    for (int m = 0; m < kEnsRegK; ++m)
                        if (m < p.K) cfma(v, ws[m], hreg[kCache ? i : 0][kCache ? j : 0][kCache ? m + 1 : 0]);
                } else {
                    v = stack[r * d + c];
                    for (int m = 0; m < p.K; ++m) cfma(v, ws[m], stack[(size_t)(m + 1) * dd + r * d + c]);
                }
                Xs[r * ld + c] = v;
                C bm1 = cscale(cmul(J[M], v), s);
                if (r == c) bm1 = cadd(bm1, J[M - 1]);
                if (M == 1) {
                    acc[i][j] = bm1;
                } else {
                    b2[i][j] = (r == c) ? J[M] : mk<C>(0.0, 0.0);
                    Bs[r * ld + c] = bm1;
                }
            }
        if (M > 1) {
            group_sync<D>(g);
            for (int k = M - 2; k >= 0; --k) {
                // acc = Bs Xs
#pragma unroll
                for (int i = 0; i < TM; ++i)
#pragma unroll
                    for (int j = 0; j < TM; ++j) acc[i][j] = mk<C>(0.0, 0.0);
                for (int q = 0; q < d; ++q) {
                    C av[TM], bv[TM];
#pragma unroll
                    for (int i = 0; i < TM; ++i) av[i] = Bs[min(ty + T * i, d - 1) * ld + q];
#pragma unroll
                    for (int j = 0; j < TM; ++j) bv[j] = Xs[q * ld + min(tx + T * j, d - 1)];
#pragma unroll
                    for (int i = 0; i < TM; ++i)
#pragma unroll
                        for (int j = 0; j < TM; ++j) cfma(acc[i][j], av[i], bv[j]);
                }
                group_sync<D>(g);
                const R beta = (k == 0) ? (R)-2 : (R)-1;
#pragma unroll
                for (int i = 0; i < TM; ++i)
#pragma unroll
                    for (int j = 0; j < TM; ++j) {
                        const int r = ty + T * i, c = tx + T * j;
                        if (r >= d || c >= d) continue;
                        C v = cscale(acc[i][j], s);
                        v.x += beta * b2[i][j].x;
                        v.y += beta * b2[i][j].y;
                        if (r == c) v = cadd(v, J[k]);
                        if (k > 0) {
                            b2[i][j] = Bs[r * ld + c];
                            Bs[r * ld + c] = v;
                        } else {
                            acc[i][j] = v;
                        }
                    }
                if (k > 0) group_sync<D>(g);
            }
        }
        if (st == it.s0) {
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) {
                    const int r = ty + T * i, c = tx + T * j;
                    if (r < d && c < d) Ps[r * ld + c] = acc[i][j];
                }
            group_sync<D>(g);
        } else {
            // U P = P + (U - I) P
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) {
                    const int r = ty + T * i, c = tx + T * j;
                    if (r >= d || c >= d) continue;
                    C u = acc[i][j];
                    if (r == c) u.x -= (R)1;
                    Bs[r * ld + c] = u;
                }
            group_sync<D>(g);
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) acc[i][j] = mk<C>(0.0, 0.0);
            for (int q = 0; q < d; ++q) {
                C av[TM], bv[TM];
#pragma unroll
                for (int i = 0; i < TM; ++i) av[i] = Bs[min(ty + T * i, d - 1) * ld + q];
#pragma unroll
                for (int j = 0; j < TM; ++j) bv[j] = Ps[q * ld + min(tx + T * j, d - 1)];
#pragma unroll
                for (int i = 0; i < TM; ++i)
#pragma unroll
                    for (int j = 0; j < TM; ++j) cfma(acc[i][j], av[i], bv[j]);
            }
            group_sync<D>(g);
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) {
                    const int r = ty + T * i, c = tx + T * j;
                    if (r < d && c < d) Ps[r * ld + c] = cadd(Ps[r * ld + c], acc[i][j]);
                }
            group_sync<D>(g);
        }
    }
    C *dst = a.chunks + p.chunk_off + (size_t)it.slot * dd;
    for (int e = gt; e < dd; e += T * T) dst[e] = Ps[(e / d) * ld + e % d];
}

template <class R>
__device__ __forceinline__ size_t ens_group_elems(int D) {
    return 3 * (size_t)D * (D + 1) + kEnsMaxK;
}

// One persistent kernel per dimension class, so each gets its own register
// budget and occupancy: CTAs pull bundles of that class from the class's
// counter until the class is exhausted.
template <class R, int TM, int D, int GROUPS, int MINB>
__global__ void __launch_bounds__(256, MINB) k_ensemble_class(const __grid_constant__ EnsArgs<R> a, int first,
                                                              int count, int *counter) {
    using C = cplx_t<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *sm = reinterpret_cast<C *>(smem_raw);
    constexpr int GT = 256 / GROUPS;  // threads per group
    __shared__ int bid;
    for (;;) {
        if (threadIdx.x == 0) bid = atomicAdd(counter, 1);
        __syncthreads();
        const int b = bid;
        __syncthreads();
        if (b >= count) break;
        const EnsBundle B = a.bundles[first + b];
        const int g = threadIdx.x / GT, gt = threadIdx.x % GT;
        if (g < B.count) {
            const EnsItem it = a.items[B.first + g];
            ens_chunk<R, TM, D>(a, a.probs[it.prob], it, g, gt, sm + g * ens_group_elems<R>(D));
        }
        __syncthreads();
    }
}

// Ordered product of each problem's chunk products (later chunk on the left),
// P <- A P formed as P + (A - I) P: a chunk product near the identity enters
// the sums without its unit diagonal, so its small terms are not rounded
// against 1 in FP32.
template <class R>
__global__ void __launch_bounds__(256) k_ensemble_reduce(const EnsProblem *probs, const cplx_t<R> *chunks,
                                                         cplx_t<R> *out) {
    using C = cplx_t<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const EnsProblem p = probs[blockIdx.x];
    const int d = p.d, dd = d * d, ld = d + 1;
    C *As = reinterpret_cast<C *>(smem_raw), *Ps = As + d * ld;
    const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
    const C *src = chunks + p.chunk_off;
    for (int e = threadIdx.x; e < dd; e += blockDim.x) Ps[(e / d) * ld + e % d] = src[e];
    __syncthreads();
    for (int c = 1; c < p.nchunks; ++c) {
        for (int e = threadIdx.x; e < dd; e += blockDim.x) {
            C v = src[(size_t)c * dd + e];
            if (e / d == e % d) v.x -= (R)1;
            As[(e / d) * ld + e % d] = v;
        }
        __syncthreads();
        C acc[4][4];
        tile_gemm<C, 4>(acc, As, Ps, d, ld, ty, tx);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int r = ty + 16 * i, cc = tx + 16 * j;
                if (r < d && cc < d) Ps[r * ld + cc] = cadd(Ps[r * ld + cc], acc[i][j]);
            }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < dd; e += blockDim.x) out[p.out_off + e] = Ps[(e / d) * ld + e % d];
}

// ---------------------------------------------------------------- host side

struct Ensemble {
    bool fp64;
    int device = 0, num_sms = 0;
    cudaStream_t stream = nullptr;
    std::vector<EnsProblem> probs;
    std::vector<int> cls;  // class of each problem
    long long carr_elems = 0, out_elems = 0;
    DevBuf d_probs, d_items, d_bundles, d_counter, d_stack, d_carr, d_J, d_chunks, d_out;
    void *h_carr = nullptr, *h_out = nullptr;  // pinned staging
    int nbundles = 0;
    int cls_first[kEnsClasses] = {0}, cls_count[kEnsClasses] = {0};
    int cls_slots[kEnsClasses] = {0};
    double granularity = 4.0;  // bundles per resident CTA (autotuned)
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_ms = -1.0f;
    int slots = 0;
};

static int class_of(int d) {
    for (int c = 0; c < kEnsClasses; ++c)
        if (d <= kClassDim[c]) return c;
    return -1;
}

static size_t ens_smem(bool fp64, int cls) {
    const size_t es = fp64 ? 16 : 8;
    const int D = kClassDim[cls];
    return es * (size_t)kClassGroups[cls] * (3 * (size_t)D * (D + 1) + kEnsMaxK);
}

// Time model of one step of a chunk: products per step times d^3 complex
// multiply-adds over the CTA's 256 threads, plus a fixed part of about one
// 32^3 product for the dependent load/synchronise chain every step pays
// (weights, assembly, barriers) -- for d <= 16 that latency, not the
// arithmetic, sets the step time, so small problems are cut into more chunks.
static double step_cost(const EnsProblem &p) { return (double)p.M * ((double)p.d * p.d * p.d + 32768.0) / 256.0; }

// Work list for a given granularity: chunk lengths chosen so that each
// bundle costs about total / (slots * granularity).
static Parament_ErrorCode build_work(Ensemble *E, double gran) {
    double total = 0.0;
    for (auto &p : E->probs) total += step_cost(p) * p.P / kClassGroups[class_of(p.d)];
    const double target = std::max(1.0, total / (E->slots * gran));  // slots: CTAs of the d=64 class
    std::vector<EnsItem> items;
    std::vector<EnsBundle> bundles;
    long long chunk_elems = 0;
    std::vector<std::vector<EnsItem>> per_class(kEnsClasses);
    for (size_t i = 0; i < E->probs.size(); ++i) {
        EnsProblem &p = E->probs[i];
        const long long L = std::max<long long>(1, (long long)(target / step_cost(p)));
        const long long n = (p.P + L - 1) / L;
        p.nchunks = (int)n;
        p.chunk_off = chunk_elems;
        chunk_elems += n * (long long)p.d * p.d;
        for (long long c = 0; c < n; ++c)
            per_class[E->cls[i]].push_back(EnsItem{(int)i, (int)c, p.P * c / n, p.P * (c + 1) / n});
    }
    // Largest classes first so the long bundles start early.
    for (int c = kEnsClasses - 1; c >= 0; --c) {
        auto &v = per_class[c];
        E->cls_first[c] = (int)bundles.size();
        for (size_t k = 0; k < v.size(); k += kClassGroups[c]) {
            const int cnt = (int)std::min<size_t>(kClassGroups[c], v.size() - k);
            bundles.push_back(EnsBundle{c, cnt, (int)items.size()});
            for (int q = 0; q < cnt; ++q) items.push_back(v[k + q]);
        }
        E->cls_count[c] = (int)bundles.size() - E->cls_first[c];
    }
    const size_t es = E->fp64 ? 16 : 8;
    if (E->d_probs.ensure(sizeof(EnsProblem) * E->probs.size()) != cudaSuccess ||
        E->d_items.ensure(sizeof(EnsItem) * std::max<size_t>(1, items.size())) != cudaSuccess ||
        E->d_bundles.ensure(sizeof(EnsBundle) * std::max<size_t>(1, bundles.size())) != cudaSuccess ||
        E->d_chunks.ensure(es * std::max<long long>(1, chunk_elems)) != cudaSuccess)
        return PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
    cudaError_t e = cudaMemcpy(E->d_probs.ptr, E->probs.data(), sizeof(EnsProblem) * E->probs.size(),
                               cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !items.empty())
        e = cudaMemcpy(E->d_items.ptr, items.data(), sizeof(EnsItem) * items.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !bundles.empty())
        e = cudaMemcpy(E->d_bundles.ptr, bundles.data(), sizeof(EnsBundle) * bundles.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return PARAMENT_FAIL;
    E->nbundles = (int)bundles.size();
    E->granularity = gran;
    return PARAMENT_STATUS_SUCCESS;
}

template <class R, int TM, int D, int GROUPS, int MINB>
static cudaError_t launch_class(Ensemble *E, const EnsArgs<R> &a, int c) {
    if (E->cls_count[c] == 0) return cudaSuccess;
    const int grid = std::max(1, std::min(E->cls_slots[c], E->cls_count[c]));
    int *counter = static_cast<int *>(E->d_counter.ptr) + c;
    k_ensemble_class<R, TM, D, GROUPS, MINB><<<grid, 256, ens_smem(E->fp64, c), E->stream>>>(
        a, E->cls_first[c], E->cls_count[c], counter);
    return cudaGetLastError();
}

template <class R>
static const void *class_kernel(int c) {
    switch (c) {
        case 0: return reinterpret_cast<const void *>(&k_ensemble_class<R, 1, 4, 16, 4>);
        case 1: return reinterpret_cast<const void *>(&k_ensemble_class<R, 1, 8, 4, 4>);
        case 2: return reinterpret_cast<const void *>(&k_ensemble_class<R, 1, 16, 1, 4>);
        case 3: return reinterpret_cast<const void *>(&k_ensemble_class<R, 2, 32, 1, sizeof(R) == 4 ? 3 : 2>);
        default: return reinterpret_cast<const void *>(&k_ensemble_class<R, 4, 64, 1, sizeof(R) == 4 ? 2 : 1>);
    }
}

template <class R>
static cudaError_t enqueue_t(Ensemble *E) {
    using C = cplx_t<R>;
    cudaError_t e = cudaMemsetAsync(E->d_counter.ptr, 0, sizeof(int) * kEnsClasses, E->stream);
    if (e != cudaSuccess) return e;
    EnsArgs<R> a;
    a.probs = static_cast<const EnsProblem *>(E->d_probs.ptr);
    a.items = static_cast<const EnsItem *>(E->d_items.ptr);
    a.bundles = static_cast<const EnsBundle *>(E->d_bundles.ptr);
    a.nbundles = E->nbundles;
    a.counter = static_cast<int *>(E->d_counter.ptr);
    a.stack = static_cast<const C *>(E->d_stack.ptr);
    a.carr = static_cast<const C *>(E->d_carr.ptr);
    a.J = static_cast<const C *>(E->d_J.ptr);
    a.chunks = static_cast<C *>(E->d_chunks.ptr);
    // Largest dimension first: its bundles are the longest.
    e = launch_class<R, 4, 64, 1, sizeof(R) == 4 ? 2 : 1>(E, a, 4);
    if (e == cudaSuccess) e = launch_class<R, 2, 32, 1, sizeof(R) == 4 ? 3 : 2>(E, a, 3);
    if (e == cudaSuccess) e = launch_class<R, 1, 16, 1, 4>(E, a, 2);
    if (e == cudaSuccess) e = launch_class<R, 1, 8, 4, 4>(E, a, 1);
    if (e == cudaSuccess) e = launch_class<R, 1, 4, 16, 4>(E, a, 0);
    if (e != cudaSuccess) return e;
    const size_t rsmem = 2 * sizeof(C) * 64 * 65;
    k_ensemble_reduce<R><<<(int)E->probs.size(), 256, rsmem, E->stream>>>(
        a.probs, a.chunks, static_cast<C *>(E->d_out.ptr));
    return cudaGetLastError();
}

static cudaError_t enqueue(Ensemble *E) { return E->fp64 ? enqueue_t<double>(E) : enqueue_t<float>(E); }

static cudaError_t capture(Ensemble *E) {
    if (E->graph) {
        cudaGraphExecDestroy(E->graph);
        E->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(E->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    cudaError_t e2 = enqueue(E);
    e = cudaStreamEndCapture(E->stream, &g);
    if (e2 != cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&E->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    return e;
}

static float timed_run(Ensemble *E) {
    cudaEventRecord(E->ev0, E->stream);
    cudaGraphLaunch(E->graph, E->stream);
    cudaEventRecord(E->ev1, E->stream);
    float ms = -1.0f;
    if (cudaEventSynchronize(E->ev1) == cudaSuccess) cudaEventElapsedTime(&ms, E->ev0, E->ev1);
    return ms;
}

template <class R>
static void set_kernel_smem(Ensemble *E) {
    for (int c = 0; c < kEnsClasses; ++c) {
        const void *fn = class_kernel<R>(c);
        const size_t m = ens_smem(E->fp64, c);
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)m);
        int per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, m);
        E->cls_slots[c] = std::max(1, per_sm) * E->num_sms;
    }
    cudaFuncSetAttribute(reinterpret_cast<const void *>(&k_ensemble_reduce<R>),
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(2 * sizeof(cplx_t<R>) * 64 * 65));
    E->slots = E->cls_slots[4];
}

}  // namespace pgb

using namespace pgb;

extern "C" {

Parament_ErrorCode Parament_ensembleCreate(Parament_Ensemble **out, int fp64, unsigned int nprob,
                                           const unsigned int *dims, const unsigned int *amps,
                                           const unsigned int *pts, const double *dts, const void *const *H0s,
                                           const void *const *H1s, int quadrature) {
    if (!out) return PARAMENT_STATUS_INVALID_VALUE;
    *out = nullptr;
    if (nprob == 0 || !dims || !amps || !pts || !dts || !H0s || !H1s) return PARAMENT_STATUS_INVALID_VALUE;
    if (quadrature != PARAMENT_QUADRATURE_NONE && quadrature != PARAMENT_QUADRATURE_MIDPOINT &&
        quadrature != PARAMENT_QUADRATURE_SIMPSON)
        return PARAMENT_STATUS_INVALID_VALUE;
    Ensemble *E = new (std::nothrow) Ensemble();
    if (!E) return PARAMENT_STATUS_HOST_ALLOC_FAILED;
    E->fp64 = fp64 != 0;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1 || cudaGetDevice(&E->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&E->num_sms, cudaDevAttrMultiProcessorCount, E->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete E;
        return PARAMENT_STATUS_CUBLAS_INIT_FAILED;
    }
    cudaEventCreate(&E->ev0);
    cudaEventCreate(&E->ev1);
    const size_t es = E->fp64 ? 16 : 8;
    long long stack_elems = 0, carr_elems = 0, out_elems = 0;
    std::vector<double> J;
    Parament_ErrorCode r = PARAMENT_STATUS_SUCCESS;
    for (unsigned i = 0; i < nprob && r == PARAMENT_STATUS_SUCCESS; ++i) {
        EnsProblem p{};
        p.d = (int)dims[i];
        p.K = (int)amps[i];
        p.mode = quadrature;
        p.pts = pts[i];
        p.P = num_steps(quadrature, false, pts[i]);
        if (p.d < 1 || p.d > 64 || p.K > kEnsMaxK || p.P <= 0 || !(dts[i] > 0.0) || !H0s[i] || (p.K && !H1s[i])) {
            r = PARAMENT_STATUS_INVALID_VALUE;
            break;
        }
        const size_t dd = (size_t)p.d * p.d;
        double hn = onenorm_host(H0s[i], p.d, E->fp64);
        for (int k = 0; k < p.K; ++k) hn += onenorm_host(static_cast<const char *>(H1s[i]) + es * dd * k, p.d, E->fp64);
        const double h = (quadrature == PARAMENT_QUADRATURE_SIMPSON) ? 2.0 * dts[i] : dts[i];
        if (hn == 0.0) {
            r = PARAMENT_STATUS_INVALID_VALUE;
            break;
        }
        p.M = select_cycles(E->fp64, hn, h);
        if (p.M < 3) {
            r = PARAMENT_STATUS_SELECT_SMALLER_DT;
            break;
        }
        p.s = 2.0 / hn;
        p.j_off = (int)(J.size() / 2);
        std::vector<double> Jp(2 * (p.M + 1));
        bessel_coeffs(p.M, h * hn, Jp.data());
        J.insert(J.end(), Jp.begin(), Jp.end());
        p.stack_off = stack_elems;
        stack_elems += (long long)dd * (1 + p.K);
        p.carr_off = carr_elems;
        carr_elems += (long long)p.K * p.pts;
        p.out_off = out_elems;
        out_elems += (long long)dd;
        E->probs.push_back(p);
        E->cls.push_back(class_of(p.d));
    }
    if (r == PARAMENT_STATUS_SUCCESS) {
        if (E->d_stack.ensure(es * stack_elems) != cudaSuccess || E->d_carr.ensure(es * std::max(1LL, carr_elems)) != cudaSuccess ||
            E->d_J.ensure(es * (J.size() / 2)) != cudaSuccess || E->d_out.ensure(es * out_elems) != cudaSuccess ||
            E->d_counter.ensure(sizeof(int) * kEnsClasses) != cudaSuccess ||
            cudaMallocHost(&E->h_carr, es * std::max(1LL, carr_elems)) != cudaSuccess ||
            cudaMallocHost(&E->h_out, es * out_elems) != cudaSuccess)
            r = PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
    }
    if (r == PARAMENT_STATUS_SUCCESS) {
        // Stacks [H0, H_1..H_K] per problem; Bessel coefficients in the context precision.
        std::vector<char> hs(es * stack_elems);
        for (size_t i = 0; i < E->probs.size(); ++i) {
            const EnsProblem &p = E->probs[i];
            const size_t dd = (size_t)p.d * p.d;
            memcpy(hs.data() + es * p.stack_off, H0s[i], es * dd);
            if (p.K) memcpy(hs.data() + es * (p.stack_off + dd), H1s[i], es * dd * p.K);
        }
        std::vector<char> hj(es * (J.size() / 2));
        for (size_t k = 0; k < J.size() / 2; ++k) {
            if (E->fp64) {
                double v[2] = {J[2 * k], J[2 * k + 1]};
                memcpy(hj.data() + 16 * k, v, 16);
            } else {
                float v[2] = {(float)J[2 * k], (float)J[2 * k + 1]};
                memcpy(hj.data() + 8 * k, v, 8);
            }
        }
        if (cudaMemcpy(E->d_stack.ptr, hs.data(), hs.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(E->d_J.ptr, hj.data(), hj.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            r = PARAMENT_FAIL;
    }
    E->carr_elems = carr_elems;
    E->out_elems = out_elems;
    if (r == PARAMENT_STATUS_SUCCESS) {
        if (E->fp64)
            set_kernel_smem<double>(E);
        else
            set_kernel_smem<float>(E);
        r = build_work(E, E->granularity);
    }
    if (r == PARAMENT_STATUS_SUCCESS && capture(E) != cudaSuccess) r = PARAMENT_STATUS_CUBLAS_FAILED;
    if (r != PARAMENT_STATUS_SUCCESS) {
        cudaGetLastError();
        Parament_ensembleDestroy(reinterpret_cast<Parament_Ensemble *>(E));
        return r;
    }
    *out = reinterpret_cast<Parament_Ensemble *>(E);
    return PARAMENT_STATUS_SUCCESS;
}

Parament_ErrorCode Parament_ensembleSetSamples(Parament_Ensemble *ens, const void *const *carrs) {
    Ensemble *E = reinterpret_cast<Ensemble *>(ens);
    if (!E || !carrs) return PARAMENT_STATUS_INVALID_VALUE;
    cudaSetDevice(E->device);
    const size_t es = E->fp64 ? 16 : 8;
    for (size_t i = 0; i < E->probs.size(); ++i) {
        const EnsProblem &p = E->probs[i];
        if (p.K && !carrs[i]) return PARAMENT_STATUS_INVALID_VALUE;
        if (p.K) memcpy(static_cast<char *>(E->h_carr) + es * p.carr_off, carrs[i], es * (size_t)p.K * p.pts);
    }
    if (cudaMemcpyAsync(E->d_carr.ptr, E->h_carr, es * std::max(1LL, E->carr_elems), cudaMemcpyHostToDevice,
                        E->stream) != cudaSuccess ||
        cudaStreamSynchronize(E->stream) != cudaSuccess) {
        cudaGetLastError();
        return PARAMENT_FAIL;
    }
    return PARAMENT_STATUS_SUCCESS;
}

Parament_ErrorCode Parament_ensembleRun(Parament_Ensemble *ens, void *const *outs) {
    Ensemble *E = reinterpret_cast<Ensemble *>(ens);
    if (!E) return PARAMENT_STATUS_INVALID_VALUE;
    cudaSetDevice(E->device);
    E->last_ms = timed_run(E);
    if (E->last_ms < 0) {
        cudaGetLastError();
        return PARAMENT_STATUS_CUBLAS_FAILED;
    }
    if (!outs) return PARAMENT_STATUS_SUCCESS;
    const size_t es = E->fp64 ? 16 : 8;
    if (cudaMemcpyAsync(E->h_out, E->d_out.ptr, es * E->out_elems, cudaMemcpyDeviceToHost, E->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(E->stream) != cudaSuccess) {
        cudaGetLastError();
        return PARAMENT_FAIL;
    }
    for (size_t i = 0; i < E->probs.size(); ++i)
        if (outs[i])
            memcpy(outs[i], static_cast<char *>(E->h_out) + es * E->probs[i].out_off,
                   es * (size_t)E->probs[i].d * E->probs[i].d);
    return PARAMENT_STATUS_SUCCESS;
}

Parament_ErrorCode Parament_ensembleTune(Parament_Ensemble *ens) {
    Ensemble *E = reinterpret_cast<Ensemble *>(ens);
    if (!E) return PARAMENT_STATUS_INVALID_VALUE;
    cudaSetDevice(E->device);
    static const double cands[] = {1.0, 2.0, 4.0, 8.0, 16.0, 32.0, 64.0};
    double best_g = E->granularity;
    float best = 1e30f;
    for (double g : cands) {
        if (build_work(E, g) != PARAMENT_STATUS_SUCCESS || capture(E) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        timed_run(E);  // warm
        float t = timed_run(E);
        if (t > 0 && t < best) {
            best = t;
            best_g = g;
        }
    }
    if (build_work(E, best_g) != PARAMENT_STATUS_SUCCESS || capture(E) != cudaSuccess) {
        cudaGetLastError();
        return PARAMENT_STATUS_CUBLAS_FAILED;
    }
    return PARAMENT_STATUS_SUCCESS;
}

double Parament_ensembleGranularity(Parament_Ensemble *ens) {
    Ensemble *E = reinterpret_cast<Ensemble *>(ens);
    return E ? E->granularity : 0.0;
}

float Parament_ensembleLastMs(Parament_Ensemble *ens) {
    Ensemble *E = reinterpret_cast<Ensemble *>(ens);
    return E ? E->last_ms : -1.0f;
}

Parament_ErrorCode Parament_ensembleDestroy(Parament_Ensemble *ens) {
    Ensemble *E = reinterpret_cast<Ensemble *>(ens);
    if (!E) return PARAMENT_STATUS_SUCCESS;
    cudaSetDevice(E->device);
    if (E->stream) cudaStreamSynchronize(E->stream);
    if (E->graph) cudaGraphExecDestroy(E->graph);
    for (DevBuf *b : {&E->d_probs, &E->d_items, &E->d_bundles, &E->d_counter, &E->d_stack, &E->d_carr, &E->d_J,
                      &E->d_chunks, &E->d_out})
        b->release();
    if (E->h_carr) cudaFreeHost(E->h_carr);
    if (E->h_out) cudaFreeHost(E->h_out);
    if (E->ev0) cudaEventDestroy(E->ev0);
    if (E->ev1) cudaEventDestroy(E->ev1);
    if (E->stream) cudaStreamDestroy(E->stream);
    delete E;
    return PARAMENT_STATUS_SUCCESS;
}

}  // extern "C"
