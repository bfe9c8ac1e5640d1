// Adjoint (reverse-mode) gradient of the equiprop propagator, d <= 64.
//
// For a seed W (d x d), computes for every real control sample u_k[i]
//
//     grad_k[i] = d/du_k[i] Re Tr(W^H U),   U = U_(P-1) ... U_1 U_0,
//
// i.e. the vector-Jacobian product of the propagator; a loss L(U) with
// dL = Re Tr(G^H dU) has dL/du = grad for W = G (the fidelity loss
// 1 - |Tr(V^H U)|^2/d^2 uses W = -(2/d^2) Tr(V^H U) V).  No counterpart in the
// reference; the forward map is the reference's: U_j = p(X_j) with p the
// Chebyshev-Bessel polynomial of src/cuda/parament.cpp:569-652.
//
// With R_j = U_(j-1)..U_0 (earlier steps) and L_j = U_(P-1)..U_(j+1) (later),
//   d Re Tr(W^H U) = Re sum_j Tr(B_j dU_j),   B_j = R_j W^H L_j,
// and, since the Frechet derivative of a matrix polynomial is self-adjoint
// under (A, B) -> Tr(A B),  Tr(B_j Dp(X_j)[dX_j]) = Tr(Gamma_j dX_j) with
// Gamma_j = Dp(X_j)[B_j].  Gamma_j comes from differentiating the Clenshaw
// recurrence in direction B_j (two extra products per order), and
// t_m[j] = Tr(Gamma_j S_m) for the expansion matrices S_m turns into sample
// gradients through the quadrature weights.
//
// Schedule (one launch per phase):
//   1. chunk products S_c of nc chunks of consecutive steps (k_small_steps),
//      nc about one per SM, so that the chunk boundaries -- the checkpoints --
//      come every P / nc steps (about sqrt(P) steps at the gradient workload,
//      16384 steps in 152 chunks);
//   2. exclusive prefix/suffix products of the chunks (Hillis-Steele scans):
//      R at every chunk start and L at every chunk end;
//   3. one CTA per chunk sweeps its steps backward carrying M_j = W^H L_j and
//      recomputing the rest: U_j from X_j, R_j = U_j^H R_(j+1) from the
//      chunk-end checkpoint R_(s1) = S_c R_(s0) (the step exponentials of the
//      automatic order are unitary to working precision), B_j = R_j M_j,
//      then U_j and Gamma_j together, and the traces t_m[j].  Nothing per
//      step is stored but the Ke traces.  A manual Chebyshev order can leave
//      U_j far from unitary; then the CTA first sweeps forward from R_(s0)
//      storing every R_j of its chunk (one d x d matrix per step) and the
//      backward sweep reads them;
//   4. sample gradients from the traces (quadrature / Magnus adjoint).
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "ctx.h"
#include "kernels.h"

namespace pgb {

template <class R>
struct AdjArgs {
    cplx_t<R> J[kMaxOrder + 1];
    const cplx_t<R> *stack;
    const cplx_t<R> *carr;
    const cplx_t<R> *pre;  // nc exclusive prefix products (R at each chunk start)
    const cplx_t<R> *suf;  // nc exclusive suffix products (L at each chunk end)
    const cplx_t<R> *W;    // seed, d x d
    const cplx_t<R> *chunks;  // nc chunk products S_c
    cplx_t<R> *Rbuf;       // P stored R_j (stored form only)
    cplx_t<R> *tr;         // P x Ke traces
    long long P;
    int nchunks;
    int d, Ke, M;
    int reversible;        // 1: R_j = U_j^H R_(j+1) in the backward sweep; 0: stored R_j
    R s;
    WeightSpec w;
};

template <class C>
__device__ __forceinline__ C warp_sum(C v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

template <class R, int TM>
__global__ void __launch_bounds__(256) k_adj_chunks(const __grid_constant__ AdjArgs<R> a) {
    using C = cplx_t<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int d = a.d, dd = d * d, ld = d + 1, sz = d * ld;
    C *Xs = reinterpret_cast<C *>(smem_raw);
    C *Bs = Xs + sz;   // B_j
    C *B1 = Bs + sz;   // b_(k+1); scratch operand
    C *D1 = B1 + sz;   // derivative of b_(k+1)
    C *Ms = D1 + sz;   // W^H L_j
    C *Rs = Ms + sz;   // R_j
    C *ws = Rs + sz;   // step weights
    C *red = ws + a.Ke;  // 8 x Ke partial traces
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15, lane = tid & 31, warp = tid >> 5;
    const long long s0 = a.P * blockIdx.x / a.nchunks;
    const long long s1 = a.P * (blockIdx.x + 1) / a.nchunks;
    const int M = a.M;
    const R s = a.s;
    const C zero = mk<C>(0.0, 0.0);

    bool own[TM][TM], dg[TM][TM];
    int eo[TM][TM], ge[TM][TM], gt[TM][TM];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TM; ++j) {
            int r = ty + 16 * i, c = tx + 16 * j;
            own[i][j] = r < d && c < d;
            eo[i][j] = r * ld + c;
            ge[i][j] = r * d + c;
            gt[i][j] = c * d + r;
            dg[i][j] = r == c;
        }
    C acc[TM][TM], acc2[TM][TM], b2[TM][TM], d2[TM][TM];

    // Weights and X_j (own elements into Xs); returns nothing, needs a sync after.
    auto assemble = [&](long long st) {
        for (int m = tid; m < a.Ke; m += blockDim.x) ws[m] = step_weight(a.carr, a.w, m, st);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j) {
                if (!own[i][j]) continue;
                C v = a.stack[ge[i][j]];
                for (int m = 0; m < a.Ke; ++m) cfma(v, ws[m], a.stack[(size_t)(m + 1) * dd + ge[i][j]]);
                Xs[eo[i][j]] = v;
            }
    };

    // U of the step in Xs by the reference's Clenshaw recurrence (own
    // elements in acc; B1 is scratch).  Starts and ends with all threads past
    // their last read of B1.
    auto clenshaw_u = [&]() {
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j) {
                if (!own[i][j]) continue;
                C x = Xs[eo[i][j]];
                C v = cscale(cmul(a.J[M], x), s);
                if (dg[i][j]) v = cadd(v, a.J[M - 1]);
                if (M == 1) {
                    acc[i][j] = v;
                } else {
                    b2[i][j] = dg[i][j] ? a.J[M] : zero;
                    B1[eo[i][j]] = v;
                }
            }
        __syncthreads();
        for (int k = M - 2; k >= 0; --k) {
            tile_gemm<C, TM>(acc, B1, Xs, d, ld, ty, tx);
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
                    if (dg[i][j]) v = cadd(v, a.J[k]);
                    if (k > 0) {
                        b2[i][j] = B1[eo[i][j]];
                        B1[eo[i][j]] = v;
                    } else {
                        acc[i][j] = v;
                    }
                }
            if (k > 0) __syncthreads();
        }
    };

    if (a.reversible) {
        // ---- checkpoint at the chunk end: R_(s1) = S_c R_(s0)
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j)
                if (own[i][j]) {
                    B1[eo[i][j]] = a.chunks[(size_t)blockIdx.x * dd + ge[i][j]];
                    Rs[eo[i][j]] = a.pre[(size_t)blockIdx.x * dd + ge[i][j]];
                }
        __syncthreads();
        tile_gemm<C, TM>(acc, B1, Rs, d, ld, ty, tx);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j)
                if (own[i][j]) Rs[eo[i][j]] = acc[i][j];
    } else {
        // ---- forward sweep: stored R_j for j in [s0, s1)
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j)
                if (own[i][j]) Rs[eo[i][j]] = a.pre[(size_t)blockIdx.x * dd + ge[i][j]];
        for (long long st = s0; st < s1; ++st) {
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j)
                    if (own[i][j]) a.Rbuf[(size_t)st * dd + ge[i][j]] = Rs[eo[i][j]];
            if (st + 1 == s1) break;
            assemble(st);
            clenshaw_u();
            // R <- U R = R + (U - I) R
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j)
                    if (own[i][j]) {
                        C u = acc[i][j];
                        if (dg[i][j]) u.x -= (R)1;
                        B1[eo[i][j]] = u;
                    }
            __syncthreads();
            tile_gemm<C, TM>(acc, B1, Rs, d, ld, ty, tx);
            __syncthreads();
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j)
                    if (own[i][j]) Rs[eo[i][j]] = cadd(Rs[eo[i][j]], acc[i][j]);
            __syncthreads();
        }
    }
    __syncthreads();

    // ---- backward sweep.  M = W^H L_(s1-1), L_(s1-1) = suffix after this chunk.
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TM; ++j)
            if (own[i][j]) {
                C w = a.W[gt[i][j]];
                B1[eo[i][j]] = mk<C>(w.x, -w.y);
                D1[eo[i][j]] = a.suf[(size_t)blockIdx.x * dd + ge[i][j]];
            }
    __syncthreads();
    tile_gemm<C, TM>(acc, B1, D1, d, ld, ty, tx);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TM; ++j)
            if (own[i][j]) Ms[eo[i][j]] = acc[i][j];

    for (long long st = s1 - 1; st >= s0; --st) {
        if (!a.reversible) {
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j)
                    if (own[i][j]) Rs[eo[i][j]] = a.Rbuf[(size_t)st * dd + ge[i][j]];
        }
        assemble(st);
        __syncthreads();
        if (a.reversible) {
            // R_j = U_j^H R_(j+1) = R_(j+1) + (U_j - I)^H R_(j+1)
            clenshaw_u();
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j)
                    if (own[i][j]) {
                        C u = acc[i][j];
                        if (dg[i][j]) u.x -= (R)1;
                        // conjugate transpose: element (r, c) of (U - I) goes to (c, r)
                        B1[(tx + 16 * j) * ld + ty + 16 * i] = mk<C>(u.x, -u.y);
                    }
            __syncthreads();
            tile_gemm<C, TM>(acc, B1, Rs, d, ld, ty, tx);
            __syncthreads();
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j)
                    if (own[i][j]) Rs[eo[i][j]] = cadd(Rs[eo[i][j]], acc[i][j]);
            __syncthreads();
        }
        // B_j = R_j M_j
        tile_gemm<C, TM>(acc, Rs, Ms, d, ld, ty, tx);
        // First Clenshaw order (b_M = J[M] I, derivative 0) needs own elements only:
        //   b_(M-1) = s J[M] X + J[M-1] I,  db_(M-1) = s J[M] B.
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j) {
                if (!own[i][j]) continue;
                const int e = eo[i][j];
                C bj = acc[i][j];
                Bs[e] = bj;
                C v = cscale(cmul(a.J[M], Xs[e]), s);
                if (dg[i][j]) v = cadd(v, a.J[M - 1]);
                C dv = cscale(cmul(a.J[M], bj), s);
                if (M == 1) {
                    acc[i][j] = v;
                    acc2[i][j] = dv;
                } else {
                    b2[i][j] = dg[i][j] ? a.J[M] : zero;
                    d2[i][j] = zero;
                    B1[e] = v;
                    D1[e] = dv;
                }
            }
        __syncthreads();
        for (int k = M - 2; k >= 0; --k) {
            tile_gemm<C, TM>(acc, B1, Xs, d, ld, ty, tx);
            tile_gemm<C, TM>(acc2, D1, Xs, d, ld, ty, tx, B1, Bs);
            __syncthreads();
            const R beta = (k == 0) ? (R)-2 : (R)-1;
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) {
                    if (!own[i][j]) continue;
                    const int e = eo[i][j];
                    C v = cscale(acc[i][j], s);
                    v.x += beta * b2[i][j].x;
                    v.y += beta * b2[i][j].y;
                    if (dg[i][j]) v = cadd(v, a.J[k]);
                    C dv = cscale(acc2[i][j], s);
                    dv.x += beta * d2[i][j].x;
                    dv.y += beta * d2[i][j].y;
                    if (k > 0) {
                        b2[i][j] = B1[e];
                        B1[e] = v;
                        d2[i][j] = D1[e];
                        D1[e] = dv;
                    } else {
                        acc[i][j] = v;    // U_j
                        acc2[i][j] = dv;  // Gamma_j
                    }
                }
            if (k > 0) __syncthreads();
        }
        // Traces t_m = Tr(Gamma S_m) = sum_(r,c) Gamma[r][c] S_m[c][r].
        for (int m = 0; m < a.Ke; ++m) {
            C p = zero;
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j)
                    if (own[i][j]) cfma(p, acc2[i][j], a.stack[(size_t)(m + 1) * dd + gt[i][j]]);
            p = warp_sum(p);
            if (lane == 0) red[warp * a.Ke + m] = p;
        }
        __syncthreads();
        for (int m = tid; m < a.Ke; m += blockDim.x) {
            C t = zero;
            for (int w8 = 0; w8 < (int)(blockDim.x >> 5); ++w8) t = cadd(t, red[w8 * a.Ke + m]);
            a.tr[(size_t)st * a.Ke + m] = t;
        }
        // M <- M U = M + M (U - I)
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j)
                if (own[i][j]) {
                    C u = acc[i][j];
                    if (dg[i][j]) u.x -= (R)1;
                    B1[eo[i][j]] = u;
                }
        __syncthreads();
        tile_gemm<C, TM>(acc, Ms, B1, d, ld, ty, tx);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j)
                if (own[i][j]) Ms[eo[i][j]] = cadd(Ms[eo[i][j]], acc[i][j]);
        __syncthreads();
    }
}

// grad[k][i] = Re sum_(j,m) t_m[j] dw_m[j]/du_k[i] for real samples
// (weights of src/cuda/control_expansion.cu:27-170, pair slots triangular).
template <class R>
__global__ void k_adj_samples(const cplx_t<R> *__restrict__ tr, const cplx_t<R> *__restrict__ carr, R *grad,
                              long long P, int Ke, WeightSpec w) {
    using C = cplx_t<R>;
    const long long pts = w.pts;
    const long long n = (long long)w.amps * pts;
    const C f = mk<C>(0.0, w.hfac);
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(idx / pts);
        const long long i = idx % pts;
        C g = mk<C>(0.0, 0.0);
        auto T = [&](long long j, int m) { return tr[(size_t)j * Ke + m]; };
        auto U = [&](int c, long long t) { return carr[(size_t)c * pts + t]; };
        if (w.magnus || w.mode == kQuadSimpson) {
            // sample i enters step j = i/2 (i even: weight 1/6 as 2j; i odd: 4/6 as 2j+1)
            // and step i/2 - 1 (i even: weight 1/6 as 2j+2)
            if (i % 2 == 1) {
                long long j = (i - 1) / 2;
                if (j < P) g = cadd(g, cscale(T(j, k), (R)(4.0 / 6.0)));
            } else {
                long long ja = i / 2, jb = i / 2 - 1;
                if (ja < P) g = cadd(g, cscale(T(ja, k), (R)(1.0 / 6.0)));
                if (jb >= 0 && jb < P) g = cadd(g, cscale(T(jb, k), (R)(1.0 / 6.0)));
                if (w.magnus) {
                    const int K = w.K;
                    // [H0, H_k]: w = f (u[2j+2] - u[2j])
                    if (ja < P) g = csub(g, cmul(f, T(ja, K + k)));
                    if (jb >= 0 && jb < P) g = cadd(g, cmul(f, T(jb, K + k)));
                    // pairs (a<b): w = f (u_a[2j] u_b[2j+2] - u_a[2j+2] u_b[2j])
                    for (int o = 0; o < w.amps; ++o) {
                        if (o == k) continue;
                        const int lo = min(o, k), hi = max(o, k);
                        const int m = 2 * K + hi * (hi - 1) / 2 + lo;
                        if (ja < P) {  // i = 2 ja
                            C c = (k == lo) ? U(hi, 2 * ja + 2) : mk<C>(-U(lo, 2 * ja + 2).x, -U(lo, 2 * ja + 2).y);
                            g = cadd(g, cmul(cmul(f, c), T(ja, m)));
                        }
                        if (jb >= 0 && jb < P) {  // i = 2 jb + 2
                            C c = (k == lo) ? mk<C>(-U(hi, 2 * jb).x, -U(hi, 2 * jb).y) : U(lo, 2 * jb);
                            g = cadd(g, cmul(cmul(f, c), T(jb, m)));
                        }
                    }
                }
            }
        } else if (w.mode == kQuadMidpoint) {
            if (i < P) g = cadd(g, cscale(T(i, k), (R)0.5));
            if (i >= 1 && i - 1 < P) g = cadd(g, cscale(T(i - 1, k), (R)0.5));
        } else {
            if (i < P) g = T(i, k);
        }
        grad[idx] = g.x;
    }
}

size_t adj_smem_bytes(bool fp64, int d, int Ke) {
    size_t c = fp64 ? 16 : 8;
    return c * (6 * (size_t)d * (d + 1) + (size_t)Ke + 8 * (size_t)std::max(Ke, 1));
}

template <class R, int TM>
static const void *adj_ptr() {
    return reinterpret_cast<const void *>(&k_adj_chunks<R, TM>);
}
static const void *pick_adj(bool fp64, int d) {
    int tm = (d + 15) / 16;
    if (fp64) {  // complex128 is limited to d <= 48 (shared memory)
        switch (tm) {
            case 1: return adj_ptr<double, 1>();
            case 2: return adj_ptr<double, 2>();
            default: return adj_ptr<double, 3>();
        }
    }
    switch (tm) {
        case 1: return adj_ptr<float, 1>();
        case 2: return adj_ptr<float, 2>();
        case 3: return adj_ptr<float, 3>();
        default: return adj_ptr<float, 4>();
    }
}

// Hillis-Steele scans over nc chunk products (all d x d, later on the left).
// prefix: out[c] = S_(c-1) ... S_0 (out[0] = I); suffix: out[c] = S_(nc-1) ... S_(c+1).
static cudaError_t chunk_scan(bool fp64, int d, const void *S, long long nc, void *out, void *t1, void *t2,
                              bool prefix, cudaStream_t st, int num_sms) {
    const size_t es = fp64 ? 16 : 8, dd = (size_t)d * d, mb = dd * es;
    cudaError_t e = cudaMemcpyAsync(t1, S, mb * nc, cudaMemcpyDeviceToDevice, st);
    char *cur = static_cast<char *>(t1), *nxt = static_cast<char *>(t2);
    for (long long o = 1; o < nc && e == cudaSuccess; o *= 2) {
        GemmLaunch g{};
        g.fp64 = fp64;
        g.d = d;
        g.batch = (int)(nc - o);
        g.alpha_re = 1.0;
        g.stream = st;
        g.num_sms = num_sms;
        if (prefix) {  // new[c] = old[c] old[c-o], c >= o
            g.A = cur + o * mb;
            g.B = cur;
            g.Cout = nxt + o * mb;
            e = cudaMemcpyAsync(nxt, cur, o * mb, cudaMemcpyDeviceToDevice, st);
        } else {  // new[c] = old[c+o] old[c], c < nc - o
            g.A = cur + o * mb;
            g.B = cur;
            g.Cout = nxt;
            e = cudaMemcpyAsync(nxt + (nc - o) * mb, cur + (nc - o) * mb, o * mb, cudaMemcpyDeviceToDevice, st);
        }
        g.strideA = g.strideB = g.strideCout = (long long)dd;
        if (e == cudaSuccess) e = launch_gemm(g);
        std::swap(cur, nxt);
    }
    if (e != cudaSuccess) return e;
    // Exclusive form: shift by one chunk and put the identity at the open end.
    char *o8 = static_cast<char *>(out);
    if (prefix) {
        if (nc > 1) e = cudaMemcpyAsync(o8 + mb, cur, (nc - 1) * mb, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = fill_identity(fp64, o8, d, 1, 1.0, 0.0, st);
    } else {
        if (nc > 1) e = cudaMemcpyAsync(o8, cur + mb, (nc - 1) * mb, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = fill_identity(fp64, o8 + (nc - 1) * mb, d, 1, 1.0, 0.0, st);
    }
    return e;
}

template <class R>
static cudaError_t launch_adj_t(Ctx *c, const void *d_carr, unsigned pts, unsigned amps, const void *d_W,
                                void *d_grad, int M, const double *J, double h, long long P, int nc, bool reversible,
                                cudaStream_t st) {
    using C = cplx_t<R>;
    const int d = (int)c->dim;
    const size_t es = sizeof(C), dd = (size_t)d * d;
    WeightSpecHost wh{pts, (int)c->K, (int)amps, c->quad, c->magnus ? 1 : 0,
                      sizeof(R) == 8 ? h / 12.0 : (double)(float)h / 12.0};
    char *chunks = static_cast<char *>(c->chunks.ptr);
    char *scan = static_cast<char *>(c->work.ptr);  // pre | suf | t1 | t2
    char *pre = scan, *suf = scan + nc * dd * es, *t1 = suf + nc * dd * es, *t2 = t1 + nc * dd * es;
    // 1. chunk products
    StepLaunch l{};
    l.fp64 = sizeof(R) == 8;
    l.d = d;
    l.Ke = (int)c->Ke;
    l.w = wh;
    l.M = M;
    l.J = J;
    l.s = 2.0 / c->hnorm;
    l.stack = c->stack.ptr;
    l.carr = d_carr;
    l.chunks = chunks;
    l.P = P;
    l.nchunks = nc;
    l.stream = st;
    cudaError_t e = launch_small_steps(l);
    // 2. scans
    if (e == cudaSuccess) e = chunk_scan(l.fp64, d, chunks, nc, pre, t1, t2, true, st, c->num_sms);
    if (e == cudaSuccess) e = chunk_scan(l.fp64, d, chunks, nc, suf, t1, t2, false, st, c->num_sms);
    if (e != cudaSuccess) return e;
    // 3. per-chunk sweeps
    AdjArgs<R> a;
    for (int k = 0; k <= M; ++k) a.J[k] = mk<C>(J[2 * k], J[2 * k + 1]);
    a.stack = static_cast<const C *>(c->stack.ptr);
    a.carr = static_cast<const C *>(d_carr);
    a.pre = reinterpret_cast<const C *>(pre);
    a.suf = reinterpret_cast<const C *>(suf);
    a.W = static_cast<const C *>(d_W);
    a.chunks = reinterpret_cast<const C *>(chunks);
    a.reversible = reversible ? 1 : 0;
    a.Rbuf = reversible ? nullptr : static_cast<C *>(c->X.ptr);
    a.tr = static_cast<C *>(c->aux.ptr);
    a.P = P;
    a.nchunks = nc;
    a.d = d;
    a.Ke = (int)c->Ke;
    a.M = M;
    a.s = (R)(2.0 / c->hnorm);
    a.w = WeightSpec{wh.pts, wh.K, wh.amps, wh.mode, wh.magnus, wh.hfac};
    const void *fn = pick_adj(l.fp64, d);
    const size_t smem = adj_smem_bytes(l.fp64, d, (int)c->Ke);
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void *args[] = {&a};
    if (c->timing) cudaEventRecord(c->ev_start, st);
    e = cudaLaunchKernel(fn, dim3(nc), dim3(256), args, smem, st);
    if (c->timing) cudaEventRecord(c->ev_stop, st);
    if (e != cudaSuccess) return e;
    // 4. sample gradients
    const long long n = (long long)amps * pts;
    if (n > 0) {
        int blocks = (int)std::min<long long>((n + 255) / 256, 4096);
        k_adj_samples<R><<<blocks, 256, 0, st>>>(a.tr, a.carr, static_cast<R *>(d_grad), P, (int)c->Ke, a.w);
        e = cudaGetLastError();
    }
    return e;
}

int adj_max_dim(bool fp64) { return fp64 ? 48 : 64; }

Parament_ErrorCode run_vjp(Ctx *c, const void *d_carr, double dt, unsigned pts, unsigned amps, const void *d_W,
                           void *d_grad, cudaStream_t stream) {
    if (!c->has_h) return PARAMENT_STATUS_NO_HAMILTONIAN;
    const int d = (int)c->dim;
    if (amps > c->K || (amps > 0 && !d_carr) || !d_W || !d_grad) return PARAMENT_STATUS_INVALID_VALUE;
    if (d > adj_max_dim(c->fp64)) return PARAMENT_STATUS_INVALID_VALUE;
    const double h = (c->magnus || c->quad == PARAMENT_QUADRATURE_SIMPSON) ? 2.0 * dt : dt;
    const long long P = num_steps(c->quad, c->magnus, pts);
    if (P <= 0 || !(dt > 0.0) || !isfinite(dt) || c->hnorm == 0.0) return PARAMENT_STATUS_INVALID_VALUE;
    int M = c->manual ? (int)c->mmax : select_cycles(c->fp64, c->hnorm, h);
    if (M < 3 && !c->manual) return PARAMENT_STATUS_SELECT_SMALLER_DT;
    std::vector<double> J(2 * (M + 1));
    bessel_coeffs(M, h * c->hnorm, J.data());
    const void *fn = pick_adj(c->fp64, d);
    const size_t smem = adj_smem_bytes(c->fp64, d, (int)c->Ke);
    int per_sm = 0;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        return PARAMENT_STATUS_CUBLAS_FAILED;
    }
    const int nc = (int)std::max<long long>(1, std::min<long long>((long long)per_sm * c->num_sms, P));
    const size_t es = c->esize(), dd = (size_t)d * d;
    // The order tables keep the truncation of every step exponential below
    // the working precision, so U_j^H inverts U_j; a manual order may not.
    const bool reversible = !c->manual;
    if (c->chunks.ensure(es * dd * nc) != cudaSuccess || c->work.ensure(4 * es * dd * nc) != cudaSuccess ||
        (!reversible && c->X.ensure(es * dd * (size_t)P) != cudaSuccess) ||
        c->aux.ensure(es * (size_t)P * std::max(1u, c->Ke)) != cudaSuccess)
        return PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
    cudaError_t e = c->fp64 ? launch_adj_t<double>(c, d_carr, pts, amps, d_W, d_grad, M, J.data(), h, P, nc,
                                                   reversible, stream)
                            : launch_adj_t<float>(c, d_carr, pts, amps, d_W, d_grad, M, J.data(), h, P, nc,
                                                  reversible, stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return PARAMENT_STATUS_CUBLAS_FAILED;
    }
    c->last_M = M;
    return PARAMENT_STATUS_SUCCESS;
}

}  // namespace pgb
