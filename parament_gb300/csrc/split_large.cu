// Split-precision complex64 form for d > 64 (the large dense workloads).
//
// The same polynomial as the d <= 64 split kernels (split.cu, split_tc.cu):
// U_j = I + E_j with the reference's Chebyshev-Bessel polynomial of
// src/cuda/parament.cpp:569-652 regrouped by powers of the step's
// Hamiltonian, here written in Z_j = h X_j:
//
//     E_j = c_0 I + a_1 Z_j + sum_(n=2..M) a_n Z_j^n,   a_n = mu_n / h^n,
//
// with c_0 = m_0 - 1 and the a_n from the Bessel coefficients in FP64.  What
// decides the precision is which terms carry the rounding:
//
//   * Z_j (assembled from the complex64 stack and the FP64 step weights),
//     c_0 and the first-order term a_1 Z_j are double-float (pairs of floats):
//     a float rounding of these repeats at every step and adds up coherently
//     over thousands of steps;
//   * p_j = sum_(n>=2) a_n Z_j^n is a few 1e-4 of the propagator and comes
//     from GEMMs by Horner's rule in Y = Z^2 with coefficients linear in Z:
//         R_top = a_(M-1) I + a_M Z,
//         R_i   = R_(i+1) Y + a_(2i+3) Z + a_(2i+2) I,   p = R_0 Y;
//   * the steps are multiplied into chunk products, one running product per
//     chunk of consecutive steps kept in double-float,
//         P <- P + E_j + E_j P          (U_j ... U_(s0) = I + P),
//     with E_j P from a GEMM of the float parts: its rounding is relative to
//     |E_j| |P|, so it does not grow with the distance of U from I;
//   * the chunk products are combined by the FP64 tree (gemm.cu).
//
// The GEMMs ask for products without a rounding bias (GemmLaunch::exact):
// the exact sliced tensor-core kernel (tc_ozaki.cu: integer bf16 slices, FP32
// accumulators that never round) for d % 64 == 0 up to 1536, the FP32 SIMT
// kernel otherwise.  Not the 3xTF32 kernel (k_tc_cgemm): the tensor core's FP32
// accumulation rounds with a bias, and at d = 512 over 700 steps the form
// measured 8.5e-6 against complex128 with every GEMM there, 5.8e-7 with only
// the Horner GEMMs there, 3.3e-8 on the SIMT kernel and 2.5e-8 on the exact
// kernel -- the error repeats at every step and the bar is 1e-6.
//
// Every chunk advances by one step per round: a round assembles Z for the
// active chunks' next steps (one batch item per chunk), runs the Horner GEMMs
// and the running-product GEMM on the batch, and updates the chunk products
// elementwise.  Chunk c covers L or L + 1 consecutive steps, the longer ones
// first, so that the chunks still active in a round are a prefix of the batch.
#include <math.h>

#include <algorithm>
#include <vector>

#include "ctx.h"
#include "kernels.h"
#include "split_common.cuh"

namespace pgb {

// Geometry of one round: chunk c starts at step c L + min(c, nlong) and has
// L + (c < nlong) steps; the round's item c is step start(c) + r.
struct SlRound {
    long long L;
    int nlong, r, nact, d;
    long long dd;
    double h;
    double2 top_a, top_b;  // R_top = top_a I + top_b Z
    double2 c0, a1;
    float2 *zhi, *zlo, *rtop, *p, *ehi, *elo, *dprod, *phi, *plo;
    int first;  // first round: the chunk product is E itself
};

__device__ __forceinline__ long long sl_step(const SlRound &q, int c) {
    return (long long)c * q.L + min(c, q.nlong) + q.r;
}

// (hi, lo) += w h for a double-float w and a float h (the product's rounding
// error and the sum's join lo; renormalised by the caller).
__device__ __forceinline__ void sl_mac(float &hi, float &lo, float wh, float wl, float h) {
    const float p = __fmul_rn(wh, h);
    float e = __fmaf_rn(wh, h, -p);
    e = __fmaf_rn(wl, h, e);
    float s, t;
    two_sum(hi, p, s, t);
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(t, e));
}

// Z = h (H_0 + sum_m w_m H_m) in double-float for the round's items, and
// R_top.  Block (x, item): the item's Ke weights go to shared memory first.
__global__ void __launch_bounds__(256) k_sl_assemble(const __grid_constant__ SplitArgs a,
                                                     const __grid_constant__ SlRound q) {
    extern __shared__ float4 wsh[];  // Ke weights: re hi, re lo, im hi, im lo
    const int item = blockIdx.y;
    const long long st = sl_step(q, item);
    for (int m = threadIdx.x; m < a.Ke; m += blockDim.x) {
        const double2 w = split_weight(a, m, st);
        const df re = df_from(w.x), im = df_from(w.y);
        wsh[m] = make_float4(re.hi, re.lo, im.hi, im.lo);
    }
    __syncthreads();
    const df hh = df_from(q.h);
    const size_t base = (size_t)item * q.dd;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < q.dd;
         e += (long long)gridDim.x * blockDim.x) {
        const float2 h0 = a.stack[e];
        float rh = h0.x, rl = 0.f, ih = h0.y, il = 0.f;
        for (int m = 0; m < a.Ke; ++m) {
            const float4 w = wsh[m];
            const float2 g = a.stack[(size_t)(m + 1) * q.dd + e];
            // (w_re + i w_im)(g_re + i g_im); the imaginary weight terms only
            // where the weight has one (uniform over the block).
            sl_mac(rh, rl, w.x, w.y, g.x);
            sl_mac(ih, il, w.x, w.y, g.y);
            if (w.z != 0.0f || w.w != 0.0f) {
                sl_mac(rh, rl, -w.z, -w.w, g.y);
                sl_mac(ih, il, w.z, w.w, g.x);
            }
        }
        const df zr = df_mul(df_norm(rh, rl), hh), zi = df_mul(df_norm(ih, il), hh);
        q.zhi[base + e] = make_float2(zr.hi, zi.hi);
        q.zlo[base + e] = make_float2(zr.lo, zi.lo);
        // R_top = top_a I + top_b Z in FP32 (it starts the small terms)
        const float br = (float)q.top_b.x, bi = (float)q.top_b.y;
        float tr = br * zr.hi - bi * zi.hi, ti = br * zi.hi + bi * zr.hi;
        if ((e / q.d) == (e % q.d)) tr += (float)q.top_a.x, ti += (float)q.top_a.y;
        q.rtop[base + e] = make_float2(tr, ti);
    }
}

// E = c_0 I + a_1 Z + p in double-float; on the first round also P = E.
__global__ void __launch_bounds__(256) k_sl_form_e(const __grid_constant__ SlRound q) {
    const long long n = q.dd * q.nact;
    const df c0r = df_from(q.c0.x), c0i = df_from(q.c0.y), a1r = df_from(q.a1.x), a1i = df_from(q.a1.y);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long e = i % q.dd;
        const float2 zh = q.zhi[i], zl = q.zlo[i], pp = q.p[i];
        const df zr = {zh.x, zl.x}, zi = {zh.y, zl.y};
        // a_1 Z = (a1r zr - a1i zi) + i (a1r zi + a1i zr)
        df er = df_add(df_mul(a1r, zr), df_neg(df_mul(a1i, zi)));
        df ei = df_add(df_mul(a1r, zi), df_mul(a1i, zr));
        if ((e / q.d) == (e % q.d)) {
            er = df_add(er, c0r);
            ei = df_add(ei, c0i);
        }
        er = df_add_f(er, pp.x);
        ei = df_add_f(ei, pp.y);
        q.ehi[i] = make_float2(er.hi, ei.hi);
        q.elo[i] = make_float2(er.lo, ei.lo);
        if (q.first) {
            q.phi[i] = make_float2(er.hi, ei.hi);
            q.plo[i] = make_float2(er.lo, ei.lo);
        }
    }
}

// P <- P + E + D (double-float), D = E P from the GEMM of the float parts.
__global__ void __launch_bounds__(256) k_sl_update(const __grid_constant__ SlRound q) {
    const long long n = q.dd * q.nact;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float2 ph = q.phi[i], pl = q.plo[i], eh = q.ehi[i], el = q.elo[i], dv = q.dprod[i];
        df wr = df_add(df{ph.x, pl.x}, df{eh.x, el.x});
        df wi = df_add(df{ph.y, pl.y}, df{eh.y, el.y});
        wr = df_add_f(wr, dv.x);
        wi = df_add_f(wi, dv.y);
        q.phi[i] = make_float2(wr.hi, wi.hi);
        q.plo[i] = make_float2(wr.lo, wi.lo);
    }
}

// Chunk products I + P in complex128.
__global__ void k_sl_finish(const float2 *phi, const float2 *plo, double2 *out, int d, long long n) {
    const long long dd = (long long)d * d;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long e = i % dd;
        double re = (double)phi[i].x + (double)plo[i].x, im = (double)phi[i].y + (double)plo[i].y;
        if ((e / d) == (e % d)) re += 1.0;
        out[i] = make_double2(re, im);
    }
}

__global__ void k_sl_to_c64(const double2 *src, float2 *dst, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = make_float2((float)src[i].x, (float)src[i].y);
}

// Number of chunks: about four waves of 128 x 128 GEMM tiles per batched
// product, between 4 and 64 chunks.
static int sl_chunks(int d, int num_sms, long long P) {
    const long long tiles = std::max<long long>(1, ((long long)d * d) / 16384);
    long long n = (4LL * num_sms + tiles - 1) / tiles;
    n = std::max<long long>(4, std::min<long long>(64, n));
    return (int)std::max<long long>(1, std::min<long long>(n, P));
}

Parament_ErrorCode run_split_large(Ctx *c, const SplitArgs &a, double h, void *d_out, cudaStream_t stream) {
    const int d = a.d, M = a.M;
    const long long dd = (long long)d * d, P = a.P;
    const int nch = sl_chunks(d, c->num_sms, P);
    const size_t mat = sizeof(float2) * (size_t)dd * nch;
    // zhi zlo y r0 r1 p ehi elo dprod phi plo
    constexpr int kBufs = 11;
    // Scratch of the exact GEMM: exponents of the row / column maxima of the
    // operands of one batched product (two operands of nch items).
    const size_t scale_bytes = sizeof(int) * 2 * (size_t)nch * d;
    if (c->xplanes.ensure(kBufs * mat + scale_bytes) != cudaSuccess ||
        c->chunks.ensure(sizeof(double2) * (size_t)dd * nch) != cudaSuccess ||
        c->work.ensure(sizeof(double2) * (size_t)dd * nch) != cudaSuccess ||
        c->aux.ensure(sizeof(double2) * (size_t)dd) != cudaSuccess)
        return PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
    float2 *buf[kBufs];
    for (int i = 0; i < kBufs; ++i)
        buf[i] = reinterpret_cast<float2 *>(static_cast<char *>(c->xplanes.ptr) + (size_t)i * mat);
    int *scales = reinterpret_cast<int *>(static_cast<char *>(c->xplanes.ptr) + (size_t)kBufs * mat);
    float2 *zhi = buf[0], *zlo = buf[1], *y = buf[2], *rb[2] = {buf[3], buf[4]}, *pp = buf[5], *ehi = buf[6],
           *elo = buf[7], *dprod = buf[8], *phi = buf[9], *plo = buf[10];
    // Coefficients in Z = h X: a_n = mu_n / h^n.
    std::vector<double2> an(M + 1);
    double hp = 1.0;
    for (int n = 1; n <= M; ++n) {
        hp *= h;
        an[n] = make_double2(a.mu[n].x / hp, a.mu[n].y / hp);
    }
    SlRound q{};
    q.L = P / nch;
    q.nlong = (int)(P % nch);
    q.d = d;
    q.dd = dd;
    q.h = h;
    q.top_a = an[M - 1];
    q.top_b = an[M];
    q.c0 = a.c0;
    q.a1 = an[1];
    q.zhi = zhi;
    q.zlo = zlo;
    q.p = pp;
    q.ehi = ehi;
    q.elo = elo;
    q.dprod = dprod;
    q.phi = phi;
    q.plo = plo;
    const long long rounds = q.L + (q.nlong > 0 ? 1 : 0);
    auto gemm = [&](const float2 *A, const float2 *B, const float2 *Cin, float2 *Cout, int batch, double2 beta,
                    double2 diag) {
        GemmLaunch g{};
        g.exact = true;
        g.scales = scales;
        g.fp64 = false;
        g.d = d;
        g.batch = batch;
        g.A = A;
        g.B = B;
        g.Cin = Cin;
        g.Cout = Cout;
        g.strideA = g.strideB = g.strideCin = g.strideCout = dd;
        g.alpha_re = 1.0;
        g.beta = beta.x;
        g.beta_im = beta.y;
        g.diag_re = diag.x;
        g.diag_im = diag.y;
        g.stream = stream;
        g.num_sms = c->num_sms;
        g.fault = c->d_fault;
        return launch_gemm(g);
    };
    const int ew_blocks = (int)std::min<long long>(8LL * c->num_sms, (dd * nch + 255) / 256);
    const int asm_bx = (int)std::max<long long>(1, std::min<long long>((dd + 255) / 256, (8LL * c->num_sms + nch - 1) / nch));
    const size_t asm_smem = sizeof(float4) * (size_t)std::max(1, a.Ke);
    int launches = 0;
    cudaError_t e = cudaSuccess;
    if (c->timing) cudaEventRecord(c->ev_start, stream);
    for (long long r = 0; r < rounds && e == cudaSuccess; ++r) {
        q.r = (int)r;
        q.nact = r < q.L ? nch : q.nlong;
        q.first = r == 0 ? 1 : 0;
        q.rtop = rb[0];
        k_sl_assemble<<<dim3(asm_bx, q.nact), 256, asm_smem, stream>>>(a, q);
        e = cudaGetLastError();
        ++launches;
        const double2 zero = make_double2(0, 0);
        // Y = Z^2, Horner in Y, p = R_0 Y.
        if (e == cudaSuccess) e = gemm(zhi, zhi, nullptr, y, q.nact, zero, zero), ++launches;
        int cur = 0;
        for (int i = (M - 3) / 2 - 1; i >= 0 && e == cudaSuccess; --i) {
            e = gemm(rb[cur], y, zhi, rb[cur ^ 1], q.nact, an[2 * i + 3], an[2 * i + 2]);
            cur ^= 1;
            ++launches;
        }
        if (e == cudaSuccess) e = gemm(rb[cur], y, nullptr, pp, q.nact, zero, zero), ++launches;
        if (e == cudaSuccess) {
            k_sl_form_e<<<ew_blocks, 256, 0, stream>>>(q);
            e = cudaGetLastError();
            ++launches;
        }
        if (r > 0 && e == cudaSuccess) {
            e = gemm(ehi, phi, nullptr, dprod, q.nact, zero, zero);
            ++launches;
            if (e == cudaSuccess) {
                k_sl_update<<<ew_blocks, 256, 0, stream>>>(q);
                e = cudaGetLastError();
                ++launches;
            }
        }
    }
    if (c->timing) cudaEventRecord(c->ev_stop, stream);
    int levels = 0;
    double2 *chunks = static_cast<double2 *>(c->chunks.ptr);
    if (e == cudaSuccess) {
        k_sl_finish<<<ew_blocks, 256, 0, stream>>>(phi, plo, chunks, d, dd * nch);
        e = cudaGetLastError();
        ++launches;
    }
    if (e == cudaSuccess)
        e = tree_product(true, d, chunks, nch, c->work.ptr, c->aux.ptr, stream, c->num_sms, &levels, c->d_fault);
    if (e == cudaSuccess) {
        k_sl_to_c64<<<(int)std::min<long long>(1024, (dd + 255) / 256), 256, 0, stream>>>(
            static_cast<const double2 *>(c->aux.ptr), static_cast<float2 *>(d_out), dd);
        e = cudaGetLastError();
        ++launches;
    }
    c->launches = launches + levels;
    if (e != cudaSuccess) {
        cudaGetLastError();
        return PARAMENT_STATUS_CUBLAS_FAILED;
    }
    return PARAMENT_STATUS_SUCCESS;
}

}  // namespace pgb
