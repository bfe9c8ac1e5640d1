// Shared pieces of the split-precision complex64 form: double-float
// arithmetic (pairs of floats), the kernel arguments and the FP64 step weights
// read from complex64 samples.  Used by the SIMT kernel (split.cu) and the
// tensor-core kernel (split_tc.cu).
#pragma once

#include "common.cuh"

namespace pgb {

constexpr int kSplitMaxOrder = 15;
constexpr double kSplitMaxX = 0.5;
// X planes of the tensor-core form: four planes of 64 rows x 68 floats per
// step (69,632 bytes), formed for batches of up to kSplitXBatch steps at a
// time (4.6 GB for a full batch).
constexpr int kSplitXStride = 4 * 64 * 68;
constexpr long long kSplitXBatch = 65536;

// ---------------------------------------------------------------- double-float

struct df {
    float hi, lo;
};

__device__ __forceinline__ df df_from(double v) {
    float h = (float)v;
    return {h, (float)(v - (double)h)};
}
// s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ df df_norm(float hi, float lo) {
    float s = __fadd_rn(hi, lo);
    return {s, __fsub_rn(lo, __fsub_rn(s, hi))};
}
__device__ __forceinline__ df df_add(df a, df b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return df_norm(s, e);
}
__device__ __forceinline__ df df_add_f(df a, float b) {
    float s, e;
    two_sum(a.hi, b, s, e);
    return df_norm(s, __fadd_rn(e, a.lo));
}
// a * b to about 2^-44 relative (the lo*lo term is dropped).
__device__ __forceinline__ df df_mul(df a, df b) {
    float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_norm(p, e);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
    float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return df_norm(p, e);
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }

struct cdf {
    df re, im;
};
__device__ __forceinline__ cdf cdf_add(cdf a, cdf b) { return {df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ cdf cdf_add_c(cdf a, float2 b) { return {df_add_f(a.re, b.x), df_add_f(a.im, b.y)}; }
__device__ __forceinline__ cdf cdf_mul(cdf a, cdf b) {
    return {df_add(df_mul(a.re, b.re), df_neg(df_mul(a.im, b.im))), df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
// a * b with b a float complex.
__device__ __forceinline__ cdf cdf_mul_c(cdf a, float2 b) {
    return {df_add(df_mul_f(a.re, b.x), df_neg(df_mul_f(a.im, b.y))), df_add(df_mul_f(a.re, b.y), df_mul_f(a.im, b.x))};
}
__device__ __forceinline__ float2 cdf_hi(cdf a) { return make_float2(a.re.hi, a.im.hi); }
__device__ __forceinline__ float2 cdf_lo(cdf a) { return make_float2(a.re.lo, a.im.lo); }

// ---------------------------------------------------------------- kernel

struct SplitArgs {
    double2 c0;                         // m_0 - 1
    double2 mu[kSplitMaxOrder + 1];     // mu_n, n = 1..M
    const float2 *stack;                // (1+Ke) complex64 matrices (commutators rounded from FP64)
    const float2 *carr;                 // samples (complex64)
    double2 *chunks;                    // nchunks products I + E^P, complex128
    long long P;
    int nchunks;
    int d, Ke, M;
    unsigned pts;
    int K, amps, mode, magnus;
    double hfac;
    const float4 *wts;                  // P x Ke step weights in double-float (re hi, re lo, im hi, im lo)
    const float *xplanes;               // X planes of the steps of one launch (tensor-core form)
    int *fault;                         // the context's counter of CTAs whose bounded waits gave up
    int herm_stack;                     // H_0, H_k exactly Hermitian and the commutators exactly anti-Hermitian
};

// Weight m of step s in FP64 from complex64 samples (src/cuda/control_expansion.cu:27-170,
// pair slots re-indexed as in step_weight).
__device__ __forceinline__ double2 split_weight(const SplitArgs &a, int m, long long s) {
    const size_t pts = a.pts;
    auto ld = [&](int k, long long i) {
        float2 v = a.carr[(size_t)k * pts + i];
        return make_double2(v.x, v.y);
    };
    if (m < a.K) {
        if (m >= a.amps) return make_double2(0, 0);
        if (a.magnus || a.mode == kQuadSimpson) {
            double2 x = ld(m, 2 * s), y = ld(m, 2 * s + 1), z = ld(m, 2 * s + 2);
            return make_double2((x.x + 4.0 * y.x + z.x) / 6.0, (x.y + 4.0 * y.y + z.y) / 6.0);
        }
        if (a.mode == kQuadMidpoint) {
            double2 x = ld(m, s), y = ld(m, s + 1);
            return make_double2(0.5 * (x.x + y.x), 0.5 * (x.y + y.y));
        }
        return ld(m, s);
    }
    const double2 f = make_double2(0.0, a.hfac);
    if (m < 2 * a.K) {
        int k = m - a.K;
        if (k >= a.amps) return make_double2(0, 0);
        return cmul(csub(ld(k, 2 * s + 2), ld(k, 2 * s)), f);
    }
    int p = m - 2 * a.K;
    int i = 1;
    while ((i + 1) * i / 2 <= p) ++i;
    int j = p - i * (i - 1) / 2;
    if (i >= a.amps) return make_double2(0, 0);
    double2 t = csub(cmul(ld(j, 2 * s), ld(i, 2 * s + 2)), cmul(ld(j, 2 * s + 2), ld(i, 2 * s)));
    return cmul(t, f);
}

// Tensor-core form of the split kernel (split_tc.cu): for each batch of up
// to kSplitXBatch steps, the X planes (xplanes: kSplitXBatch x kSplitXStride
// floats) and then one CTA per SM over the batch.  *nchunks receives the
// number of chunk products written, at most ceil(P / kSplitXBatch) x num_sms.
// Non-null ev0 / ev1 are recorded just before the first and after the last
// step-kernel launch (one batch: around k_split_tc alone).
cudaError_t launch_split_tc(const SplitArgs &a, int num_sms, float *xplanes, int *nchunks, cudaStream_t stream,
                            cudaEvent_t ev0 = nullptr, cudaEvent_t ev1 = nullptr);

}  // namespace pgb
