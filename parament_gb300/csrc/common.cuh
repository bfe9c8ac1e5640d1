// Shared device helpers for the GB300 equiprop kernels.
//
// Complex numbers are float2/double2 (real part in .x), matching the
// interleaved layout of the C-ABI.  Matrices are row-major d x d.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"

namespace pgb {

template <class R>
struct V2;
template <>
struct V2<float> {
    using T = float2;
};
template <>
struct V2<double> {
    using T = double2;
};
template <class R>
using cplx_t = typename V2<R>::T;

template <class C>
__host__ __device__ __forceinline__ C mk(double re, double im) {
    C c;
    c.x = re;
    c.y = im;
    return c;
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

// acc += a * b with four fused multiply-adds.
__device__ __forceinline__ void cfma(float2 &acc, float2 a, float2 b) {
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(-a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(a.y, b.x, acc.y);
}
__device__ __forceinline__ void cfma(double2 &acc, double2 a, double2 b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}

// Quadrature modes (values of Parament_QuadratureSpec).
enum : int { kQuadNone = 0x00000000, kQuadMidpoint = 0x01000000, kQuadSimpson = 0x02000000 };

// Parameters that describe how the step weights are formed from the samples.
struct WeightSpec {
    unsigned pts;   // samples per control array
    int K;          // controls loaded with the Hamiltonian
    int amps;       // control arrays passed to equiprop (<= K); the rest are zero
    int mode;       // quadrature mode
    int magnus;     // 1: Magnus commutator terms (implies Simpson)
    double hfac;    // h/12 for the Magnus commutator coefficients
};

// Weight of expansion matrix m (1-based slot m+1 of the stack; slot 0 is H0)
// for step s.  Slots: [0,K) controls, [K,2K) commutators [H0,H_k],
// [2K, 2K+K(K-1)/2) pair commutators [H_j,H_i], j<i, at slot 2K+i(i-1)/2+j.
// Follows src/cuda/control_expansion.cu:27-170 with the pair slot re-indexed.
template <class C>
__device__ __forceinline__ C step_weight(const C *__restrict__ carr, const WeightSpec &w, int m, long long s) {
    using R = decltype(C().x);
    C zero = mk<C>(0.0, 0.0);
    const size_t pts = w.pts;
    if (m < w.K) {
        if (m >= w.amps) return zero;
        const C *u = carr + (size_t)m * pts;
        if (w.magnus || w.mode == kQuadSimpson) {
            C a = u[2 * s], b = u[2 * s + 1], c = u[2 * s + 2];
            C t = cadd(cadd(a, cscale(b, (R)4)), c);
            return mk<C>(t.x / (R)6, t.y / (R)6);
        }
        if (w.mode == kQuadMidpoint) return cscale(cadd(u[s], u[s + 1]), (R)0.5);
        return u[s];
    }
    const C f = mk<C>(0.0, w.hfac);
    if (m < 2 * w.K) {
        int k = m - w.K;
        if (k >= w.amps) return zero;
        const C *u = carr + (size_t)k * pts;
        return cmul(csub(u[2 * s + 2], u[2 * s]), f);
    }
    int p = m - 2 * w.K;
    int i = 1;
    while ((i + 1) * i / 2 <= p) ++i;
    int j = p - i * (i - 1) / 2;
    if (i >= w.amps) return zero;
    const C *ui = carr + (size_t)i * pts;
    const C *uj = carr + (size_t)j * pts;
    C t = csub(cmul(uj[2 * s], ui[2 * s + 2]), cmul(uj[2 * s + 2], ui[2 * s]));
    return cmul(t, f);
}

// acc[i][j] = sum_k A[r_i][k] B[k][c_j] (plus A2[r_i][k] B2[k][c_j] when A2 is
// given) for a thread's TM x TM micro-tile of a d x d product held in shared
// memory: 256 threads as 16 x 16, rows r_i = ty + 16 i, columns
// c_j = tx + 16 j.  Rows/columns past d are clamped reads whose results the
// caller discards.  Shared-memory matrices have row stride ld = d + 1, so the
// two rows a warp reads of A sit in different banks.
template <class C, int TM>
__device__ __forceinline__ void tile_gemm(C (&acc)[TM][TM], const C *__restrict__ A, const C *__restrict__ B, int d,
                                          int ld, int ty, int tx, const C *__restrict__ A2 = nullptr,
                                          const C *__restrict__ B2 = nullptr) {
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TM; ++j) acc[i][j] = mk<C>(0.0, 0.0);
    int ro[TM], co[TM];
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        ro[i] = min(ty + 16 * i, d - 1) * ld;
        co[i] = min(tx + 16 * i, d - 1);
    }
#pragma unroll 4
    for (int k = 0; k < d; ++k) {
        C a[TM], b[TM];
#pragma unroll
        for (int i = 0; i < TM; ++i) a[i] = A[ro[i] + k];
#pragma unroll
        for (int j = 0; j < TM; ++j) b[j] = B[k * ld + co[j]];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TM; ++j) cfma(acc[i][j], a[i], b[j]);
        if (A2) {
#pragma unroll
            for (int i = 0; i < TM; ++i) a[i] = A2[ro[i] + k];
#pragma unroll
            for (int j = 0; j < TM; ++j) b[j] = B2[k * ld + co[j]];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TM; ++j) cfma(acc[i][j], a[i], b[j]);
        }
    }
}

}  // namespace pgb
