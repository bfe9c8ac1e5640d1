// Host-side launch interface of the equiprop kernels (no CUDA device code here).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace pgb {

// Maximum Chebyshev order accepted by the kernels (the fp64 order table stops at 41).
constexpr int kMaxOrder = 63;

struct WeightSpecHost {
    unsigned pts;
    int K;
    int amps;
    int mode;
    int magnus;
    double hfac;
};

// One plain-path propagation over the steps [0, P): the fused small-d kernel
// (d <= kSmallMaxDim) writes one ordered product per chunk of consecutive
// steps into `chunks`.
constexpr int kSmallMaxDim = 64;

struct StepLaunch {
    bool fp64;
    int d;
    int Ke;                   // expansion matrices beside H0
    WeightSpecHost w;
    int M;                    // odd Chebyshev order
    const double *J;          // 2*(M+1) doubles: (-i)^k J_k(x), k=0..M
    double s;                 // 2 / Hnorm
    const void *stack;        // (1+Ke) d x d matrices, context precision
    const void *carr;         // amps x pts samples, context precision
    void *chunks;             // nchunks d x d products (output)
    long long P;              // steps
    int nchunks;
    cudaStream_t stream;
};

// Number of chunks the small kernel uses for P steps (one wave of resident CTAs).
int small_chunk_count(bool fp64, int d, int Ke, long long P, int num_sms);
size_t small_smem_bytes(bool fp64, int d, int Ke);
cudaError_t launch_small_steps(const StepLaunch &a);

// The same plain complex64 propagation at d = 64 on the tcgen05 tensor cores
// (small_tc.cu): per batch of up to 65536 steps, the X planes of the batch
// (xplanes: small_tc_xplane_bytes(P)) and then one CTA per SM over the batch.
// *nchunks receives the number of chunk products written (complex64), at most
// small_tc_max_chunks(P, num_sms).  Non-null ev0 / ev1 are recorded around the
// step-kernel launches; `fault` is the context's counter of bounded waits that
// gave up.
bool small_tc_applies(bool fp64, int d, int Ke, int M);
size_t small_tc_xplane_bytes(long long P);
int small_tc_max_chunks(long long P, int num_sms);
cudaError_t launch_small_tc(const StepLaunch &l, int num_sms, float *xplanes, int *fault, int *nchunks,
                            cudaEvent_t ev0, cudaEvent_t ev1);

// C_b = alpha * A_b B_b + beta * Cin_b + diag * I for b < batch (all d x d,
// row-major; strides in elements; beta = beta + i beta_im).  Cin may alias
// Cout.  Cin may be null when beta == 0.
struct GemmLaunch {
    bool fp64;
    int d;
    int batch;
    const void *A;
    long long strideA;
    const void *B;
    long long strideB;
    const void *Cin;
    long long strideCin;
    void *Cout;
    long long strideCout;
    double alpha_re, alpha_im;
    double beta;
    double diag_re, diag_im;
    double beta_im;
    cudaStream_t stream;
    int num_sms;
    bool a_minus_identity;  // use A - I in place of A
    int *fault;             // device counter of bounded waits that gave up (tensor-core kernel)
    bool simt_only;         // FP32/FP64 SIMT kernel even where the tensor-core kernel applies
    // complex64 products without a rounding bias: the exact sliced tensor-core
    // kernel (tc_ozaki.cu) where it applies, the FP32 SIMT kernel otherwise.
    // `scales` is its scratch: oz_scale_ints(g) ints (null: SIMT).
    bool exact;
    int *scales;
};
cudaError_t launch_gemm(const GemmLaunch &g);

// Exact sliced complex64 GEMM (integer bf16 slices, tcgen05): d % 64 == 0,
// 128 <= d <= 2048, no A - I.
bool oz_gemm_applies(const GemmLaunch &g);
size_t oz_scale_ints(const GemmLaunch &g);
cudaError_t launch_oz_gemm(const GemmLaunch &g, int *scales);

// tcgen05 tensor-core complex64 GEMM (3xTF32), used by launch_gemm for
// complex64 with d >= 256 and d % 128 == 0.  A CTA whose bounded waits gave
// up adds one to *g.fault (the calling context's device counter).
bool tc_gemm_applies(const GemmLaunch &g);
cudaError_t launch_tc_gemm(const GemmLaunch &g);

// Tensor-core form of the split complex64 kernel (d = 64): whether it serves
// this problem.
bool split_tc_applies(int d, int Ke, int M);

// Ordered product of n d x d matrices (later index on the left), pairwise tree
// as src/cuda/parament.cpp:677-714.  `work` holds n*d*d elements and may be
// overwritten; `in` is overwritten too.  The result is copied into `out`.
// *levels (if given) receives the number of kernel launches.
cudaError_t tree_product(bool fp64, int d, void *in, long long n, void *work, void *out, cudaStream_t stream,
                         int num_sms, int *levels = nullptr, int *fault = nullptr);

// Fused plain-path kernel for 64 < d <= 128 (step_mid.cu): clusters of four
// CTAs, one cluster per chunk of steps, writing one product per chunk into
// `chunks` (l.nchunks = clusters).  mid_applies: whether the kernel's shared
// memory holds this dimension and precision.
bool mid_applies(bool fp64, int d, int Ke);
int mid_chunk_count(int num_sms, long long P);
cudaError_t launch_mid_steps(const StepLaunch &l);

// n complex numbers converted between complex64 and complex128 (to_fp64:
// complex64 -> complex128).
cudaError_t convert_complex(bool to_fp64, const void *src, void *dst, long long n, cudaStream_t stream);

// Ordered product of n complex64 chunk products (d <= 64) into the complex64
// result through the double-float tree (split.cu): buf128 holds n, bufb
// ceil(n / 2) d x d complex128-sized matrices.  *levels receives the launches.
cudaError_t tree_df_c64(int d, const float2 *chunks, long long n, void *buf128, void *bufb, float2 *out,
                        cudaStream_t stream, int *levels);

// Large-d plain path: the steps [s0, s1) are assembled, exponentiated and
// multiplied into one product written to `out`.  Buffers: X, B1, B2 each hold
// `batch` matrices.
struct LargeLaunch {
    bool fp64;
    int d;
    int Ke;
    WeightSpecHost w;
    int M;
    const double *J;
    double s;
    const void *stack;
    const void *carr;
    long long s0, s1;
    int batch;
    void *X, *B1, *B2;
    void *out;
    cudaStream_t stream;
    int num_sms;
    int *fault;  // device fault counter of the context (tensor-core products)
};
cudaError_t launch_large_range(const LargeLaunch &a, int *launches = nullptr);

// Device-side copies and fills.
cudaError_t fill_identity(bool fp64, void *dst, int d, long long count, double scale_re, double scale_im,
                          cudaStream_t stream);

}  // namespace pgb
