/*
 * parament-gb300: C-ABI of the GB300-native equiprop library (libparament.so).
 *
 * The first block of declarations is the reference library's public interface,
 * kept name-for-name and type-for-type so that existing callers (the pyparament
 * ctypes wrapper, C programs) link and run unchanged.  Each declaration cites
 * the reference declaration it replaces (src/cuda/parament.h, src/cuda/mathhelper.h,
 * src/cuda/deviceInfo.c inside the parament project).
 *
 * The second block adds entry points that the reference does not have
 * (device-resident inputs, the split-precision form, the adjoint gradient and
 * batched ensembles).  They take plain pointers and sizes only.
 *
 * All matrices are row-major (C order) arrays of interleaved complex numbers.
 */
#ifndef PARAMENT_GB300_H_
#define PARAMENT_GB300_H_

#ifdef __cplusplus
extern "C" {
#else
#include <stdbool.h>
#endif

#if defined(__GNUC__)
#define PARAMENT_API __attribute__((visibility("default")))
#else
#define PARAMENT_API
#endif

#ifndef PARAMENT_NO_CUDA_TYPES
/* Opaque stand-ins for CUDA's complex types when cuComplex.h is not included:
 * two floats (cuComplex) or two doubles (cuDoubleComplex), real part first. */
typedef struct cuComplex cuComplex;
typedef struct cuDoubleComplex cuDoubleComplex;
#endif

typedef struct Parament_Context_f32 Parament_Context_f32;
typedef struct Parament_Context_f64 Parament_Context_f64;

/* Quadrature rule; same values as src/cuda/parament.h:64-69. */
typedef enum Parament_QuadratureSpec {
    PARAMENT_QUADRATURE_NONE = 0x00000000,
    PARAMENT_QUADRATURE_MIDPOINT = 0x01000000,
    PARAMENT_QUADRATURE_SIMPSON = 0x02000000
} Parament_QuadratureSpec;

/* Error codes; values 0..1000 as src/cuda/parament.h:74-130.  Codes above 1000
 * are new: they report conditions the reference left undefined. */
typedef enum Parament_ErrorCode {
    PARAMENT_STATUS_SUCCESS = 0,
    PARAMENT_STATUS_HOST_ALLOC_FAILED = 10,
    PARAMENT_STATUS_DEVICE_ALLOC_FAILED = 20,
    PARAMENT_STATUS_CUBLAS_INIT_FAILED = 30, /* kept for ABI compatibility; also reported when no CUDA device is usable */
    PARAMENT_STATUS_INVALID_VALUE = 50,
    PARAMENT_STATUS_CUBLAS_FAILED = 60, /* kept for ABI compatibility; reported when a kernel launch fails */
    PARAMENT_STATUS_SELECT_SMALLER_DT = 70,
    PARAMENT_STATUS_NO_HAMILTONIAN = 80,
    PARAMENT_STATUS_INVALID_QUADRATURE_SELECTION = 90,
    PARAMENT_FAIL = 1000,
    PARAMENT_STATUS_KERNEL_TIMEOUT = 1010, /* a bounded device-side wait of a tensor-core kernel gave up */
    PARAMENT_STATUS_SCRATCH_EXCEEDED = 1020 /* problem larger than Parament_equipropNoAlloc_fp64's fixed scratch */
} Parament_ErrorCode;

/* ---------------------------------------------------------------- reference ABI */

/* src/cuda/parament.h:155 */
PARAMENT_API Parament_ErrorCode Parament_create(Parament_Context_f32 **handle_p);
/* src/cuda/parament.h:177 */
PARAMENT_API Parament_ErrorCode Parament_destroy(Parament_Context_f32 *handle);
/* src/cuda/parament.h:219-220.  H1 holds `amps` matrices of dim*dim, back to back. */
PARAMENT_API Parament_ErrorCode Parament_setHamiltonian(Parament_Context_f32 *handle, cuComplex *H0, cuComplex *H1,
                                                        unsigned int dim, unsigned int amps, bool use_magnus,
                                                        Parament_QuadratureSpec quadrature_mode);
/* src/cuda/parament.h:261-262.  carr holds `amps` arrays of `pts` samples, back to back. */
PARAMENT_API Parament_ErrorCode Parament_equiprop(Parament_Context_f32 *handle, cuComplex *carr, double dt,
                                                  unsigned int pts, unsigned int amps, cuComplex *out);
/* src/cuda/parament.h:286 */
PARAMENT_API int Parament_selectIterationCycles_fp32(double H_norm, double dt);
/* src/cuda/parament.h:308 */
PARAMENT_API Parament_ErrorCode Parament_setIterationCyclesManually(Parament_Context_f32 *handle, unsigned int cycles);
/* src/cuda/parament.h:327 */
PARAMENT_API Parament_ErrorCode Parament_automaticIterationCycles(Parament_Context_f32 *handle);
/* src/cuda/parament.h:347 */
PARAMENT_API Parament_ErrorCode Parament_peekAtLastError(Parament_Context_f32 *handle);
/* src/cuda/parament.h:357 */
PARAMENT_API const char *Parament_errorMessage(Parament_ErrorCode errorCode);

/* src/cuda/parament.h:363 */
PARAMENT_API Parament_ErrorCode Parament_create_fp64(Parament_Context_f64 **handle_p);
/* src/cuda/parament.h:368 */
PARAMENT_API Parament_ErrorCode Parament_destroy_fp64(Parament_Context_f64 *handle);
/* src/cuda/parament.h:373-374 */
PARAMENT_API Parament_ErrorCode Parament_setHamiltonian_fp64(Parament_Context_f64 *handle, cuDoubleComplex *H0,
                                                             cuDoubleComplex *H1, unsigned int dim, unsigned int amps,
                                                             bool use_magnus, Parament_QuadratureSpec quadrature_mode);
/* src/cuda/parament.h:379-380 */
PARAMENT_API Parament_ErrorCode Parament_equiprop_fp64(Parament_Context_f64 *handle, cuDoubleComplex *carr, double dt,
                                                       unsigned int pts, unsigned int amps, cuDoubleComplex *out);
/* src/cuda/parament.h:385 */
PARAMENT_API Parament_ErrorCode Parament_setIterationCyclesManually_fp64(Parament_Context_f64 *handle,
                                                                         unsigned int cycles);
/* src/cuda/parament.h:390 */
PARAMENT_API Parament_ErrorCode Parament_automaticIterationCycles_fp64(Parament_Context_f64 *handle);
/* src/cuda/parament.h:395 */
PARAMENT_API Parament_ErrorCode Parament_peekAtLastError_fp64(Parament_Context_f64 *handle);
/* src/cuda/parament.h:400 */
PARAMENT_API int Parament_selectIterationCycles_fp64(double H_norm, double dt);

/* src/cuda/mathhelper.h:67 -- maximum absolute row sum of a dim x dim matrix */
PARAMENT_API double OneNorm(cuComplex *arr, unsigned int dim);
/* src/cuda/mathhelper.h:68 */
PARAMENT_API double OneNorm_fp64(cuDoubleComplex *arr, unsigned int dim);
/* src/cuda/deviceInfo.c:30 -- prints the CUDA devices to stdout */
PARAMENT_API void device_info(void);

/* ---------------------------------------------------------------- extensions */

/* Precision forms of a context (new; no reference counterpart).
 *   PARAMENT_PRECISION_PLAIN : the reference scheme in the context's own precision
 *                              (default; complex128 or complex64 arithmetic).
 *   PARAMENT_PRECISION_SPLIT : complex64 contexts only.  Step exponentials are
 *                              formed as U_j = I + E_j from the same
 *                              Chebyshev-Bessel polynomial regrouped by powers
 *                              of X_j: the step's Hamiltonian X_j and the
 *                              first-order term in double-float (pairs of
 *                              floats), the higher powers as sliced products
 *                              (bf16 slices of integers, accumulated exactly on
 *                              the tensor cores) at d = 64 and at d > 64 with
 *                              d % 64 == 0, FP32 products otherwise; each chunk
 *                              of consecutive steps is multiplied into a
 *                              double-float running product (sliced products
 *                              again on the tensor cores) and the chunk
 *                              products are combined by a double-float tree
 *                              (d <= 64) or an FP64 tree (d > 64).
 *                              The Chebyshev order is the smallest odd order
 *                              whose truncation summed over all steps stays
 *                              below 1e-9. */
typedef enum Parament_PrecisionMode {
    PARAMENT_PRECISION_PLAIN = 0,
    PARAMENT_PRECISION_SPLIT = 1
} Parament_PrecisionMode;

PARAMENT_API Parament_ErrorCode Parament_setPrecisionMode(Parament_Context_f32 *handle, int mode);
PARAMENT_API int Parament_getPrecisionMode(Parament_Context_f32 *handle);

/* Chebyshev order used by the last successful equiprop (0 before the first). */
PARAMENT_API int Parament_lastIterationCycles(Parament_Context_f32 *handle);
PARAMENT_API int Parament_lastIterationCycles_fp64(Parament_Context_f64 *handle);

/* Norm bound Hnorm = ||H0||_inf + sum_k ||H_k||_inf of the loaded Hamiltonian (0 if none). */
PARAMENT_API double Parament_hamiltonianNorm(Parament_Context_f32 *handle);
PARAMENT_API double Parament_hamiltonianNorm_fp64(Parament_Context_f64 *handle);

/* equiprop on device-resident buffers (new; the reference copies from host
 * memory at src/cuda/parament.cpp:477 and back at :846).  d_carr and d_out are
 * device pointers; the work is queued on `stream` (a cudaStream_t, or NULL for
 * the context's own stream) and the call returns without waiting. */
PARAMENT_API Parament_ErrorCode Parament_equipropDevice(Parament_Context_f32 *handle, const void *d_carr, double dt,
                                                        unsigned int pts, unsigned int amps, void *d_out,
                                                        void *stream);
PARAMENT_API Parament_ErrorCode Parament_equipropDevice_fp64(Parament_Context_f64 *handle, const void *d_carr,
                                                             double dt, unsigned int pts, unsigned int amps,
                                                             void *d_out, void *stream);

/* Adjoint gradient (new; no reference counterpart).  For a seed W (d x d,
 * row-major) returns, for every real control sample,
 *     grad[k*pts + i] = d/du_k[i]  Re Tr(W^H U),
 * U the propagator equiprop would return for the same arguments (the exact
 * derivative of the computed Chebyshev propagator, including the quadrature
 * and Magnus weights).  A loss L(U) with dL = Re Tr(G^H dU) has dL/du = grad
 * for W = G; for L = 1 - |Tr(V^H U)|^2 / d^2 use W = -(2/d^2) Tr(V^H U) V.
 * Controls are taken as real: the imaginary parts of the samples enter U but
 * get no derivative.  grad is float for complex64 contexts and double for
 * complex128 ones.  Limits: dim <= 64 (complex64) or 48 (complex128).
 * Memory: Ke traces per step plus five d x d matrices per chunk of steps
 * (about one chunk per resident CTA; the chunk boundaries are the
 * checkpoints, the propagators between them are recomputed).  With a manual
 * Chebyshev order the step exponentials need not be unitary, and one d x d
 * matrix per step is stored instead. */
PARAMENT_API Parament_ErrorCode Parament_equipropVJP(Parament_Context_f32 *handle, cuComplex *carr, double dt,
                                                     unsigned int pts, unsigned int amps, cuComplex *W, float *grad);
PARAMENT_API Parament_ErrorCode Parament_equipropVJP_fp64(Parament_Context_f64 *handle, cuDoubleComplex *carr,
                                                          double dt, unsigned int pts, unsigned int amps,
                                                          cuDoubleComplex *W, double *grad);
/* Same on device buffers, queued on `stream` (NULL: the context's stream). */
PARAMENT_API Parament_ErrorCode Parament_equipropVJPDevice(Parament_Context_f32 *handle, const void *d_carr, double dt,
                                                           unsigned int pts, unsigned int amps, const void *d_W,
                                                           void *d_grad, void *stream);
PARAMENT_API Parament_ErrorCode Parament_equipropVJPDevice_fp64(Parament_Context_f64 *handle, const void *d_carr,
                                                                double dt, unsigned int pts, unsigned int amps,
                                                                const void *d_W, void *d_grad, void *stream);

/* Batched ensembles (new; no reference counterpart).  nprob independent
 * problems, each with its own dim (<= 64), control count (<= 16), step count
 * and dt, one precision (fp64 = 1: complex128, else complex64) and one
 * quadrature (NONE, MIDPOINT or SIMPSON; no Magnus terms).  H0s[i] is dim x dim
 * and H1s[i] holds amps[i] matrices back to back, as for setHamiltonian.
 * Create uploads the Hamiltonians, plans the work and captures the persistent
 * launch in a CUDA graph; SetSamples copies carrs[i] (amps[i] x pts[i]) to the
 * device; Run replays the graph and copies each propagator to outs[i] (NULL:
 * leave on the device); Tune times candidate work granularities on this
 * ensemble and keeps the fastest.  Each problem uses the reference's scheme
 * (norm bound, order table of the precision, Clenshaw, time-ordered product). */
typedef struct Parament_Ensemble Parament_Ensemble;
PARAMENT_API Parament_ErrorCode Parament_ensembleCreate(Parament_Ensemble **out, int fp64, unsigned int nprob,
                                                        const unsigned int *dims, const unsigned int *amps,
                                                        const unsigned int *pts, const double *dts,
                                                        const void *const *H0s, const void *const *H1s,
                                                        int quadrature);
PARAMENT_API Parament_ErrorCode Parament_ensembleSetSamples(Parament_Ensemble *ens, const void *const *carrs);
PARAMENT_API Parament_ErrorCode Parament_ensembleRun(Parament_Ensemble *ens, void *const *outs);
PARAMENT_API Parament_ErrorCode Parament_ensembleTune(Parament_Ensemble *ens);
PARAMENT_API double Parament_ensembleGranularity(Parament_Ensemble *ens);
/* Device time of the last Run (graph launch to completion), milliseconds. */
PARAMENT_API float Parament_ensembleLastMs(Parament_Ensemble *ens);
PARAMENT_API Parament_ErrorCode Parament_ensembleDestroy(Parament_Ensemble *ens);

/* equiprop that allocates no device memory (no counterpart in the reference).
 * For callers that must not call cudaMalloc while they propagate: real-time
 * loops that cannot wait on the allocator, applications whose device memory
 * belongs to their own pool, plug-ins where runtime allocation is forbidden.
 * The Hamiltonian must be loaded beforehand (Parament_setHamiltonian_fp64
 * allocates once, at set-up); d_carr and d_out are the caller's device
 * buffers; the work goes to `stream` (NULL: the context's stream) and the call
 * returns without waiting.  Scratch lives in a fixed 24 MiB device array inside
 * the library (held on each GPU that loads it until exit).  Limits: complex128
 * contexts with dim <= 64; larger problems return
 * PARAMENT_STATUS_SCRATCH_EXCEEDED.  The first call on a device (and the first
 * after a cudaDeviceReset, which gives the device a new context) looks up the
 * array's address (cudaGetSymbolAddress) -- make it before any stream capture.
 * All calls share the array: calls that overlap on the GPU race; serialise them. */
PARAMENT_API Parament_ErrorCode Parament_equipropNoAlloc_fp64(Parament_Context_f64 *handle, const void *d_carr,
                                                              double dt, unsigned int pts, unsigned int amps,
                                                              void *d_out, void *stream);

/* Completion and faults (new).  The device-buffer entry points queue their
 * work and return.  Parament_synchronize waits until the last call's work on
 * the context is done and returns PARAMENT_STATUS_KERNEL_TIMEOUT if a bounded
 * device-side wait of one of its tensor-core kernels gave up since the last
 * report (that call's result is then not valid), PARAMENT_STATUS_SUCCESS
 * otherwise.  Such a give-up is also reported by the host-buffer entry point
 * that ran the kernel, and by the next device-buffer call on the context once
 * it is known (that call then queues nothing). */
PARAMENT_API Parament_ErrorCode Parament_synchronize(Parament_Context_f32 *handle);
PARAMENT_API Parament_ErrorCode Parament_synchronize_fp64(Parament_Context_f64 *handle);
/* Bytes of device memory the context's buffers hold (Hamiltonian and work
 * buffers; grow-only until Parament_destroy). */
PARAMENT_API unsigned long long Parament_deviceMemoryBytes(Parament_Context_f32 *handle);
PARAMENT_API unsigned long long Parament_deviceMemoryBytes_fp64(Parament_Context_f64 *handle);

/* Instrumentation (new).  With timing enabled, each equiprop records CUDA
 * events on its stream around its dominant kernel (the fused step kernel, or
 * the step batches of the large-d path); Parament_lastKernelMs waits for the
 * stop event and returns that duration in milliseconds (-1 when disabled).
 * Parament_lastLaunchCount returns the number of kernels the last call launched. */
PARAMENT_API Parament_ErrorCode Parament_setKernelTiming(Parament_Context_f32 *handle, int enable);
PARAMENT_API Parament_ErrorCode Parament_setKernelTiming_fp64(Parament_Context_f64 *handle, int enable);
PARAMENT_API float Parament_lastKernelMs(Parament_Context_f32 *handle);
PARAMENT_API float Parament_lastKernelMs_fp64(Parament_Context_f64 *handle);
PARAMENT_API int Parament_lastLaunchCount(Parament_Context_f32 *handle);
PARAMENT_API int Parament_lastLaunchCount_fp64(Parament_Context_f64 *handle);

#ifdef __cplusplus
}
#endif

#endif /* PARAMENT_GB300_H_ */
