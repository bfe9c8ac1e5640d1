// Context state behind the opaque Parament_Context_f32/_f64 handles.
//
// Mirrors what src/cuda/parament_context.hpp:26-78 keeps (dimension, norm
// bound, order control, quadrature settings, last error) with a new layout:
// one expansion stack [H0, H_k, commutators] instead of separate H0/H1
// buffers, grow-only work buffers, and a private non-blocking stream.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "parament.h"

namespace pgb {

bool fault_inject_alloc();

struct DevBuf {
    void *ptr = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes);
    void release();
};

struct Ctx {
    bool fp64 = false;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    Parament_ErrorCode last_error = PARAMENT_STATUS_SUCCESS;

    // Hamiltonian (src/cuda/parament_context.hpp:37-56)
    bool has_h = false;
    unsigned dim = 0, K = 0, Ke = 0;
    bool magnus = true;                          // defaults as src/cuda/parament.cpp:72-75
    int quad = PARAMENT_QUADRATURE_SIMPSON;
    double hnorm = 0.0;
    DevBuf stack;                                // (1+Ke) d x d, context precision

    // Chebyshev order control (src/cuda/parament_context.hpp:72-73)
    unsigned mmax = 11;
    bool manual = false;
    int last_M = 0;

    // Precision form (complex64 contexts)
    int precision = PARAMENT_PRECISION_PLAIN;
    DevBuf split_stack;                          // split form's stack (commutators from FP64)
    bool split_ready = false;
    bool split_herm = false;                     // split stack exactly (anti-)Hermitian per slot

    // Instrumentation: CUDA events around the dominant kernel of the last call
    // and the number of kernels it launched.
    bool timing = false;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    int launches = 0;

    // Work buffers (grow-only, like src/cuda/parament.cpp:418-474)
    DevBuf carr, out, chunks, work, X, B1, B2, aux, grad, wts, xplanes;

    // Bounded-wait faults of this context's tensor-core kernels.  The kernels
    // add to a device counter (d_fault, zero at creation, never reset); after
    // each call that may run such a kernel the counter is copied into pinned
    // host memory (h_fault) on the call's stream and ev_fault is recorded
    // there.  A count above faults_seen is reported as
    // PARAMENT_STATUS_KERNEL_TIMEOUT by the call itself (host-buffer entry
    // points), by Parament_synchronize, or by the next device-buffer call on
    // the context.
    int *d_fault = nullptr;
    int *h_fault = nullptr;
    int faults_seen = 0;
    cudaEvent_t ev_fault = nullptr;  // h_fault refreshed
    bool fault_recorded = false;
    cudaEvent_t ev_done = nullptr;   // end of the last call's work
    bool done_recorded = false;

    size_t esize() const { return fp64 ? 16 : 8; }
    size_t device_bytes() const {
        return stack.cap + split_stack.cap + carr.cap + out.cap + chunks.cap + work.cap + X.cap + B1.cap + B2.cap +
               aux.cap + grad.cap + wts.cap + xplanes.cap;
    }
    void release_all() {
        stack.release();
        split_stack.release();
        carr.release();
        out.release();
        chunks.release();
        work.release();
        X.release();
        B1.release();
        B2.release();
        aux.release();
        grad.release();
        wts.release();
        xplanes.release();
    }
};

// Marks the end of a call's work on `stream`; with tensor_kernels set, the
// fault counter is copied to the host there.  new_faults() reports whether a
// kernel gave up since the last report (wait: block until the last call's
// work is done; otherwise only look if it already is).
void note_call_end(Ctx *c, cudaStream_t stream, bool tensor_kernels);
bool new_faults(Ctx *c, bool wait);

double onenorm_host(const void *m, unsigned d, bool fp64);
int select_cycles(bool fp64, double hnorm, double dt);
void bessel_coeffs(int M, double x, double *J);
long long num_steps(int quad, bool magnus, unsigned pts);

// Split-precision form (complex64 contexts): order choice and propagation;
// run_split_large serves d > 64 (split_large.cu).
struct SplitArgs;
int split_order(double hnorm, double h, long long P);
Parament_ErrorCode run_split(Ctx *c, const void *d_carr, unsigned pts, unsigned amps, double h, int M, long long P,
                             void *d_out, cudaStream_t stream);
Parament_ErrorCode run_split_large(Ctx *c, const SplitArgs &a, double h, void *d_out, cudaStream_t stream);

// Adjoint: d/du_k[i] Re Tr(W^H U) for real samples, d <= adj_max_dim.
int adj_max_dim(bool fp64);
Parament_ErrorCode run_vjp(Ctx *c, const void *d_carr, double dt, unsigned pts, unsigned amps, const void *d_W,
                           void *d_grad, cudaStream_t stream);

}  // namespace pgb
