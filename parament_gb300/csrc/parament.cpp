// Host side of libparament.so: the reference's C-ABI (context life cycle,
// Hamiltonian upload, equiprop, cycle control, error strings) re-built on the
// GB300 kernels in this directory.  No cuBLAS: every product runs in a kernel
// written here.
//
// Reference anchors (paths inside the parament project): life cycle
// src/cuda/parament.cpp:51-205, setHamiltonian :210-368, coefficients :373-409,
// transfer :415-481, equiprop :791-851, cycles :723-786, errors :854-882.
#include <cuComplex.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#define PARAMENT_NO_CUDA_TYPES
#include "parament.h"
#include "ctx.h"
#include "kernels.h"

using namespace pgb;

namespace pgb {

cudaError_t DevBuf::ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    if (fault_inject_alloc()) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(&ptr, bytes);
    if (e != cudaSuccess) {
        ptr = nullptr;
        cudaGetLastError();
        return e;
    }
    cap = bytes;
    return cudaSuccess;
}

void DevBuf::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
}

// Host-side fault injection: PARAMENT_FAIL_ALLOC_AFTER=n makes the (n+1)-th
// device allocation of this process (and only that one) report failure, so
// the allocation-failure paths can be tested without exhausting the GPU.
bool fault_inject_alloc() {
    static long long budget = [] {
        const char *v = getenv("PARAMENT_FAIL_ALLOC_AFTER");
        return v ? atoll(v) : -1LL;
    }();
    if (budget < 0) return false;
    if (budget == 0) {
        budget = -1;  // that one allocation fails; later ones proceed
        return true;
    }
    --budget;
    return false;
}

double onenorm_host(const void *m, unsigned d, bool fp64) {
    double best = 0.0;
    for (unsigned i = 0; i < d; ++i) {
        double sum = 0.0;
        for (unsigned j = 0; j < d; ++j) {
            size_t e = (size_t)i * d + j;
            if (fp64) {
                const double *p = static_cast<const double *>(m) + 2 * e;
                sum += hypot(p[0], p[1]);
            } else {
                const float *p = static_cast<const float *>(m) + 2 * e;
                sum += (double)hypotf(p[0], p[1]);
            }
        }
        best = std::max(best, sum);
    }
    return best;
}

// Order tables: thresholds on Hnorm*dt (src/cuda/parament.cpp:723-766).
static const double kFp32Limits[14] = {0.032516793, 0.219062571, 0.619625593, 1.218059203, 1.979888284,
                                       2.873301187, 3.872963682, 4.959398466, 6.117657121, 7.336154907,
                                       8.605792444, 9.919320831, 11.27088616, 12.65570085};
static const double kFp64Limits[20] = {0.000213616, 0.00768149, 0.0501474, 0.162592, 0.368382, 0.676861, 1.08784,
                                       1.59605,     2.19402,    2.87366,   3.62716,  4.44725,  5.3274,   6.26179,
                                       7.2453,      8.27338,    9.34206,   10.4478,  11.5875,  12.7584};

int select_cycles(bool fp64, double hnorm, double dt) {
    const double *lim = fp64 ? kFp64Limits : kFp32Limits;
    const int n = fp64 ? 20 : 14;
    const double v = hnorm * dt;
    for (int i = 0; i < n; ++i)
        if (v <= lim[i]) return 3 + 2 * i;
    return -1;
}

void bessel_coeffs(int M, double x, double *J) {
    // (-i)^k J_k(x) (src/cuda/mathhelper.cpp:35-80), glibc jn on the host.
    static const double pr[4] = {1, 0, -1, 0}, pi[4] = {0, -1, 0, 1};
    for (int k = 0; k <= M; ++k) {
        double v = jn(k, x);
        J[2 * k] = pr[k % 4] * v;
        J[2 * k + 1] = pi[k % 4] * v;
    }
}

long long num_steps(int quad, bool magnus, unsigned pts) {
    if (magnus || quad == PARAMENT_QUADRATURE_SIMPSON) return pts >= 1 ? (long long)((pts - 1) / 2) : 0;
    if (quad == PARAMENT_QUADRATURE_MIDPOINT) return pts >= 1 ? (long long)pts - 1 : 0;
    return pts;
}

void note_call_end(Ctx *c, cudaStream_t stream, bool tensor_kernels) {
    if (tensor_kernels &&
        cudaMemcpyAsync(c->h_fault, c->d_fault, sizeof(int), cudaMemcpyDeviceToHost, stream) == cudaSuccess &&
        cudaEventRecord(c->ev_fault, stream) == cudaSuccess)
        c->fault_recorded = true;
    if (cudaEventRecord(c->ev_done, stream) == cudaSuccess) c->done_recorded = true;
    cudaGetLastError();
}

bool new_faults(Ctx *c, bool wait) {
    if (!c->fault_recorded) return false;
    cudaError_t e = wait ? cudaEventSynchronize(c->ev_fault) : cudaEventQuery(c->ev_fault);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const int v = *static_cast<volatile int *>(c->h_fault);
    if (v <= c->faults_seen) return false;
    c->faults_seen = v;
    return true;
}

}  // namespace pgb

// ------------------------------------------------------------------ life cycle

static Parament_ErrorCode ctx_create(Ctx **out, bool fp64) {
    Ctx *c = new (std::nothrow) Ctx();
    *out = c;
    if (!c) return PARAMENT_STATUS_HOST_ALLOC_FAILED;
    c->fp64 = fp64;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1 || cudaGetDevice(&c->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        *out = nullptr;
        return PARAMENT_STATUS_CUBLAS_INIT_FAILED;
    }
    // The fault counter and its host mirror (set-up allocations, not counted by
    // the allocation-failure injection of the work buffers).
    if (cudaMalloc(&c->d_fault, sizeof(int)) != cudaSuccess ||
        cudaHostAlloc(&c->h_fault, sizeof(int), cudaHostAllocDefault) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fault, cudaEventDisableTiming) != cudaSuccess ||
        cudaMemsetAsync(c->d_fault, 0, sizeof(int), c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
        cudaGetLastError();
        if (c->d_fault) cudaFree(c->d_fault);
        if (c->h_fault) cudaFreeHost(c->h_fault);
        if (c->ev_done) cudaEventDestroy(c->ev_done);
        if (c->ev_fault) cudaEventDestroy(c->ev_fault);
        cudaStreamDestroy(c->stream);
        delete c;
        *out = nullptr;
        return PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
    }
    *c->h_fault = 0;
    c->last_error = PARAMENT_STATUS_SUCCESS;
    return PARAMENT_STATUS_SUCCESS;
}

static Parament_ErrorCode ctx_destroy(Ctx *c) {
    if (!c) return PARAMENT_STATUS_SUCCESS;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    if (c->done_recorded) cudaEventSynchronize(c->ev_done);
    if (c->fault_recorded) cudaEventSynchronize(c->ev_fault);
    c->release_all();
    if (c->ev_start) cudaEventDestroy(c->ev_start);
    if (c->ev_stop) cudaEventDestroy(c->ev_stop);
    cudaEventDestroy(c->ev_done);
    cudaEventDestroy(c->ev_fault);
    cudaFree(c->d_fault);
    cudaFreeHost(c->h_fault);
    cudaStreamDestroy(c->stream);
    delete c;
    return PARAMENT_STATUS_SUCCESS;
}

// ------------------------------------------------------------ setHamiltonian

static Parament_ErrorCode set_hamiltonian(Ctx *c, const void *H0, const void *H1, unsigned dim, unsigned amps,
                                          bool use_magnus, int quad) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    c->has_h = false;
    c->stack.release();
    c->split_stack.release();
    if (use_magnus) {
        c->magnus = true;
        if (quad != PARAMENT_QUADRATURE_SIMPSON) return c->last_error = PARAMENT_STATUS_INVALID_QUADRATURE_SELECTION;
        c->quad = PARAMENT_QUADRATURE_SIMPSON;
    } else {
        if (quad != PARAMENT_QUADRATURE_NONE && quad != PARAMENT_QUADRATURE_MIDPOINT &&
            quad != PARAMENT_QUADRATURE_SIMPSON)
            return c->last_error = PARAMENT_STATUS_INVALID_VALUE;
        c->magnus = false;
        c->quad = quad;
    }
    if (dim == 0 || !H0 || (amps > 0 && !H1)) return c->last_error = PARAMENT_STATUS_INVALID_VALUE;
    const size_t es = c->esize(), dd = (size_t)dim * dim;
    const unsigned Ke = use_magnus ? 2 * amps + amps * (amps - 1) / 2 : amps;
    if (c->stack.ensure(es * dd * (1 + Ke)) != cudaSuccess) return c->last_error = PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
    char *st = static_cast<char *>(c->stack.ptr);
    cudaError_t e = cudaMemcpyAsync(st, H0, es * dd, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && amps)
        e = cudaMemcpyAsync(st + es * dd, H1, es * dd * amps, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) {
        c->stack.release();
        return c->last_error = PARAMENT_FAIL;
    }
    // Norm bound on the host input arrays (src/cuda/parament.cpp:279-287).
    double hn = onenorm_host(H0, dim, c->fp64);
    for (unsigned k = 0; k < amps; ++k)
        hn += onenorm_host(static_cast<const char *>(H1) + es * dd * k, dim, c->fp64);
    // Magnus commutators (src/cuda/parament.cpp:289-359; pair slots triangular).
    auto commutator = [&](size_t a, size_t b, size_t dst) -> cudaError_t {
        GemmLaunch g{};
        g.fp64 = c->fp64;
        g.d = (int)dim;
        g.batch = 1;
        g.A = st + es * dd * a;
        g.B = st + es * dd * b;
        g.Cout = st + es * dd * dst;
        g.alpha_re = 1.0;
        g.stream = c->stream;
        g.num_sms = c->num_sms;
        g.fault = c->d_fault;
        cudaError_t r = launch_gemm(g);
        if (r != cudaSuccess) return r;
        g.A = st + es * dd * b;
        g.B = st + es * dd * a;
        g.Cin = st + es * dd * dst;
        g.alpha_re = -1.0;
        g.beta = 1.0;
        return launch_gemm(g);
    };
    if (use_magnus) {
        for (unsigned k = 0; k < amps && e == cudaSuccess; ++k) e = commutator(0, 1 + k, 1 + amps + k);
        for (unsigned i = 1; i < amps && e == cudaSuccess; ++i)
            for (unsigned j = 0; j < i && e == cudaSuccess; ++j)
                e = commutator(1 + j, 1 + i, 1 + 2 * amps + i * (i - 1) / 2 + j);
    }
    if (use_magnus) note_call_end(c, c->stream, true);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        c->stack.release();
        return c->last_error = PARAMENT_STATUS_CUBLAS_FAILED;
    }
    if (new_faults(c, true)) {
        c->stack.release();
        return c->last_error = PARAMENT_STATUS_KERNEL_TIMEOUT;
    }
    c->dim = dim;
    c->K = amps;
    c->Ke = Ke;
    c->hnorm = hn;
    c->has_h = true;
    c->split_ready = false;
    return c->last_error = PARAMENT_STATUS_SUCCESS;
}

// ------------------------------------------------------------------ equiprop

// Plain path: propagate the P steps and leave the product in d_out (device).
static Parament_ErrorCode run_plain(Ctx *c, const void *d_carr, unsigned pts, unsigned amps, double h, int M,
                                    long long P, void *d_out, cudaStream_t stream) {
    const int d = (int)c->dim;
    const size_t es = c->esize(), dd = (size_t)d * d;
    std::vector<double> J(2 * (M + 1));
    bessel_coeffs(M, h * c->hnorm, J.data());
    WeightSpecHost w{pts, (int)c->K, (int)amps, c->quad, c->magnus ? 1 : 0,
                     c->fp64 ? h / 12.0 : (double)(float)h / 12.0};
    const double s = 2.0 / c->hnorm;
    cudaError_t e;
    // complex64 at d = 64: the same scheme with the products on the tensor
    // cores (small_tc.cu); X planes per batch of steps, one complex64 chunk
    // product per CTA, combined by the double-float tree.  Where the planes
    // (up to 2.3 GB) cannot be allocated, the FP32 SIMT kernel below runs,
    // which needs only the chunk buffers.
    const int nmax = small_tc_max_chunks(P, c->num_sms);
    if (small_tc_applies(c->fp64, d, (int)c->Ke, M) && c->chunks.ensure(es * dd * nmax) == cudaSuccess &&
        c->work.ensure(16 * dd * nmax) == cudaSuccess && c->X.ensure(16 * dd * ((nmax + 1) / 2)) == cudaSuccess &&
        c->xplanes.ensure(small_tc_xplane_bytes(P)) == cudaSuccess) {
        StepLaunch l{};
        l.fp64 = false;
        l.d = d;
        l.Ke = (int)c->Ke;
        l.w = w;
        l.M = M;
        l.J = J.data();
        l.s = s;
        l.stack = c->stack.ptr;
        l.carr = d_carr;
        l.chunks = c->chunks.ptr;
        l.P = P;
        l.stream = stream;
        int nch = 0;
        e = launch_small_tc(l, c->num_sms, static_cast<float *>(c->xplanes.ptr), c->d_fault, &nch,
                            c->timing ? c->ev_start : nullptr, c->timing ? c->ev_stop : nullptr);
        int levels = 0;
        if (e == cudaSuccess)
            e = tree_df_c64(d, static_cast<const float2 *>(c->chunks.ptr), nch, c->work.ptr, c->X.ptr,
                            static_cast<float2 *>(d_out), stream, &levels);
        const long long batches = (P + 65535) / 65536;
        c->launches = 2 * (int)batches + levels;
    } else if (d <= kSmallMaxDim) {
        const int nch = small_chunk_count(c->fp64, d, (int)c->Ke, P, c->num_sms);
        // complex64: the chunk products are combined by the double-float tree
        // (complex128-sized buffers); complex128: by the FP64 tree.
        if (c->chunks.ensure(es * dd * nch) != cudaSuccess || c->work.ensure(16 * dd * nch) != cudaSuccess ||
            (!c->fp64 && c->X.ensure(16 * dd * ((nch + 1) / 2)) != cudaSuccess))
            return PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
        StepLaunch l{};
        l.fp64 = c->fp64;
        l.d = d;
        l.Ke = (int)c->Ke;
        l.w = w;
        l.M = M;
        l.J = J.data();
        l.s = s;
        l.stack = c->stack.ptr;
        l.carr = d_carr;
        l.chunks = c->chunks.ptr;
        l.P = P;
        l.nchunks = nch;
        l.stream = stream;
        if (c->timing) cudaEventRecord(c->ev_start, stream);
        e = launch_small_steps(l);
        if (c->timing) cudaEventRecord(c->ev_stop, stream);
        int levels = 0;
        if (e == cudaSuccess && c->fp64)
            e = tree_product(true, d, c->chunks.ptr, nch, c->work.ptr, d_out, stream, c->num_sms, &levels,
                             c->d_fault);
        else if (e == cudaSuccess)
            e = tree_df_c64(d, static_cast<const float2 *>(c->chunks.ptr), nch, c->work.ptr, c->X.ptr,
                            static_cast<float2 *>(d_out), stream, &levels);
        c->launches = 1 + levels;
    } else {
        // Batches of G steps held as X, b_(k+1), b_(k+2): 3 G d^2 elements, capped near 4 GiB.
        const size_t per = 3 * es * dd;
        long long G = std::max<long long>(1, std::min<long long>(P, (long long)((4ULL << 30) / per)));
        G = std::min<long long>(G, 4096);
        const long long nb = (P + G - 1) / G;
        if (c->X.ensure(es * dd * G) != cudaSuccess || c->B1.ensure(es * dd * G) != cudaSuccess ||
            c->B2.ensure(es * dd * G) != cudaSuccess || c->chunks.ensure(es * dd * nb) != cudaSuccess ||
            c->work.ensure(es * dd * nb) != cudaSuccess) {
            if (!mid_applies(c->fp64, d, (int)c->Ke)) return PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
            // 64 < d <= 128 (96 in complex128) without room for the batches:
            // clusters of four CTAs with the step resident in their shared
            // memory, one d x d product per cluster (the batched path is about
            // twice as fast where its buffers fit); the chunk products are
            // combined by the FP64 tree.
            const int nch = mid_chunk_count(c->num_sms, P);
            if (c->chunks.ensure(es * dd * nch) != cudaSuccess || c->work.ensure(16 * dd * nch) != cudaSuccess ||
                c->X.ensure(16 * dd * nch) != cudaSuccess || c->aux.ensure(16 * dd) != cudaSuccess)
                return PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
            StepLaunch l{};
            l.fp64 = c->fp64;
            l.d = d;
            l.Ke = (int)c->Ke;
            l.w = w;
            l.M = M;
            l.J = J.data();
            l.s = s;
            l.stack = c->stack.ptr;
            l.carr = d_carr;
            l.chunks = c->chunks.ptr;
            l.P = P;
            l.nchunks = nch;
            l.stream = stream;
            if (c->timing) cudaEventRecord(c->ev_start, stream);
            e = launch_mid_steps(l);
            if (c->timing) cudaEventRecord(c->ev_stop, stream);
            int levels = 0;
            if (c->fp64) {
                if (e == cudaSuccess)
                    e = tree_product(true, d, c->chunks.ptr, nch, c->work.ptr, d_out, stream, c->num_sms, &levels,
                                     c->d_fault);
                c->launches = 1 + levels;
            } else {
                if (e == cudaSuccess) e = convert_complex(true, c->chunks.ptr, c->work.ptr, dd * nch, stream);
                if (e == cudaSuccess)
                    e = tree_product(true, d, c->work.ptr, nch, c->X.ptr, c->aux.ptr, stream, c->num_sms, &levels,
                                     c->d_fault);
                if (e == cudaSuccess) e = convert_complex(false, c->aux.ptr, d_out, dd, stream);
                c->launches = 3 + levels;
            }
            if (e != cudaSuccess) {
                cudaGetLastError();
                return PARAMENT_STATUS_CUBLAS_FAILED;
            }
            return PARAMENT_STATUS_SUCCESS;
        }
        LargeLaunch l{};
        l.fp64 = c->fp64;
        l.d = d;
        l.Ke = (int)c->Ke;
        l.w = w;
        l.M = M;
        l.J = J.data();
        l.s = s;
        l.stack = c->stack.ptr;
        l.carr = d_carr;
        l.s0 = 0;
        l.s1 = P;
        l.batch = (int)G;
        l.X = c->X.ptr;
        l.B1 = c->B1.ptr;
        l.B2 = c->B2.ptr;
        l.out = c->chunks.ptr;
        l.stream = stream;
        l.num_sms = c->num_sms;
        l.fault = c->d_fault;
        if (c->timing) cudaEventRecord(c->ev_start, stream);
        int launched = 0;
        e = launch_large_range(l, &launched);
        if (c->timing) cudaEventRecord(c->ev_stop, stream);
        int levels = 0;
        if (e == cudaSuccess)
            e = tree_product(c->fp64, d, c->chunks.ptr, nb, c->work.ptr, d_out, stream, c->num_sms, &levels,
                             c->d_fault);
        c->launches = launched + levels;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return PARAMENT_STATUS_CUBLAS_FAILED;
    }
    return PARAMENT_STATUS_SUCCESS;
}

// Whether an equiprop of this context may launch a kernel with bounded waits
// (the tensor-core GEMM of complex64 contexts with d > 64, the tensor-core
// split kernel, the tensor-core plain kernel at d = 64).
static bool uses_tensor_kernels(const Ctx *c) {
    return !c->fp64 && (c->dim >= (unsigned)kSmallMaxDim || c->precision == PARAMENT_PRECISION_SPLIT);
}

// Checks, order selection and dispatch shared by the host and device entry
// points.  d_carr: device samples; d_out: device result (d x d).
static Parament_ErrorCode equiprop_device(Ctx *c, const void *d_carr, double dt, unsigned pts, unsigned amps,
                                          void *d_out, cudaStream_t stream) {
    if (!c->has_h) return PARAMENT_STATUS_NO_HAMILTONIAN;
    if (amps > c->K) return PARAMENT_STATUS_INVALID_VALUE;
    const double h = (c->magnus || c->quad == PARAMENT_QUADRATURE_SIMPSON) ? 2.0 * dt : dt;
    const long long P = num_steps(c->quad, c->magnus, pts);
    if (P <= 0 || !(dt >= 0.0) || !isfinite(dt)) return PARAMENT_STATUS_INVALID_VALUE;
    if (amps > 0 && !d_carr) return PARAMENT_STATUS_INVALID_VALUE;
    const bool split = (!c->fp64 && c->precision == PARAMENT_PRECISION_SPLIT);
    int M;
    if (c->manual) {
        M = (int)c->mmax;
    } else if (split) {
        M = split_order(c->hnorm, h, P);
        if (M < 3) return PARAMENT_STATUS_SELECT_SMALLER_DT;
    } else {
        M = select_cycles(c->fp64, c->hnorm, h);
        if (M < 3) return PARAMENT_STATUS_SELECT_SMALLER_DT;
    }
    if (c->hnorm == 0.0 || dt == 0.0) {
        // exp(0) = I for every step: the product is the identity.
        cudaError_t e = fill_identity(c->fp64, d_out, (int)c->dim, 1, 1.0, 0.0, stream);
        c->last_M = M;
        c->launches = 1;
        return e == cudaSuccess ? PARAMENT_STATUS_SUCCESS : PARAMENT_STATUS_CUBLAS_FAILED;
    }
    Parament_ErrorCode r = split ? run_split(c, d_carr, pts, amps, h, M, P, d_out, stream)
                                 : run_plain(c, d_carr, pts, amps, h, M, P, d_out, stream);
    if (r == PARAMENT_STATUS_SUCCESS) c->last_M = M;
    return r;
}

static Parament_ErrorCode equiprop_host(Ctx *c, const void *carr, double dt, unsigned pts, unsigned amps,
                                        void *out) {
    cudaSetDevice(c->device);
    if (!c->has_h) return c->last_error = PARAMENT_STATUS_NO_HAMILTONIAN;
    if (!out || (amps > 0 && !carr)) return c->last_error = PARAMENT_STATUS_INVALID_VALUE;
    const size_t es = c->esize(), dd = (size_t)c->dim * c->dim;
    const size_t cbytes = es * (size_t)amps * pts;
    if (c->carr.ensure(std::max<size_t>(cbytes, 16)) != cudaSuccess || c->out.ensure(es * dd) != cudaSuccess)
        return c->last_error = PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
    // Transfer of the samples (src/cuda/parament.cpp:477).
    if (cbytes && cudaMemcpyAsync(c->carr.ptr, carr, cbytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) {
        cudaGetLastError();
        return c->last_error = PARAMENT_FAIL;
    }
    Parament_ErrorCode r = equiprop_device(c, c->carr.ptr, dt, pts, amps, c->out.ptr, c->stream);
    if (r != PARAMENT_STATUS_SUCCESS) {
        cudaStreamSynchronize(c->stream);
        return c->last_error = r;
    }
    note_call_end(c, c->stream, uses_tensor_kernels(c));
    // Result back to the host (src/cuda/parament.cpp:846).
    cudaError_t e = cudaMemcpyAsync(out, c->out.ptr, es * dd, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return c->last_error = PARAMENT_STATUS_CUBLAS_FAILED;
    }
    if (new_faults(c, true)) return c->last_error = PARAMENT_STATUS_KERNEL_TIMEOUT;
    return c->last_error = PARAMENT_STATUS_SUCCESS;
}

static Ctx *as_ctx(void *p) { return static_cast<Ctx *>(p); }

// Device-buffer entry points: the work is queued and not waited for.  A
// bounded wait that gave up in an earlier call of the context is reported
// here, once it is known, before anything new is queued.
static Parament_ErrorCode equiprop_device_call(Ctx *c, const void *d_carr, double dt, unsigned pts, unsigned amps,
                                               void *d_out, void *stream_p) {
    cudaSetDevice(c->device);
    if (new_faults(c, false)) return c->last_error = PARAMENT_STATUS_KERNEL_TIMEOUT;
    cudaStream_t stream = stream_p ? static_cast<cudaStream_t>(stream_p) : c->stream;
    Parament_ErrorCode r = equiprop_device(c, d_carr, dt, pts, amps, d_out, stream);
    if (r == PARAMENT_STATUS_SUCCESS) note_call_end(c, stream, uses_tensor_kernels(c));
    return c->last_error = r;
}

// ------------------------------------------------------------ exported C-ABI

extern "C" {

Parament_ErrorCode Parament_create(Parament_Context_f32 **handle_p) {
    if (!handle_p) return PARAMENT_STATUS_INVALID_VALUE;
    Ctx *c = nullptr;
    Parament_ErrorCode r = ctx_create(&c, false);
    *handle_p = reinterpret_cast<Parament_Context_f32 *>(c);
    return r;
}

Parament_ErrorCode Parament_create_fp64(Parament_Context_f64 **handle_p) {
    if (!handle_p) return PARAMENT_STATUS_INVALID_VALUE;
    Ctx *c = nullptr;
    Parament_ErrorCode r = ctx_create(&c, true);
    *handle_p = reinterpret_cast<Parament_Context_f64 *>(c);
    return r;
}

Parament_ErrorCode Parament_destroy(Parament_Context_f32 *handle) { return ctx_destroy(as_ctx(handle)); }
Parament_ErrorCode Parament_destroy_fp64(Parament_Context_f64 *handle) { return ctx_destroy(as_ctx(handle)); }

Parament_ErrorCode Parament_setHamiltonian(Parament_Context_f32 *handle, cuComplex *H0, cuComplex *H1,
                                           unsigned int dim, unsigned int amps, bool use_magnus,
                                           Parament_QuadratureSpec quadrature_mode) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    return set_hamiltonian(as_ctx(handle), H0, H1, dim, amps, use_magnus, (int)quadrature_mode);
}

Parament_ErrorCode Parament_setHamiltonian_fp64(Parament_Context_f64 *handle, cuDoubleComplex *H0,
                                                cuDoubleComplex *H1, unsigned int dim, unsigned int amps,
                                                bool use_magnus, Parament_QuadratureSpec quadrature_mode) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    return set_hamiltonian(as_ctx(handle), H0, H1, dim, amps, use_magnus, (int)quadrature_mode);
}

Parament_ErrorCode Parament_equiprop(Parament_Context_f32 *handle, cuComplex *carr, double dt, unsigned int pts,
                                     unsigned int amps, cuComplex *out) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    return equiprop_host(as_ctx(handle), carr, dt, pts, amps, out);
}

Parament_ErrorCode Parament_equiprop_fp64(Parament_Context_f64 *handle, cuDoubleComplex *carr, double dt,
                                          unsigned int pts, unsigned int amps, cuDoubleComplex *out) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    return equiprop_host(as_ctx(handle), carr, dt, pts, amps, out);
}

int Parament_selectIterationCycles_fp32(double H_norm, double dt) { return select_cycles(false, H_norm, dt); }
int Parament_selectIterationCycles_fp64(double H_norm, double dt) { return select_cycles(true, H_norm, dt); }

static Parament_ErrorCode set_cycles(Ctx *c, unsigned cycles) {
    // The reference accepts any value (src/cuda/parament.cpp:771-776); an even
    // order would read J[-1] there, so only odd orders 1..63 are taken here.
    if (cycles < 1 || cycles > (unsigned)kMaxOrder || cycles % 2 == 0) return PARAMENT_STATUS_INVALID_VALUE;
    c->mmax = cycles;
    c->manual = true;
    return PARAMENT_STATUS_SUCCESS;
}

Parament_ErrorCode Parament_setIterationCyclesManually(Parament_Context_f32 *handle, unsigned int cycles) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    return set_cycles(as_ctx(handle), cycles);
}
Parament_ErrorCode Parament_setIterationCyclesManually_fp64(Parament_Context_f64 *handle, unsigned int cycles) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    return set_cycles(as_ctx(handle), cycles);
}

Parament_ErrorCode Parament_automaticIterationCycles(Parament_Context_f32 *handle) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    as_ctx(handle)->mmax = 11;
    as_ctx(handle)->manual = false;
    return PARAMENT_STATUS_SUCCESS;
}
Parament_ErrorCode Parament_automaticIterationCycles_fp64(Parament_Context_f64 *handle) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    as_ctx(handle)->mmax = 11;
    as_ctx(handle)->manual = false;
    return PARAMENT_STATUS_SUCCESS;
}

Parament_ErrorCode Parament_peekAtLastError(Parament_Context_f32 *handle) {
    return handle ? as_ctx(handle)->last_error : PARAMENT_STATUS_INVALID_VALUE;
}
Parament_ErrorCode Parament_peekAtLastError_fp64(Parament_Context_f64 *handle) {
    return handle ? as_ctx(handle)->last_error : PARAMENT_STATUS_INVALID_VALUE;
}

const char *Parament_errorMessage(Parament_ErrorCode errorCode) {
    // Strings as src/cuda/parament.cpp:859-882 (callers match on them).
    switch (errorCode) {
        case PARAMENT_STATUS_SUCCESS: return "Success";
        case PARAMENT_STATUS_HOST_ALLOC_FAILED: return "Memory allocation on the host failed.";
        case PARAMENT_STATUS_DEVICE_ALLOC_FAILED: return "Memory allocation on the device failed.";
        case PARAMENT_STATUS_CUBLAS_INIT_FAILED: return "Failed to initialize the cuBLAS library.";
        case PARAMENT_STATUS_INVALID_VALUE: return "Invalid value.";
        case PARAMENT_STATUS_CUBLAS_FAILED: return "Failed to execute cuBLAS function.";
        case PARAMENT_STATUS_SELECT_SMALLER_DT: return "Timestep too large";
        case PARAMENT_STATUS_INVALID_QUADRATURE_SELECTION: return "Invalid quadrature selection.";
        case PARAMENT_STATUS_NO_HAMILTONIAN: return "No hamiltonian set";
        case PARAMENT_STATUS_KERNEL_TIMEOUT: return "A bounded device-side wait timed out.";
        case PARAMENT_STATUS_SCRATCH_EXCEEDED:
            return "Problem too large for the fixed scratch of the no-allocation entry point (complex128, dim <= 64).";
        default: return "Unknown error code";
    }
}

double OneNorm(cuComplex *arr, unsigned int dim) { return arr ? onenorm_host(arr, dim, false) : 0.0; }
double OneNorm_fp64(cuDoubleComplex *arr, unsigned int dim) { return arr ? onenorm_host(arr, dim, true) : 0.0; }

void device_info(void) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        printf("Failed to query the number of CUDA devices. Error code: %d\n", (int)e);
        return;
    }
    printf("PARAMENT_INFO:\n");
    printf("Total number of CUDA devices: %d\n", n);
    printf("-----------------------------------\n");
    for (int i = 0; i < n; ++i) {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, i) != cudaSuccess) {
            printf("Failed to query device properties.");
            return;
        }
        int clk = 0, bus = 0;
        cudaDeviceGetAttribute(&clk, cudaDevAttrMemoryClockRate, i);
        cudaDeviceGetAttribute(&bus, cudaDevAttrGlobalMemoryBusWidth, i);
        printf("Device Number: %d\n", i);
        printf("  Device name: %s\n", prop.name);
        printf("  Memory Clock Rate (KHz): %d\n", clk);
        printf("  Memory Bus Width (bits): %d\n", bus);
        printf("  Peak Memory Bandwidth (GB/s): %f\n", 2.0 * clk * (bus / 8) / 1.0e6);
        printf("  Total global memory: %zu MB\n\n", (size_t)(prop.totalGlobalMem / 1024 / 1024));
    }
    fflush(stdout);
}

Parament_ErrorCode Parament_setPrecisionMode(Parament_Context_f32 *handle, int mode) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    if (mode != PARAMENT_PRECISION_PLAIN && mode != PARAMENT_PRECISION_SPLIT) return PARAMENT_STATUS_INVALID_VALUE;
    as_ctx(handle)->precision = mode;
    return PARAMENT_STATUS_SUCCESS;
}
int Parament_getPrecisionMode(Parament_Context_f32 *handle) { return handle ? as_ctx(handle)->precision : -1; }

int Parament_lastIterationCycles(Parament_Context_f32 *handle) { return handle ? as_ctx(handle)->last_M : 0; }
int Parament_lastIterationCycles_fp64(Parament_Context_f64 *handle) { return handle ? as_ctx(handle)->last_M : 0; }

double Parament_hamiltonianNorm(Parament_Context_f32 *handle) {
    return (handle && as_ctx(handle)->has_h) ? as_ctx(handle)->hnorm : 0.0;
}
double Parament_hamiltonianNorm_fp64(Parament_Context_f64 *handle) {
    return (handle && as_ctx(handle)->has_h) ? as_ctx(handle)->hnorm : 0.0;
}

Parament_ErrorCode Parament_equipropDevice(Parament_Context_f32 *handle, const void *d_carr, double dt,
                                           unsigned int pts, unsigned int amps, void *d_out, void *stream) {
    if (!handle || !d_out) return PARAMENT_STATUS_INVALID_VALUE;
    return equiprop_device_call(as_ctx(handle), d_carr, dt, pts, amps, d_out, stream);
}

Parament_ErrorCode Parament_equipropDevice_fp64(Parament_Context_f64 *handle, const void *d_carr, double dt,
                                                unsigned int pts, unsigned int amps, void *d_out, void *stream) {
    if (!handle || !d_out) return PARAMENT_STATUS_INVALID_VALUE;
    return equiprop_device_call(as_ctx(handle), d_carr, dt, pts, amps, d_out, stream);
}

static Parament_ErrorCode vjp_host(Ctx *c, const void *carr, double dt, unsigned pts, unsigned amps, const void *W,
                                   void *grad) {
    cudaSetDevice(c->device);
    if (!c->has_h) return c->last_error = PARAMENT_STATUS_NO_HAMILTONIAN;
    if (!W || !grad || (amps > 0 && !carr)) return c->last_error = PARAMENT_STATUS_INVALID_VALUE;
    const size_t es = c->esize(), dd = (size_t)c->dim * c->dim;
    const size_t cbytes = es * (size_t)amps * pts, gbytes = (es / 2) * (size_t)amps * pts;
    if (c->carr.ensure(std::max<size_t>(cbytes, 16)) != cudaSuccess || c->out.ensure(es * dd) != cudaSuccess ||
        c->grad.ensure(std::max<size_t>(gbytes, 16)) != cudaSuccess)
        return c->last_error = PARAMENT_STATUS_DEVICE_ALLOC_FAILED;
    cudaError_t e = cudaSuccess;
    if (cbytes) e = cudaMemcpyAsync(c->carr.ptr, carr, cbytes, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->out.ptr, W, es * dd, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return c->last_error = PARAMENT_FAIL;
    }
    Parament_ErrorCode r = run_vjp(c, c->carr.ptr, dt, pts, amps, c->out.ptr, c->grad.ptr, c->stream);
    if (r != PARAMENT_STATUS_SUCCESS) {
        cudaStreamSynchronize(c->stream);
        return c->last_error = r;
    }
    if (gbytes) e = cudaMemcpyAsync(grad, c->grad.ptr, gbytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return c->last_error = PARAMENT_STATUS_CUBLAS_FAILED;
    }
    return c->last_error = PARAMENT_STATUS_SUCCESS;
}

static Parament_ErrorCode vjp_device_call(Ctx *c, const void *d_carr, double dt, unsigned pts, unsigned amps,
                                          const void *d_W, void *d_grad, void *stream_p) {
    cudaSetDevice(c->device);
    if (new_faults(c, false)) return c->last_error = PARAMENT_STATUS_KERNEL_TIMEOUT;
    cudaStream_t stream = stream_p ? static_cast<cudaStream_t>(stream_p) : c->stream;
    Parament_ErrorCode r = run_vjp(c, d_carr, dt, pts, amps, d_W, d_grad, stream);
    if (r == PARAMENT_STATUS_SUCCESS) note_call_end(c, stream, false);
    return c->last_error = r;
}

Parament_ErrorCode Parament_equipropVJP(Parament_Context_f32 *handle, cuComplex *carr, double dt, unsigned int pts,
                                        unsigned int amps, cuComplex *W, float *grad) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    return vjp_host(as_ctx(handle), carr, dt, pts, amps, W, grad);
}
Parament_ErrorCode Parament_equipropVJP_fp64(Parament_Context_f64 *handle, cuDoubleComplex *carr, double dt,
                                             unsigned int pts, unsigned int amps, cuDoubleComplex *W, double *grad) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    return vjp_host(as_ctx(handle), carr, dt, pts, amps, W, grad);
}
Parament_ErrorCode Parament_equipropVJPDevice(Parament_Context_f32 *handle, const void *d_carr, double dt,
                                              unsigned int pts, unsigned int amps, const void *d_W, void *d_grad,
                                              void *stream) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    return vjp_device_call(as_ctx(handle), d_carr, dt, pts, amps, d_W, d_grad, stream);
}
Parament_ErrorCode Parament_equipropVJPDevice_fp64(Parament_Context_f64 *handle, const void *d_carr, double dt,
                                                   unsigned int pts, unsigned int amps, const void *d_W, void *d_grad,
                                                   void *stream) {
    if (!handle) return PARAMENT_STATUS_INVALID_VALUE;
    return vjp_device_call(as_ctx(handle), d_carr, dt, pts, amps, d_W, d_grad, stream);
}

static Parament_ErrorCode set_timing(Ctx *c, int enable) {
    cudaSetDevice(c->device);
    if (enable && !c->ev_start) {
        if (cudaEventCreate(&c->ev_start) != cudaSuccess || cudaEventCreate(&c->ev_stop) != cudaSuccess) {
            cudaGetLastError();
            return PARAMENT_FAIL;
        }
    }
    c->timing = enable != 0;
    return PARAMENT_STATUS_SUCCESS;
}

static float kernel_ms(Ctx *c) {
    if (!c->timing || !c->ev_stop) return -1.0f;
    float ms = -1.0f;
    if (cudaEventSynchronize(c->ev_stop) != cudaSuccess || cudaEventElapsedTime(&ms, c->ev_start, c->ev_stop) != cudaSuccess) {
        cudaGetLastError();
        return -1.0f;
    }
    return ms;
}

Parament_ErrorCode Parament_setKernelTiming(Parament_Context_f32 *handle, int enable) {
    return handle ? set_timing(as_ctx(handle), enable) : PARAMENT_STATUS_INVALID_VALUE;
}
Parament_ErrorCode Parament_setKernelTiming_fp64(Parament_Context_f64 *handle, int enable) {
    return handle ? set_timing(as_ctx(handle), enable) : PARAMENT_STATUS_INVALID_VALUE;
}
float Parament_lastKernelMs(Parament_Context_f32 *handle) { return handle ? kernel_ms(as_ctx(handle)) : -1.0f; }
float Parament_lastKernelMs_fp64(Parament_Context_f64 *handle) { return handle ? kernel_ms(as_ctx(handle)) : -1.0f; }
static Parament_ErrorCode ctx_synchronize(Ctx *c) {
    cudaSetDevice(c->device);
    cudaError_t e = cudaSuccess;
    if (c->done_recorded) e = cudaEventSynchronize(c->ev_done);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return c->last_error = PARAMENT_FAIL;
    }
    return c->last_error = new_faults(c, true) ? PARAMENT_STATUS_KERNEL_TIMEOUT : PARAMENT_STATUS_SUCCESS;
}

Parament_ErrorCode Parament_synchronize(Parament_Context_f32 *handle) {
    return handle ? ctx_synchronize(as_ctx(handle)) : PARAMENT_STATUS_INVALID_VALUE;
}
Parament_ErrorCode Parament_synchronize_fp64(Parament_Context_f64 *handle) {
    return handle ? ctx_synchronize(as_ctx(handle)) : PARAMENT_STATUS_INVALID_VALUE;
}
unsigned long long Parament_deviceMemoryBytes(Parament_Context_f32 *handle) {
    return handle ? (unsigned long long)as_ctx(handle)->device_bytes() : 0ULL;
}
unsigned long long Parament_deviceMemoryBytes_fp64(Parament_Context_f64 *handle) {
    return handle ? (unsigned long long)as_ctx(handle)->device_bytes() : 0ULL;
}

int Parament_lastLaunchCount(Parament_Context_f32 *handle) { return handle ? as_ctx(handle)->launches : 0; }
int Parament_lastLaunchCount_fp64(Parament_Context_f64 *handle) { return handle ? as_ctx(handle)->launches : 0; }

}  // extern "C"
