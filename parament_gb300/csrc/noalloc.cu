// equiprop without any device allocation: Parament_equipropNoAlloc_fp64.
//
// Who needs this: code that may not call cudaMalloc at the moment it
// propagates -- a real-time control loop that must not stall on the driver's
// allocator, a host application whose GPU memory is handed out by its own pool
// and forbids the CUDA runtime from taking more, or a plug-in running where
// device allocation is disallowed.  The regular entry points grow per-context
// work buffers on demand; this one instead keeps the per-chunk products and the
// tree's ping-pong buffer in one fixed array of device memory that is part of
// the library image (kNoAllocScratchBytes, held on every GPU that loads the
// library until the process exits).  The Hamiltonian must already be on the
// device (Parament_setHamiltonian_fp64 allocates, once, at set-up time); the
// caller passes device pointers for the samples and the result.
//
// Limits and rules:
//  - complex128 contexts with dim <= 64 only (the fused shared-memory kernel);
//    anything larger returns PARAMENT_STATUS_SCRATCH_EXCEEDED.  If a GPU has so
//    many SMs that one chunk per resident CTA would not fit, fewer chunks are
//    used (same result, less parallelism).
//  - The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (once per device and CUDA context, with that device
//    current).  Make that first call before any stream capture.  After a
//    cudaDeviceReset the device gets a new context and the library image is
//    loaded again, possibly at another address: the next call sees the new
//    context and looks the address up again (make it outside capture too).
//  - All calls share the one array and it keeps the previous call's contents.
//    Nothing here reads a scratch element before writing it, so nothing needs
//    clearing -- but two calls whose work overlaps on the GPU (different
//    streams, different contexts, different host threads) race on the array.
//    Serialise them.
#include <cuda.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "ctx.h"
#include "kernels.h"

namespace pgb {

constexpr size_t kNoAllocScratchBytes = 24u << 20;  // 24 MiB
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[kNoAllocMaxDevices];
static CUcontext g_noalloc_ctx[kNoAllocMaxDevices];

// The calling thread's current CUDA context (the driver's cuCtxGetCurrent,
// reached through the runtime's entry-point query so that no link against the
// driver library is needed); null if unavailable.
static CUcontext current_context() {
    using GetCurrent = CUresult (*)(CUcontext *);
    static GetCurrent fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<GetCurrent>(p);
    }();
    CUcontext ctx = nullptr;
    if (!fn || fn(&ctx) != CUDA_SUCCESS) return nullptr;
    return ctx;
}

// Device address of the scratch array on `device` (which must be current).
// Looked up once per device and context: a reset device has a new context.
static cudaError_t noalloc_scratch(int device, void **out) {
    if (device < 0 || device >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    const CUcontext ctx = current_context();
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[device] || !ctx || g_noalloc_ctx[device] != ctx) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            g_noalloc_ptr[device] = nullptr;
            return e != cudaSuccess ? e : cudaErrorInvalidSymbol;
        }
        g_noalloc_ptr[device] = p;
        g_noalloc_ctx[device] = ctx;
    }
    *out = g_noalloc_ptr[device];
    return cudaSuccess;
}

// Usable scratch bytes: the whole array, or less when the environment variable
// PARAMENT_NOALLOC_SCRATCH_BYTES asks for less (read once; a test hook that
// forces the reduced chunk count a GPU with very many SMs would get).
static size_t usable_scratch_bytes() {
    static const size_t n = [] {
        const char *v = getenv("PARAMENT_NOALLOC_SCRATCH_BYTES");
        const long long b = v ? atoll(v) : 0;
        return (b > 0 && (size_t)b < kNoAllocScratchBytes) ? (size_t)b : kNoAllocScratchBytes;
    }();
    return n;
}

}  // namespace pgb

using namespace pgb;

extern "C" Parament_ErrorCode Parament_equipropNoAlloc_fp64(Parament_Context_f64 *handle, const void *d_carr,
                                                            double dt, unsigned int pts, unsigned int amps,
                                                            void *d_out, void *stream_p) {
    if (!handle || !d_out) return PARAMENT_STATUS_INVALID_VALUE;
    Ctx *c = reinterpret_cast<Ctx *>(handle);
    if (!c->fp64) return c->last_error = PARAMENT_STATUS_INVALID_VALUE;
    if (cudaSetDevice(c->device) != cudaSuccess) {
        cudaGetLastError();
        return c->last_error = PARAMENT_FAIL;
    }
    cudaStream_t stream = stream_p ? static_cast<cudaStream_t>(stream_p) : c->stream;
    // Argument checks in the order of the regular device entry point, then the
    // size limit of the scratch array.
    if (!c->has_h) return c->last_error = PARAMENT_STATUS_NO_HAMILTONIAN;
    if (amps > c->K) return c->last_error = PARAMENT_STATUS_INVALID_VALUE;
    const double h = (c->magnus || c->quad == PARAMENT_QUADRATURE_SIMPSON) ? 2.0 * dt : dt;
    const long long P = num_steps(c->quad, c->magnus, pts);
    if (P <= 0 || !(dt >= 0.0) || !isfinite(dt)) return c->last_error = PARAMENT_STATUS_INVALID_VALUE;
    if (amps > 0 && !d_carr) return c->last_error = PARAMENT_STATUS_INVALID_VALUE;
    int M = c->manual ? (int)c->mmax : select_cycles(true, c->hnorm, h);
    if (M < 3 && !c->manual) return c->last_error = PARAMENT_STATUS_SELECT_SMALLER_DT;
    const int d = (int)c->dim;
    if (d > kSmallMaxDim) return c->last_error = PARAMENT_STATUS_SCRATCH_EXCEEDED;
    void *scratch = nullptr;
    if (noalloc_scratch(c->device, &scratch) != cudaSuccess) return c->last_error = PARAMENT_FAIL;
    if (c->hnorm == 0.0 || dt == 0.0) {
        if (fill_identity(true, d_out, d, 1, 1.0, 0.0, stream) != cudaSuccess) {
            cudaGetLastError();
            return c->last_error = PARAMENT_STATUS_CUBLAS_FAILED;
        }
        c->last_M = M;
        c->launches = 1;
        return c->last_error = PARAMENT_STATUS_SUCCESS;
    }
    // Chunk products and the tree's second buffer: 2 * nchunks * d^2 complex128.
    const size_t per_chunk = 2 * sizeof(double) * 2 * (size_t)d * d;
    const long long fit = (long long)(usable_scratch_bytes() / per_chunk);
    const int nch = (int)std::min<long long>(small_chunk_count(true, d, (int)c->Ke, P, c->num_sms), fit);
    if (nch < 1) return c->last_error = PARAMENT_STATUS_SCRATCH_EXCEEDED;
    char *chunks = static_cast<char *>(scratch);
    char *work = chunks + (size_t)nch * d * d * 2 * sizeof(double);
    std::vector<double> J(2 * (M + 1));
    bessel_coeffs(M, h * c->hnorm, J.data());
    StepLaunch l{};
    l.fp64 = true;
    l.d = d;
    l.Ke = (int)c->Ke;
    l.w = WeightSpecHost{pts, (int)c->K, (int)amps, c->quad, c->magnus ? 1 : 0, h / 12.0};
    l.M = M;
    l.J = J.data();
    l.s = 2.0 / c->hnorm;
    l.stack = c->stack.ptr;
    l.carr = d_carr;
    l.chunks = chunks;
    l.P = P;
    l.nchunks = nch;
    l.stream = stream;
    if (c->timing) cudaEventRecord(c->ev_start, stream);
    cudaError_t e = launch_small_steps(l);
    if (c->timing) cudaEventRecord(c->ev_stop, stream);
    int levels = 0;
    if (e == cudaSuccess) e = tree_product(true, d, chunks, nch, work, d_out, stream, c->num_sms, &levels);
    c->launches = 1 + levels;
    if (e != cudaSuccess) {
        cudaGetLastError();
        return c->last_error = PARAMENT_STATUS_CUBLAS_FAILED;
    }
    c->last_M = M;
    return c->last_error = PARAMENT_STATUS_SUCCESS;
}
