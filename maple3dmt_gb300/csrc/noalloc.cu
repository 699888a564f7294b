// m3d_dot_batched_noalloc: the batched Hermitian dot of m3d_dot_batched with
// no solver handle and no device allocation.
//
// Who needs it: a caller that owns every byte of device memory itself and
// may not allocate, e.g. an inversion driver that has given the whole of HBM
// to its own field and model-vector pool and evaluates misfit and model
// norms there, or a driver that runs these norms next to solves in flight on
// other streams, where a cudaMalloc/cudaFree could stall the device.  The
// solver-bound entry needs m3d_solver_setup, which allocates the mesh,
// matrix and Krylov vectors (gigabytes); this one needs nothing but its
// inputs.
//
// How: the reduction scratch is a file-scope device array of fixed size,
// K <= 16 right-hand sides x 1024 blocks of partial sums (256 KiB per
// device).  Its address is looked up once per device context with
// cudaGetSymbolAddress while that device is current, and cached together with
// the context's id (cuCtxGetId).  The first call on a device, and the first
// call after that device's context was replaced (cudaDeviceReset, or a new
// primary context), does this set-up (the runtime may load the module there),
// so make it before any latency-critical region and before any stream
// capture.  Larger K is rejected with M3D_ERR_TOO_LARGE; n is unlimited (the
// kernel strides over the grid).
//
// The only scratch state that must start at zero is the arrival counter of
// the grid reduction; each call clears it on the caller's stream before the
// launch (the kernel's last block also leaves it at zero).  The partial sums
// need no clearing: every block writes its own before the last block reads.
//
// There is one scratch array per device, so calls on the same device must not
// overlap: two calls in flight at once (different streams, or host threads
// without a lock) race on the partial sums and the counter and give wrong
// results.  Issue them on one stream, or serialise them.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "m3d_gb300.h"
#include "cuda/dot.cuh"

namespace {

constexpr int kNoAllocMaxRhs = 16;
constexpr int kNoAllocMaxBlocks = m3d::dev::kDotMaxBlocks;

struct NoAllocScratch {
    double2 partial[kNoAllocMaxBlocks * kNoAllocMaxRhs];
    double2 final_[kNoAllocMaxRhs];
    unsigned int counter;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
NoAllocScratch* g_addr[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Id of the calling thread's current context (unique for the life of the
// process), or 0 when it cannot be read.  The driver functions are reached
// through the runtime's entry-point query, so the library needs no -lcuda.
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1{}, q2{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
            get_id = reinterpret_cast<CtxGetIdFn>(f2);
        }
        cudaGetLastError();
        looked_up = true;
    }
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of this device's scratch; looked up with that device
// current on the first call, and again whenever the device's context differs
// from the one the cached address belongs to.
int scratch_of_current_device(NoAllocScratch** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return M3D_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices) return M3D_ERR_TOO_LARGE;
    std::lock_guard<std::mutex> lock(g_addr_mu);
    const unsigned long long ctx = current_context_id();
    if (!g_addr[dev] || ctx == 0 || ctx != g_ctx_id[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return M3D_ERR_CUDA;
        }
        g_addr[dev] = static_cast<NoAllocScratch*>(p);
        // the lookup made the context current if it was not yet
        g_ctx_id[dev] = current_context_id();
    }
    *out = g_addr[dev];
    return M3D_OK;
}

}  // namespace

extern "C" int m3d_dot_batched_noalloc(const double* x, const double* y, long long n, int K, double* out,
                                       void* stream) {
    if (K > kNoAllocMaxRhs) return M3D_ERR_TOO_LARGE;
    if (K != 1 && K != 2 && K != 4 && K != 8 && K != 16) return M3D_ERR_ARG;
    if (n < 0 || !out || (n > 0 && (!x || !y))) return M3D_ERR_ARG;
    NoAllocScratch* sc = nullptr;
    const int rc = scratch_of_current_device(&sc);
    if (rc != M3D_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(&sc->counter, 0, sizeof(unsigned int), st) != cudaSuccess) {
        cudaGetLastError();
        return M3D_ERR_CUDA;
    }
    m3d::dev::RedScratch rs{sc->partial, sc->final_, &sc->counter, kNoAllocMaxBlocks};
    if (m3d::dev::launch_dot_batched(reinterpret_cast<const double2*>(x), reinterpret_cast<const double2*>(y), n,
                                     K, kNoAllocMaxBlocks, rs, reinterpret_cast<double2*>(out), st) != cudaSuccess) {
        cudaGetLastError();
        return M3D_ERR_CUDA;
    }
    return M3D_OK;
}
