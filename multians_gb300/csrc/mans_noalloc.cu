// Decode without any allocation: the decoder's workspace lives in a
// file-scope device array instead of caller- or library-allocated memory.
//
// Who needs this: callers that may not allocate device memory at the
// moment they decode -- a plugin running inside a host application that
// owns all device memory through its own pool, a request path that must
// not stall behind cudaMalloc/cudaFree (both can synchronise the device),
// or a recovery path that runs when device memory is already exhausted.
// They pass their input and output buffers as usual; the workspace is this
// library's.
//
// Limits and rules:
//  * the array holds kScratchBytes (32 MiB); every GPU that loads the
//    library's kernels keeps it until the process exits.  Under CUDA's
//    default lazy module loading the array is reserved on a device when
//    this file's module is first used there, which is the first call's
//    address look-up: callers that rely on the entry point once device
//    memory is exhausted make one call early (a warm-up decode at start-up);
//  * a stream is accepted when some plan of it fits the array, tried in
//    the order mans_decode_sync tries them: the planner's geometry, then
//    without symbol capture, then with fewer walk slots (measured with the
//    planner: about 28 million units, ~114 MB compressed, at 6 or 8.6
//    bits per symbol; about 7.7 million units at 0.67 bits per symbol,
//    L = 1024); larger streams get MANS_ERR_AUX_SMALL before any GPU work;
//  * every call on a device shares the one array and it keeps the last
//    call's contents: calls that overlap on the GPU (another stream, another
//    host thread) race and must be serialised by the caller.  The decode
//    itself clears what has to start at zero (status word, scan flags);
//  * the first call on a device (and the first after that device's context
//    is re-created, e.g. by cudaDeviceReset) looks up the array's device
//    address with that device current (cudaGetSymbolAddress) and caches it
//    under the context's ID; make that first call before any stream capture.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "multians_gb300.h"

namespace {

constexpr size_t kScratchBytes = 32ull << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

std::mutex g_mu;
struct Cached {
    unsigned long long ctx_id;
    void* addr;
};
Cached g_cache[kMaxDevices] = {};

// ID of the current device's current context (0 if it cannot be read): the
// cache key, so a context re-created after a reset looks the address up
// again.  The driver calls come through the runtime's entry-point query,
// so the library needs no link against the driver library.
unsigned long long current_ctx_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_current = (CtxGetCurrentFn) f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_id = (CtxGetIdFn) f;
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx ||
        get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// Device address of g_scratch on the current device, looked up once per
// device context.
int scratch_address(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return MANS_ERR_CUDA;
    // makes the device's primary context current (created if need be), so
    // that its ID can be read before the look-up
    if (cudaSetDevice(dev) != cudaSuccess) return MANS_ERR_CUDA;
    const unsigned long long id = current_ctx_id();
    std::lock_guard<std::mutex> lock(g_mu);
    Cached& c = g_cache[dev];
    if (!c.addr || id == 0 || c.ctx_id != id) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            c.addr = nullptr;
            return MANS_ERR_CUDA;
        }
        c.addr = p;
        c.ctx_id = id;
    }
    *out = c.addr;
    return MANS_OK;
}

}  // namespace

extern "C" {

size_t mans_noalloc_scratch_bytes(void) { return kScratchBytes; }

int mans_decode_noalloc(const uint32_t* d_units, size_t n_units, uint8_t* d_out, size_t n_out,
                        const uint32_t* d_table, uint32_t L, uint32_t first_state,
                        uint32_t first_bit, void* stream, uint32_t* status_out) {
    if (status_out) *status_out = 0;
    if (n_out == 0) return MANS_OK;
    // the arguments first, as mans_decode_sync checks them (the workspace
    // pointer it also checks is this file's)
    if (!d_units || ((uintptr_t) d_units & 15) || !d_out || !d_table || n_units == 0 ||
        n_units > 0xffffffffull || L < 2 || L > 8192 || first_state < L ||
        first_state >= 2 * L || first_bit > 32)
        return MANS_ERR_ARG;
    void* scratch = nullptr;
    const int sc = scratch_address(&scratch);
    if (sc != MANS_OK) return sc;
    // plans that do not fit the array fall back (no capture, fewer walk
    // slots) or return MANS_ERR_AUX_SMALL inside, before any GPU work
    return mans_decode_sync(d_units, n_units, d_out, n_out, d_table, L, first_state, first_bit,
                            scratch, kScratchBytes, nullptr, stream, status_out);
}

}  // extern "C"
