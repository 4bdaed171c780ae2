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
//  * the array holds kScratchBytes (32 MiB) and every GPU that loads the
//    library keeps it until the process exits;
//  * a stream is accepted when the workspace of its planned geometry fits
//    (about 6.4 million units, ~26 MB of compressed input, at 6 bits per
//    symbol; about 1.7 million units at 0.67 bits per symbol); larger
//    streams get MANS_ERR_AUX_SMALL before any GPU work;
//  * every call on a device shares the one array and it keeps the last
//    call's contents: calls that overlap on the GPU (another stream, another
//    host thread) race and must be serialised by the caller.  The decode
//    itself clears what has to start at zero (status word, scan flags);
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current) and caches it; make
//    that first call before any stream capture.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "multians_gb300.h"

namespace {

constexpr size_t kScratchBytes = 32ull << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// Device address of g_scratch on the current device (looked up once).
int scratch_address(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return MANS_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return MANS_ERR_CUDA;
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
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
    mans_cfg plan;
    int rc = mans_plan(n_units, n_out, L, nullptr, &plan);
    if (rc != MANS_OK) return rc;
    if (plan.capture_bytes && mans_aux_size(n_units, &plan) > kScratchBytes) {
        // the capture slices do not fit: decode every block in the final pass
        mans_cfg hint = {0, 0, 0, 0, MANS_DECODE_NO_CAPTURE, 0};
        rc = mans_plan(n_units, n_out, L, &hint, &plan);
        if (rc != MANS_OK) return rc;
    }
    if (mans_aux_size(n_units, &plan) > kScratchBytes) return MANS_ERR_AUX_SMALL;
    void* scratch = nullptr;
    const int sc = scratch_address(&scratch);
    if (sc != MANS_OK) return sc;
    return mans_decode_sync(d_units, n_units, d_out, n_out, d_table, L, first_state, first_bit,
                            scratch, kScratchBytes, &plan, stream, status_out);
}

}  // extern "C"
