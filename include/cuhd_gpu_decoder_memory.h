// Decoder scratch memory (reference include/cuhd_gpu_decoder_memory.h:20-45).
// Same constructor and methods.  It holds this decoder's sync workspace
// (per-block entry records, per-region merge data, scan state, prepared
// tables), sized for the largest geometry the planner may choose for
// num_units units; the subsequence size and thread count of the reference
// constructor are accepted and kept, and used as planning hints.
// reserve() grows the workspace before a decode whose plan captures
// symbols (the capture slices scale with the output size, which the
// constructor does not see).
// get_sync_info() returns the start of the workspace, get_output_sizes()
// and the sync-flag getters return null: this decoder has no host
// round-trips and no per-subsequence count array.
#ifndef CUHD_GPU_DECODER_MEMORY_
#define CUHD_GPU_DECODER_MEMORY_

#include <cstddef>
#include <cstdint>

#include "cuhd_constants.h"
#include "cuhd_cuda_definitions.h"
#include "cuhd_subsequence_sync_point.h"
#include "cuhd_util.h"

namespace cuhd {
class CUHDGPUDecoderMemory {
public:
    CUHDGPUDecoderMemory(size_t num_units, size_t subsequence_size, size_t num_threads);
    ~CUHDGPUDecoderMemory();

    void allocate();
    void free();
    void retrieve_sync_data();

    cuhd::CUHDSubsequenceSyncPoint* get_sync_info();
    std::uint32_t* get_output_sizes();
    std::uint8_t* get_sequence_synced_device();
    std::uint8_t* get_sequence_synced_host();

    // workspace for the C ABI (mans_decode)
    void reserve(size_t bytes);
    void* get_workspace() { return workspace_; }
    size_t get_workspace_size() const { return bytes_; }
    size_t get_subsequence_size() const { return subsequence_size_; }
    size_t get_num_threads() const { return num_threads_; }

private:
    const size_t num_units_;
    const size_t subsequence_size_;
    const size_t num_threads_;
    size_t bytes_ = 0;
    void* workspace_ = nullptr;
    bool is_allocated_ = false;
};
}  // namespace cuhd

#endif
