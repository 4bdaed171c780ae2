// Decoder scratch memory (reference include/cuhd_gpu_decoder_memory.h:20-45).
// Same constructor and methods.  allocate() reserves this decoder's sync
// workspace (per-block entry records, per-region merge data, scan state,
// prepared tables, and symbol-capture slices) at the size every plan the
// planner may choose for num_units units fits, whatever the output size and
// table size: decode then allocates nothing, as the reference's does.  It
// also allocates the reference's four arrays with the reference's shapes
// (src/multians_gpu_decoder_memory.cc:25-50; num_subseq = units / S and
// num_blocks = num_subseq / threads, rounded up, S and threads from the
// constructor):
//   get_sync_info()               num_subseq CUHDSubsequenceSyncPoint, zero
//   get_output_sizes()            num_subseq uint32, zero
//   get_sequence_synced_device()  num_blocks bytes: 0 after allocate(), 1
//                                 after every successful decode (this
//                                 decoder synchronises every sequence
//                                 before it returns)
//   get_sequence_synced_host()    page-locked copy of those flags, filled by
//                                 retrieve_sync_data()
// The sync points and output sizes stay zero: this decoder's own sync data
// (block records, merge points) lives in the workspace in its own layout,
// and its output offsets come from a prefix over regions, not subsequences.
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

    // workspace for the C ABI (mans_decode); flags set after a decode
    void mark_synced();
    bool is_allocated() const { return is_allocated_; }
    void* get_workspace() { return workspace_; }
    size_t get_workspace_size() const { return bytes_; }
    size_t get_subsequence_size() const { return subsequence_size_; }
    size_t get_num_threads() const { return num_threads_; }

private:
    const size_t num_units_;
    const size_t subsequence_size_;
    const size_t num_threads_;
    const size_t num_subseq_;
    const size_t num_blocks_;
    size_t bytes_ = 0;
    void* workspace_ = nullptr;
    cuhd::CUHDSubsequenceSyncPoint* sync_info_ = nullptr;
    std::uint32_t* output_sizes_ = nullptr;
    std::uint8_t* synced_device_ = nullptr;
    std::uint8_t* synced_host_ = nullptr;
    bool is_allocated_ = false;
};
}  // namespace cuhd

#endif
