// GPU-side classes of the reference API: device copies of the table, the
// input and the output (src/multians_gpu_{codetable,input_buffer,
// output_buffer}.cc), decoder scratch memory
// (src/multians_gpu_decoder_memory.cc) and the decode call
// (src/multians_gpu_decoder.cu:575-687), all over the C ABI of
// include/multians_gb300.h.
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <iostream>

#include <cuda_runtime.h>

#include "cuhd_gpu_codetable.h"
#include "cuhd_gpu_decoder.h"
#include "cuhd_gpu_decoder_memory.h"
#include "cuhd_gpu_input_buffer.h"
#include "cuhd_gpu_output_buffer.h"
#include "multians_gb300.h"

cuhd::CUHDGPUCodetable::CUHDGPUCodetable(std::shared_ptr<CUHDCodetable> codetable)
    : CUHDGPUMemoryBuffer<CUHDCodetableItem>(codetable->get(), codetable->get_size()),
      table_(codetable) {}

cuhd::CUHDGPUInputBuffer::CUHDGPUInputBuffer(std::shared_ptr<CUHDInputBuffer> input_buffer)
    : CUHDGPUMemoryBuffer<UNIT_TYPE>(input_buffer->get_compressed_data(),
                                     input_buffer->get_compressed_size() + 4),
      input_buffer_(input_buffer) {}

cuhd::CUHDGPUOutputBuffer::CUHDGPUOutputBuffer(std::shared_ptr<CUHDOutputBuffer> output_buffer)
    : CUHDGPUMemoryBuffer<SYMBOL_TYPE>(output_buffer->get_decompressed_data().get(),
                                       output_buffer->get_uncompressed_size()),
      output_buffer_(output_buffer) {}

namespace {

size_t sdiv(size_t a, size_t b) { return b ? (a + b - 1) / b : 0; }

}  // namespace

cuhd::CUHDGPUDecoderMemory::CUHDGPUDecoderMemory(size_t num_units, size_t subsequence_size,
                                                 size_t num_threads)
    : num_units_(num_units), subsequence_size_(subsequence_size), num_threads_(num_threads),
      num_subseq_(sdiv(num_units, subsequence_size ? subsequence_size : 4)),
      num_blocks_(sdiv(num_subseq_, num_threads ? num_threads : 128)) {}

cuhd::CUHDGPUDecoderMemory::~CUHDGPUDecoderMemory() { free(); }

void cuhd::CUHDGPUDecoderMemory::allocate() {
    if (is_allocated_) return;
    bytes_ = mans_aux_size_max_any(num_units_ ? num_units_ : 1);
    cudaMalloc(&workspace_, bytes_);
    CUERR
    // the reference's arrays, same shapes (src/multians_gpu_decoder_memory.cc
    // :25-50): zero-filled sync points and sizes, and the per-sequence sync
    // flags on the device and in page-locked host memory
    const size_t ns = num_subseq_ ? num_subseq_ : 1, nb = num_blocks_ ? num_blocks_ : 1;
    cudaMalloc((void**) &sync_info_, ns * sizeof(CUHDSubsequenceSyncPoint));
    cudaMemset(sync_info_, 0, ns * sizeof(CUHDSubsequenceSyncPoint));
    cudaMalloc((void**) &output_sizes_, ns * sizeof(std::uint32_t));
    cudaMemset(output_sizes_, 0, ns * sizeof(std::uint32_t));
    cudaMalloc((void**) &synced_device_, nb);
    cudaMemset(synced_device_, 0, nb);
    cudaMallocHost((void**) &synced_host_, nb);
    CUERR
    std::memset(synced_host_, 0, nb);
    is_allocated_ = true;
}

void cuhd::CUHDGPUDecoderMemory::mark_synced() {
    if (is_allocated_) cudaMemset(synced_device_, 1, num_blocks_ ? num_blocks_ : 1);
}

void cuhd::CUHDGPUDecoderMemory::free() {
    if (!is_allocated_) return;
    cudaFree(workspace_);
    cudaFree(sync_info_);
    cudaFree(output_sizes_);
    cudaFree(synced_device_);
    cudaFreeHost(synced_host_);
    workspace_ = nullptr;
    sync_info_ = nullptr;
    output_sizes_ = nullptr;
    synced_device_ = nullptr;
    synced_host_ = nullptr;
    bytes_ = 0;
    is_allocated_ = false;
}

void cuhd::CUHDGPUDecoderMemory::retrieve_sync_data() {
    if (!is_allocated_) return;
    cudaMemcpy(synced_host_, synced_device_, num_blocks_ ? num_blocks_ : 1,
               cudaMemcpyDeviceToHost);
    CUERR
}

cuhd::CUHDSubsequenceSyncPoint* cuhd::CUHDGPUDecoderMemory::get_sync_info() { return sync_info_; }
std::uint32_t* cuhd::CUHDGPUDecoderMemory::get_output_sizes() { return output_sizes_; }
std::uint8_t* cuhd::CUHDGPUDecoderMemory::get_sequence_synced_device() { return synced_device_; }
std::uint8_t* cuhd::CUHDGPUDecoderMemory::get_sequence_synced_host() { return synced_host_; }

int cuhd::CUHDGPUDecoder::decode_status(
    std::shared_ptr<cuhd::CUHDGPUInputBuffer> input, size_t input_size,
    std::shared_ptr<cuhd::CUHDGPUOutputBuffer> output, size_t output_size,
    std::shared_ptr<cuhd::CUHDGPUCodetable> table, std::shared_ptr<cuhd::CUHDGPUDecoderMemory> aux,
    STATE_TYPE initial_state, std::uint32_t initial_bit, std::uint32_t number_of_states,
    size_t /*max_codeword_length: unused, as in the reference*/,
    size_t /*preferred_subsequence_size*/, size_t /*threads_per_block*/) {
    if (!input || !output || !table || !aux) return MANS_ERR_ARG;
    // the reference's decode allocates nothing (src/multians_gpu_decoder.cu
    // :575-687): the workspace is what allocate() reserved, which every plan
    // fits; decoder memory that was never allocated is an argument error
    if (!aux->is_allocated()) return MANS_ERR_ARG;
    uint32_t dev_status = 0;
    const int rc = mans_decode_sync(input->get(), input_size, output->get(), output_size,
                                    reinterpret_cast<const uint32_t*>(table->get()),
                                    number_of_states, initial_state, initial_bit,
                                    aux->get_workspace(), aux->get_workspace_size(), nullptr,
                                    nullptr, &dev_status);
    // every sequence is synchronised once the decode has returned
    if (rc == MANS_OK) aux->mark_synced();
    return rc;
}

void cuhd::CUHDGPUDecoder::decode(
    std::shared_ptr<cuhd::CUHDGPUInputBuffer> input, size_t input_size,
    std::shared_ptr<cuhd::CUHDGPUOutputBuffer> output, size_t output_size,
    std::shared_ptr<cuhd::CUHDGPUCodetable> table, std::shared_ptr<cuhd::CUHDGPUDecoderMemory> aux,
    STATE_TYPE initial_state, std::uint32_t initial_bit, std::uint32_t number_of_states,
    size_t max_codeword_length, size_t preferred_subsequence_size, size_t threads_per_block) {
    const int rc = decode_status(input, input_size, output, output_size, table, aux,
                                 initial_state, initial_bit, number_of_states,
                                 max_codeword_length, preferred_subsequence_size,
                                 threads_per_block);
    if (rc != MANS_OK) {
        std::cout << "multians_gb300 decode error: status " << rc << " ("
                  << cudaGetErrorString(cudaGetLastError()) << ")" << std::endl;
        std::exit(1);
    }
}
