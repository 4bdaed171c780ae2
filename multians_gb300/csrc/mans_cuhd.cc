// GPU-side classes of the reference API: device copies of the table, the
// input and the output (src/multians_gpu_{codetable,input_buffer,
// output_buffer}.cc), decoder scratch memory
// (src/multians_gpu_decoder_memory.cc) and the decode call
// (src/multians_gpu_decoder.cu:575-687), all over the C ABI of
// include/multians_gb300.h.
#include <cstdio>
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

cuhd::CUHDGPUDecoderMemory::CUHDGPUDecoderMemory(size_t num_units, size_t subsequence_size,
                                                 size_t num_threads)
    : num_units_(num_units), subsequence_size_(subsequence_size), num_threads_(num_threads) {}

cuhd::CUHDGPUDecoderMemory::~CUHDGPUDecoderMemory() { free(); }

void cuhd::CUHDGPUDecoderMemory::allocate() {
    if (is_allocated_) return;
    bytes_ = mans_aux_size_max(num_units_ ? num_units_ : 1);
    cudaMalloc(&workspace_, bytes_);
    CUERR
    is_allocated_ = true;
}

void cuhd::CUHDGPUDecoderMemory::reserve(size_t bytes) {
    allocate();
    if (bytes <= bytes_) return;
    void* grown = nullptr;
    if (cudaMalloc(&grown, bytes) != cudaSuccess) {
        cudaGetLastError();   // keep the smaller workspace: the decode runs without capture
        return;
    }
    cudaFree(workspace_);
    workspace_ = grown;
    bytes_ = bytes;
}

void cuhd::CUHDGPUDecoderMemory::free() {
    if (!is_allocated_) return;
    cudaFree(workspace_);
    workspace_ = nullptr;
    bytes_ = 0;
    is_allocated_ = false;
}

void cuhd::CUHDGPUDecoderMemory::retrieve_sync_data() {}

cuhd::CUHDSubsequenceSyncPoint* cuhd::CUHDGPUDecoderMemory::get_sync_info() {
    return reinterpret_cast<cuhd::CUHDSubsequenceSyncPoint*>(workspace_);
}
std::uint32_t* cuhd::CUHDGPUDecoderMemory::get_output_sizes() { return nullptr; }
std::uint8_t* cuhd::CUHDGPUDecoderMemory::get_sequence_synced_device() { return nullptr; }
std::uint8_t* cuhd::CUHDGPUDecoderMemory::get_sequence_synced_host() { return nullptr; }

int cuhd::CUHDGPUDecoder::decode_status(
    std::shared_ptr<cuhd::CUHDGPUInputBuffer> input, size_t input_size,
    std::shared_ptr<cuhd::CUHDGPUOutputBuffer> output, size_t output_size,
    std::shared_ptr<cuhd::CUHDGPUCodetable> table, std::shared_ptr<cuhd::CUHDGPUDecoderMemory> aux,
    STATE_TYPE initial_state, std::uint32_t initial_bit, std::uint32_t number_of_states,
    size_t /*max_codeword_length: unused, as in the reference*/,
    size_t /*preferred_subsequence_size*/, size_t /*threads_per_block*/) {
    if (!input || !output || !table || !aux) return MANS_ERR_ARG;
    aux->allocate();
    mans_cfg plan;
    if (input_size && mans_plan(input_size, output_size, number_of_states, nullptr, &plan) == MANS_OK)
        aux->reserve(mans_aux_size(input_size, &plan));
    uint32_t dev_status = 0;
    return mans_decode_sync(input->get(), input_size, output->get(), output_size,
                            reinterpret_cast<const uint32_t*>(table->get()), number_of_states,
                            initial_state, initial_bit, aux->get_workspace(),
                            aux->get_workspace_size(), nullptr, nullptr, &dev_status);
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
