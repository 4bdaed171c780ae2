// The decode call of the reference API (include/cuhd_gpu_decoder.h:21-37,
// src/multians_gpu_decoder.cu:575-687): same signature and meaning.
// Decodes `input_size` units into `output_size` symbols in decode order
// (reversed, like the reference) on the current device and returns when
// the result is in `output`.  On an error it prints and exits like the
// reference's CUERR; decode_status() is the same call returning the
// mans_status code instead.  max_codeword_length is unused (as in the
// reference).  preferred_subsequence_size and threads_per_block are
// accepted and ignored: the geometry (units per block, blocks per region,
// threads per CTA) is the planner's, keyed on the table size and the
// compression ratio; the reference's S = 4 / 128-thread geometry would give
// this decoder blocks of 4 units and 16 B of records per 16 B of input.
// The decoder memory must have been allocate()d (MANS_ERR_ARG otherwise);
// the call itself allocates nothing.
#ifndef CUHD_GPU_DECODER_
#define CUHD_GPU_DECODER_

#include <cstddef>
#include <memory>

#include "cuhd_constants.h"
#include "cuhd_gpu_codetable.h"
#include "cuhd_gpu_decoder_memory.h"
#include "cuhd_gpu_input_buffer.h"
#include "cuhd_gpu_output_buffer.h"
#include "cuhd_subsequence_sync_point.h"

namespace cuhd {
class CUHDGPUDecoder {
public:
    static void decode(std::shared_ptr<cuhd::CUHDGPUInputBuffer> input, size_t input_size,
                       std::shared_ptr<cuhd::CUHDGPUOutputBuffer> output, size_t output_size,
                       std::shared_ptr<cuhd::CUHDGPUCodetable> table,
                       std::shared_ptr<cuhd::CUHDGPUDecoderMemory> aux,
                       STATE_TYPE initial_state, std::uint32_t initial_bit,
                       std::uint32_t number_of_states, size_t max_codeword_length,
                       size_t preferred_subsequence_size, size_t threads_per_block);

    static int decode_status(std::shared_ptr<cuhd::CUHDGPUInputBuffer> input, size_t input_size,
                             std::shared_ptr<cuhd::CUHDGPUOutputBuffer> output,
                             size_t output_size, std::shared_ptr<cuhd::CUHDGPUCodetable> table,
                             std::shared_ptr<cuhd::CUHDGPUDecoderMemory> aux,
                             STATE_TYPE initial_state, std::uint32_t initial_bit,
                             std::uint32_t number_of_states, size_t max_codeword_length,
                             size_t preferred_subsequence_size, size_t threads_per_block);
};
}  // namespace cuhd

#endif
