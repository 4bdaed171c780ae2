// Device copy of a compressed stream, with the reference's four padding
// units (reference include/cuhd_gpu_input_buffer.h:19-29,
// src/multians_gpu_input_buffer.cc:13-19).
#ifndef CUHD_GPU_INPUT_BUFFER_
#define CUHD_GPU_INPUT_BUFFER_

#include <memory>

#include "cuhd_gpu_memory_buffer.h"
#include "cuhd_input_buffer.h"

namespace cuhd {
class CUHDGPUInputBuffer : public CUHDGPUMemoryBuffer<UNIT_TYPE> {
public:
    explicit CUHDGPUInputBuffer(std::shared_ptr<CUHDInputBuffer> input_buffer);

private:
    std::shared_ptr<CUHDInputBuffer> input_buffer_;
};
}  // namespace cuhd

#endif
