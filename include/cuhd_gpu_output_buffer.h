// Device buffer for decoded symbols (reference include/cuhd_gpu_output_buffer.h:19-29).
#ifndef CUHD_GPU_OUTPUT_BUFFER_
#define CUHD_GPU_OUTPUT_BUFFER_

#include <memory>

#include "cuhd_gpu_memory_buffer.h"
#include "cuhd_output_buffer.h"

namespace cuhd {
class CUHDGPUOutputBuffer : public CUHDGPUMemoryBuffer<SYMBOL_TYPE> {
public:
    explicit CUHDGPUOutputBuffer(std::shared_ptr<CUHDOutputBuffer> output_buffer);

private:
    std::shared_ptr<CUHDOutputBuffer> output_buffer_;
};
}  // namespace cuhd

#endif
