// Device copy of a decoder table (reference include/cuhd_gpu_codetable.h:17-25).
#ifndef CUHD_GPU_CODETABLE_
#define CUHD_GPU_CODETABLE_

#include <memory>

#include "cuhd_codetable.h"
#include "cuhd_gpu_memory_buffer.h"

namespace cuhd {
class CUHDGPUCodetable : public CUHDGPUMemoryBuffer<CUHDCodetableItem> {
public:
    explicit CUHDGPUCodetable(std::shared_ptr<CUHDCodetable> codetable);

private:
    std::shared_ptr<CUHDCodetable> table_;
};
}  // namespace cuhd

#endif
