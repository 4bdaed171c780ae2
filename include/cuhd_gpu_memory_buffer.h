// Device buffer mirroring a host buffer, as in the reference API
// (include/cuhd_gpu_memory_buffer.h:19-39): allocate() reserves and zeroes
// device memory, cpy_host_to_device() allocates on first use and copies,
// cpy_device_to_host() copies back, the destructor frees.  CUDA errors end
// the process through CUERR as in the reference.
#ifndef CUHD_GPU_MEMORY_BUFFER_
#define CUHD_GPU_MEMORY_BUFFER_

#include <cstddef>
#include <memory>

#include "cuhd_constants.h"

namespace cuhd {
template <typename T>
class CUHDGPUMemoryBuffer {
public:
    CUHDGPUMemoryBuffer(T* buffer, size_t size);
    ~CUHDGPUMemoryBuffer();

    T* get();
    void allocate();
    void free();
    void cpy_host_to_device();
    void cpy_device_to_host();

    size_t get_size() const { return size_; }

private:
    T* buffer_;
    T* buffer_device_ = nullptr;
    bool is_allocated_ = false;
    size_t size_;
};
}  // namespace cuhd

#include "cuhd_gpu_memory_buffer.hxx"

#endif
