// Decoded output of the reference API (include/cuhd_output_buffer.h:19-39).
// The GPU decoder writes symbols in decode order (last encoded first);
// reverse() restores source order.
#ifndef CUHD_OUTPUT_BUFFER_
#define CUHD_OUTPUT_BUFFER_

#include <cstddef>
#include <memory>

#include "cuhd_constants.h"
#include "cuhd_definitions.h"

class CUHDOutputBuffer {
public:
    explicit CUHDOutputBuffer(size_t size);

    std::shared_ptr<SYMBOL_TYPE[]>& get_decompressed_data();
    void reverse();
    size_t get_uncompressed_size();
    size_t get_symbol_size();

private:
    size_t uncompressed_size_;
    const size_t symbol_size_ = sizeof(SYMBOL_TYPE);
    cuhd_out_buf(SYMBOL_TYPE, buffer_);
};

#endif
