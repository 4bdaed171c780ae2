// Compressed input of the reference API (include/cuhd_input_buffer.h:19-48):
// holds the encoder's units in reversed order plus four zero padding units,
// the bit count of the last encoded unit and the encoder's final state.
#ifndef CUHD_INPUT_BUFFER_
#define CUHD_INPUT_BUFFER_

#include <cstddef>
#include <memory>

#include "cuhd_constants.h"
#include "cuhd_definitions.h"

class CUHDInputBuffer {
public:
    CUHDInputBuffer(UNIT_TYPE* buffer, size_t size, size_t first_bit, size_t first_state);

    UNIT_TYPE* get_compressed_data();
    size_t get_first_bit();
    size_t get_first_state();
    size_t get_compressed_size();
    size_t get_unit_size();

private:
    size_t first_bit_;
    size_t first_state_;
    size_t compressed_size_;
    const size_t unit_size_ = sizeof(UNIT_TYPE);
    cuhd_buf(UNIT_TYPE, buffer_);
};

#endif
