// Decoder table of the reference API (include/cuhd_codetable.h:20-45).  An
// item is 4 bytes: {u16 next_state, u8 symbol, u8 min_num_bits}; the GPU
// reads it as one little-endian word.
#ifndef CUHD_CODETABLE_
#define CUHD_CODETABLE_

#include <cstddef>
#include <memory>

#include "cuhd_constants.h"
#include "cuhd_definitions.h"

struct CUHDCodetableItem {
    std::uint16_t next_state;
    std::uint8_t symbol;
    std::uint8_t min_num_bits;
};
static_assert(sizeof(CUHDCodetableItem) == 4, "table items are packed 4-byte words");

class CUHDCodetable {
public:
    explicit CUHDCodetable(size_t num_entries);

    size_t get_size();
    size_t get_num_entries();
    size_t get_max_codeword_length();
    CUHDCodetableItem* get();

private:
    size_t size_;
    size_t num_entries_;
    cuhd_buf(CUHDCodetableItem, table_);
};

#endif
