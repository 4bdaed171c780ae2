// Single-state tANS encoder of the reference API (include/ans_encoder.h:22-45).
// encode() returns the stream as a CUHDInputBuffer (units reversed, first
// bit and first state set).  `in` must be readable one symbol past size_in:
// like the reference, the encoder looks one symbol ahead at the end.
#ifndef ANS_ENCODER_
#define ANS_ENCODER_

#include <cstddef>
#include <memory>

#include "ans_encoder_table.h"
#include "ans_table_generator.h"
#include "cuhd_constants.h"
#include "cuhd_definitions.h"
#include "cuhd_input_buffer.h"

struct Decoder_Info {
    UNIT_TYPE state;
    size_t bit;
    size_t size;   // encoded size in units
};

class ANSEncoder {
public:
    static std::shared_ptr<CUHDInputBuffer> encode(SYMBOL_TYPE* in, size_t size_in,
                                                   std::shared_ptr<ANSEncoderTable> encoder_table);

private:
    static void encode_memory(UNIT_TYPE* out, size_t size_out, SYMBOL_TYPE* in, size_t size_in,
                              std::shared_ptr<ANSEncoderTable> encoder_table,
                              std::shared_ptr<Decoder_Info> decoder_info);
};

#endif
