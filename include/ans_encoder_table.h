// Encoder table of the reference API (include/ans_encoder_table.h:19-45):
// table[symbol][state index] = {next state, emitted bits, their count}.
#ifndef ANS_ENCODER_TABLE_
#define ANS_ENCODER_TABLE_

#include <cstddef>
#include <vector>

#include "cuhd_constants.h"

struct ANSEncoderTable {
    struct ANSEncoderTableItem {
        std::uint32_t next_state;
        std::uint32_t code_sequence;
        std::uint32_t code_length;
        SYMBOL_TYPE symbol;
    };
    size_t max_number_of_symbols;
    size_t number_of_symbols;
    size_t number_of_states;
    std::vector<std::vector<ANSEncoderTableItem>> table;
};

#endif
