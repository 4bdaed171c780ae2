// Type configuration of the decoder; the same macros as the reference's
// include/cuhd_constants.h:14-27 (they are part of its public API).
#ifndef CUHD_CONSTANTS_
#define CUHD_CONSTANTS_

#include <cstdint>

// longest codeword the reference's demo assumes (decode ignores it)
#define MAX_CODEWORD_LENGTH 11

#define UNIT_TYPE std::uint32_t
#define STATE_TYPE std::uint32_t
#define SYMBOL_TYPE std::uint8_t
#define BIT_COUNT_TYPE std::uint8_t

#endif
