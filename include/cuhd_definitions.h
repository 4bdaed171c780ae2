// Buffer member macros of the reference API (include/cuhd_definitions.h:14-15).
#ifndef CUHD_DEFINITIONS_
#define CUHD_DEFINITIONS_

#include <memory>

#define cuhd_buf(TYPE, IDENTIFIER) std::shared_ptr<TYPE[]> IDENTIFIER
#define cuhd_out_buf(TYPE, IDENTIFIER) std::shared_ptr<TYPE[]> IDENTIFIER

#endif
