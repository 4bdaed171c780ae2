// Umbrella header of the reference API (include/multians.h:11-30).  The
// GPU classes are always included here (the reference gates them behind
// -DCUDA); the reference's std::thread decoder (MULTI) is not part of this
// library.
#ifndef MULTIANS_H_
#define MULTIANS_H_

#include "ans_encoder.h"
#include "ans_encoder_table.h"
#include "ans_table_generator.h"
#include "cuhd_codetable.h"
#include "cuhd_constants.h"
#include "cuhd_input_buffer.h"
#include "cuhd_output_buffer.h"
#include "cuhd_util.h"

#include "cuhd_gpu_codetable.h"
#include "cuhd_gpu_decoder.h"
#include "cuhd_gpu_decoder_memory.h"
#include "cuhd_gpu_input_buffer.h"
#include "cuhd_gpu_output_buffer.h"

#include "multians_gb300.h"

#endif
