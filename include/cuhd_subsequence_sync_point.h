// Sync point layout of the reference API
// (include/cuhd_subsequence_sync_point.h:16-23): 16 bytes per subsequence.
#ifndef CUHD_SUBSEQUENCE_SYNC_POINT_
#define CUHD_SUBSEQUENCE_SYNC_POINT_

#include "cuhd_constants.h"

namespace cuhd {
struct CUHDSubsequenceSyncPoint {
    std::uint32_t unit;
    std::uint32_t bit;
    std::uint32_t output_size;
    std::uint32_t state;
};
}  // namespace cuhd

#endif
