// Device building blocks of the GB300 MULTIANS decoder: the shared-memory
// decode tables and the per-thread bit cursor.
//
// Decode step (the reference's per-symbol body, src/multians_gpu_decoder.cu
// :131-167): with state x in [L, 2L) and table word t = table[x - L] =
// {next_state, symbol, k}, the decoder reads k stream bits b (LSB first)
// and moves to x' = (next_state << k) | b; the symbol is emitted.  Every
// table the reference generator builds keeps x' in [L, 2L), so the
// reference's extra-bit loop (lines 141-145) never runs; the table check
// enforces that form and rejects anything else.
//
// Shared-memory entry (8 bytes per state index j = x - L):
//   x  byte address (shared window) of the entry of state index
//      base = (next_state << k) - L; the next entry is at x + 8 * b
//   y  bits  0..15  mask = (1 << k) - 1
//      bits 16..23  k
//      bits 24..31  (counting table) codewords this step stands for
//                   (symbol table)   the symbol
// so one step is: e = lds64(a); b = buf & e.y & 0xffff; a = e.x + 8 * b --
// two integer operations between dependent shared loads.
//
// The counting table folds runs of zero-bit codewords: from state j the
// decoder may pass z zero-bit codewords (no bits read, state strictly
// decreasing) before a codeword that reads bits.  Its entry for j is the
// entry of that last codeword with a count of z + 1, so one step advances
// to the next bit position.  Positions where a step starts are exactly the
// first codewords at each bit position, which is all the sync logic needs.
#pragma once

#include <cstdint>

namespace mans {

constexpr uint32_t kMaxBits = 16;      // longest code a table word can carry
constexpr uint32_t kMaxStates = 8192;  // L limit of the shared tables
constexpr uint32_t kIncMax = 255;      // longest folded run (8 bits)

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint2 lds64(uint32_t a) {
    uint2 v;
    asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(a));
    return v;
}

// Copies a prepared table (global, x fields relative to the table start)
// into shared memory, rebasing x to shared addresses.  All threads.
__device__ __forceinline__ void load_prepared(uint2* s_tab, const uint2* __restrict__ g_tab,
                                              uint32_t L) {
    const uint32_t base = smem_addr(s_tab);
    for (uint32_t j = threadIdx.x; j < L; j += blockDim.x) {
        uint2 e = __ldg(g_tab + j);
        e.x += base;
        s_tab[j] = e;
    }
    __syncthreads();
}

__device__ __forceinline__ uint32_t entry_index(uint32_t a, uint32_t tab_base) {
    return (a - tab_base) >> 3;
}

}  // namespace mans
