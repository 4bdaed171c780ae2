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

// Stream bit reader for one decoder, LSB first.  A 64-bit window lo:hi
// holds 32..63 valid bits; the next unit is prefetched into `pre` one
// refill ahead so the global load latency stays off the decode chain.  The
// prefetch reads a clamped (always in-bounds) address and keeps the
// "past the end" test apart, applying it only when the unit is used: a
// select right after the load would make every refill wait for memory.
// Positions are bit offsets relative to `origin` (a 64-bit bit address).
// Units at index >= n read as zero.
struct Cursor {
    uint32_t a;      // shared address of the current state's entry
    uint32_t lo, hi; // bit window
    uint32_t avail;  // valid bits in the window
    uint32_t pos;    // bit position of the next codeword (relative)
    uint32_t next;   // global index of the unit in `pre`
    uint32_t pre;    // prefetched unit (valid only if next < n)

    __device__ __forceinline__ static uint32_t ld(const uint32_t* __restrict__ in,
                                                  uint32_t n, uint32_t i) {
        return i < n ? __ldg(in + i) : 0u;
    }

    // Places the cursor at absolute bit position `abs` (pos = abs - origin).
    __device__ __forceinline__ void init(const uint32_t* __restrict__ in, uint32_t n,
                                         uint64_t origin, uint64_t abs,
                                         uint32_t entry_addr) {
        a = entry_addr;
        pos = (uint32_t) (abs - origin);
        const uint32_t u = (uint32_t) (abs >> 5), o = (uint32_t) (abs & 31);
        const uint32_t w0 = ld(in, n, u), w1 = ld(in, n, u + 1);
        lo = __funnelshift_r(w0, w1, o);
        hi = w1 >> o;
        avail = 64 - o;
        next = u + 2;
        pre = __ldg(in + min(next, n - 1));
    }

    // One step; returns the entry's y word (mask / k / count or symbol).
    __device__ __forceinline__ uint32_t step(const uint32_t* __restrict__ in, uint32_t n) {
        const uint2 e = lds64(a);
        const uint32_t b = lo & e.y & 0xffffu;
        a = e.x + (b << 3);
        const uint32_t k = __byte_perm(e.y, 0, 0x4442);
        lo = __funnelshift_r(lo, hi, k);
        hi >>= k;
        avail -= k;
        pos += k;
        if (avail < 32) {
            const uint32_t u = next < n ? pre : 0u;
            lo |= u << avail;
            hi = u >> (32 - avail);
            avail += 32;
            ++next;
            pre = __ldg(in + min(next, n - 1));
        }
        return e.y;
    }
};

__device__ __forceinline__ uint32_t entry_index(uint32_t a, uint32_t tab_base) {
    return (a - tab_base) >> 3;
}

}  // namespace mans
