// Device building blocks of the GB300 MULTIANS decoder: the shared-memory
// decode table and the per-thread bit cursor.
//
// Decode step (the reference's per-symbol body, src/multians_gpu_decoder.cu
// :131-167): with state x in [L, 2L) and table word t = table[x - L] =
// {next_state, symbol, k}, the decoder reads k stream bits b (LSB first)
// and moves to x' = (next_state << k) | b; the symbol is emitted.  Every
// table the reference generator builds keeps x' in [L, 2L), so the
// reference's extra-bit loop (lines 141-145) never runs; the table check
// below enforces that form and rejects anything else.
//
// Internal table word (one per state index j = x - L), 32 bits:
//   bits  0..15  base  = (next_state << k) - L  (next index = base + b)
//   bits 16..20  k     (bits consumed, 0..16)
//   bits 24..31  symbol
#pragma once

#include <cstdint>

namespace mans {

constexpr uint32_t kMaxBits = 16;  // longest code a table word can carry

// Converts one reference table word into the internal form.  Entries that
// would leave [L, 2L), or zero-bit entries that do not strictly decrease
// the state index (a zero-bit cycle would never advance the stream), are
// replaced by a safe one-bit entry and reported through `bad`.  `selfloop`
// reports zero-bit entries that map a state to itself (all entries of a
// single-symbol table look like that).
__device__ __forceinline__ uint32_t convert_entry(uint32_t raw, uint32_t j,
                                                  uint32_t L, bool& bad,
                                                  bool& selfloop) {
    const uint32_t ns = raw & 0xffffu;
    const uint32_t sym = (raw >> 16) & 0xffu;
    const uint32_t k = raw >> 24;
    selfloop = false;
    if (k <= kMaxBits) {
        const uint64_t lo = (uint64_t) ns << k;
        const uint64_t hi = (uint64_t) (ns + 1) << k;
        if (lo >= L && hi <= 2ull * L) {
            const uint32_t base = (uint32_t) (lo - L);
            if (k > 0 || base < j) return base | (k << 16) | (sym << 24);
            selfloop = (base == j);
        }
    }
    bad = true;
    return (1u << 16) | (sym << 24);
}

// Loads and converts the table into shared memory (all threads of the CTA
// take part).  Returns through the flags whether any entry was invalid and
// whether every entry was a zero-bit self loop (single-symbol table).
__device__ __forceinline__ void load_table(uint32_t* s_tbl,
                                           const uint32_t* __restrict__ raw,
                                           uint32_t L, int& any_bad,
                                           int& all_selfloop) {
    int bad_local = 0, loop_all = 1;
    for (uint32_t j = threadIdx.x; j < L; j += blockDim.x) {
        bool bad = false, sl = false;
        s_tbl[j] = convert_entry(__ldg(raw + j), j, L, bad, sl);
        bad_local |= bad ? 1 : 0;
        loop_all &= sl ? 1 : 0;
    }
    any_bad = __syncthreads_or(bad_local);
    all_selfloop = __syncthreads_and(loop_all);
}

// Sequential reader of the stream bits, LSB first, starting at any bit
// position.  Keeps 32..63 valid bits in a 64-bit buffer; units at index
// >= n read as zero (the padding of the reference input buffer).
struct BitCursor {
    const uint32_t* __restrict__ in;
    uint64_t buf;
    uint64_t pos;      // global bit position of the next unread bit
    uint32_t n;        // units in the stream
    uint32_t next;     // next unit to load into buf
    uint32_t nbits;    // valid bits in buf

    __device__ __forceinline__ uint32_t unit(uint32_t i) const {
        return i < n ? __ldg(in + i) : 0u;
    }

    __device__ __forceinline__ void init(const uint32_t* __restrict__ src,
                                         uint32_t n_units, uint64_t p) {
        in = src;
        n = n_units;
        pos = p;
        const uint32_t u = (uint32_t) (p >> 5);
        const uint32_t o = (uint32_t) (p & 31);
        buf = ((uint64_t) unit(u) | ((uint64_t) unit(u + 1) << 32)) >> o;
        nbits = 64 - o;
        next = u + 2;
    }

    // One decode step from state index `idx`; returns the table word used.
    __device__ __forceinline__ uint32_t step(const uint32_t* s_tbl,
                                             uint32_t& idx) {
        const uint32_t e = s_tbl[idx];
        const uint32_t k = (e >> 16) & 31u;
        const uint32_t bits = (uint32_t) buf & ((1u << k) - 1u);
        idx = (e & 0xffffu) + bits;
        buf >>= k;
        nbits -= k;
        pos += k;
        if (nbits < 32) {
            buf |= (uint64_t) unit(next) << nbits;
            ++next;
            nbits += 32;
        }
        return e;
    }
};

}  // namespace mans
