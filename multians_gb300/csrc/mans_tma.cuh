// TMA bulk copies (cp.async.bulk) and mbarriers for staging compressed
// units into shared memory, plus the shared-memory bit cursor.
//
// Why shared memory: a decoder refills its 64-bit window every few symbols,
// at a different step on every lane.  A refill from global memory leaves a
// load in flight on the warp's register; the next step some other lane
// refills and the warp waits for that load, so global latency lands on
// nearly every step.  Shared-memory refills cost a shared load that
// overlaps the table lookup of the next step.
#pragma once

#include <cstdint>

#include "mans_device.cuh"

namespace mans {

__device__ __forceinline__ uint32_t lds32(uint32_t a) {
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a));
    return v;
}

__device__ __forceinline__ void sts32(uint32_t a, uint32_t v) {
    asm volatile("st.shared.u32 [%0], %1;" :: "r"(a), "r"(v) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(count) : "memory");
}

// Retires an mbarrier whose phases have all completed, so its word can be
// initialised again.
__device__ __forceinline__ void mbar_inval(uint32_t bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" :: "r"(bar) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity; gives up after a bounded
// number of polls (returns false) instead of spinning forever.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < (1u << 22); ++i)
        if (mbar_test(bar, parity)) return true;
    return false;
}

// 1-D bulk copy global -> shared, completion counted on `bar` (bytes).
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void tma_load(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        :: "r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

// Where a cursor finds its units: the unit with global index i lives at
// `base + min((i - u0) & wrap, last) * 4`.  A per-lane ring of 128 units
// uses u0 = 0, wrap = last = 127; a flat tile uses wrap = ~0 and
// last = tile length - 1.  The clamp keeps every shared address inside the
// caller's buffer whatever the stream contents.
struct UnitSrc {
    uint32_t base, u0, wrap, last;
    __device__ __forceinline__ uint32_t operator()(uint32_t i) const {
        return lds32(base + (min((i - u0) & wrap, last) << 2));
    }
};

// Bit cursor over units held in shared memory, software-pipelined: the
// table entry of the current state is already in registers (e), and each
// step issues the shared load of the next entry before anything that
// depends on this step's result, so the dependent chain per symbol is one
// shared load plus two integer operations.  The window is two units w0:w1
// (the units next - 2 and next - 1) and the next codeword starts at bit
// o < 32 of it: a step extracts 32 bits at o (one funnel shift, computed
// from the previous step's o before the entry arrives), moves o by k <= 16,
// and when o reaches 32 shifts the window by one unit (selects, no
// branch).
//
// Every step loads the unit a refill would take, next to the table entry
// and before either is needed.  Loading it only on refilling lanes (a
// branch some lane of the warp takes on most steps, about a fifth of the
// unit wavefronts) was measured slower in every pass on GB300: the
// branch-free step saves more issue slots than the extra wavefronts cost
// (G pass 0.345 -> 0.310 ms, final pass 0.349 -> 0.339 ms).
struct SCursor {
    uint2 e;         // table entry of the current state
    uint32_t a;      // shared address of that entry
    uint32_t w0, w1; // window: units next - 2 and next - 1
    uint32_t o;      // bit offset of the next codeword in w0:w1 (< 32)
    uint32_t pos;    // bit position of the next codeword (relative)
    uint32_t next;   // global index of the next unit a refill takes

    __device__ __forceinline__ void init(const UnitSrc& src, uint64_t origin, uint64_t abs,
                                         uint32_t entry_addr) {
        a = entry_addr;
        e = lds64(a);
        pos = (uint32_t) (abs - origin);
        const uint32_t u = (uint32_t) (abs >> 5);
        o = (uint32_t) (abs & 31);
        w0 = src(u);
        w1 = src(u + 1);
        next = u + 2;
    }

    // One step; returns y (mask | k << 16 | count-or-symbol << 24).
    __device__ __forceinline__ uint32_t step(const UnitSrc& src) {
        const uint32_t u = src(next);
        const uint32_t y = e.y;
        const uint32_t bits = __funnelshift_r(w0, w1, o);
        a = e.x + ((bits & y & 0xffffu) << 3);
        e = lds64(a);
        const uint32_t k = __byte_perm(y, 0, 0x4442);
        pos += k;
        o += k;
        const bool r = o >= 32;    // at most one unit per step: o < 32, k <= 16
        w0 = r ? w1 : w0;
        w1 = r ? u : w1;
        o = r ? o - 32 : o;
        next += r ? 1u : 0u;
        return y;
    }
};

}  // namespace mans
