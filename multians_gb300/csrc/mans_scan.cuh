// Exclusive prefix max and prefix sum over per-piece (m, delta) pairs, the
// scan both the decoder (regions) and the encoder (chunks) run between
// their sync and final passes.
#pragma once

#include <cstdint>

#include "multians_gb300.h"

namespace mans {

// Scan tiling: elements per tile.  In the decoder the word after the
// tiles' flags is the scan ticket and the next two count the merge-walk
// jobs.
constexpr uint32_t kScanThreads = 256;
constexpr uint32_t kScanPer = 8;
constexpr uint32_t kScanTile = kScanThreads * kScanPer;

// Exclusive prefix max of m (identity 0) and prefix sum of delta over the
// regions: single-pass decoupled look-back.  Tiles of kScanTile regions are
// taken in launch order through an atomic ticket, so a tile only ever waits
// on tiles that are already running or done; each wait is bounded and a
// timeout sets MANS_DEV_SCAN_TIMEOUT instead of spinning on.

struct ScanTile {               // one per tile, 32 bytes
    unsigned long long agg_m;   // tile max
    long long agg_s;            // tile sum
    unsigned long long inc_m;   // inclusive prefix max through this tile
    long long inc_s;            // inclusive prefix sum
};

// P is any parameter block with the fields m, delta, Mpre, Dpre (one per
// element, nreg elements), scan_tiles, scan_flags and status.
template <class P>
__device__ __forceinline__ void scan_body(const P& p, uint32_t tile) {
    __shared__ unsigned long long s_m[kScanThreads];
    __shared__ long long s_s[kScanThreads];
    __shared__ unsigned long long s_pm;
    __shared__ long long s_ps;
    ScanTile* tiles = p.scan_tiles;
    uint32_t* flags = p.scan_flags;
    const uint32_t t = threadIdx.x;
    const uint32_t base = tile * kScanTile + t * kScanPer;
    unsigned long long vm[kScanPer];
    long long vs[kScanPer];
    unsigned long long lm = 0;
    long long ls = 0;
#pragma unroll
    for (uint32_t i = 0; i < kScanPer; ++i) {
        const uint32_t r = base + i;
        vm[i] = r < p.nreg ? p.m[r] : 0ull;
        vs[i] = r < p.nreg ? p.delta[r] : 0ll;
        lm = max(lm, vm[i]);
        ls += vs[i];
    }
    s_m[t] = lm;
    s_s[t] = ls;
    __syncthreads();
    for (uint32_t off = 1; off < kScanThreads; off <<= 1) {
        unsigned long long xm = 0;
        long long xs = 0;
        if (t >= off) { xm = s_m[t - off]; xs = s_s[t - off]; }
        __syncthreads();
        if (t >= off) { s_m[t] = max(s_m[t], xm); s_s[t] += xs; }
        __syncthreads();
    }
    // the tile's aggregate, then its exclusive prefix by a warp-wide look-back:
    // lane l reads tile j - l, so one round trip covers 32 predecessors
    // (their aggregates up to the nearest inclusive prefix)
    __shared__ unsigned long long s_am;
    __shared__ long long s_as;
    if (t == kScanThreads - 1) {
        s_am = s_m[t];
        s_as = s_s[t];
    }
    __syncthreads();
    if (t < 32) {
        const unsigned long long am = s_am;
        const long long as = s_as;
        unsigned long long pm = 0;
        long long ps = 0;
        if (tile == 0) {
            if (t == 0) {
                tiles[0].inc_m = am;
                tiles[0].inc_s = as;
                __threadfence();
                atomicExch(flags + 0, 2u);
            }
        } else {
            if (t == 0) {
                tiles[tile].agg_m = am;
                tiles[tile].agg_s = as;
                __threadfence();
                atomicExch(flags + tile, 1u);
            }
            int32_t j = (int32_t) tile - 1;
            uint32_t spins = 0;
            while (j >= 0) {
                const int32_t q = j - (int32_t) t;
                uint32_t f = 0;
                unsigned long long vm = 0;
                long long vs = 0;
                if (q >= 0) {
                    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(f) : "l"(flags + q) : "memory");
                    if (f == 2) {
                        vm = *(volatile unsigned long long*) &tiles[q].inc_m;
                        vs = *(volatile long long*) &tiles[q].inc_s;
                    } else if (f == 1) {
                        vm = *(volatile unsigned long long*) &tiles[q].agg_m;
                        vs = *(volatile long long*) &tiles[q].agg_s;
                    }
                }
                // lanes 0 .. stop: the predecessors down to the nearest
                // inclusive prefix (tile 0's always is one)
                const uint32_t incl = __ballot_sync(0xffffffffu, q >= 0 && f == 2);
                const uint32_t stop = incl ? __ffs(incl) - 1 : 31u;
                const uint32_t upto = stop == 31 ? 0xffffffffu : ((2u << stop) - 1u);
                const uint32_t valid = __ballot_sync(0xffffffffu, q >= 0);
                if (__ballot_sync(0xffffffffu, q >= 0 && f == 0) & upto & valid) {
                    if (++spins > (1u << 24)) {   // a predecessor never published
                        if (t == 0) atomicOr(p.status, MANS_DEV_SCAN_TIMEOUT);
                        break;
                    }
                    continue;
                }
                unsigned long long wm = t <= stop ? vm : 0ull;
                long long ws = t <= stop ? vs : 0ll;
#pragma unroll
                for (uint32_t o = 16; o; o >>= 1) {
                    wm = max(wm, __shfl_xor_sync(0xffffffffu, wm, o));
                    ws += __shfl_xor_sync(0xffffffffu, ws, o);
                }
                pm = max(pm, wm);
                ps += ws;
                if (incl) break;
                j -= 32;
            }
            if (t == 0) {
                tiles[tile].inc_m = max(pm, am);
                tiles[tile].inc_s = ps + as;
                __threadfence();
                atomicExch(flags + tile, 2u);
            }
        }
        if (t == 0) {
            s_pm = pm;
            s_ps = ps;
        }
    }
    __syncthreads();
    unsigned long long run_m = max(s_pm, t ? s_m[t - 1] : 0ull);
    long long run_s = s_ps + (t ? s_s[t - 1] : 0ll);
#pragma unroll
    for (uint32_t i = 0; i < kScanPer; ++i) {
        const uint32_t r = base + i;
        if (r < p.nreg) {
            p.Mpre[r] = run_m;
            p.Dpre[r] = run_s;
        }
        run_m = max(run_m, vm[i]);
        run_s += vs[i];
    }
}

}  // namespace mans
