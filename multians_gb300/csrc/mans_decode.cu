// Plain single-stream decode: the reference's four phases (guessed-state
// decode, sync extension, exclusive prefix sum, final write pass) rebuilt
// as sm_103a kernels that never stop for the host (k_prep, k_gwalk,
// k_wwalk, k_scan, then k_final, or with symbol capture k_copy and
// k_final_fb), and the batched form of the same kernels.
//
// Geometry.  The stream is cut into blocks of B units (final-pass work
// items) and regions of nb blocks (sync work items, R = nb * B units).
//
//  k_gwalk  one thread per region k.  It decodes region k from a guessed
//           start (bit 0 of the region, state = the stream's first state;
//           region 0 starts from the true start), the trajectory Gamma_k,
//           and records for every block of the region the first codeword
//           at or after the block start and Gamma_k's symbol count before
//           it, and Gamma_k's entry at the first block of region k + 1.
//  k_wwalk  keeps walking Gamma_k past its region end (the G pass starts
//           each walk; this pass finishes the longer ones), comparing it
//           at every block start with Gamma_{k+1}, until the
//           two trajectories meet at the same bit position in the same
//           state: the merge point m_k.  Gamma_k's count minus
//           Gamma_{k+1}'s count at m_k is delta_k.  Blocks the walk crosses
//           before m_k get Gamma_k's records in walk slot (region - k).
//           Together these are the reference's guessed-state decode and
//           sync extension (src/multians_gpu_decoder.cu:195-361, 363-466),
//           with the check made at every block start instead of at
//           subsequence ends and with no host round trip per pass.
//  k_scan   M_k = max(0, m_0..m_{k-1}) and D_k = sum(delta_0..delta_{k-1}).
//           After M_k the true trajectory is Gamma_k and its global symbol
//           index is D_k + Gamma_k's count (by induction from Gamma_0,
//           which starts at the true start).  Replaces the reference's
//           thrust::exclusive_scan of per-subsequence counts
//           (src/multians_gpu_decoder.cu:658-670).
//  k_final  one thread per block b: the largest k <= region(b) with
//           M_k <= start(b) owns the block; its record gives the true entry
//           (bit, state) and output offset D_k + count.  The block is
//           decoded and its symbols written (the reference's phase 4,
//           src/multians_gpu_decoder.cu:492-573).
//  capture  (long streams, 2+ bits per symbol) k_gwalk and k_wwalk also
//           keep the symbols they decode, count c of Gamma_k at byte c of
//           region k's slice; k_copy then copies every block whose owner's
//           symbols are in a slice (Gamma_r's, or the owner's own) and lists
//           the warps that hold any other block for k_final_fb, the k_final
//           decode over those warps only.
//
// No pass waits on another thread: correctness needs only that every walk
// ends inside its slots, which the host checks and cures by re-planning.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "mans_device.cuh"
#include "mans_scan.cuh"
#include "mans_tma.cuh"
#include "mans_tune_table.h"
#include "multians_gb300.h"

namespace mans {

struct DecodeParams {
    const uint32_t* units;
    uint8_t* out;
    const uint32_t* table;      // reference-format table (L words)
    uint2* tab_sync;            // [L] prepared counting table
    uint2* tab_sym;             // [L] prepared symbol table
    uint2* rec_g;               // [nblk]       Gamma_region records
    uint2* rec_w;               // [nblk*dmax]  walk records, slot d-1 = Gamma_{r-d}
    unsigned long long* m;      // [nreg] merge bit position (~0 = none)
    long long* delta;           // [nreg]
    unsigned long long* Mpre;   // [nreg] prefix max of m
    long long* Dpre;            // [nreg] prefix sum of delta
    uint32_t* status;
    struct ScanTile* scan_tiles;   // [ntiles] look-back records
    struct WJob* walk_jobs;        // [nreg] merge-walk jobs
    uint32_t* scan_flags;          // [ntiles] look-back flags, then the tile ticket
    unsigned long long n_out;
    uint32_t n_units;
    uint32_t L;
    uint32_t first_idx;    // first_state - L
    uint32_t first_pos;    // 32 - first_bit
    uint32_t B;            // units per block
    uint32_t nb;           // blocks per region
    uint32_t dmax;         // walk slots
    uint32_t nblk;
    uint32_t nreg;
    uint32_t stage_cap;    // staging bytes per warp in k_final (multiple of 16)
    uint32_t wcap;         // blocks a merge walk may run inside the G pass
    uint32_t flags;        // MANS_DECODE_*
    uint8_t* cap;          // [nreg * cap_bytes + 16] captured symbols, by region
    uint32_t* cap_valid;   // [nreg] leading symbols of Gamma_k captured in slice k
    uint32_t cap_bytes;    // capture bytes per region (0: no capture)
    uint32_t* fb_list;     // [nblk / 32] warps the copy pass leaves to the decoding pass
    uint2* seed_ring;      // [kSeedSlots * 32 * kSeedRing] seeded-walk records (null: no seeds)
};

// Checks and converts the reference table, then builds both shared-memory
// tables (see mans_device.cuh).  One CTA.  Invalid entries (outside
// [L, 2L), or zero-bit entries that do not strictly decrease the state)
// become safe one-bit entries and set MANS_DEV_BAD_TABLE; a table whose
// every entry is a zero-bit self loop is a single-symbol table and sets
// MANS_DEV_DEGENERATE.  Zero-bit runs are folded by pointer doubling over
// the run-successor links (runs are strictly decreasing, so they end).
__device__ __forceinline__ void prep_body(const DecodeParams& p) {
    extern __shared__ uint32_t sm[];
    const uint32_t L = p.L;
    uint32_t* plain = sm;                        // base | k << 16 | sym << 24
    uint16_t* nxt0 = reinterpret_cast<uint16_t*>(sm + L);
    uint16_t* nxt1 = nxt0 + L;
    uint16_t* z0 = nxt1 + L;
    uint16_t* z1 = z0 + L;
    int bad_l = 0, loop_l = 1;
    for (uint32_t j = threadIdx.x; j < L; j += blockDim.x) {
        const uint32_t raw = __ldg(p.table + j);
        const uint32_t ns = raw & 0xffffu, sym = (raw >> 16) & 0xffu, k = raw >> 24;
        bool ok = false, sl = false;
        uint32_t base = 0;
        if (k <= kMaxBits) {
            const uint64_t lo = (uint64_t) ns << k, hi = (uint64_t) (ns + 1) << k;
            if (lo >= L && hi <= 2ull * L) {
                base = (uint32_t) (lo - L);
                ok = k > 0 || base < j;
                sl = k == 0 && base == j;
            }
        }
        uint32_t kk = k;
        if (!ok) { base = 0; kk = 1; }
        bad_l |= ok ? 0 : 1;
        loop_l &= sl ? 1 : 0;
        plain[j] = base | (kk << 16) | (sym << 24);
        nxt0[j] = (uint16_t) (kk == 0 ? base : j);
        z0[j] = (uint16_t) (kk == 0 ? 1 : 0);
    }
    const int any_bad = __syncthreads_or(bad_l);
    const int all_loop = __syncthreads_and(loop_l);
    if (threadIdx.x == 0 && any_bad)
        atomicOr(p.status, all_loop ? MANS_DEV_DEGENERATE : MANS_DEV_BAD_TABLE);
    // pointer doubling: nxt -> last state of the run, z -> run length
    uint16_t *na = nxt0, *nb = nxt1, *za = z0, *zb = z1;
    for (uint32_t span = 1; span < L; span <<= 1) {
        for (uint32_t j = threadIdx.x; j < L; j += blockDim.x) {
            const uint32_t t = na[j];
            nb[j] = na[t];
            const uint32_t zz = (uint32_t) za[j] + za[t];
            zb[j] = (uint16_t) min(zz, 0xffffu);
        }
        __syncthreads();
        uint16_t* tmp = na; na = nb; nb = tmp;
        tmp = za; za = zb; zb = tmp;
    }
    for (uint32_t j = threadIdx.x; j < L; j += blockDim.x) {
        const uint32_t e = plain[j];
        const uint32_t k = (e >> 16) & 31u;
        const uint32_t mask = (1u << k) - 1u;
        p.tab_sym[j] = make_uint2((e & 0xffffu) * 8u, mask | (k << 16) | (e & 0xff000000u));
        const uint32_t run = za[j];
        if (run + 1 <= kIncMax) {
            const uint32_t t = plain[na[j]];
            const uint32_t kt = (t >> 16) & 31u;
            p.tab_sync[j] = make_uint2((t & 0xffffu) * 8u,
                                       ((1u << kt) - 1u) | (kt << 16) | ((run + 1) << 24));
        } else {
            p.tab_sync[j] = make_uint2((e & 0xffffu) * 8u, mask | (k << 16) | (1u << 24));
        }
    }
}

__global__ void k_prep(DecodeParams p) { prep_body(p); }

__device__ __forceinline__ uint2 make_rec(uint32_t rel, uint32_t idx, uint32_t cnt) {
    return make_uint2(rel | (idx << 8), cnt);
}


// A merge walk the G pass did not finish, in the job list of the
// merge-walk pass (see k_wwalk).
struct WJob {          // stored as two uint4
    uint32_t k;       // region whose merge walk this is
    uint32_t b;       // block the cursors stand at (its start)
    uint32_t a_rec;   // Gamma_k's entry at block b: rel | idx << 8
    uint32_t ca;      // Gamma_k's count from region k's start (while A
                      // follows the region's trajectory: the offset to it)
    uint32_t g_rec;   // Gamma_{k+1}'s entry (replay cursor), ~0 = not started
    uint32_t cg;      // Gamma_{k+1}'s count from region k + 1's start (or offset)
    uint32_t flags;   // 1: A follows, 2: G follows the current region's trajectory
    uint32_t pad;
};
static_assert(sizeof(WJob) == 32, "job record layout");

// A merge walk still running: the G pass marks every walk it hands over,
// the walk pass publishes the result (delta first, then m, after a fence).
constexpr unsigned long long kMergePending = ~1ull;

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* a) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(a) : "memory");
    return v;
}

__device__ __forceinline__ void publish_merge(const DecodeParams& p, uint32_t k,
                                              unsigned long long m, long long delta) {
    p.delta[k] = delta;
    if (p.seed_ring) __threadfence();   // only seeded walks read other walks' results
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" :: "l"(p.m + k), "l"(m) : "memory");
}

// Sync stage, G pass (k_gwalk): every lane owns a ring of kRingSlots chunks
// of kChunk units in shared memory, filled by TMA bulk copies.  The warp
// works in rounds; in one round every lane advances its cursor to the next
// half-block boundary, so its unit loads advance at most
// kMaxBlockUnits / 2 + 3 = 11 units.  At the start of a round each lane
// releases its oldest chunk w once its cursor has loaded past unit
// 16(w+1) + kRelease and refills that slot with chunk w + 4; the cursor is
// then less than 11 units past that threshold, so rounds r and r + 1 read
// below unit 16(w+1) + 36 < 16(w+4), the start of the new chunk: a chunk
// copied in round r is first read in round r + 2, and round r waits only
// for the copies of round r - 2.  The small ring (272 bytes a lane) keeps
// 20 warps of walks resident per SM (16 with symbol capture, whose rings
// take shared memory too).
constexpr uint32_t kChunk = 16;                    // units per ring slot
constexpr uint32_t kRingSlots = 4;
constexpr uint32_t kRingUnits = kChunk * kRingSlots;
constexpr uint32_t kRingStride = kRingUnits * 4 + 16;   // bytes per lane: 68 words, 8 bank groups
constexpr uint32_t kRelease = 4;
constexpr uint32_t kSyncThreads = 128;      // batch launches; plain launches use
constexpr uint32_t kSyncThreadsMax = 256;   // 256 for L >= 4096 (one table per 8 warps)
constexpr uint32_t kMaxBlockUnits = 16;
constexpr uint32_t kMaxWalkSlots = 12;
constexpr uint32_t kMaxQueries = 1024;   // positions per mans_trajectory_query

__device__ __forceinline__ void ring_fill(uint32_t slot_addr, const uint32_t* __restrict__ in,
                                          uint32_t n, uint32_t chunk, uint32_t bar,
                                          uint32_t& bytes) {
    const uint32_t u = chunk * kChunk;
    if (u + kChunk <= n) {
        tma_load(slot_addr, in + u, kChunk * 4, bar);
        bytes = kChunk * 4;
    } else {
        for (uint32_t i = 0; i < kChunk; ++i)
            sts32(slot_addr + i * 4, u + i < n ? __ldg(in + u + i) : 0u);
        bytes = 0;
    }
}

// Symbol capture in the sync passes (DecodeParams::cap_bytes != 0).  A lane
// keeps the symbols of its trajectory in a ring of 32 words: its column of
// a warp-wide block of shared memory, row r at byte 128 r, so the 32 lanes
// of a warp store to 32 different banks whatever their counts.  Symbol c
// lies in byte c mod 4 of row (c / 4) mod 32.  Each step shifts the symbol
// into the register word of the last four symbols and stores that word to
// its row; the row holds the right bytes once its fourth symbol is in.
// Completed 16-byte groups go to the trajectory's slice of the capture
// buffer at the start of every round; a lane whose ring wrapped before a
// flush, or whose count passed the slice, stops capturing, and cap_valid
// records how many leading symbols of the slice are right.
constexpr uint32_t kCapRing = 128;                  // symbols a lane's ring holds
constexpr uint32_t kCapWarpBytes = kCapRing * 32;   // shared bytes per warp

struct CapLane {
    uint32_t col;    // shared address of the lane's word in row 0
    uint32_t acc;    // the last four symbols, newest in byte 3
    uint32_t done;   // leading symbols copied to the slice
    bool on;         // capture still complete
};

__device__ __forceinline__ uint32_t cap_row(uint32_t col, uint32_t c) {
    return col + ((c << 5) & 0xF80u);   // row (c / 4) mod 32
}

// Decodes trajectory A with capture until its cursor reaches relative bit
// `be`; cs is 32 x its count (bits 7..11: the ring row).  kAligned: the
// capture rows start on a 4 KB boundary, so a row address is the column OR
// the offset (one logic operation).
template <bool kAligned>
__device__ __forceinline__ uint32_t cap_run(SCursor& A, const UnitSrc& src, CapLane& cl,
                                            uint32_t cs, uint32_t be) {
    // unrolled by four (a test before every step): measured at 256 MiB
    // against no unrolling, 375-377 -> 378-380 GB/s at lambda = 0.05,
    // 234-236 -> 240-242 at lambda = 0.2 (G pass and walks both faster),
    // 422 -> 424 at lambda = 0.005; by two: in between
#pragma unroll 4
    while (A.pos < be) {
        cl.acc = __byte_perm(cl.acc, A.step(src), 0x7321);
        sts32(kAligned ? (cl.col | (cs & 0xF80u)) : cl.col + (cs & 0xF80u), cl.acc);
        cs += 32;
    }
    return cs;
}

// Largest code length k of the shared table's L entries (all threads of
// the CTA; a barrier per bit).
__device__ __forceinline__ uint32_t table_kmax(const uint2* s_tab, uint32_t L) {
    uint32_t km = 0;
    for (uint32_t j = threadIdx.x; j < L; j += blockDim.x) km = max(km, (s_tab[j].y >> 16) & 0xffu);
    uint32_t kmax = 0;
    for (uint32_t bit = 16; bit; bit >>= 1)
        if (__syncthreads_or(km >= kmax + bit)) kmax += bit;
    return kmax;
}

// Copies the completed groups of the first `count` symbols (all of them,
// the last group padded, when `final`) to dst, at most `limit` bytes
// (a multiple of 16).
__device__ __forceinline__ void cap_flush(CapLane& cl, uint8_t* __restrict__ dst,
                                          uint32_t count, uint32_t limit, bool final) {
    if (!cl.on) return;
    if (count - cl.done > kCapRing) {   // the ring wrapped before this flush
        cl.on = false;
        return;
    }
    if (final && (count & 3u)) sts32(cap_row(cl.col, count), cl.acc >> (8u * (4u - (count & 3u))));
    uint32_t upto = final ? (count + 15u) & ~15u : count & ~15u;
    upto = min(upto, limit);
    for (; cl.done + 16 <= upto; cl.done += 16) {
        const uint32_t a = cap_row(cl.col, cl.done);
        uint4 v;
        v.x = lds32(a);
        v.y = lds32(a + 128);
        v.z = lds32(a + 256);
        v.w = lds32(a + 384);
        *reinterpret_cast<uint4*>(dst + cl.done) = v;
    }
    if (count > limit) cl.on = false;   // the slice is full
}

// One lane per region k: decode Gamma_k over the region's blocks, record
// every block's entry (rec_g) and, for k + 1 < nreg, Gamma_k's entry at the
// first block of region k + 1 (walk slot 0 of that block).  Then the lane
// starts region k's merge walk in the same ring: region k + 1 belongs to
// the next lane, whose block records were written rounds earlier, so at
// every block start of region k + 1 the lane compares Gamma_k with
// Gamma_{k+1}'s record (read from L2, one block ahead).  A walk that has not
// merged after kWalkCapUnits units, and the walk of the warp's last lane
// (whose successor region belongs to another warp), go to the job list of
// the merge-walk pass (k_wwalk).  The cap trades the G pass's lane
// efficiency (a warp waits for its longest walk) against the merge-walk
// pass's load; measured at 256 MiB, 6 bits per symbol: 32 units 356 GB/s,
// 64 units 370, 128 units 363; measured again with the current passes, 48
// and 96 units against 64: 369-375 and 371-373 GB/s against 375-378, the
// G pass 0.365 and 0.387 ms against 0.373, the walks 0.188 and 0.167-0.169
// against 0.175.
constexpr uint32_t kWalkCapUnits = 64;
template <bool kCap>
__device__ __forceinline__ void gwalk_body(const DecodeParams& p, uint32_t rbase) {
    extern __shared__ __align__(16) uint2 s_tab[];
    // capture decodes symbol by symbol; otherwise zero-bit runs are folded
    load_prepared(s_tab, kCap ? p.tab_sym : p.tab_sync, p.L);
    // the uncaptured pass steps four at a time while the fourth step surely
    // starts before the half-block end (a step moves at most kmax bits)
    const uint32_t kgrp = kCap ? 0u : 3 * table_kmax(s_tab, p.L);
    if (*(volatile uint32_t*) p.status & (MANS_DEV_BAD_TABLE | MANS_DEV_DEGENERATE)) return;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t tb = smem_addr(s_tab);
    const uint32_t tab_bytes = (p.L * 8 + 15) & ~15u;
    const uint32_t ring = tb + tab_bytes + threadIdx.x * kRingStride;
    const uint32_t bars = tb + tab_bytes + blockDim.x * kRingStride + warp * 40;  // 5 mbarriers
    const uint32_t k = rbase + threadIdx.x;
    const uint32_t* __restrict__ in = p.units;
    const uint32_t n = p.n_units;
    const uint32_t Bbits = p.B * 32, Hbits = p.B * 16;
    const UnitSrc rs{ring, 0u, kRingUnits - 1, kRingUnits - 1};

    if ((rbase + (warp << 5)) >= p.nreg) return;   // whole warp idle
    if (lane == 0) {
        for (uint32_t i = 0; i < 5; ++i) mbar_init(bars + 8 * i, 1);
        fence_mbar_init();
    }
    __syncwarp();

    bool active = k < p.nreg;
    bool walking = false;   // merge walk (after the region's own blocks)
    const uint32_t b0 = min(k * p.nb, p.nblk);
    const uint32_t b1 = min(b0 + p.nb, p.nblk);
    const uint64_t origin = (uint64_t) b0 * Bbits;
    const uint64_t start = k == 0 ? (uint64_t) p.first_pos : origin;
    uint32_t w = (uint32_t) (start >> 5) / kChunk;   // oldest chunk held
    bool timed_out = false;

    // initial fill: chunks w .. w+3, completion on barrier 4
    {
        uint32_t mine = 0;
        if (active) {
            fence_proxy_async();
            for (uint32_t i = 0; i < kRingSlots; ++i) {
                uint32_t by;
                ring_fill(ring + ((w + i) & (kRingSlots - 1)) * kChunk * 4, in, n, w + i,
                          bars + 32, by);
                mine += by;
            }
        }
        const uint32_t total = __reduce_add_sync(0xffffffffu, mine);
        if (lane == 0) mbar_arrive_expect_tx(bars + 32, total);
        if (!mbar_wait(bars + 32, 0)) {
            timed_out = true;
            mbar_wait(bars + 32, 0);
        }
        __syncwarp();
    }

    // a unit load every step (one more shared wavefront) beats a refill
    // branch that some lane of the warp takes on most steps: the pass runs
    // near its issue limit as well as its shared-memory limit (measured:
    // capturing 0.430 -> 0.398 ms, uncaptured 0.345 -> 0.310 ms)
    SCursor A;
    uint32_t ca = 0;
    // the capture rows start on a 4 KB boundary, so a row address is the
    // lane's column OR the row offset (one logic operation per step)
    CapLane cl;
    cl.col = ((tb + tab_bytes + blockDim.x * kRingStride + (blockDim.x >> 5) * 40 + 4095) &
              ~4095u) + warp * kCapWarpBytes + lane * 4;
    cl.acc = 0;
    cl.done = 0;
    cl.on = kCap;
    uint8_t* const cdst = kCap ? p.cap + (size_t) k * p.cap_bytes : nullptr;
    uint32_t b = b0;        // block being decoded
    uint32_t bs = 0;        // relative start bit of the current half block
    uint32_t half = 0;      // 0: first half of block b, 1: second half
    uint32_t wend = 0;      // merge walk: last block start it may compare at
    uint2 rg = make_uint2(0, 0);       // Gamma_{k+1}'s record at block b
    uint2 rg_next = make_uint2(0, 0);  // ... at block b + 1 (loaded ahead)
    if (active) {
        A.init(rs, origin, start, tb + 8u * p.first_idx);
        p.rec_g[b0] = make_rec(A.pos, entry_index(A.a, tb), 0);
        if (b0 == b1) {
            active = false;
            if (kCap) p.cap_valid[k] = 0;
        }
    }

    const uint32_t ntile = (p.nreg + kScanTile - 1) / kScanTile;
    uint32_t r = 0;
    while (__any_sync(0xffffffffu, active)) {
        __syncwarp();   // orders the records of earlier rounds for the other lanes
        const bool was_active = active;
        if (kCap && active) cap_flush(cl, cdst, ca, p.cap_bytes, false);
        // refill: wait for round r-2's copies, then issue this round's
        if (r >= 2 && !mbar_wait(bars + 8 * ((r - 2) & 3), ((r - 2) >> 2) & 1)) {
            timed_out = true;
            mbar_wait(bars + 8 * ((r - 2) & 3), ((r - 2) >> 2) & 1);
        }
        uint32_t mine = 0;
        if (active && A.next >= (w + 1) * kChunk + kRelease) {
            fence_proxy_async();
            ring_fill(ring + (w & (kRingSlots - 1)) * kChunk * 4, in, n, w + kRingSlots,
                      bars + 8 * (r & 3), mine);
            ++w;
        }
        const uint32_t total = __reduce_add_sync(0xffffffffu, mine);
        if (lane == 0) mbar_arrive_expect_tx(bars + 8 * (r & 3), total);
        ++r;

        if (active && walking && half == 0) {
            // merge walk at the start of block b (inside region k + 1)
            const uint32_t ax = (A.pos - bs) | (entry_index(A.a, tb) << 8);
            if (ax == rg.x) {
                p.m[k] = (uint64_t) b * Bbits + (ax & 0xffu);
                p.delta[k] = (long long) ca - (long long) rg.y;
                active = false;
            } else if (b == wend) {
                p.m[k] = kMergePending;
                const uint32_t slot = atomicAdd(p.scan_flags + ntile + 1, 1u);
                uint4* dst = reinterpret_cast<uint4*>(p.walk_jobs + slot);
                dst[0] = make_uint4(k, b, ax, ca);
                dst[1] = make_uint4(~0u, 0u, 0u, 0u);
                active = false;
            } else if (b + 1 < p.nblk) {
                rg_next = __ldcg(p.rec_g + b + 1);   // written rounds ago
            }
        }
        if (active) {
            // decode to the end of the half block
            const uint32_t be = bs + Hbits;
            if (kCap) {
                ca = cap_run<true>(A, rs, cl, ca << 5, be) >> 5;
            } else {
                // measured at 256 MiB: 0.319 -> 0.314 ms (6 bits per symbol), L = 4096
                // at 1.5 bits per symbol 1.91 -> 1.82 ms
                while (A.pos + kgrp < be) {
                    const uint32_t y0 = A.step(rs), y1 = A.step(rs);
                    const uint32_t y2 = A.step(rs), y3 = A.step(rs);
                    ca += (y0 >> 24) + (y1 >> 24) + (y2 >> 24) + (y3 >> 24);
                }
                while (A.pos < be) ca += A.step(rs) >> 24;
            }
            bs = be;
            half ^= 1u;
            if (half == 0) {
                // block b done: record block b+1's entry
                ++b;
                const uint2 rec = make_rec(A.pos - bs, entry_index(A.a, tb), ca);
                if (walking) {
                    if (b >= p.nblk) {
                        p.m[k] = ~0ull;   // no merge before the stream end
                        p.delta[k] = 0;
                        active = false;
                    } else {
                        p.rec_w[(size_t) b * p.dmax] = rec;
                        rg = rg_next;
                    }
                } else if (b < b1) {
                    p.rec_g[b] = rec;
                } else if (k + 1 >= p.nreg) {
                    p.m[k] = ~0ull;   // the last region has no successor
                    p.delta[k] = 0;
                    active = false;
                } else {
                    p.rec_w[(size_t) b1 * p.dmax] = rec;
                    if (lane < 31) {
                        // the successor region is the next lane's: walk on here
                        walking = true;
                        wend = b1 + p.wcap;
                        rg = __ldcg(p.rec_g + b1);
                    } else {
                        p.m[k] = kMergePending;
                        const uint32_t slot = atomicAdd(p.scan_flags + ntile + 1, 1u);
                        uint4* dst = reinterpret_cast<uint4*>(p.walk_jobs + slot);
                        dst[0] = make_uint4(k, b1, rec.x, rec.y);
                        dst[1] = make_uint4(~0u, 0u, 0u, 0u);
                        active = false;
                    }
                }
            }
        }
        if (kCap && was_active && !active) {
            // the trajectory ends here (merged, at the stream end, or handed
            // to the merge-walk pass, which does not capture)
            cap_flush(cl, cdst, ca, p.cap_bytes, true);
            p.cap_valid[k] = cl.on ? ca : cl.done;
        }
    }
    // drain: no copy may still be writing this CTA's shared memory at exit
    for (uint32_t q = (r >= 2 ? r - 2 : 0); q < r; ++q) {
        if (!mbar_wait(bars + 8 * (q & 3), (q >> 2) & 1)) {
            timed_out = true;
            mbar_wait(bars + 8 * (q & 3), (q >> 2) & 1);
        }
    }
    if (timed_out) atomicOr(p.status, MANS_DEV_SCAN_TIMEOUT);
}

template <bool kCap>
__global__ void __launch_bounds__(kSyncThreadsMax) k_gwalk(DecodeParams p) {
    gwalk_body<kCap>(p, blockIdx.x * blockDim.x);
}

// Sync stage, merge walks (k_wwalk): region k's walk continues Gamma_k from
// where the G pass left it and stops at the first block start where it
// meets Gamma_{k+1}: inside region k + 1 Gamma_{k+1} is known from its block
// records (rec_g), so one cursor suffices; past region k + 1 a second
// cursor replays Gamma_{k+1} from its entry at region k + 2 (walk slot 0 of
// that block, written by region k + 1's G pass).
//
// The walks the G pass hands over (its job list) vary a lot in length, so
// warps take them one lane at a time: a warp works in rounds; at the start
// of a round every lane without a walk takes the next job (one atomic per
// warp), then each lane stages a window of kWindowUnits units (plus 4 of
// look-ahead) with one TMA copy and walks at most that window.  A lane's
// state between windows is its job record.  The grid is persistent (at most
// a few CTAs per SM); warps leave when the list is exhausted and their
// lanes are done.
//
// Past region k + 1 both trajectories are cursors (A = Gamma_k, G =
// Gamma_{k+1}), stepped interleaved.  A cursor that meets the current
// region's own trajectory Gamma_j at a block start stops being stepped: it
// equals Gamma_j from there on, so its entry at every later block of region
// j is rec_g's and its count is rec_g's plus a fixed offset; at the next
// region start it resumes from Gamma_j's entry there (walk slot 0, from the
// G pass).  Once both cursors follow Gamma_j their entries coincide, which
// is the merge.
// With capture, a walk that the G pass handed over while its capture was
// complete (cap_valid == its count) keeps capturing Gamma_k through region
// k + 1, where Gamma_k owns the blocks before its merge: in the lane's ring
// of capture words as in the G pass, flushed every half block, after the
// ring is primed with the partial group the G pass wrote.
constexpr uint32_t kWalkThreads = 64;
constexpr uint32_t kWalkCtasMax = 152 * 8;
constexpr uint32_t kWindowUnits = 128;   // 256 measured slower (fewer CTAs per SM)
constexpr uint32_t kWindowTile = (kWindowUnits + 4) * 4;     // bytes per lane
constexpr uint32_t kWindowStride = kWindowTile;   // 132 words: 8 bank groups, 16-byte aligned

// Seeded walks (the tail of the walk pass).  The walk pass lasts as long
// as its longest walk, a dependent chain of table lookups.  When a warp has
// one walk left and the job list is empty, its 31 idle lanes become seeds:
// trajectories decoded from a guessed state (the stream's first state, bit
// 0 of the block) at the blocks just ahead of the walker, each recording its
// entry and count at every block start in a ring.  Decodes that stand at the
// same bit in the same state are identical from there on, so when the
// walker's entry at block b equals a seed's record at b, the walker's
// trajectory is that seed's from b: the seed writes its records for the
// blocks after b as the walk's (counts shifted by the difference at b) and
// carries the walk on, from where it stands.  The farthest matching seed is
// taken; idle lanes are seeded again ahead of the others at window ends.
//
// The walk ends where its trajectory meets Gamma_{k+1}'s at a block start.
// Every lane looks Gamma_{k+1} up in memory: its G-pass records inside region
// k + 1, and past that the records of the walks that continue it (walk k + 1
// up to its merge, then Gamma_{k+2}, and so on, counts shifted by the deltas).
// A seed that meets Gamma_{k+1} stops there; a walker that takes such a seed
// ends the walk at the seed's stop.  A merge found later than the first one
// is still a block start where both trajectories agree (they stay equal), so
// m and delta are valid either way.
constexpr uint32_t kSeedSlots = 32;    // warps that may seed at once
constexpr uint32_t kSeedRing = 32;     // blocks of records a seed keeps
constexpr uint32_t kSeedMinWindows = 2;   // windows a walk runs in the walk pass first
constexpr uint32_t kBmUnknown = 0xfffffffeu;

// Where Gamma_{k+1} stands at block starts, read from memory.
struct NextLookup {
    uint32_t j;       // Gamma_{k+1} runs on Gamma_j here (with a count offset)
    uint32_t bm;      // block of walk j's merge (~0: none; kBmUnknown: not read yet)
    long long off;    // Gamma_{k+1}'s count - Gamma_j's count
};

// Gamma_{k+1}'s entry and count at block b (blocks asked in increasing order).
// 0: found; 1: a walk it depends on is still running; 2: not available.
__device__ __forceinline__ int next_lookup(const DecodeParams& p, NextLookup& L, uint32_t b,
                                           uint32_t& x, uint32_t& c) {
    const uint32_t r = b / p.nb;
    for (uint32_t it = 0; it < kMaxWalkSlots + 2; ++it) {
        if (r < L.j) return 2;
        if (r == L.j) {
            const uint2 e = __ldcg(p.rec_g + b);
            x = e.x;
            c = (uint32_t) ((long long) e.y + L.off);
            return 0;
        }
        if (L.bm == kBmUnknown) {
            const unsigned long long mj = ld_acquire_u64(p.m + L.j);
            if (mj == kMergePending) return 1;
            L.bm = mj == ~0ull ? ~0u : (uint32_t) (mj / (p.B * 32));
        }
        if (b <= L.bm) {
            const uint32_t d = r - L.j;
            if (d > p.dmax) return 2;
            const uint2 e = __ldcg(p.rec_w + (size_t) b * p.dmax + (d - 1));
            x = e.x;
            c = (uint32_t) ((long long) e.y + L.off);
            return 0;
        }
        L.off += __ldcg(p.delta + L.j);
        ++L.j;
        L.bm = kBmUnknown;
    }
    return 2;
}

// Stages units [u0, u0 + tile_units) of the lanes with `on` into their
// tiles and waits for the copies (phase `win` of the warp's barrier).
__device__ __forceinline__ void stage_window(const DecodeParams& p, bool on, uint32_t u0,
                                             uint32_t tile, uint32_t tile_units, uint32_t bar,
                                             uint32_t win, bool& timed_out) {
    const uint32_t n = p.n_units;
    const uint32_t avail = (on && u0 < n) ? min(tile_units, n - u0) : 0u;
    const uint32_t bulk = avail & ~3u;
    const uint32_t total = __reduce_add_sync(0xffffffffu, bulk * 4);
    if ((threadIdx.x & 31) == 0) mbar_arrive_expect_tx(bar, total);
    __syncwarp();
    if (bulk) {
        fence_proxy_async();
        tma_load(tile, p.units + u0, bulk * 4, bar);
    }
    if (on)
        for (uint32_t i = bulk; i < tile_units; ++i)
            sts32(tile + i * 4, i < avail ? __ldg(p.units + u0 + i) : 0u);
    if (!mbar_wait(bar, win & 1)) {
        timed_out = true;
        mbar_wait(bar, win & 1);
    }
    __syncwarp();
}


// Runs walk k (the walker lane wl stands at block jb with entry arec and
// count cnt) to its end with the warp's other lanes as seeds; ring: the
// lane's part of the warp's slot of seed records.  All lanes call it.  The
// memory every block start needs (Gamma_{k+1}'s entry there, and a seed's
// record at the walker's next block) is loaded one block ahead, while the
// lane decodes its current block.
// A call, not inlined: inlined it pushed the uncaptured walk loop into
// spills.
template <bool kCap>
__device__ __noinline__ void seeded_walk(const DecodeParams& p, uint32_t tb, uint32_t tile, uint32_t bar,
                            uint32_t& win, bool& timed_out, uint32_t wl, uint32_t k,
                            uint32_t jb, uint32_t arec, uint32_t cnt, uint2* __restrict__ ring) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t B = p.B, Bbits = p.B * 32, nwb = kWindowUnits / p.B;
    const uint32_t tile_units = kWindowUnits + 4;
    const uint32_t kgrp = kCap ? 0u : 3 * 16u;   // a step moves at most 16 bits
    // lane roles: 0 idle, 1 walker, 2 seed
    uint32_t role = lane == wl ? 1u : 0u;
    uint32_t pb = jb, st = jb;
    bool stopped = false;
    uint32_t sgc = 0;    // a stopped seed: Gamma_{k+1}'s count at its stop
    NextLookup L{k + 1, kBmUnknown, 0};
    // Gamma_{k+1} at this lane's block pb, looked up ahead (nrc: 0 found,
    // 1 pending, 2 unavailable, 3 not looked up yet)
    uint32_t ngx = 0, ngc = 0;
    int nrc = 3;
    // the record at the walker's block, loaded ahead (for block rwb)
    uint2 rw = make_uint2(0, 0);
    uint32_t rwb = ~0u;
    uint32_t cur_wl = wl;
    bool done = false;   // the walk has ended (warp-uniform)
    const uint32_t max_iter = (p.dmax + 2) * p.nb + 2 * kSeedRing;
    uint32_t iter = 0;
    for (;;) {
        // seed the idle lanes ahead of every active lane, within reach of the
        // walker's comparisons (kSeedRing blocks)
        {
            const uint32_t pbw = __shfl_sync(0xffffffffu, pb, cur_wl);
            const uint32_t front = __reduce_max_sync(0xffffffffu, role ? pb : 0u);
            const uint32_t idle = __ballot_sync(0xffffffffu, role == 0);
            if (role == 0) {
                const uint32_t rank = __popc(idle & ((1u << lane) - 1));
                const uint32_t nb0 = front + 1 + rank;
                if (nb0 < p.nblk && nb0 < pbw + kSeedRing &&
                    nb0 / p.nb <= k + p.dmax) {
                    role = 2;
                    st = pb = nb0;
                    arec = p.first_idx << 8;
                    cnt = 0;
                    stopped = false;
                    L = NextLookup{k + 1, kBmUnknown, 0};
                    nrc = 3;
                    rwb = ~0u;
                }
            }
        }
        const bool mov = role != 0 && !stopped;
        const uint32_t u0 = pb * B;
        stage_window(p, mov, u0, tile, tile_units, bar, win, timed_out);
        ++win;
        const UnitSrc src{tile, u0, ~0u, tile_units - 1};
        const uint64_t origin = (uint64_t) u0 * 32;
        SCursor A;
        if (mov) A.init(src, origin, origin + (arec & 0xffu), tb + 8u * min(arec >> 8, p.L - 1));
        uint32_t bs = 0;
        const bool moved = mov;   // this lane's cursor stands in this window's tile
        for (uint32_t i = 0; i < nwb; ++i, bs += Bbits) {
            bool fin = false;
            unsigned long long fm = 0;
            long long fd = 0;
            uint32_t ex = 0;
            const bool act = role != 0 && !stopped && moved;
            if (act) {
                ex = (A.pos - bs) | (entry_index(A.a, tb) << 8);
                const uint32_t d = pb / p.nb - k;
                if (pb >= p.nblk || d > p.dmax || d == 0) {
                    if (role == 1) {
                        if (pb < p.nblk) atomicOr(p.status, MANS_DEV_SYNC_OVERFLOW);
                        fin = true;
                        fm = ~0ull;
                    }
                    role = 0;
                } else {
                    uint32_t gx = ngx, gc = ngc;
                    int rc = nrc;
                    if (rc == 3) rc = next_lookup(p, L, pb, gx, gc);
                    if (role == 1) {
                        // the walker waits (bounded) for the walk it needs
                        for (uint32_t w = 0; rc == 1 && w < (1u << 20); ++w) {
                            __nanosleep(256);
                            rc = next_lookup(p, L, pb, gx, gc);
                        }
                        p.rec_w[(size_t) pb * p.dmax + (d - 1)] = make_uint2(ex, cnt);
                        if (rc != 0) {
                            atomicOr(p.status, MANS_DEV_SYNC_OVERFLOW);
                            fin = true;
                            fm = ~0ull;
                        } else if (ex == gx) {
                            fin = true;
                            fm = (uint64_t) pb * Bbits + (ex & 0xffu);
                            fd = (long long) cnt - (long long) gc;
                        }
                    } else {
                        ring[pb % kSeedRing] = make_uint2(ex, cnt);
                        if (rc == 0 && ex == gx) {   // a running walk: not checked here
                            stopped = true;
                            sgc = gc;
                        }
                    }
                }
            }
            // the walker's entry against the seeds' records at its block
            const uint32_t pbw = __shfl_sync(0xffffffffu, pb, cur_wl);
            const uint32_t exw = __shfl_sync(0xffffffffu, ex, cur_wl);
            const uint32_t cw = __shfl_sync(0xffffffffu, cnt, cur_wl);
            const bool wact = __shfl_sync(0xffffffffu, (int) act, cur_wl) != 0;
            const bool anyfin = __any_sync(0xffffffffu, fin);
            uint32_t key = 0;
            if (wact && !anyfin && role == 2 && (moved || stopped) && st <= pbw && pbw < pb &&
                pb - pbw < kSeedRing) {
                if (rwb != pbw) rw = ring[pbw % kSeedRing];
                if (rw.x == exw) key = pb + 1;
            }
            const uint32_t kmx = __reduce_max_sync(0xffffffffu, key);
            if (kmx) {
                const uint32_t ns = __ffs(__ballot_sync(0xffffffffu, key == kmx)) - 1;
                if (lane == ns) {
                    // the walk runs on this seed's trajectory from pbw on
                    const long long off = (long long) cw - (long long) rw.y;
                    for (uint32_t b = pbw + 1; b <= pb; ++b) {
                        const uint2 r = ring[b % kSeedRing];
                        p.rec_w[(size_t) b * p.dmax + (b / p.nb - k - 1)] =
                            make_uint2(r.x, (uint32_t) ((long long) r.y + off));
                    }
                    cnt = (uint32_t) ((long long) cnt + off);
                    if (stopped) {
                        fin = true;
                        fm = (uint64_t) pb * Bbits + (ring[pb % kSeedRing].x & 0xffu);
                        fd = (long long) cnt - (long long) sgc;
                        role = 0;
                    } else {
                        role = 1;
                    }
                } else if (lane == cur_wl || (role == 2 && pb <= kmx - 1)) {
                    role = 0;   // behind the new walker
                }
                cur_wl = ns;
            }
            if (__any_sync(0xffffffffu, fin)) {
                if (fin) publish_merge(p, k, fm, fd);
                done = true;
                break;
            }
            // look ahead: Gamma_{k+1} at this lane's next block, and the
            // record at the walker's next block
            const bool step = role != 0 && !stopped && moved;
            nrc = 3;
            if (step && pb + 1 < p.nblk) nrc = next_lookup(p, L, pb + 1, ngx, ngc);
            const uint32_t pbn = __shfl_sync(0xffffffffu, pb, cur_wl) + 1;
            rwb = ~0u;
            if (role == 2 && st <= pbn && pbn <= pb && pb - pbn < kSeedRing) {
                rw = ring[pbn % kSeedRing];
                rwb = pbn;
            }
            // every moving lane walks its block
            if (step) {
                const uint32_t be = bs + Bbits;
                if (kCap) {
                    while (A.pos < be) { A.step(src); ++cnt; }
                } else {
                    while (A.pos + kgrp < be) {
                        const uint32_t y0 = A.step(src), y1 = A.step(src);
                        const uint32_t y2 = A.step(src), y3 = A.step(src);
                        cnt += (y0 >> 24) + (y1 >> 24) + (y2 >> 24) + (y3 >> 24);
                    }
                    while (A.pos < be) cnt += A.step(src) >> 24;
                }
                ++pb;
            }
        }
        if (done) break;
        if (role != 0 && !stopped && moved) arec = (A.pos - bs) | (entry_index(A.a, tb) << 8);
        // a stopped seed behind the walker is of no more use
        const uint32_t pbw = __shfl_sync(0xffffffffu, pb, cur_wl);
        if (role == 2 && stopped && pb < pbw) role = 0;
        if (++iter > max_iter) {   // cannot happen for a walk within its slots
            if (lane == cur_wl) {
                atomicOr(p.status, MANS_DEV_SYNC_OVERFLOW);
                publish_merge(p, k, ~0ull, 0);
            }
            break;
        }
    }
}

template <bool kCap, bool kSeeds>
__device__ __forceinline__ void wwalk_body(const DecodeParams& p) {
    extern __shared__ __align__(16) uint2 s_tab[];
    const uint32_t ntile = (p.nreg + kScanTile - 1) / kScanTile;
    uint32_t* const job_next = p.scan_flags + ntile + 2;   // next job to take
    const uint32_t njobs = *(volatile uint32_t*) (p.scan_flags + ntile + 1);
    {   // nothing left: one thread decides for the CTA (other CTAs take jobs
        // meanwhile), which then leaves as a whole
        __shared__ uint32_t s_go;
        if (threadIdx.x == 0) s_go = njobs != 0 && *(volatile uint32_t*) job_next < njobs;
        __syncthreads();
        if (!s_go) return;
    }
    load_prepared(s_tab, kCap ? p.tab_sym : p.tab_sync, p.L);
    // the uncaptured walks step four at a time while the fourth step surely
    // starts before the block end (a lone long walk runs at the latency of
    // its dependent chain, where a loop test per step weighs most)
    const uint32_t kgrp = kCap ? 0u : 3 * table_kmax(s_tab, p.L);
    if (*(volatile uint32_t*) p.status & (MANS_DEV_BAD_TABLE | MANS_DEV_DEGENERATE)) return;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t tb = smem_addr(s_tab);
    const uint32_t tab_bytes = (p.L * 8 + 15) & ~15u;
    const uint32_t tile = tb + tab_bytes + threadIdx.x * kWindowStride;
    const uint32_t bar = tb + tab_bytes + blockDim.x * kWindowStride + warp * 8;
    const uint32_t* __restrict__ in = p.units;
    const uint32_t n = p.n_units;
    const uint32_t B = p.B, Bbits = p.B * 32, nwb = kWindowUnits / p.B;
    const uint32_t tile_units = kWindowUnits + 4;
    const WJob* lists = p.walk_jobs;
    constexpr uint32_t kAFollow = 1u, kGFollow = 2u;

    if (lane == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncwarp();

    bool open = false, exhausted = false;
    // job: region jk, block jb; A: entry a_rec, count ca (offset to Gamma_j's
    // count while following); G likewise (g_rec = ~0: not a cursor yet)
    uint32_t jk = 0, jb = 0, a_rec = 0, ca = 0, g_rec = ~0u, cg = 0, fl = 0;
    uint32_t wins = 0;   // windows walked on the current job
    bool timed_out = false;
    CapLane cl;
    cl.col = ((tb + tab_bytes + blockDim.x * kWindowStride + (blockDim.x >> 5) * 8 + 15) & ~15u) +
             warp * kCapWarpBytes + lane * 4;
    cl.acc = 0;
    cl.done = 0;
    cl.on = false;
    uint8_t* slice = nullptr;
    for (uint32_t win = 0;; ++win) {
        // lanes without a walk take the next jobs
        const uint32_t need = __ballot_sync(0xffffffffu, !open);
        if (need && !exhausted) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(job_next, __popc(need));
            base = __shfl_sync(0xffffffffu, base, 0);
            exhausted = base + __popc(need) >= njobs;
            if (!open) {
                const uint32_t jj = base + __popc(need & ((1u << lane) - 1));
                if (jj < njobs) {
                    const uint4* src = reinterpret_cast<const uint4*>(lists + jj);
                    const uint4 v0 = src[0], v1 = src[1];
                    jk = v0.x; jb = v0.y; a_rec = v0.z; ca = v0.w;
                    g_rec = v1.x; cg = v1.y; fl = v1.z;
                    open = true;
                    wins = 0;
                    if (kCap) {
                        // capture goes on where the G pass's was complete
                        slice = p.cap + (size_t) jk * p.cap_bytes;
                        cl.on = !(fl & kAFollow) && jb / p.nb == jk + 1 &&
                                __ldcg(p.cap_valid + jk) == ca;
                        if (cl.on) {
                            // the open group's bytes below ca, as the G pass wrote them
                            const uint32_t g0 = ca & ~15u;
                            const uint4 g = *reinterpret_cast<const uint4*>(slice + g0);
                            sts32(cap_row(cl.col, g0), g.x);
                            sts32(cap_row(cl.col, g0 + 4), g.y);
                            sts32(cap_row(cl.col, g0 + 8), g.z);
                            sts32(cap_row(cl.col, g0 + 12), g.w);
                            const uint32_t wi = (ca >> 2) & 3u, j = ca & 3u;
                            const uint32_t part = wi == 0 ? g.x : (wi == 1 ? g.y : (wi == 2 ? g.z : g.w));
                            cl.acc = j ? part << (8u * (4u - j)) : 0u;
                            cl.done = g0;
                        }
                    }
                }
            }
        }
        if (!__any_sync(0xffffffffu, open)) break;
        if (kSeeds && p.seed_ring && exhausted) {
            // one long walk left in this warp and no jobs: seed it
            const uint32_t om = __ballot_sync(0xffffffffu, open);
            const uint32_t wl = __ffs(om) - 1;
            if (__popc(om) == 1 && __shfl_sync(0xffffffffu, wins, wl) >= kSeedMinWindows) {
                uint32_t* const mask = p.scan_flags + ntile + 4;
                uint32_t slot = ~0u;
                if (lane == 0)
                    for (int t = 0; t < 4 && slot == ~0u; ++t) {
                        const uint32_t m = *(volatile uint32_t*) mask;
                        if (m == ~0u) break;
                        const uint32_t bit = __ffs(~m) - 1;
                        if (!(atomicOr(mask, 1u << bit) & (1u << bit))) slot = bit;
                    }
                slot = __shfl_sync(0xffffffffu, slot, 0);
                if (slot != ~0u) {
                    if (lane == wl) {
                        if (fl & kAFollow) {
                            // the walk stands on Gamma_j's trajectory: inside
                            // region j its G-pass record, at the next region's
                            // first block Gamma_j's walk record there
                            const uint2 r0 = (jb % p.nb == 0 && jb / p.nb >= jk + 2)
                                                 ? __ldcg(p.rec_w + (size_t) jb * p.dmax)
                                                 : __ldcg(p.rec_g + jb);
                            a_rec = r0.x;
                            ca += r0.y;
                        }
                        if (kCap && cl.on) {   // the seeded walk does not capture
                            cap_flush(cl, slice, ca, p.cap_bytes, true);
                            p.cap_valid[jk] = cl.on ? ca : cl.done;
                            cl.on = false;
                        }
                    }
                    seeded_walk<kCap>(p, tb, tile, bar, win, timed_out, wl,
                                      __shfl_sync(0xffffffffu, jk, wl), jb, a_rec, ca,
                                      p.seed_ring + ((size_t) slot * 32 + lane) * kSeedRing);
                    if (lane == 0) {
                        atomicAnd(mask, ~(1u << slot));
                        atomicAdd(p.scan_flags + ntile + 5, 1u);   // seeded walks (statistics)
                    }
                    open = false;
                    break;   // the warp's last walk has ended
                }
            }
        }
        // stage units [jb * B, jb * B + kWindowUnits + 4) of every open lane
        const uint32_t u0 = jb * B;
        const uint32_t avail = (open && u0 < n) ? min(tile_units, n - u0) : 0u;
        const uint32_t bulk = avail & ~3u;
        const uint32_t total = __reduce_add_sync(0xffffffffu, bulk * 4);
        if (lane == 0) mbar_arrive_expect_tx(bar, total);
        __syncwarp();
        if (bulk) {
            fence_proxy_async();
            tma_load(tile, in + u0, bulk * 4, bar);
        }
        if (open)
            for (uint32_t i = bulk; i < tile_units; ++i)
                sts32(tile + i * 4, i < avail ? __ldg(in + u0 + i) : 0u);
        // Gamma_j's record at the window's first block, while the copy lands
        uint2 rg = (open && jb < p.nblk) ? __ldcg(p.rec_g + jb) : make_uint2(0, 0);
        if (!mbar_wait(bar, win & 1)) {
            timed_out = true;
            mbar_wait(bar, win & 1);
        }
        __syncwarp();
        if (!open) continue;

        const UnitSrc src{tile, u0, ~0u, tile_units - 1};
        const uint64_t origin = (uint64_t) u0 * 32;
        SCursor A, G;
        if (!(fl & kAFollow))
            A.init(src, origin, origin + (a_rec & 0xffu), tb + 8u * min(a_rec >> 8, p.L - 1));
        if (g_rec != ~0u && !(fl & kGFollow))
            G.init(src, origin, origin + (g_rec & 0xffu), tb + 8u * min(g_rec >> 8, p.L - 1));
        uint32_t reg = jb / p.nb;                 // region of block jb
        uint32_t reg_end = (reg + 1) * p.nb;      // first block of the next region
        uint32_t bs = 0;
        for (uint32_t i = 0; i < nwb && open; ++i) {
            const uint32_t b = jb;
            const uint32_t d = reg - jk;
            if (d > p.dmax) {
                atomicOr(p.status, MANS_DEV_SYNC_OVERFLOW);
                publish_merge(p, jk, ~0ull, 0);
                open = false;
                break;
            }
            if (d >= 2 && b == reg * p.nb) {
                // region start: a following cursor resumes from Gamma_{j-1}'s
                // entry here; G starts here as Gamma_{k+1}'s entry
                const uint2 r1 = p.rec_w[(size_t) b * p.dmax];
                if (fl & kAFollow) {
                    A.init(src, origin, origin + bs + (r1.x & 0xffu), tb + 8u * min(r1.x >> 8, p.L - 1));
                    ca += r1.y;
                    fl &= ~kAFollow;
                }
                if (g_rec == ~0u || (fl & kGFollow)) {
                    G.init(src, origin, origin + bs + (r1.x & 0xffu), tb + 8u * min(r1.x >> 8, p.L - 1));
                    cg = g_rec == ~0u ? r1.y : cg + r1.y;
                    g_rec = 0;   // G is a cursor from here on
                    fl &= ~kGFollow;
                }
            }
            // entries and counts of both trajectories at block b
            const bool af = fl & kAFollow, gf = fl & kGFollow;
            const uint32_t ax = af ? rg.x : (A.pos - bs) | (entry_index(A.a, tb) << 8);
            const uint32_t cab = af ? rg.y + ca : ca;
            uint32_t gx, cgb;
            if (d == 1) {
                gx = rg.x;
                cgb = rg.y;
            } else {
                gx = gf ? rg.x : (G.pos - bs) | (entry_index(G.a, tb) << 8);
                cgb = gf ? rg.y + cg : cg;
            }
            p.rec_w[(size_t) b * p.dmax + (d - 1)] = make_uint2(ax, cab);
            if (ax == gx) {
                publish_merge(p, jk, (uint64_t) b * Bbits + (ax & 0xffu),
                              (long long) cab - (long long) cgb);
                open = false;
                break;
            }
            if (d >= 2) {
                // a cursor meeting Gamma_j follows it from here
                if (!af && ax == rg.x) { fl |= kAFollow; ca -= rg.y; }
                if (!gf && gx == rg.x) { fl |= kGFollow; cg -= rg.y; }
            }
            const uint2 rg_next = b + 1 < p.nblk ? __ldcg(p.rec_g + b + 1) : make_uint2(0, 0);
            // walk block b with the cursors that do not follow
            const uint32_t be = bs + Bbits;
            const bool sa = !(fl & kAFollow), sg = d >= 2 && !(fl & kGFollow);
            if (kCap) {
                // symbol table: one symbol per step; only A (at d == 1) captures
                if (sa && sg) {
                    while (A.pos < be && G.pos < be) {
                        A.step(src);
                        ++ca;
                        G.step(src);
                        ++cg;
                    }
                }
                if (sa && cl.on) {
                    // d == 1: capture, flushing at the half block and the block end
                    uint32_t cs = cap_run<false>(A, src, cl, ca << 5, bs + (Bbits >> 1));
                    cap_flush(cl, slice, cs >> 5, p.cap_bytes, false);
                    ca = cap_run<false>(A, src, cl, cs, be) >> 5;
                    cap_flush(cl, slice, ca, p.cap_bytes, false);
                    if (!cl.on) p.cap_valid[jk] = cl.done;   // the capture broke off
                }
                if (sa) while (A.pos < be) { A.step(src); ++ca; }
                if (sg) while (G.pos < be) { G.step(src); ++cg; }
            } else {
                // measured at 256 MiB, L = 4096, 1.5 bits per symbol: walks 2.92 -> 2.70 ms
                if (sa && sg) {
                    while (A.pos + kgrp < be && G.pos + kgrp < be) {
                        const uint32_t a0 = A.step(src), g0 = G.step(src), a1 = A.step(src),
                                       g1 = G.step(src), a2 = A.step(src), g2 = G.step(src),
                                       a3 = A.step(src), g3 = G.step(src);
                        ca += (a0 >> 24) + (a1 >> 24) + (a2 >> 24) + (a3 >> 24);
                        cg += (g0 >> 24) + (g1 >> 24) + (g2 >> 24) + (g3 >> 24);
                    }
                    while (A.pos < be && G.pos < be) {
                        ca += A.step(src) >> 24;
                        cg += G.step(src) >> 24;
                    }
                }
                if (sa) while (A.pos + kgrp < be) {
                    const uint32_t y0 = A.step(src), y1 = A.step(src);
                    const uint32_t y2 = A.step(src), y3 = A.step(src);
                    ca += (y0 >> 24) + (y1 >> 24) + (y2 >> 24) + (y3 >> 24);
                }
                if (sg) while (G.pos + kgrp < be) {
                    const uint32_t y0 = G.step(src), y1 = G.step(src);
                    const uint32_t y2 = G.step(src), y3 = G.step(src);
                    cg += (y0 >> 24) + (y1 >> 24) + (y2 >> 24) + (y3 >> 24);
                }
                if (sa) while (A.pos < be) ca += A.step(src) >> 24;
                if (sg) while (G.pos < be) cg += G.step(src) >> 24;
            }
            bs = be;
            jb = b + 1;
            rg = rg_next;
            if (jb == reg_end) { ++reg; reg_end += p.nb; }
            if (jb >= p.nblk) {
                publish_merge(p, jk, ~0ull, 0);   // no merge before the stream end
                open = false;
            }
            // the capture covers region k + 1 only
            if (kCap && cl.on && (!open || reg != jk + 1)) {
                cap_flush(cl, slice, ca, p.cap_bytes, true);
                p.cap_valid[jk] = cl.on ? ca : cl.done;
                cl.on = false;
            }
        }
        if (kCap && cl.on && !open) {   // merged, or out of slots
            cap_flush(cl, slice, ca, p.cap_bytes, true);
            p.cap_valid[jk] = cl.on ? ca : cl.done;
            cl.on = false;
        }
        if (open) {
            if (!(fl & kAFollow)) a_rec = (A.pos - bs) | (entry_index(A.a, tb) << 8);
            if (g_rec != ~0u && !(fl & kGFollow)) g_rec = (G.pos - bs) | (entry_index(G.a, tb) << 8);
            ++wins;
        }
    }
    __syncwarp();
    if (lane == 0) mbar_inval(bar);   // every phase completed: free for the next stream
    if (timed_out) atomicOr(p.status, MANS_DEV_SCAN_TIMEOUT);
}

template <bool kCap>
__global__ void __launch_bounds__(kWalkThreads) k_wwalk(DecodeParams p) { wwalk_body<kCap, true>(p); }

// Tiles are taken in launch order through an atomic ticket (the word after
// the flags), so a tile only waits on tiles that have already started.
__global__ void __launch_bounds__(kScanThreads) k_scan(DecodeParams p) {
    __shared__ uint32_t s_tile;
    if (threadIdx.x == 0) s_tile = atomicAdd(p.scan_flags + (p.nreg + kScanTile - 1) / kScanTile, 1u);
    __syncthreads();
    scan_body(p, s_tile);
}

__device__ __forceinline__ void sts8(uint32_t a, uint32_t v) {
    asm volatile("st.shared.u8 [%0], %1;" :: "r"(a), "r"(v) : "memory");
}

// Owner of block b: d = region(b) - k for the owning trajectory Gamma_k, its
// record at b and its output offset there.  Returns false when no
// trajectory owns the block (a walk ran out of slots).
__device__ __forceinline__ bool block_owner(const DecodeParams& p, uint32_t b, uint32_t& d,
                                            uint2& rec, unsigned long long& off) {
    const uint64_t bs = (uint64_t) b * p.B * 32;
    const uint32_t r = b / p.nb;
    for (d = 0;; ++d) {
        if (d > r || d > p.dmax) return false;
        if (p.Mpre[r - d] <= bs) break;
    }
    rec = d == 0 ? p.rec_g[b] : p.rec_w[(size_t) b * p.dmax + (d - 1)];
    off = (unsigned long long) (p.Dpre[r - d] + (long long) rec.y);
    return true;
}

// Entry (bit offset from the block start, state index) and global output
// offset of block b.
__device__ __forceinline__ bool block_entry(const DecodeParams& p, uint32_t b,
                                            uint32_t& rel, uint32_t& idx,
                                            unsigned long long& off) {
    uint32_t d;
    uint2 rec;
    if (!block_owner(p, b, d, rec, off)) return false;
    idx = min(rec.x >> 8, p.L - 1);   // records come from the sync stage; the clamp keeps
    rel = rec.x & 0xffu;              // table addresses in range regardless
    return true;
}

// Trajectory queries (mans_trajectory_query): for a bit position q, the
// decode's first codeword at or after q -- its bit position, its state and
// how many symbols come before it -- from the owner record of q's block and
// a short decode from the block's entry.  One thread per query, the table
// read from global memory: a query decodes less than one block.
struct QueryPoint {
    unsigned long long pos;
    uint32_t state;
    uint32_t found;
    unsigned long long count;
};

__global__ void k_query(DecodeParams p, const unsigned long long* __restrict__ q, uint32_t nq,
                        QueryPoint* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    QueryPoint r = {0, 0, 0, 0};
    const uint32_t st = *(volatile uint32_t*) p.status;
    if (!(st & (MANS_DEV_BAD_TABLE | MANS_DEV_DEGENERATE | MANS_DEV_SYNC_OVERFLOW |
                MANS_DEV_SCAN_TIMEOUT))) {
        const unsigned long long Bbits = (unsigned long long) p.B * 32;
        const unsigned long long qq = q[i];
        const uint32_t b = (uint32_t) min(qq / Bbits, (unsigned long long) p.nblk - 1);
        uint32_t d;
        uint2 rec;
        unsigned long long off;
        if (block_owner(p, b, d, rec, off)) {
            unsigned long long pos = b * Bbits + (rec.x & 0xffu);
            uint32_t j = min(rec.x >> 8, p.L - 1);
            unsigned long long cnt = off;
            // a block holds at most B * 32 + 17 bit positions, each with
            // fewer than L codewords: the bound keeps the loop finite
            const unsigned long long cap = (Bbits + 17) * p.L;
            for (unsigned long long s = 0; pos < qq && s < cap; ++s) {
                const uint2 t = p.tab_sym[j];
                const unsigned long long u = pos >> 5;
                const uint32_t w0 = u < p.n_units ? __ldg(p.units + u) : 0u;
                const uint32_t w1 = u + 1 < p.n_units ? __ldg(p.units + u + 1) : 0u;
                const uint32_t bits = __funnelshift_r(w0, w1, (uint32_t) (pos & 31u));
                j = min((t.x >> 3) + (bits & t.y & 0xffffu), p.L - 1);
                pos += (t.y >> 16) & 0xffu;
                ++cnt;
            }
            r.pos = pos;
            r.state = j + p.L;
            r.count = cnt;
            r.found = pos >= qq ? 1u : 0u;
        }
    }
    out[i] = r;
}

__device__ __forceinline__ void sts128(uint32_t a, uint4 v) {
    asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};"
                 :: "r"(a), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w) : "memory");
}

// Copies len captured bytes into the staging buffer: staging byte t0 + j
// gets cap[s0 + j], or with kRev cap[s0 + len - 1 - j].  Single bytes up to
// the first 16-byte staging boundary and after the last; in between every
// lane takes 16-byte chunks, four at a time (their 20 source words in
// flight together: the copy is bound by load latency otherwise), and
// assembles each from five aligned source words by funnel shifts.  Source
// words may extend up to 4 bytes past the range (inside the buffer's pad).
template <bool kRev>
__device__ __forceinline__ void stage_copy(uint32_t t0, const uint8_t* __restrict__ cap,
                                           unsigned long long s0, uint32_t len, uint32_t lane) {
    const uint32_t head = min(len, (16u - (t0 & 15u)) & 15u);
    const uint32_t nc = (len - head) >> 4;
    const uint32_t tail = (len - head) & 15u;
    if (lane < head + tail) {
        const uint32_t j = lane < head ? lane : head + nc * 16 + (lane - head);
        sts8(t0 + j, cap[kRev ? s0 + len - 1 - j : s0 + j]);
    }
    constexpr int kU = 4;
    for (uint32_t c0 = 0; c0 < nc; c0 += kU * 32) {
        uint32_t w[kU][5];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t c = c0 + u * 32 + lane;
            const uint32_t j = head + 16 * c;
            const unsigned long long e = kRev ? s0 + len - 16 - j : s0 + j;   // lowest source byte
            const uint32_t* q = reinterpret_cast<const uint32_t*>(cap + (e & ~3ull));
#pragma unroll
            for (int i = 0; i < 5; ++i) w[u][i] = c < nc ? __ldg(q + i) : 0u;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t c = c0 + u * 32 + lane;
            if (c < nc) {
                const uint32_t j = head + 16 * c;
                const unsigned long long e = kRev ? s0 + len - 16 - j : s0 + j;
                const uint32_t sh = (uint32_t) (e & 3u) * 8u;
                uint4 v;
                if (!kRev) {
                    v.x = __funnelshift_r(w[u][0], w[u][1], sh);
                    v.y = __funnelshift_r(w[u][1], w[u][2], sh);
                    v.z = __funnelshift_r(w[u][2], w[u][3], sh);
                    v.w = __funnelshift_r(w[u][3], w[u][4], sh);
                } else {
                    v.x = __byte_perm(__funnelshift_r(w[u][3], w[u][4], sh), 0, 0x0123);
                    v.y = __byte_perm(__funnelshift_r(w[u][2], w[u][3], sh), 0, 0x0123);
                    v.z = __byte_perm(__funnelshift_r(w[u][1], w[u][2], sh), 0, 0x0123);
                    v.w = __byte_perm(__funnelshift_r(w[u][0], w[u][1], sh), 0, 0x0123);
                }
                sts128(t0 + j, v);
            }
        }
    }
}

// One warp per 32 consecutive blocks, one lane per block.  The 32 blocks'
// symbols form one contiguous output range; lanes fill a shared staging
// buffer laid out with the same 16-byte phase as the output, then the warp
// writes the range with 16-byte stores (bytes at the unaligned ends).  A
// range larger than the staging buffer is written byte by byte instead.
//
// A block whose owning trajectory was captured by the sync passes is
// copied: its symbols are Gamma_r's (r = its region) when the owner's entry
// equals Gamma_r's record at the block, else the owner's own, and either
// slice holds them when cap_valid covers the block's count range.  Lanes
// whose blocks abut in both the capture and the output form segments that
// the warp copies together.  Every other block is decoded: its input (the
// block plus four units of look-ahead) arrives in shared memory by a TMA
// bulk copy into a lane-private tile (tiles kTileStride bytes apart, so
// lanes reading the same relative unit spread over eight bank groups), and
// the lane decodes exactly the block's symbol count, known from the scan,
// checking that it ended at the next block start.
constexpr uint32_t kFinalThreads = 256;   // eight warps share one table copy

// Shared-memory address of a final-pass warp's mbarrier.
__device__ __forceinline__ uint32_t final_bar(const DecodeParams& p, uint32_t tb, uint32_t warp) {
    const uint32_t tile_units = p.B + 4;
    const uint32_t tile_stride = tile_units * 4 + (((tile_units * 4) & 127) == 0 ? 16 : 0);
    const uint32_t per_warp = 32 * tile_stride + 16 + p.stage_cap + 16;
    const uint32_t tab_bytes = (p.L * 8 + 15) & ~15u;
    return tb + tab_bytes + warp * per_warp + 32 * tile_stride;
}

// CTA prologue of the final passes: the symbol table into shared memory;
// a single-symbol table fills the output (when `fill`).  Returns false when
// the CTA has nothing more to do.
__device__ __forceinline__ bool final_prologue(const DecodeParams& p, uint32_t cta,
                                               uint32_t nctas, bool fill) {
    extern __shared__ __align__(16) uint2 s_tab[];
    load_prepared(s_tab, p.tab_sym, p.L);
    const uint32_t st = *(volatile uint32_t*) p.status;
    if (st & MANS_DEV_DEGENERATE) {
        // single-symbol table: every state decodes that symbol
        if (!fill) return false;
        const uint8_t sym = (uint8_t) (__ldg(p.table) >> 16);
        const unsigned long long stride = (unsigned long long) nctas * blockDim.x;
        for (unsigned long long i = (unsigned long long) cta * blockDim.x + threadIdx.x;
             i < p.n_out; i += stride)
            p.out[i] = sym;
        return false;
    }
    return !(st & (MANS_DEV_BAD_TABLE | MANS_DEV_SYNC_OVERFLOW | MANS_DEV_SCAN_TIMEOUT));
}

// The final pass for the warp of blocks b0 .. b0 + 31 (its mbarrier
// initialised, expecting parity `phase`).  Returns false after an error
// (reported in the status word).
template <bool kRev>
__device__ __forceinline__ bool final_warp(const DecodeParams& p, uint32_t tb, uint32_t b0,
                                           uint32_t phase) {
    extern __shared__ __align__(16) uint2 s_tab[];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t tile_units = p.B + 4;                 // 16-byte multiple (B % 4 == 0)
    const uint32_t tile_stride = tile_units * 4 + (((tile_units * 4) & 127) == 0 ? 16 : 0);
    const uint32_t per_warp = 32 * tile_stride + 16 + p.stage_cap + 16;
    const uint32_t tab_bytes = (p.L * 8 + 15) & ~15u;
    const uint32_t wbase = tb + tab_bytes + warp * per_warp;
    const uint32_t tile = wbase + lane * tile_stride;
    const uint32_t bar = wbase + 32 * tile_stride;       // 16 bytes reserved
    const uint32_t stage_addr = bar + 16;

    const uint32_t b = b0 + lane;
    const bool have = b < p.nblk;

    uint32_t d = 0;
    uint2 rec = make_uint2(0, 0);
    unsigned long long off = 0;
    bool ok = have ? block_owner(p, b, d, rec, off) : true;
    // offset of block b + 1; the last block runs to the end of the output
    // (writes stop at n_out), which may lie before or after its start
    unsigned long long off_nx = max((unsigned long long) p.n_out, off);
    const unsigned long long from_next = __shfl_down_sync(0xffffffffu, off, 1);
    if (lane < 31 && b + 1 < p.nblk) off_nx = from_next;
    if (lane == 31 && b + 1 < p.nblk) {
        uint32_t tr, ti;
        ok &= block_entry(p, b + 1, tr, ti, off_nx);
    }
    __syncwarp();
    if (__any_sync(0xffffffffu, !ok)) {
        if (lane == 0) atomicOr(p.status, MANS_DEV_SYNC_OVERFLOW);
        return false;
    }
    const unsigned long long off0 = __shfl_sync(0xffffffffu, off, 0);
    const uint32_t last_lane = min(31u, p.nblk - 1 - b0);
    const unsigned long long off_end = __shfl_sync(0xffffffffu, off_nx, last_lane);
    const unsigned long long lo = min(off0, p.n_out);
    const unsigned long long hi = min(max(off_end, off0), p.n_out);
    // the warp writes output indices [wlo, whi): decode indices [lo, hi), or
    // in source order their mirror images n_out - 1 - i; the staging buffer
    // holds output index j at byte sb + (j - wlo), with the output's 16-byte
    // phase
    const unsigned long long wlo = kRev ? p.n_out - hi : lo;
    const unsigned long long whi = kRev ? p.n_out - lo : hi;
    const uint32_t sb = (uint32_t) (((uintptr_t) p.out + wlo) & 15u);
    const bool staged = whi - wlo + sb <= p.stage_cap;

    // every lane's range must lie inside the warp's range (offsets are
    // monotonic in the block index); anything else is reported, not written
    const bool lane_ok = !have || (off >= off0 && max(off_nx, off) <= max(off_end, off0));
    if (__any_sync(0xffffffffu, !lane_ok)) {
        if (lane == 0) atomicOr(p.status, MANS_DEV_COUNT_MISMATCH);
        return false;
    }
    // symbols of this block that land in [.., n_out)
    const unsigned long long end = min(max(off_nx, off), p.n_out);
    // a valid block holds at most (B * 32 + 17) bit positions, each with
    // fewer than L codewords: the cap keeps a corrupted offset from
    // running the loop (or its tile reads) away
    const unsigned long long cap_sym = (unsigned long long) (p.B * 32 + 17) * p.L;
    const uint32_t cnt = have && off < end ? (uint32_t) min(end - off, cap_sym) : 0u;

    // captured blocks: slice ck from count cy
    bool capd = false;
    unsigned long long csrc = 0;
    if (p.cap_bytes && staged && cnt) {
        const uint32_t r = b / p.nb;
        uint32_t ck = r - d, cy = rec.y;
        if (d > 0) {
            const uint2 g = __ldg(p.rec_g + b);
            if (g.x == rec.x) {   // the owner runs on Gamma_r's trajectory here
                ck = r;
                cy = g.y;
            }
        }
        capd = (unsigned long long) cy + cnt <= __ldg(p.cap_valid + ck);
        csrc = (unsigned long long) ck * p.cap_bytes + cy;
    }
    const bool dec = have && !capd;

    // stage the tiles of the lanes that decode
    const uint32_t* __restrict__ in = p.units;
    const uint32_t n = p.n_units;
    const uint32_t u0 = b * p.B;
    const uint32_t avail_units = (dec && u0 < n) ? min(tile_units, n - u0) : 0u;
    const uint32_t bulk_units = avail_units & ~3u;
    const uint32_t total = __reduce_add_sync(0xffffffffu, bulk_units * 4);
    if (lane == 0) mbar_arrive_expect_tx(bar, total);
    __syncwarp();
    if (bulk_units) {
        fence_proxy_async();
        tma_load(tile, in + u0, bulk_units * 4, bar);
    }
    if (dec)
        for (uint32_t i = bulk_units; i < tile_units; ++i)
            sts32(tile + i * 4, i < avail_units ? __ldg(in + u0 + i) : 0u);
    bool staged_in = mbar_wait(bar, phase);
    if (!staged_in) mbar_wait(bar, phase);   // never exit with the copy in flight
    __syncwarp();
    if (__any_sync(0xffffffffu, !staged_in)) {
        if (lane == 0) atomicOr(p.status, MANS_DEV_SCAN_TIMEOUT);
        return false;
    }

    if (dec) {
        const uint32_t pos_cap = p.B * 32 + kMaxBits + 1;
        const uint32_t full = off_nx >= off ? (uint32_t) min(off_nx - off, 0xffffffffull) : 0u;
        SCursor c;
        const UnitSrc ts{tile, u0, ~0u, tile_units - 1};
        const uint64_t bs = (uint64_t) b * p.B * 32;   // cursor units are global indices
        c.init(ts, bs, bs + (rec.x & 0xffu), tb + 8u * min(rec.x >> 8, p.L - 1));
        if (staged && !kRev) {
            // bytes up to a word boundary, then four symbols per 32-bit
            // store, then the remaining bytes
            uint32_t q = stage_addr + sb + (uint32_t) (off - wlo);
            uint32_t i = 0;
            for (; i < cnt && (q & 3u) && c.pos < pos_cap; ++i, ++q)
                sts8(q, c.step(ts) >> 24);
            for (; i + 4 <= cnt && c.pos < pos_cap; i += 4, q += 4) {
                const uint32_t y0 = c.step(ts), y1 = c.step(ts);
                const uint32_t y2 = c.step(ts), y3 = c.step(ts);
                const uint32_t lo2 = __byte_perm(y0, y1, 0x0073);   // sym0 | sym1 << 8
                const uint32_t hi2 = __byte_perm(y2, y3, 0x7300);   // sym2 << 16 | sym3 << 24
                sts32(q, __byte_perm(lo2, hi2, 0x7610));
            }
            for (; i < cnt && c.pos < pos_cap; ++i, ++q)
                sts8(q, c.step(ts) >> 24);
        } else if (staged) {
            // source order: decode index i goes to output n_out - 1 - i, so
            // the lane fills its staging bytes downwards, four symbols per
            // 32-bit store once the address is the top byte of a word
            uint32_t q = stage_addr + sb + (uint32_t) (p.n_out - 1 - off - wlo);
            uint32_t i = 0;
            for (; i < cnt && (q & 3u) != 3u && c.pos < pos_cap; ++i, --q)
                sts8(q, c.step(ts) >> 24);
            for (; i + 4 <= cnt && c.pos < pos_cap; i += 4, q -= 4) {
                const uint32_t y0 = c.step(ts), y1 = c.step(ts);
                const uint32_t y2 = c.step(ts), y3 = c.step(ts);
                const uint32_t lo2 = __byte_perm(y3, y2, 0x0073);   // sym3 | sym2 << 8
                const uint32_t hi2 = __byte_perm(y1, y0, 0x7300);   // sym1 << 16 | sym0 << 24
                sts32(q - 3, __byte_perm(lo2, hi2, 0x7610));
            }
            for (; i < cnt && c.pos < pos_cap; ++i, --q)
                sts8(q, c.step(ts) >> 24);
        } else if (!kRev) {
            uint8_t* dst = p.out + off;
            for (uint32_t i = 0; i < cnt && c.pos < pos_cap; ++i)
                dst[i] = (uint8_t) (c.step(ts) >> 24);
        } else {
            uint8_t* dst = p.out + (p.n_out - 1 - off);
            for (uint32_t i = 0; i < cnt && c.pos < pos_cap; ++i)
                *(dst - i) = (uint8_t) (c.step(ts) >> 24);
        }
        // a block decoded to its full count ends at the next block start
        if (cnt == full && b + 1 < p.nblk &&
            (c.pos < p.B * 32 || c.pos >= p.B * 32 + kMaxBits + 1))
            atomicOr(p.status, MANS_DEV_COUNT_MISMATCH);
    }
    if (!staged || wlo >= whi) return true;
    if (p.cap_bytes) {
        // captured segments: runs of lanes whose capture and output ranges abut
        __syncwarp();
        const unsigned long long s_end = csrc + cnt, o_end = off + cnt;
        const unsigned long long ps = __shfl_up_sync(0xffffffffu, s_end, 1);
        const unsigned long long po = __shfl_up_sync(0xffffffffu, o_end, 1);
        const int pc = __shfl_up_sync(0xffffffffu, (int) capd, 1);
        const bool cont = lane > 0 && capd && pc && ps == csrc && po == off;
        const uint32_t starts = __ballot_sync(0xffffffffu, capd && !cont);
        const uint32_t conts = __ballot_sync(0xffffffffu, cont);
        for (uint32_t rest = starts; rest; rest &= rest - 1) {
            const uint32_t s0 = __ffs(rest) - 1;
            const uint32_t after = ~conts & (0xfffffffeu << s0);   // lanes past s0 that start anew
            const uint32_t e = after ? __ffs(after) - 2 : 31u;     // last lane of the segment
            const unsigned long long src0 = __shfl_sync(0xffffffffu, csrc, s0);
            const unsigned long long o0 = __shfl_sync(0xffffffffu, off, s0);
            const unsigned long long o1 = __shfl_sync(0xffffffffu, o_end, e);
            const uint32_t t0 = stage_addr + sb + (uint32_t) (kRev ? p.n_out - o1 - wlo : o0 - wlo);
            stage_copy<kRev>(t0, p.cap, src0, (uint32_t) (o1 - o0), lane);
        }
    }
    __syncwarp();
    // [wlo, whi) from stage[sb + (j - wlo)]; aligned middle in 16 B words
    const uint8_t* stage = reinterpret_cast<const uint8_t*>(s_tab) + (stage_addr - tb);
    const uintptr_t base = (uintptr_t) p.out;
    unsigned long long a0 = wlo + ((16 - ((base + wlo) & 15)) & 15);
    unsigned long long a1 = whi - ((base + whi) & 15);
    if (a0 > a1) a0 = a1 = whi;
    for (unsigned long long i = wlo + lane; i < a0; i += 32)
        p.out[i] = stage[sb + (i - wlo)];
    for (unsigned long long i = a1 + lane; i < whi; i += 32)
        p.out[i] = stage[sb + (i - wlo)];
    const uint4* src = reinterpret_cast<const uint4*>(stage + sb + (a0 - wlo));
    uint4* dst = reinterpret_cast<uint4*>(p.out + a0);
    const uint32_t nvec = (uint32_t) ((a1 - a0) >> 4);
    for (uint32_t v = lane; v < nvec; v += 32) dst[v] = src[v];
    return true;
}

template <bool kRev>
__device__ __forceinline__ void final_body(const DecodeParams& p, uint32_t cta, uint32_t nctas) {
    extern __shared__ __align__(16) uint2 s_tab[];
    if (!final_prologue(p, cta, nctas, true)) return;
    const uint32_t tb = smem_addr(s_tab);
    const uint32_t warp = threadIdx.x >> 5;
    const uint32_t b0 = cta * blockDim.x + (warp << 5);
    if (b0 >= p.nblk) return;
    if ((threadIdx.x & 31) == 0) {
        mbar_init(final_bar(p, tb, warp), 1);
        fence_mbar_init();
    }
    final_warp<kRev>(p, tb, b0, 0);
}

// Final pass with capture, first kernel (k_copy): warps whose 32 blocks
// were all captured copy the symbols straight from the capture slices to
// the output; every other warp is listed for the decoding kernel
// (k_final_fb, the final pass above run over the listed warps).  No shared
// memory, so many warps per SM keep their loads in flight: a warp is a
// short chain of global loads (owners and records, issued together for
// walk depths up to 2, then the symbols) and 16-byte stores.
constexpr uint32_t kCopyThreads = 256;
constexpr uint32_t kCopyEarlyBlocks = 12;
static_assert(kCopyThreads == kFinalThreads, "batch items give both kernels the same CTA blocks");

struct CopyEntry {
    unsigned long long off;   // output offset of the block's first symbol
    unsigned long long src;   // capture byte of that symbol
    uint32_t cy;              // its count in the slice
    uint32_t valid;           // the slice's captured count
    bool ok;                  // owner at walk depth <= 2
};

__device__ __forceinline__ CopyEntry copy_entry(const DecodeParams& p, uint32_t b) {
    CopyEntry e;
    e.off = e.src = 0;
    e.cy = e.valid = 0;
    e.ok = false;
    const uint64_t bs = (uint64_t) b * p.B * 32;
    const uint32_t r = b / p.nb;
    const uint32_t r1 = r >= 1 ? r - 1 : r, r2 = r >= 2 ? r - 2 : r;
    const unsigned long long M0 = __ldg(p.Mpre + r), M1 = __ldg(p.Mpre + r1),
                             M2 = __ldg(p.Mpre + r2);
    const long long D0 = __ldg(p.Dpre + r), D1 = __ldg(p.Dpre + r1), D2 = __ldg(p.Dpre + r2);
    const uint32_t V0 = __ldg(p.cap_valid + r), V1 = __ldg(p.cap_valid + r1),
                   V2 = __ldg(p.cap_valid + r2);
    const uint2 g = __ldg(p.rec_g + b);
    // blocks near their region's start are mostly owned by the previous
    // region's walk: their walk record is loaded with the rest
    const bool early = b - r * p.nb < kCopyEarlyBlocks;
    const uint2 w1 = early ? __ldg(p.rec_w + (size_t) b * p.dmax) : make_uint2(0, 0);
    uint32_t d;
    if (M0 <= bs) d = 0;
    else if (r >= 1 && M1 <= bs) d = 1;
    else if (r >= 2 && p.dmax >= 2 && M2 <= bs) d = 2;
    else return e;   // a deeper owner (or none): left to the decoding kernel
    const uint2 rec = d == 0 ? g : ((d == 1 && early) ? w1 : __ldg(p.rec_w + (size_t) b * p.dmax + (d - 1)));
    e.off = (unsigned long long) ((d == 0 ? D0 : (d == 1 ? D1 : D2)) + (long long) rec.y);
    const bool own = d == 0 || rec.x == g.x;   // on Gamma_r's trajectory here
    e.cy = own ? g.y : rec.y;
    e.valid = own ? V0 : (d == 1 ? V1 : V2);
    e.src = (unsigned long long) (own ? r : r - d) * p.cap_bytes + e.cy;
    e.ok = true;
    return e;
}

// Decode indices [o0, o1) from cap[src0 ..] to the output (index i, or
// n_out - 1 - i with kRev): single bytes up to the first 16-byte output
// boundary and after the last, 16-byte stores in between, each assembled
// from five aligned source words (two chunks per lane in flight).
template <bool kRev>
__device__ __forceinline__ void out_copy(uint8_t* __restrict__ out, unsigned long long n_out,
                                         unsigned long long o0, unsigned long long o1,
                                         const uint8_t* __restrict__ cap,
                                         unsigned long long src0, uint32_t lane) {
    const unsigned long long y0 = kRev ? n_out - o1 : o0;
    const uint32_t len = (uint32_t) (o1 - o0);
    const uint32_t head = min(len, (uint32_t) ((16u - (((uintptr_t) out + y0) & 15u)) & 15u));
    const uint32_t nc = (len - head) >> 4;
    const uint32_t tail = (len - head) & 15u;
    if (lane < head + tail) {
        const uint32_t j = lane < head ? lane : head + nc * 16 + (lane - head);
        out[y0 + j] = cap[kRev ? src0 + len - 1 - j : src0 + j];
    }
    constexpr int kU = 2;   // measured: 4 chunks 0.141 ms, 2 and 1 0.138 (fewer registers)
    for (uint32_t c0 = 0; c0 < nc; c0 += kU * 32) {
        uint32_t w[kU][5];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t c = c0 + u * 32 + lane;
            const uint32_t j = head + 16 * c;
            const unsigned long long e = kRev ? src0 + len - 16 - j : src0 + j;
            const uint32_t* q = reinterpret_cast<const uint32_t*>(cap + (e & ~3ull));
#pragma unroll
            for (int i = 0; i < 5; ++i) w[u][i] = c < nc ? __ldg(q + i) : 0u;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t c = c0 + u * 32 + lane;
            if (c < nc) {
                const uint32_t j = head + 16 * c;
                const unsigned long long e = kRev ? src0 + len - 16 - j : src0 + j;
                const uint32_t sh = (uint32_t) (e & 3u) * 8u;
                uint4 v;
                if (!kRev) {
                    v.x = __funnelshift_r(w[u][0], w[u][1], sh);
                    v.y = __funnelshift_r(w[u][1], w[u][2], sh);
                    v.z = __funnelshift_r(w[u][2], w[u][3], sh);
                    v.w = __funnelshift_r(w[u][3], w[u][4], sh);
                } else {
                    v.x = __byte_perm(__funnelshift_r(w[u][3], w[u][4], sh), 0, 0x0123);
                    v.y = __byte_perm(__funnelshift_r(w[u][2], w[u][3], sh), 0, 0x0123);
                    v.z = __byte_perm(__funnelshift_r(w[u][1], w[u][2], sh), 0, 0x0123);
                    v.w = __byte_perm(__funnelshift_r(w[u][0], w[u][1], sh), 0, 0x0123);
                }
                __stcs(reinterpret_cast<uint4*>(out + y0 + j), v);
            }
        }
    }
}

// Staging bytes per warp of k_copy: a segment whose aligned source range
// (plus a word of read slack) fits is copied through shared memory.
constexpr uint32_t kCopyStage = 4096;

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" :: "r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// out_copy through the warp's staging buffer: the segment's 16-byte aligned
// source chunks are copied in with cp.async (all of them in flight at once,
// one DRAM round trip), then every lane assembles its 16-byte output chunks
// from five shared words, as out_copy does from global ones.
template <bool kRev>
__device__ __forceinline__ void out_copy_staged(uint8_t* __restrict__ out, unsigned long long n_out,
                                                unsigned long long o0, unsigned long long o1,
                                                const uint8_t* __restrict__ cap,
                                                unsigned long long src0, uint32_t lane,
                                                uint32_t stage) {
    const uint32_t len = (uint32_t) (o1 - o0);
    const unsigned long long s_lo = src0 & ~15ull;
    const uint32_t sh0 = (uint32_t) (src0 - s_lo);
    const uint32_t nsrc = (sh0 + len + 15) >> 4;
    for (uint32_t c = lane; c < nsrc; c += 32) cp_async16(stage + c * 16, cap + s_lo + c * 16);
    cp_async_wait_all();
    __syncwarp();
    const unsigned long long y0 = kRev ? n_out - o1 : o0;
    const uint32_t head = min(len, (uint32_t) ((16u - (((uintptr_t) out + y0) & 15u)) & 15u));
    const uint32_t nc = (len - head) >> 4;
    const uint32_t tail = (len - head) & 15u;
    if (lane < head + tail) {
        const uint32_t j = lane < head ? lane : head + nc * 16 + (lane - head);
        const uint32_t e = kRev ? sh0 + len - 1 - j : sh0 + j;
        out[y0 + j] = (uint8_t) (lds32(stage + (e & ~3u)) >> (8u * (e & 3u)));
    }
    for (uint32_t c = lane; c < nc; c += 32) {
        const uint32_t j = head + 16 * c;
        const uint32_t e = kRev ? sh0 + len - 16 - j : sh0 + j;
        const uint32_t q = stage + (e & ~3u), sh = (e & 3u) * 8u;
        const uint32_t w0 = lds32(q), w1 = lds32(q + 4), w2 = lds32(q + 8), w3 = lds32(q + 12),
                       w4 = lds32(q + 16);
        uint4 v;
        if (!kRev) {
            v.x = __funnelshift_r(w0, w1, sh);
            v.y = __funnelshift_r(w1, w2, sh);
            v.z = __funnelshift_r(w2, w3, sh);
            v.w = __funnelshift_r(w3, w4, sh);
        } else {
            v.x = __byte_perm(__funnelshift_r(w3, w4, sh), 0, 0x0123);
            v.y = __byte_perm(__funnelshift_r(w2, w3, sh), 0, 0x0123);
            v.z = __byte_perm(__funnelshift_r(w1, w2, sh), 0, 0x0123);
            v.w = __byte_perm(__funnelshift_r(w0, w1, sh), 0, 0x0123);
        }
        __stcs(reinterpret_cast<uint4*>(out + y0 + j), v);
    }
    __syncwarp();   // the buffer is refilled by the next segment
}

template <bool kRev>
__device__ __forceinline__ void copy_body(const DecodeParams& p, uint32_t cta, uint32_t nctas,
                                          uint32_t stage_base) {
    const uint32_t st = *(volatile uint32_t*) p.status;
    if (st & MANS_DEV_DEGENERATE) {
        const uint8_t sym = (uint8_t) (__ldg(p.table) >> 16);
        const unsigned long long stride = (unsigned long long) nctas * blockDim.x;
        for (unsigned long long i = (unsigned long long) cta * blockDim.x + threadIdx.x;
             i < p.n_out; i += stride)
            p.out[i] = sym;
        return;
    }
    if (st & (MANS_DEV_BAD_TABLE | MANS_DEV_SYNC_OVERFLOW | MANS_DEV_SCAN_TIMEOUT)) return;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t b0 = cta * blockDim.x + (threadIdx.x & ~31u);
    if (b0 >= p.nblk) return;
    const uint32_t b = b0 + lane;
    const bool have = b < p.nblk;
    CopyEntry e = have ? copy_entry(p, b) : CopyEntry{0, 0, 0, 0, true};
    // the next block's offset (lane 31: the first block of the next warp)
    CopyEntry en{0, 0, 0, 0, true};
    if (lane == 31 && b + 1 < p.nblk) en = copy_entry(p, b + 1);
    unsigned long long off_nx = max((unsigned long long) p.n_out, e.off);
    const unsigned long long from_next = __shfl_down_sync(0xffffffffu, e.off, 1);
    if (b + 1 < p.nblk) off_nx = lane < 31 ? from_next : en.off;
    const unsigned long long off0 = __shfl_sync(0xffffffffu, e.off, 0);
    const uint32_t last_lane = min(31u, p.nblk - 1 - b0);
    const unsigned long long off_end = __shfl_sync(0xffffffffu, off_nx, last_lane);
    const bool lane_ok = !have || (e.off >= off0 && max(off_nx, e.off) <= max(off_end, off0));
    const unsigned long long end = min(max(off_nx, e.off), p.n_out);
    const uint32_t cnt = have && e.off < end ? (uint32_t) min(end - e.off, 0xffffffffull) : 0u;
    const bool capd = cnt == 0 || (unsigned long long) e.cy + cnt <= e.valid;
    if (__any_sync(0xffffffffu, !e.ok || !en.ok || !lane_ok || !capd)) {
        if (lane == 0) {
            const uint32_t ntile = (p.nreg + kScanTile - 1) / kScanTile;
            p.fb_list[atomicAdd(p.scan_flags + ntile + 3, 1u)] = b0 >> 5;
        }
        return;
    }
    // runs of lanes whose capture and output ranges abut: one copy each
    const bool cp = cnt > 0;
    const unsigned long long s_end = e.src + cnt, o_end = e.off + cnt;
    const unsigned long long ps = __shfl_up_sync(0xffffffffu, s_end, 1);
    const unsigned long long po = __shfl_up_sync(0xffffffffu, o_end, 1);
    const int pc = __shfl_up_sync(0xffffffffu, (int) cp, 1);
    const bool cont = lane > 0 && cp && pc && ps == e.src && po == e.off;
    const uint32_t starts = __ballot_sync(0xffffffffu, cp && !cont);
    const uint32_t conts = __ballot_sync(0xffffffffu, cont);
    for (uint32_t rest = starts; rest; rest &= rest - 1) {
        const uint32_t s0 = __ffs(rest) - 1;
        const uint32_t after = ~conts & (0xfffffffeu << s0);
        const uint32_t last = after ? __ffs(after) - 2 : 31u;
        const unsigned long long src0 = __shfl_sync(0xffffffffu, e.src, s0);
        const unsigned long long o0 = __shfl_sync(0xffffffffu, e.off, s0);
        const unsigned long long o1 = __shfl_sync(0xffffffffu, o_end, last);
        // measured at 256 MiB, 6 bits per symbol: copy pass 0.138 -> 0.130 ms
        if ((src0 & 15ull) + (o1 - o0) + 32 <= kCopyStage) {
            out_copy_staged<kRev>(p.out, p.n_out, o0, o1, p.cap, src0, lane,
                                  stage_base + (threadIdx.x >> 5) * kCopyStage);
            continue;
        }
        out_copy<kRev>(p.out, p.n_out, o0, o1, p.cap, src0, lane);
    }
}

template <bool kRev>
__global__ void __launch_bounds__(kCopyThreads) k_copy(DecodeParams p) {
    __shared__ __align__(16) uint8_t s_stage[(kCopyThreads / 32) * kCopyStage];
    copy_body<kRev>(p, blockIdx.x, gridDim.x, smem_addr(s_stage));
}

// The decoding final pass over the warps k_copy listed (persistent grid).
template <bool kRev>
__device__ __forceinline__ void final_fb_body(const DecodeParams& p, uint32_t cta,
                                              uint32_t nctas) {
    extern __shared__ __align__(16) uint2 s_tab[];
    const uint32_t ntile = (p.nreg + kScanTile - 1) / kScanTile;
    const uint32_t count = *(volatile uint32_t*) (p.scan_flags + ntile + 3);
    const uint32_t wpc = blockDim.x >> 5;
    if (cta * wpc >= count) return;   // the whole CTA is idle
    if (!final_prologue(p, cta, nctas, false)) return;
    const uint32_t tb = smem_addr(s_tab);
    const uint32_t warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        mbar_init(final_bar(p, tb, warp), 1);
        fence_mbar_init();
    }
    __syncwarp();
    uint32_t phase = 0;
    for (uint32_t i = cta * wpc + warp; i < count; i += nctas * wpc) {
        if (!final_warp<kRev>(p, tb, p.fb_list[i] << 5, phase)) return;
        phase ^= 1u;
    }
}

template <bool kRev>
__global__ void __launch_bounds__(kFinalThreads) k_final_fb(DecodeParams p) {
    final_fb_body<kRev>(p, blockIdx.x, gridDim.x);
}

// Plain decodes run k_final with 256 threads, or 384 for L >= 4096 (one
// table per 12 warps: with a 32 KB table two CTAs fit an SM either way).
constexpr uint32_t kFinalThreadsWide = 384;

template <bool kRev>
__global__ void __launch_bounds__(kFinalThreadsWide) k_final(DecodeParams p) {
    // persistent: the table is loaded once per CTA, then every warp takes
    // every (grid x warps)-th group of 32 blocks
    extern __shared__ __align__(16) uint2 s_tab[];
    if (!final_prologue(p, blockIdx.x, gridDim.x, true)) return;
    const uint32_t tb = smem_addr(s_tab);
    const uint32_t warp = threadIdx.x >> 5, wpc = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        mbar_init(final_bar(p, tb, warp), 1);
        fence_mbar_init();
    }
    __syncwarp();
    const uint32_t ngroups = (p.nblk + 31) >> 5;
    uint32_t phase = 0;
    for (uint32_t g = blockIdx.x * wpc + warp; g < ngroups; g += gridDim.x * wpc) {
        if (!final_warp<kRev>(p, tb, g << 5, phase)) return;
        phase ^= 1u;
    }
}

// ---------------------------------------------------------------------------
// Batched launches: every CTA takes one work item {stream, first region /
// tile / CTA index} from a host-built list and the parameters of its stream
// from the stream table, so one launch of each kernel covers every stream
// of the batch.

struct BatchItem {
    uint32_t stream;
    uint32_t index;    // first region (sync), tile (scan) or CTA of the stream (final)
    uint32_t count;    // CTAs the stream has in this launch (final)
    uint32_t pad;
};

__device__ __forceinline__ void load_params(DecodeParams& dst, const DecodeParams* src) {
    static_assert(sizeof(DecodeParams) % 4 == 0, "word copy");
    const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
    uint32_t* d = reinterpret_cast<uint32_t*>(&dst);
    for (uint32_t i = threadIdx.x; i < sizeof(DecodeParams) / 4; i += blockDim.x) d[i] = s[i];
    __syncthreads();
}

__global__ void k_prep_batch(const DecodeParams* ps) {
    __shared__ DecodeParams sp;
    load_params(sp, ps + blockIdx.x);
    prep_body(sp);
}

__global__ void __launch_bounds__(kSyncThreads) k_gwalk_batch(const DecodeParams* ps,
                                                              const BatchItem* items) {
    __shared__ DecodeParams sp;
    const BatchItem it = items[blockIdx.x];
    load_params(sp, ps + it.stream);
    if (sp.cap_bytes) gwalk_body<true>(sp, it.index);
    else gwalk_body<false>(sp, it.index);
}

// Merge walks of a batch.  After the G pass k_walk_items appends, per
// stream, one item per 64 open walks (at most the stream's static share of
// CTAs) to one list; a persistent grid then takes items through a ticket,
// each CTA running the stream's walk pass (whose lanes take that stream's
// jobs until its list is exhausted).  A launch with one CTA per region
// group of every stream would run in waves, each as long as its longest
// walk.
__device__ __forceinline__ uint32_t walk_ctas_for(uint32_t nreg) {
    if (nreg < 2) return 0;
    return min((nreg - 1 + kWalkThreads - 1) / kWalkThreads, kWalkCtasMax);
}

__global__ void k_walk_items(const DecodeParams* ps, uint32_t n, uint32_t* list,
                             uint32_t* count) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const DecodeParams* p = ps + s;
    const uint32_t nreg = p->nreg;
    if (nreg < 2) return;   // inactive streams have nreg 0
    const uint32_t ntile = (nreg + kScanTile - 1) / kScanTile;
    const uint32_t jobs = *(volatile uint32_t*) (p->scan_flags + ntile + 1);
    const uint32_t want = min((jobs + kWalkThreads - 1) / kWalkThreads, walk_ctas_for(nreg));
    if (!want) return;
    const uint32_t at = atomicAdd(count, want);
    for (uint32_t i = 0; i < want; ++i) list[at + i] = s;
}

__global__ void __launch_bounds__(kWalkThreads) k_wwalk_batch(const DecodeParams* ps,
                                                              const uint32_t* list,
                                                              uint32_t* count) {
    __shared__ DecodeParams sp;
    __shared__ uint32_t s_item;
    const uint32_t total = *(volatile uint32_t*) count;   // written by k_walk_items
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(count + 1, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if (it >= total) return;
        load_params(sp, ps + list[it]);
        if (sp.cap_bytes) wwalk_body<true, false>(sp);
        else wwalk_body<false, false>(sp);
        __syncthreads();   // sp and s_item are rewritten next
    }
}

// The batch ticket hands out items in list order; the list holds each
// stream's tiles in increasing order, so a tile only waits on tiles of its
// own stream that have already started.
__global__ void __launch_bounds__(kScanThreads) k_scan_batch(const DecodeParams* ps,
                                                             const BatchItem* items,
                                                             uint32_t* ticket) {
    __shared__ DecodeParams sp;
    __shared__ uint32_t s_item;
    if (threadIdx.x == 0) s_item = atomicAdd(ticket, 1u);
    __syncthreads();
    const BatchItem it = items[s_item];
    load_params(sp, ps + it.stream);
    scan_body(sp, it.index);
}

// Final pass of a batch: streams with capture copy here first (k_copy_batch)
// and decode only their listed warps in k_final_batch; the others decode
// every block in k_final_batch.
__global__ void __launch_bounds__(kCopyThreads) k_copy_batch(const DecodeParams* ps,
                                                             const BatchItem* items) {
    __shared__ DecodeParams sp;
    const BatchItem it = items[blockIdx.x];
    load_params(sp, ps + it.stream);
    if (!sp.cap_bytes) return;
    __shared__ __align__(16) uint8_t s_stage[(kCopyThreads / 32) * kCopyStage];
    const uint32_t stage = smem_addr(s_stage);
    if (sp.flags & MANS_DECODE_SOURCE_ORDER) copy_body<true>(sp, it.index, it.count, stage);
    else copy_body<false>(sp, it.index, it.count, stage);
}

__global__ void __launch_bounds__(kFinalThreads) k_final_batch(const DecodeParams* ps,
                                                               const BatchItem* items) {
    __shared__ DecodeParams sp;
    const BatchItem it = items[blockIdx.x];
    load_params(sp, ps + it.stream);
    const bool rev = (sp.flags & MANS_DECODE_SOURCE_ORDER) != 0;
    if (sp.cap_bytes) {
        if (rev) final_fb_body<true>(sp, it.index, it.count);
        else final_fb_body<false>(sp, it.index, it.count);
    } else if (rev) {
        final_body<true>(sp, it.index, it.count);
    } else {
        final_body<false>(sp, it.index, it.count);
    }
}

// ---------------------------------------------------------------------------
// host side

struct AuxLayout {
    size_t rec_g, rec_w, m, delta, Mpre, Dpre, status, tab_sync, tab_sym, scan_tiles,
        scan_flags, walk_jobs, cap_valid, fb_list, cap, seed_ring, total;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t) 255; }

// CTAs of the merge-walk pass for a stream of nreg regions (persistent:
// warps take jobs until the list is exhausted).
static uint32_t walk_ctas(size_t nreg) {
    if (nreg < 2) return 0;
    return (uint32_t) std::min<size_t>((nreg - 1 + kWalkThreads - 1) / kWalkThreads, kWalkCtasMax);
}

// Blocks a merge walk may run inside the G pass before it goes to the
// merge-walk pass: at most kWalkCapUnits units and half a region (the warp
// waits for its longest walk, so the cap bounds that wait).
static uint32_t walk_cap(const mans_cfg& c) {
    const uint32_t cap = std::min<uint32_t>(kWalkCapUnits / c.block_units,
                                            std::max<uint32_t>(2, c.region_blocks / 2));
    return std::max<uint32_t>(1, std::min<uint32_t>(cap, c.region_blocks - 1));
}

// Shared memory of a G-pass CTA: table, lane rings, mbarriers and, with
// capture, the warps' capture rings (4 KB aligned: up to 4 KB of slack;
// two 256-thread CTAs at L = 1024 still fit an SM).
static size_t sync_smem(uint32_t L, uint32_t threads, bool capture) {
    return (((size_t) L * 8 + 15) & ~(size_t) 15) + (size_t) threads * kRingStride +
           (threads / 32) * 40 + (capture ? 4096 + (size_t) (threads / 32) * kCapWarpBytes : 0);
}

// Resident lanes of a capturing G pass with `threads`-thread CTAs: shared
// memory bounds it (228 KB per SM, 1 KB of it reserved per CTA).
static uint64_t capture_lanes(uint32_t L, uint32_t threads) {
    const uint64_t per_sm = std::min<uint64_t>(233472 / (sync_smem(L, threads, true) + 1024),
                                               2048 / threads);
    return 152ull * std::max<uint64_t>(per_sm, 1) * threads;
}

// CTA size of a capturing G pass over nreg regions: 128 threads (finer
// balance over the SMs) while their resident lanes hold the regions in one
// wave or outnumber those of 256-thread CTAs, else 256.
static uint32_t capture_threads(uint32_t L, size_t nreg) {
    const uint64_t small = capture_lanes(L, kSyncThreads);
    const uint64_t big = capture_lanes(L, kSyncThreadsMax);
    return (nreg <= small || small >= big) ? kSyncThreads : kSyncThreadsMax;
}

static size_t walk_smem(uint32_t L, bool capture) {
    return (((size_t) L * 8 + 15) & ~(size_t) 15) + (size_t) kWalkThreads * kWindowStride +
           (kWalkThreads / 32) * 8 + (capture ? 16 + (kWalkThreads / 32) * kCapWarpBytes : 0);
}

// Staging bytes per warp of the final pass: 1.25x the expected symbols of
// 32 blocks, 16 B rounded (a warp whose range does not fit writes it
// directly, byte by byte; 1.5x put the batched final pass at two CTAs per
// SM), and never more than lets `warps` warps and the table fit the final
// passes' shared-memory opt-in (long blocks at few bits per symbol would
// otherwise ask for more and the launch would be refused).
constexpr size_t kFinalSmemMax = 200 * 1024;
static uint32_t stage_cap_for(double per_unit, uint32_t B, uint32_t L, uint32_t warps) {
    uint64_t cap = (uint64_t) (per_unit * 32.0 * B * 1.25) + 128;
    cap = std::min<uint64_t>(std::max<uint64_t>(cap, 512), 16384);
    const size_t tab = ((size_t) L * 8 + 15) & ~(size_t) 15;
    const uint32_t tile_bytes = (B + 4) * 4;
    const uint32_t tile_stride = tile_bytes + ((tile_bytes & 127) == 0 ? 16 : 0);
    const size_t fixed = (size_t) 32 * tile_stride + 32;
    const size_t room = (kFinalSmemMax - tab) / std::max<uint32_t>(warps, 1);
    const uint64_t fit = room >= fixed + 16 ? ((room - fixed) & ~(size_t) 15) : 16;
    cap = std::min<uint64_t>(cap, fit);
    return (uint32_t) ((cap + 15) & ~(uint64_t) 15);
}

// Opts the kernels in to large dynamic shared memory, once per device.
static void set_kernel_attributes() {
    static std::mutex mu;
    static uint64_t done = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 64 && ((done >> dev) & 1)) return;
    cudaFuncSetAttribute(k_prep, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    cudaFuncSetAttribute(k_gwalk<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_gwalk<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_wwalk<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    cudaFuncSetAttribute(k_wwalk<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    cudaFuncSetAttribute(k_final<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFinalSmemMax);
    cudaFuncSetAttribute(k_final<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFinalSmemMax);
    cudaFuncSetAttribute(k_final_fb<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFinalSmemMax);
    cudaFuncSetAttribute(k_final_fb<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFinalSmemMax);
    cudaFuncSetAttribute(k_prep_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    cudaFuncSetAttribute(k_gwalk_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    cudaFuncSetAttribute(k_wwalk_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    cudaFuncSetAttribute(k_final_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, kFinalSmemMax);
    if (dev < 64) done |= 1ull << dev;
}

// seeds: room for the seeded walks' records (plain decodes; batches run
// without seeds)
static AuxLayout layout_for(size_t nblk, size_t nreg, size_t dmax, size_t cap_bytes,
                            bool seeds = true) {
    AuxLayout a;
    size_t o = 0;
    a.status = o; o += 256;
    a.tab_sync = o; o += (size_t) kMaxStates * 8;
    a.tab_sym = o; o += (size_t) kMaxStates * 8;
    a.rec_g = o; o += align256(nblk * sizeof(uint2));
    a.rec_w = o; o += align256(nblk * dmax * sizeof(uint2));
    a.m = o; o += align256(nreg * 8);
    a.delta = o; o += align256(nreg * 8);
    a.Mpre = o; o += align256(nreg * 8);
    a.Dpre = o; o += align256(nreg * 8);
    const size_t ntiles = (nreg + kScanTile - 1) / kScanTile;
    a.scan_tiles = o; o += align256(ntiles * sizeof(ScanTile));
    // flags, ticket, job count, next job, fallback warp count, seed slots,
    // seeded walks
    a.scan_flags = o; o += align256((ntiles + 6) * 4);
    a.walk_jobs = o; o += align256(nreg * sizeof(WJob));
    a.cap_valid = o; o += cap_bytes ? align256(nreg * 4) : 0;
    a.fb_list = o; o += cap_bytes ? align256((nblk + 31) / 32 * 4) : 0;
    a.cap = o; o += cap_bytes ? align256(nreg * cap_bytes + 16) : 0;
    a.seed_ring = o; o += seeds ? align256((size_t) kSeedSlots * 32 * kSeedRing * sizeof(uint2)) : 0;
    a.total = o;
    return a;
}

static uint32_t pow2_floor(uint64_t x) {
    uint32_t r = 1;
    while ((uint64_t) r * 2 <= x && r < (1u << 30)) r *= 2;
    return r;
}

static thread_local uint32_t g_last_launches = 0;

// Optional per-kernel timing: events recorded around each kernel of every
// decode into a ring of slots, summed by mans_timing_collect.
constexpr int kTimedKernels = 5;   // prep, gwalk, wwalk (3 passes), scan, final
struct TimingState {
    bool on = false;
    int cap = 0, used = 0;
    cudaEvent_t* ev = nullptr;     // cap * (kTimedKernels + 1)
};
static TimingState g_timing;

static void timing_mark(int slot_evt, cudaStream_t st) {
    if (!g_timing.on || g_timing.used >= g_timing.cap) return;
    cudaEventRecord(g_timing.ev[g_timing.used * (kTimedKernels + 1) + slot_evt], st);
}

// Blocks cover bit positions [0, 32 * n_units] inclusive: the first encoded
// symbols can be zero-bit codewords sitting exactly at the stream end
// (bit 32 * n_units), after the last bit the decoder consumes.  The
// reference stops at the last unit and leaves them unwritten (its output
// buffers are zero-filled, src/multicore_decoder.cc:176, and byte 0 is the
// most frequent symbol of its generator, so its round trip passes).
static size_t num_blocks(size_t n_units, size_t B) { return n_units / B + 1; }

}  // namespace mans

using namespace mans;

extern "C" {

const char* mans_version(void) { return "multians_gb300 0.1"; }

uint32_t mans_last_launch_count(void) { return g_last_launches; }

// Mean distance (units) after which a decode started from the guessed
// state meets the true one, measured on the generator's data (CPU
// simulation over 4 M symbols per point) at L = 1024 and L = 4096 for
// 0.67 .. 8.6 bits per symbol; interpolated linearly in bits per symbol and
// in log2(L), extrapolated in proportion to L outside that range.
static double mean_meeting_units(uint32_t L, double bits_per_symbol) {
    static const double kBps[6] = {0.67, 1.5, 2.5, 3.8, 6.0, 8.6};
    static const double kD1024[6] = {65, 143, 175, 153, 75, 28};
    static const double kD4096[6] = {278, 567, 700, 630, 324, 65};
    const double x = std::min(std::max(bits_per_symbol, kBps[0]), kBps[5]);
    int i = 0;
    while (i < 4 && x > kBps[i + 1]) ++i;
    const double t = (x - kBps[i]) / (kBps[i + 1] - kBps[i]);
    const double d1 = kD1024[i] + t * (kD1024[i + 1] - kD1024[i]);
    const double d4 = kD4096[i] + t * (kD4096[i + 1] - kD4096[i]);
    const double lg = std::log2((double) std::max<uint32_t>(L, 2));
    if (lg <= 10) return d1 * (double) L / 1024.0;
    if (lg >= 12) return d4 * (double) L / 4096.0;
    const double u = (lg - 10) / 2;
    return d1 + u * (d4 - d1);
}

// Symbol capture (MANS_DECODE_NO_CAPTURE): from this many bits per symbol
// on average zero-bit runs are rare, so the sync passes lose little by
// decoding symbol by symbol, and a half block holds few enough symbols for
// a lane's capture ring.  Capture costs the G pass a roughly fixed time
// (measured 0.05 ms: its rings take shared memory, so fewer warps per SM)
// and saves the final pass time in proportion to the output (0.8 us per
// MiB at 6 bits per symbol): from 16 M units on it pays.
constexpr double kCaptureMinBits = 2.0;
constexpr uint32_t kCaptureMaxL = 4096;   // larger tables leave too little shared memory
constexpr size_t kCaptureMinUnits = 16u << 20;
// Seeded walks from 1 to 4.5 bits per symbol, to 7 bits at L >= 4096
// (measured at 256 MiB, seeds on against off: L = 1024 at 3.8 bits per
// symbol +7.7 %, 1.5 bits +2.2 %; L = 4096 at 6.0 bits +3.2 %, 1.5 bits
// +6.5 %; at 8.6 and 0.67 bits, and 6.0 bits with L = 1024, 0.4-1.5 %
// slower: their walks are short, and the rest of their seeds fall on the
// next region's trajectory)
constexpr double kSeedMinBits = 1.0;
constexpr double kSeedMaxBits = 4.5;
constexpr double kSeedMaxBitsLarge = 7.0;   // L >= 4096

// The planner's choices a measured table entry overrides (see
// mans_tune_table.h): units per block, the shortest region in mean meeting
// distances, and symbol capture.
struct PlanKnobs {
    uint32_t block_units;
    double meet_mult;
    bool capture;
};

static int plan_core(size_t n_units, size_t n_out, uint32_t L, const mans_cfg* hint,
                     const PlanKnobs* kn, mans_cfg* out) {
    if (!out || n_units == 0 || L < 2 || L > kMaxStates) return MANS_ERR_ARG;
    mans_cfg c = {0, 0, 0, 0, 0, 0};
    if (hint) c = *hint;
    const double sym_per_unit = n_out ? (double) n_out / (double) n_units : 1.0;
    const double bps = 32.0 / std::max(sym_per_unit, 1e-3);
    const bool capture =
        !(c.flags & MANS_DECODE_NO_CAPTURE) &&
        (c.capture_bytes != 0 ||
         (kn ? (kn->capture && n_out > 0 && L <= kCaptureMaxL)
             : (n_out > 0 && L <= kCaptureMaxL && bps >= kCaptureMinBits &&
                (n_units >= kCaptureMinUnits || (c.flags & MANS_DECODE_CAPTURE)))));
    if (kn && c.block_units == 0) c.block_units = kn->block_units;
    if (!capture) c.capture_bytes = 0;
    if (c.block_units == 0) {
        // about 128 symbols per block
        uint64_t b = (uint64_t) (128.0 / std::max(sym_per_unit, 1e-3));
        c.block_units = std::min<uint32_t>(std::max<uint32_t>(pow2_floor(std::max<uint64_t>(b, 1)), 4), 256);
    }
    c.block_units = std::min<uint32_t>(std::max<uint32_t>(c.block_units & ~3u, 4), kMaxBlockUnits);
    // Sync walks: a walk runs from a region's end until its trajectory meets
    // the next region's guessed one, crossing up to walk_slots regions.  The
    // meeting distance grows with L (on the generator's data its mean is
    // about 0.08 L units and its tail passes 1.5 L units about once per
    // thousand regions), so slots are sized for R * (slots - 1) >= 4 L.  A
    // walk that still runs out is reported (MANS_DEV_SYNC_OVERFLOW) and
    // redone with longer regions.
    //
    // Region length R: one lane decodes a region, so R sets the parallelism
    // (about 78 k lanes, 16 warps on every SM, when the stream is long
    // enough) against the walk work (a walk per region, of the mean meeting
    // distance).  R is the length that gives that many regions, kept between
    // three mean meeting distances and 512 units (2048 for L > 1024; more
    // when three meeting distances are longer): measured over 0.67 .. 8.6
    // bits per symbol and L = 1024 / 4096, between about 2.5 and 4 meeting
    // distances is best.  With capture the lanes are those the capturing G
    // pass keeps resident (16 warps per SM at L = 1024, 12 at L = 2048, 8 at
    // L = 4096: the rings and the table fill shared memory), and R may grow to
    // 4096 units to keep them one wave.
    const uint64_t tail = std::max<uint64_t>(256, 4ull * L);
    const double meet = mean_meeting_units(L, bps);
    if (c.region_blocks == 0) {
        const uint64_t lanes =
            capture ? std::max(capture_lanes(L, kSyncThreads), capture_lanes(L, kSyncThreadsMax))
                    : 152ull * 16 * 32;
        const uint64_t r_sync = (uint64_t) ((kn ? kn->meet_mult : 3.0) * meet);
        const uint64_t r_max = std::max<uint64_t>(capture ? 4096 : (L <= 1024 ? 512 : 2048), r_sync);
        uint64_t R = (n_units + lanes - 1) / lanes;
        R = std::min<uint64_t>(std::max<uint64_t>(R, std::max<uint64_t>(r_sync, 64)), r_max);
        // an odd block count keeps lanes of a warp (one region each) off
        // power-of-two strides, which would pile them into the same L1 sets;
        // rounded up, so the regions never outnumber the lanes of one wave
        c.region_blocks =
            (uint32_t) std::max<uint64_t>(8, (R + c.block_units - 1) / c.block_units) | 1u;
    }
    if (c.walk_slots == 0) {
        const uint64_t R = (uint64_t) c.region_blocks * c.block_units;
        c.walk_slots = (uint32_t) std::min<uint64_t>(kMaxWalkSlots, std::max<uint64_t>(2, (tail + R - 1) / R + 1));
    }
    if (c.threads == 0) c.threads = 128;
    c.threads = std::min<uint32_t>(128, std::max<uint32_t>(32, c.threads & ~31u));
    if (capture && c.capture_bytes == 0) {
        // the region's symbols and those of the first stretch of its merge
        // walk, with a quarter to spare; blocks past the slice are decoded
        const double R = (double) c.region_blocks * c.block_units;
        const double walk = std::min(R, std::max((double) kWalkCapUnits, 3.0 * meet));
        const double bytes = sym_per_unit * (R + walk) * 1.25 + 64.0;
        c.capture_bytes = (uint32_t) std::min(bytes, (double) (1u << 30));
    }
    c.capture_bytes = (c.capture_bytes + 15) & ~15u;
    // a table plan without capture says so, so that the plan given back as
    // a hint (its geometry fixed) keeps deciding the same way
    if (kn && !capture) c.flags |= MANS_DECODE_NO_CAPTURE;
    // seeded walks where walks are long
    if (!(c.flags & (MANS_DECODE_SEEDS | MANS_DECODE_NO_SEEDS)) && bps >= kSeedMinBits &&
        bps < (L >= 4096 ? kSeedMaxBitsLarge : kSeedMaxBits))
        c.flags |= MANS_DECODE_SEEDS;
    *out = c;
    return MANS_OK;
}


// The measured table's entry for a decode of this size, table size and
// compression ratio: the same L (or, inside the table's range of L, the
// nearest power of two), the same size class (more or less than 32 MiB of
// symbols), and the nearest bits per symbol (by ratio).  False when the
// table has none.
static bool tune_lookup(uint32_t L, double bps, uint64_t n_out, TuneEntry* out) {
    const uint32_t large = n_out > (32ull << 20) ? 1u : 0u;
    uint32_t lo = ~0u, hi = 0;
    for (uint32_t i = 0; i < kTuneCount; ++i) {
        lo = std::min(lo, kTuneTable[i].L);
        hi = std::max(hi, kTuneTable[i].L);
    }
    if (kTuneCount == 0 || L < lo || L > hi) return false;
    const double lg = std::log2((double) L);
    double best = 1e300;
    bool found = false;
    for (uint32_t i = 0; i < kTuneCount; ++i) {
        const TuneEntry& t = kTuneTable[i];
        if (t.large != large) continue;
        const double dl = std::fabs(std::log2((double) t.L) - lg);
        const double db = std::fabs(std::log(std::max(bps, 1e-3) / (double) t.bps));
        const double d = dl * 100.0 + db;   // L first, then bits per symbol
        if (d < best) {
            best = d;
            *out = t;
            found = true;
        }
    }
    return found;
}

int mans_plan(size_t n_units, size_t n_out, uint32_t L, const mans_cfg* hint,
              mans_cfg* out) {
    if (!out || n_units == 0 || L < 2 || L > kMaxStates) return MANS_ERR_ARG;
    // the measured table applies when the caller fixes neither the geometry
    // nor the capture and does not ask for the model
    const bool free_plan =
        !hint || (hint->block_units == 0 && hint->region_blocks == 0 &&
                  hint->capture_bytes == 0 &&
                  !(hint->flags & (MANS_PLAN_MODEL | MANS_DECODE_NO_CAPTURE | MANS_DECODE_CAPTURE)));
    TuneEntry t;
    if (free_plan && n_out > 0 &&
        tune_lookup(L, 32.0 * (double) n_units / (double) n_out, n_out, &t)) {
        // capture as measured, from the length on where it pays at all
        // (the table's streams are 16 MiB and 256 MiB of symbols; shorter
        // streams of the large class stay below that length)
        const PlanKnobs kn = {t.block_units, (double) t.meet_mult,
                              t.capture != 0 && n_units >= kCaptureMinUnits};
        return plan_core(n_units, n_out, L, hint, &kn, out);
    }
    return plan_core(n_units, n_out, L, hint, nullptr, out);
}

int mans_plan_tuned(size_t n_units, size_t n_out, uint32_t L, uint32_t block_units,
                    double meet_mult, int capture, mans_cfg* out) {
    if (!out || n_units == 0 || L < 2 || L > kMaxStates || block_units < 4 ||
        block_units > kMaxBlockUnits || (block_units & 3) || !(meet_mult > 0.0) ||
        meet_mult > 64.0)
        return MANS_ERR_ARG;
    const PlanKnobs kn = {block_units, meet_mult, capture != 0};
    return plan_core(n_units, n_out, L, nullptr, &kn, out);
}

int mans_tune_lookup(uint32_t L, double bits_per_symbol, uint64_t n_out, mans_tune_entry* out) {
    if (!out) return MANS_ERR_ARG;
    TuneEntry t;
    if (!tune_lookup(L, bits_per_symbol, n_out, &t)) return 0;
    out->L = t.L;
    out->bits_per_symbol = t.bps;
    out->large = t.large;
    out->block_units = t.block_units;
    out->meet_mult = t.meet_mult;
    out->capture = t.capture;
    out->gbps = t.gbps;
    out->model_gbps = t.model_gbps;
    return 1;
}

size_t mans_aux_size(size_t n_units, const mans_cfg* cfg) {
    if (!cfg || cfg->block_units == 0 || cfg->region_blocks == 0 || cfg->walk_slots == 0)
        return 0;
    const size_t nblk = num_blocks(n_units, cfg->block_units);
    const size_t nreg = (nblk + cfg->region_blocks - 1) / cfg->region_blocks;
    return layout_for(nblk, nreg, cfg->walk_slots, cfg->capture_bytes).total;
}

size_t mans_aux_size_max(size_t n_units) {
    // smallest blocks (4 units), fewest blocks per region (8), most slots,
    // no capture (a decode whose plan captures into less memory than it
    // needs runs without)
    mans_cfg c = {4, 8, kMaxWalkSlots, 128, 0, 0};
    return mans_aux_size(n_units, &c);
}

size_t mans_aux_size_max_any(size_t n_units) {
    // symbol capture needs at least 2 bits per symbol (at most 16 symbols
    // per unit) and L <= 4096; the capture slices grow with the output, and
    // the region length the planner picks with it depends on L
    size_t best = mans_aux_size_max(n_units);
    static const double kSymPerUnit[] = {16, 14, 12, 10, 8, 6, 16.0 / 3, 4, 3.2, 8.0 / 3, 2};
    for (uint32_t L = 2; L <= kCaptureMaxL; L *= 2)
        for (double spu : kSymPerUnit) {
            mans_cfg plan;
            if (mans_plan(n_units, (size_t) (spu * (double) n_units), L, nullptr, &plan) == MANS_OK)
                best = std::max(best, mans_aux_size(n_units, &plan));
        }
    return best;
}

int mans_table_check(const uint32_t* t, uint32_t L) {
    if (!t || L < 2 || L > 32768) return -1;
    int loops = 0;
    for (uint32_t j = 0; j < L; ++j) {
        const uint32_t ns = t[j] & 0xffffu, k = t[j] >> 24;
        if (k > kMaxBits) return -1;
        const uint64_t lo = (uint64_t) ns << k, hi = (uint64_t) (ns + 1) << k;
        if (lo < L || hi > 2ull * L) return -1;
        if (k == 0 && lo - L >= j) {
            if (lo - L == j) ++loops;
            else return -1;
        }
    }
    if (loops == 0) return 0;
    return loops == (int) L ? 1 : -1;
}

// The plan a decode with these arguments runs with: the planner's, or the
// same without symbol capture when capture was the planner's choice and
// its slices do not fit the workspace (a workspace of mans_aux_size_max
// bytes always suffices then).
static int resolve_plan(size_t n_units, size_t n_out, uint32_t L, const mans_cfg* cfg_in,
                        size_t aux_bytes, mans_cfg* cfg) {
    int rc = mans_plan(n_units, n_out, L, cfg_in, cfg);
    if (rc != MANS_OK) return rc;
    if (cfg->capture_bytes && !(cfg_in && cfg_in->capture_bytes) &&
        mans_aux_size(n_units, cfg) > aux_bytes) {
        mans_cfg h = cfg_in ? *cfg_in : mans_cfg{0, 0, 0, 0, 0, 0};
        h.flags |= MANS_DECODE_NO_CAPTURE;
        h.capture_bytes = 0;
        rc = mans_plan(n_units, n_out, L, &h, cfg);
    }
    return rc;
}

// The arguments of a decode with output, checked before any CUDA call.
// first_bit: the reference's count of valid bits in unit 0 (the decode
// starts at bit 32 - first_bit), or with MANS_DECODE_START_OFFSET the start
// itself, a bit offset < 128 from the first unit's least significant bit.
static bool decode_args_ok(const uint32_t* d_units, size_t n_units, const uint8_t* d_out,
                           const uint32_t* d_table, uint32_t L, uint32_t first_state,
                           uint32_t first_bit, const void* d_aux, uint32_t flags = 0) {
    return d_units && ((uintptr_t) d_units & 15) == 0 &&   // TMA needs 16-byte alignment
           d_out && d_table && d_aux && n_units != 0 && n_units <= 0xffffffffull &&
           L >= 2 && L <= kMaxStates && first_state >= L && first_state < 2 * L &&
           first_bit <= ((flags & MANS_DECODE_START_OFFSET) ? 127u : 32u);
}

static uint32_t start_pos(uint32_t first_bit, uint32_t flags) {
    return (flags & MANS_DECODE_START_OFFSET) ? first_bit : 32 - first_bit;
}

// The decode's launch sequence; with sync_only the final pass is left out
// (d_out is not used) and the parameters the passes ran with go to *p_out.
static int decode_impl(const uint32_t* d_units, size_t n_units, uint8_t* d_out,
                       size_t n_out, const uint32_t* d_table, uint32_t L,
                       uint32_t first_state, uint32_t first_bit, void* d_aux,
                       size_t aux_bytes, const mans_cfg* cfg_in, void* stream, bool sync_only,
                       DecodeParams* p_out) {
    g_last_launches = 0;
    if (n_out == 0) return MANS_OK;
    const uint32_t in_flags = cfg_in ? cfg_in->flags : 0u;
    if (!decode_args_ok(d_units, n_units, sync_only ? (const uint8_t*) d_aux : d_out, d_table, L,
                        first_state, first_bit, d_aux, in_flags))
        return MANS_ERR_ARG;
    mans_cfg cfg;
    int rc = resolve_plan(n_units, n_out, L, cfg_in, aux_bytes, &cfg);
    if (rc != MANS_OK) return rc;
    const size_t nblk = num_blocks(n_units, cfg.block_units);
    const size_t nreg = (nblk + cfg.region_blocks - 1) / cfg.region_blocks;
    const AuxLayout lay = layout_for(nblk, nreg, cfg.walk_slots, cfg.capture_bytes);
    if (aux_bytes < lay.total) return MANS_ERR_AUX_SMALL;
    if ((uint64_t) nblk * cfg.block_units * 32 >= (1ull << 40)) return MANS_ERR_ARG;

    cudaStream_t st = (cudaStream_t) stream;
    char* base = (char*) d_aux;
    DecodeParams p;
    p.units = d_units;
    p.out = d_out;
    p.table = d_table;
    p.rec_g = (uint2*) (base + lay.rec_g);
    p.rec_w = (uint2*) (base + lay.rec_w);
    p.m = (unsigned long long*) (base + lay.m);
    p.delta = (long long*) (base + lay.delta);
    p.Mpre = (unsigned long long*) (base + lay.Mpre);
    p.Dpre = (long long*) (base + lay.Dpre);
    p.status = (uint32_t*) (base + lay.status);
    p.tab_sync = (uint2*) (base + lay.tab_sync);
    p.tab_sym = (uint2*) (base + lay.tab_sym);
    p.scan_tiles = (ScanTile*) (base + lay.scan_tiles);
    p.scan_flags = (uint32_t*) (base + lay.scan_flags);
    p.walk_jobs = (WJob*) (base + lay.walk_jobs);
    p.n_out = n_out;
    p.n_units = (uint32_t) n_units;
    p.L = L;
    p.first_idx = first_state - L;
    p.first_pos = start_pos(first_bit, in_flags);
    p.B = cfg.block_units;
    p.nb = cfg.region_blocks;
    p.dmax = cfg.walk_slots;
    p.nblk = (uint32_t) nblk;
    p.nreg = (uint32_t) nreg;
    p.wcap = walk_cap(cfg);
    p.flags = cfg.flags & MANS_DECODE_SOURCE_ORDER;
    p.cap_bytes = cfg.capture_bytes;
    p.cap = cfg.capture_bytes ? (uint8_t*) (base + lay.cap) : nullptr;
    p.cap_valid = cfg.capture_bytes ? (uint32_t*) (base + lay.cap_valid) : nullptr;
    p.fb_list = cfg.capture_bytes ? (uint32_t*) (base + lay.fb_list) : nullptr;
    p.seed_ring = (cfg.flags & MANS_DECODE_SEEDS) && !(cfg.flags & MANS_DECODE_NO_SEEDS)
                      ? (uint2*) (base + lay.seed_ring) : nullptr;
    const bool capture = cfg.capture_bytes != 0;

    const size_t ntiles = (nreg + kScanTile - 1) / kScanTile;
    if (cudaMemsetAsync(p.status, 0, sizeof(uint32_t), st) != cudaSuccess ||
        cudaMemsetAsync(base + lay.scan_flags, 0, (ntiles + 6) * 4, st) != cudaSuccess)
        return MANS_ERR_CUDA;
    const size_t smem = ((size_t) L * sizeof(uint2) + 15) & ~(size_t) 15;
    set_kernel_attributes();
    const uint32_t fthreads = L >= 4096 ? kFinalThreadsWide : kFinalThreads;
    p.stage_cap = stage_cap_for((double) n_out / (double) n_units, cfg.block_units, L,
                                std::max(fthreads, kFinalThreads) / 32);
    // G-pass CTAs: 256 threads share a table for L >= 4096; with capture as
    // capture_threads picks
    const uint32_t gthreads =
        capture ? capture_threads(L, nreg) : (L >= 4096 ? kSyncThreadsMax : kSyncThreads);
    const size_t smem_sync = sync_smem(L, gthreads, capture);
    const size_t smem_walk = walk_smem(L, capture);
    const uint32_t tile_bytes = (cfg.block_units + 4) * 4;
    const uint32_t tile_stride = tile_bytes + ((tile_bytes & 127) == 0 ? 16 : 0);
    const size_t per_warp_final = (size_t) 32 * tile_stride + 16 + p.stage_cap + 16;
    const size_t smem_final = smem + (size_t) (kFinalThreads / 32) * per_warp_final;
    const size_t smem_final_p = smem + (size_t) (fthreads / 32) * per_warp_final;
    timing_mark(0, st);
    k_prep<<<1, 1024, (size_t) L * 12, st>>>(p);
    timing_mark(1, st);
    const unsigned gg = (unsigned) ((nreg + gthreads - 1) / gthreads);
    if (capture) k_gwalk<true><<<gg, gthreads, smem_sync, st>>>(p);
    else k_gwalk<false><<<gg, gthreads, smem_sync, st>>>(p);
    timing_mark(2, st);
    uint32_t launches = 4;
    if (const uint32_t ww = walk_ctas(nreg)) {
        if (capture) k_wwalk<true><<<ww, kWalkThreads, smem_walk, st>>>(p);
        else k_wwalk<false><<<ww, kWalkThreads, smem_walk, st>>>(p);
        ++launches;
    }
    timing_mark(3, st);
    k_scan<<<(unsigned) ntiles, kScanThreads, 0, st>>>(p);
    timing_mark(4, st);
    if (sync_only) {
        if (p_out) *p_out = p;
        g_last_launches = launches;
        return cudaGetLastError() == cudaSuccess ? MANS_OK : MANS_ERR_CUDA;
    }
    const unsigned gf = (unsigned) ((nblk + kFinalThreads - 1) / kFinalThreads);
    const bool rev = (p.flags & MANS_DECODE_SOURCE_ORDER) != 0;
    if (capture) {
        // copy the captured warps, then decode the listed ones
        const unsigned gc = (unsigned) ((nblk + kCopyThreads - 1) / kCopyThreads);
        const unsigned gfb = std::min<unsigned>(gf, 152 * 3);
        if (rev) {
            k_copy<true><<<gc, kCopyThreads, 0, st>>>(p);
            k_final_fb<true><<<gfb, kFinalThreads, smem_final, st>>>(p);
        } else {
            k_copy<false><<<gc, kCopyThreads, 0, st>>>(p);
            k_final_fb<false><<<gfb, kFinalThreads, smem_final, st>>>(p);
        }
        ++launches;
    } else {
        // persistent final pass: as many CTAs as stay resident
        int per_sm = 0, sms = 152, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &per_sm, rev ? k_final<true> : k_final<false>, fthreads, smem_final_p) !=
                cudaSuccess || per_sm < 1)
            per_sm = 1;
        const unsigned need = (unsigned) ((nblk + fthreads - 1) / fthreads);
        const unsigned gp = std::min<unsigned>(need, (unsigned) (per_sm * std::max(sms, 1)));
        if (rev) k_final<true><<<gp, fthreads, smem_final_p, st>>>(p);
        else k_final<false><<<gp, fthreads, smem_final_p, st>>>(p);
    }
    timing_mark(5, st);
    if (g_timing.on && g_timing.used < g_timing.cap) ++g_timing.used;
    g_last_launches = launches;
    if (cudaGetLastError() != cudaSuccess) return MANS_ERR_CUDA;
    return MANS_OK;
}

int mans_decode(const uint32_t* d_units, size_t n_units, uint8_t* d_out,
                size_t n_out, const uint32_t* d_table, uint32_t L,
                uint32_t first_state, uint32_t first_bit, void* d_aux,
                size_t aux_bytes, const mans_cfg* cfg_in, void* stream) {
    return decode_impl(d_units, n_units, d_out, n_out, d_table, L, first_state, first_bit, d_aux,
                       aux_bytes, cfg_in, stream, false, nullptr);
}

// Query buffers after the sync workspace: positions, then results.
static size_t query_bytes(uint32_t nq) {
    return align256((size_t) nq * 8) + align256((size_t) nq * sizeof(QueryPoint));
}

static mans_cfg query_plan_hint() {
    mans_cfg h = {0, 0, 0, 0, MANS_DECODE_NO_CAPTURE | MANS_PLAN_MODEL, 0};
    return h;
}

size_t mans_trajectory_aux_size(size_t n_units, size_t n_out_hint, uint32_t L, uint32_t nq) {
    if (n_units == 0 || nq == 0 || nq > kMaxQueries) return 0;
    const size_t n_out = n_out_hint ? n_out_hint : n_units * 8;
    mans_cfg plan;
    const mans_cfg h = query_plan_hint();
    if (mans_plan(n_units, n_out, L, &h, &plan) != MANS_OK) return 0;
    // re-plans with longer regions need less; the largest of the first plan
    // and the worst case without capture
    return std::max(mans_aux_size(n_units, &plan), mans_aux_size_max(n_units)) + query_bytes(nq);
}

int mans_trajectory_query(const uint32_t* d_units, size_t n_units, const uint32_t* d_table,
                          uint32_t L, uint32_t first_state, uint32_t first_bit, uint32_t flags,
                          size_t n_out_hint, void* d_aux, size_t aux_bytes,
                          const uint64_t* h_pos, uint32_t nq, mans_point* h_out, void* stream,
                          uint32_t* dev_status) {
    if (dev_status) *dev_status = 0;
    if (!h_pos || !h_out || nq == 0 || nq > kMaxQueries || !d_aux ||
        aux_bytes < query_bytes(nq) + 256)
        return MANS_ERR_ARG;
    flags &= MANS_DECODE_START_OFFSET;
    if (!decode_args_ok(d_units, n_units, (const uint8_t*) d_aux, d_table, L, first_state,
                        first_bit, d_aux, flags))
        return MANS_ERR_ARG;
    const size_t n_out = n_out_hint ? n_out_hint : n_units * 8;
    // the sync workspace, then the query buffers (a multiple of 256 bytes)
    const size_t work_bytes = (aux_bytes - query_bytes(nq)) & ~(size_t) 255;
    char* qbase = (char*) d_aux + work_bytes;
    unsigned long long* d_q = (unsigned long long*) qbase;
    QueryPoint* d_r = (QueryPoint*) (qbase + align256((size_t) nq * 8));
    cudaStream_t st = (cudaStream_t) stream;
    mans_cfg c = query_plan_hint();
    c.flags |= flags;
    uint32_t status = 0;
    for (int attempt = 0; attempt < 8; ++attempt) {
        mans_cfg plan;
        int rc = mans_plan(n_units, n_out, L, &c, &plan);
        if (rc != MANS_OK) return rc;
        if (mans_aux_size(n_units, &plan) > work_bytes) {
            if (plan.walk_slots > 1) { c = plan; c.walk_slots = plan.walk_slots / 2; continue; }
            return MANS_ERR_AUX_SMALL;
        }
        DecodeParams p;
        rc = decode_impl(d_units, n_units, nullptr, n_out, d_table, L, first_state, first_bit,
                         d_aux, work_bytes, &plan, stream, true, &p);
        if (rc != MANS_OK) return rc;
        if (cudaMemcpyAsync(d_q, h_pos, (size_t) nq * 8, cudaMemcpyHostToDevice, st) !=
            cudaSuccess)
            return MANS_ERR_CUDA;
        k_query<<<(nq + 127) / 128, 128, 0, st>>>(p, d_q, nq, d_r);
        if (cudaGetLastError() != cudaSuccess) return MANS_ERR_CUDA;
        rc = mans_aux_status(d_aux, stream, &status);
        if (rc != MANS_OK) return rc;
        if (!(status & MANS_DEV_SYNC_OVERFLOW)) {
            std::vector<QueryPoint> r(nq);
            if (cudaMemcpy(r.data(), d_r, (size_t) nq * sizeof(QueryPoint),
                           cudaMemcpyDeviceToHost) != cudaSuccess)
                return MANS_ERR_CUDA;
            for (uint32_t i = 0; i < nq; ++i) {
                h_out[i].pos = r[i].pos;
                h_out[i].state = r[i].state;
                h_out[i].found = r[i].found;
                h_out[i].count = r[i].count;
            }
            break;
        }
        // a walk outran its slots: longer regions, as the synchronous decode
        c = plan;
        c.region_blocks = plan.region_blocks * 4;
        c.flags |= flags;
    }
    if (dev_status) *dev_status = status;
    if (status & MANS_DEV_DEGENERATE) return MANS_ERR_TABLE;
    return mans_status_code(status);
}

int mans_timing_enable(int max_decodes) {
    if (g_timing.ev) {
        for (int i = 0; i < g_timing.cap * (kTimedKernels + 1); ++i) cudaEventDestroy(g_timing.ev[i]);
        delete[] g_timing.ev;
        g_timing.ev = nullptr;
    }
    g_timing.on = max_decodes > 0;
    g_timing.cap = max_decodes > 0 ? max_decodes : 0;
    g_timing.used = 0;
    if (!g_timing.on) return MANS_OK;
    g_timing.ev = new cudaEvent_t[(size_t) g_timing.cap * (kTimedKernels + 1)];
    for (int i = 0; i < g_timing.cap * (kTimedKernels + 1); ++i)
        if (cudaEventCreate(&g_timing.ev[i]) != cudaSuccess) return MANS_ERR_CUDA;
    return MANS_OK;
}

int mans_timing_collect(float* ms_per_kernel, int n_kernels, int* n_decodes) {
    if (!ms_per_kernel || n_kernels < kTimedKernels) return MANS_ERR_ARG;
    for (int k = 0; k < n_kernels; ++k) ms_per_kernel[k] = 0.f;
    for (int d = 0; d < g_timing.used; ++d) {
        cudaEvent_t* e = g_timing.ev + d * (kTimedKernels + 1);
        if (cudaEventSynchronize(e[kTimedKernels]) != cudaSuccess) return MANS_ERR_CUDA;
        for (int k = 0; k < kTimedKernels; ++k) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, e[k], e[k + 1]) != cudaSuccess) return MANS_ERR_CUDA;
            ms_per_kernel[k] += ms;
        }
    }
    if (n_decodes) *n_decodes = g_timing.used;
    g_timing.used = 0;
    return MANS_OK;
}

int mans_aux_status(const void* d_aux, void* stream, uint32_t* status_out) {
    if (!d_aux || !status_out) return MANS_ERR_ARG;
    uint32_t v = 0;
    cudaStream_t st = (cudaStream_t) stream;
    if (cudaMemcpyAsync(&v, d_aux, sizeof(v), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return MANS_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MANS_ERR_CUDA;
    *status_out = v;
    return MANS_OK;
}

int mans_sync_stats_get(const void* d_aux, size_t aux_bytes, size_t n_units, size_t n_out,
                        uint32_t L, const mans_cfg* cfg_in, void* stream,
                        mans_sync_stats* out) {
    if (!d_aux || !out || n_units == 0 || n_units > 0xffffffffull || n_out == 0 || L < 2 ||
        L > kMaxStates)
        return MANS_ERR_ARG;
    mans_cfg cfg;
    int rc = resolve_plan(n_units, n_out, L, cfg_in, aux_bytes, &cfg);
    if (rc != MANS_OK) return rc;
    const size_t nblk = num_blocks(n_units, cfg.block_units);
    const size_t nreg = (nblk + cfg.region_blocks - 1) / cfg.region_blocks;
    const AuxLayout lay = layout_for(nblk, nreg, cfg.walk_slots, cfg.capture_bytes);
    if (aux_bytes < lay.total) return MANS_ERR_AUX_SMALL;
    const size_t ntiles = (nreg + kScanTile - 1) / kScanTile;
    // the merge point of every region and the counters behind the scan
    // flags (flags, ticket, job count, next job, fallback warp count): all
    // inside the workspace whose size was checked above
    std::vector<unsigned long long> m(nreg);
    uint32_t cnt[6] = {0, 0, 0, 0, 0, 0};
    cudaStream_t st = (cudaStream_t) stream;
    const char* base = (const char*) d_aux;
    if (cudaMemcpyAsync(m.data(), base + lay.m, nreg * 8, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(cnt, base + lay.scan_flags + ntiles * 4, sizeof(cnt),
                        cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return MANS_ERR_CUDA;
    const uint64_t bbits = (uint64_t) cfg.block_units * 32;
    const uint64_t rbits = bbits * cfg.region_blocks;
    const uint64_t end_bit = (uint64_t) n_units * 32;
    mans_sync_stats s{};
    s.regions = nreg;
    s.blocks = nblk;
    s.walks = nreg > 0 ? nreg - 1 : 0;
    s.open_walks = cnt[1];
    s.fallback_warps = cfg.capture_bytes ? cnt[3] : 0;
    s.seeded_walks = cnt[5];
    uint64_t walk_bits = 0;
    for (size_t k = 0; k + 1 < nreg; ++k) {
        // region k's walk starts at the first bit of region k + 1 and ends
        // at the merge point (or at the stream end when it never merged)
        const uint64_t start = (uint64_t) (k + 1) * rbits;
        uint64_t stop = m[k];
        if (stop == ~0ull) {
            ++s.unmerged;
            stop = std::max(start, end_bit);
        }
        const uint64_t bits = stop > start ? stop - start : 0;
        walk_bits += bits;
        s.walk_max_units = std::max<uint64_t>(s.walk_max_units, (bits + 31) / 32);
        s.walk_blocks += (bits + bbits - 1) / bbits;
    }
    s.walk_units = (walk_bits + 31) / 32;
    s.metadata_bytes = nblk * sizeof(uint2) + s.walk_blocks * sizeof(uint2) + nreg * 4 * 8 +
                       s.open_walks * sizeof(WJob);
    *out = s;
    return MANS_OK;
}

int mans_aux_alloc(size_t n_units, size_t n_out, uint32_t L, const mans_cfg* hint,
                   void** d_aux, size_t* bytes) {
    if (!d_aux || !bytes) return MANS_ERR_ARG;
    *d_aux = nullptr;
    *bytes = 0;
    mans_cfg plan;
    const int rc = mans_plan(n_units ? n_units : 1, n_out, L, hint, &plan);
    if (rc != MANS_OK) return rc;
    const size_t need = mans_aux_size(n_units ? n_units : 1, &plan);
    if (cudaMalloc(d_aux, need) != cudaSuccess) {
        cudaGetLastError();
        *d_aux = nullptr;
        return MANS_ERR_NOMEM;
    }
    *bytes = need;
    return MANS_OK;
}

int mans_aux_free(void* d_aux) {
    if (!d_aux) return MANS_OK;
    return cudaFree(d_aux) == cudaSuccess ? MANS_OK : MANS_ERR_CUDA;
}

int mans_table_upload(const uint32_t* h_table, uint32_t L, uint32_t** d_table) {
    if (!h_table || !d_table || L < 2 || L > kMaxStates) return MANS_ERR_ARG;
    *d_table = nullptr;
    if (mans_table_check(h_table, L) < 0) return MANS_ERR_TABLE;
    void* p = nullptr;
    if (cudaMalloc(&p, (size_t) L * 4) != cudaSuccess) {
        cudaGetLastError();
        return MANS_ERR_NOMEM;
    }
    if (cudaMemcpy(p, h_table, (size_t) L * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(p);
        return MANS_ERR_CUDA;
    }
    *d_table = (uint32_t*) p;
    return MANS_OK;
}

int mans_table_free(uint32_t* d_table) {
    if (!d_table) return MANS_OK;
    return cudaFree(d_table) == cudaSuccess ? MANS_OK : MANS_ERR_CUDA;
}

int mans_status_code(uint32_t st) {
    if (st & MANS_DEV_BAD_TABLE) return MANS_ERR_TABLE;
    if (st & (MANS_DEV_SYNC_OVERFLOW | MANS_DEV_COUNT_MISMATCH)) return MANS_ERR_SYNC;
    if (st & MANS_DEV_SCAN_TIMEOUT) return MANS_ERR_CUDA;
    return MANS_OK;
}

int mans_decode_sync(const uint32_t* d_units, size_t n_units, uint8_t* d_out,
                     size_t n_out, const uint32_t* d_table, uint32_t L,
                     uint32_t first_state, uint32_t first_bit, void* d_aux,
                     size_t aux_bytes, const mans_cfg* hint, void* stream,
                     uint32_t* status_out) {
    if (n_out != 0 && !decode_args_ok(d_units, n_units, d_out, d_table, L, first_state,
                                      first_bit, d_aux, hint ? hint->flags : 0u))
        return MANS_ERR_ARG;
    mans_cfg c = {0, 0, 0, 0, 0, 0};
    if (hint) c = *hint;
    mans_cfg plan;
    uint32_t st = 0;
    for (int attempt = 0; attempt < 8; ++attempt) {
        int rc = mans_plan(n_units, n_out, L, &c, &plan);
        if (rc != MANS_OK) return rc;
        if (mans_aux_size(n_units, &plan) > aux_bytes) {
            if (plan.capture_bytes) {
                // no capture first, then fewer slots, fit in the same memory
                c.capture_bytes = 0;
                c.flags |= MANS_DECODE_NO_CAPTURE;
                continue;
            }
            if (plan.walk_slots > 1) { c = plan; c.walk_slots = plan.walk_slots / 2; continue; }
            return MANS_ERR_AUX_SMALL;
        }
        rc = mans_decode(d_units, n_units, d_out, n_out, d_table, L, first_state,
                         first_bit, d_aux, aux_bytes, &plan, stream);
        if (rc != MANS_OK) return rc;
        if (n_out == 0) { st = 0; break; }
        rc = mans_aux_status(d_aux, stream, &st);
        if (rc != MANS_OK) return rc;
        if (!(st & MANS_DEV_SYNC_OVERFLOW)) break;
        // a walk outran its slots: longer regions, same slot count (and a
        // capture slice sized for them)
        c = plan;
        c.region_blocks = plan.region_blocks * 4;
        c.capture_bytes = 0;
    }
    if (status_out) *status_out = st;
    return mans_status_code(st);
}


int mans_decode_loop(const mans_stream_desc* streams, uint32_t n, const mans_cfg* plans,
                     void* const* d_aux, const size_t* aux_bytes, void* stream,
                     void* const* events) {
    if (n && (!streams || !plans || !d_aux || !aux_bytes)) return MANS_ERR_ARG;
    uint32_t launches = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const mans_stream_desc& d = streams[i];
        if (d.n_out != 0) {
            mans_cfg c = plans[i];
            c.flags |= d.flags & MANS_DECODE_SOURCE_ORDER;
            const int rc = mans_decode(d.d_units, d.n_units, d.d_out, d.n_out, d.d_table, d.L,
                                       d.first_state, d.first_bit, d_aux[i], aux_bytes[i], &c,
                                       stream);
            if (rc != MANS_OK) return rc;
            launches += g_last_launches;
        }
        if (events && events[i] &&
            cudaEventRecord((cudaEvent_t) events[i], (cudaStream_t) stream) != cudaSuccess)
            return MANS_ERR_CUDA;
    }
    g_last_launches = launches;
    return MANS_OK;
}

// ---------------------------------------------------------------------------
// Batched decode of many independent streams (one launch of each kernel for
// the whole batch; see the BatchItem kernels above).

}  // extern "C"

namespace mans {

struct BatchStreamPlan {
    mans_cfg cfg;
    size_t nblk, nreg, ntiles;
    size_t data_off;     // offset of this stream's slice in the data region
    size_t flags_off;    // word offset of its scan flags in the flag array
    uint32_t stage_cap;
    bool active;
};

struct BatchLayout {
    size_t status, flags, ticket, params, items, data, total;
    size_t n_sync, n_walk, n_scan, n_final, n_items;
    bool any_capture;
    size_t smem_sync, smem_walk, smem_final, smem_prep;
    // G-pass and final-pass launches per table class (0: L <= 1024, 1:
    // larger), each with its own shared memory: a batch's large tables
    // then leave the small-table streams at their own occupancy
    size_t n_sync_c[2], n_final_c[2], smem_sync_c[2], smem_final_c[2];
    size_t walk_list;     // [n_walk] stream of each merge-walk CTA (device-built)
    uint32_t walk_grid;   // persistent merge-walk grid
};

static size_t stream_data_bytes(const BatchStreamPlan& sp) {
    const AuxLayout a = layout_for(sp.nblk, sp.nreg, sp.cfg.walk_slots, sp.cfg.capture_bytes, false);
    return a.total;
}


constexpr uint64_t kBatchRegionMax = 8192;   // units

static int batch_class(uint32_t L) { return L <= 1024 ? 0 : 1; }

static int plan_batch(const mans_stream_desc* d, uint32_t n, const mans_cfg* hint,
                      std::vector<BatchStreamPlan>& plans, BatchLayout& lay) {
    plans.assign(n, BatchStreamPlan{});
    size_t data = 0, flag_words = 0;
    lay.n_sync = lay.n_walk = lay.n_scan = lay.n_final = 0;
    lay.any_capture = false;
    for (int c = 0; c < 2; ++c)
        lay.n_sync_c[c] = lay.n_final_c[c] = lay.smem_sync_c[c] = lay.smem_final_c[c] = 0;
    lay.smem_sync = lay.smem_walk = lay.smem_final = lay.smem_prep = 0;
    // A batch finds its parallelism across streams: regions are sized so the
    // whole batch gives about one G-pass wave of lanes (152 SMs x 16 warps),
    // each with a similar number of symbols, but every stream keeps at least
    // 128 regions, and never below the planner's length for the stream
    // alone.  Longer regions mean fewer merge walks and fewer walks that
    // cross a whole region.
    double batch_sym = 0;
    for (uint32_t i = 0; i < n; ++i) batch_sym += (double) d[i].n_out;
    const double sym_per_lane = batch_sym / (152.0 * 16 * 32);
    for (uint32_t i = 0; i < n; ++i) {
        BatchStreamPlan& sp = plans[i];
        sp.active = d[i].n_out > 0;
        if (!sp.active) continue;
        if (!d[i].d_units || !d[i].d_out || !d[i].d_table || d[i].n_units == 0 ||
            d[i].n_units > 0xffffffffull || d[i].L < 2 || d[i].L > kMaxStates ||
            d[i].first_state < d[i].L || d[i].first_state >= 2 * d[i].L ||
            d[i].first_bit > ((d[i].flags & MANS_DECODE_START_OFFSET) ? 127u : 32u) ||
            ((uintptr_t) d[i].d_units & 15) != 0)
            return MANS_ERR_ARG;
        mans_cfg h = {0, 0, 0, 0, 0, 0};
        if (hint) h = *hint;
        h.flags |= d[i].flags & (MANS_DECODE_NO_CAPTURE | MANS_DECODE_CAPTURE);
        // batches plan each stream with the model: the measured table is
        // tuned for streams decoded alone (capture lost on batches of short
        // streams: the capturing G pass holds fewer warps per SM)
        h.flags |= MANS_PLAN_MODEL;
        int rc = mans_plan(d[i].n_units, d[i].n_out, d[i].L, &h, &sp.cfg);
        if (rc != MANS_OK) return rc;
        if (h.region_blocks == 0) {
            const double spu = (double) d[i].n_out / (double) d[i].n_units;
            const uint64_t B = sp.cfg.block_units;
            // at least a full G-pass CTA (128 regions) per stream: a CTA's
            // idle warps still hold its slot on the SM
            const uint64_t want = (uint64_t) std::min(
                {sym_per_lane / std::max(spu, 1e-3), (double) d[i].n_units / kSyncThreads,
                 (double) kBatchRegionMax});
            const uint64_t cur = (uint64_t) sp.cfg.region_blocks * B;
            if (want > cur) {
                h.block_units = (uint32_t) B;
                h.region_blocks =
                    (uint32_t) std::max<uint64_t>(1, std::min<uint64_t>(want, d[i].n_units + B) / B) | 1u;
                h.walk_slots = 0;
                h.capture_bytes = 0;
                rc = mans_plan(d[i].n_units, d[i].n_out, d[i].L, &h, &sp.cfg);
                if (rc != MANS_OK) return rc;
            }
        }
        sp.cfg.flags = d[i].flags & (MANS_DECODE_SOURCE_ORDER | MANS_DECODE_START_OFFSET);
        sp.nblk = num_blocks(d[i].n_units, sp.cfg.block_units);
        sp.nreg = (sp.nblk + sp.cfg.region_blocks - 1) / sp.cfg.region_blocks;
        sp.ntiles = (sp.nreg + kScanTile - 1) / kScanTile;
        sp.data_off = data;
        data += align256(stream_data_bytes(sp));
        sp.flags_off = flag_words;
        flag_words += sp.ntiles + 4;
        sp.stage_cap = stage_cap_for((double) d[i].n_out / (double) d[i].n_units,
                                     sp.cfg.block_units, d[i].L, kFinalThreads / 32);
        const int cls = batch_class(d[i].L);
        lay.n_sync += (sp.nreg + kSyncThreads - 1) / kSyncThreads;
        lay.n_sync_c[cls] += (sp.nreg + kSyncThreads - 1) / kSyncThreads;
        lay.n_walk += walk_ctas(sp.nreg);
        lay.smem_walk = std::max(lay.smem_walk, walk_smem(d[i].L, sp.cfg.capture_bytes != 0));
        lay.n_scan += sp.ntiles;
        lay.n_final += (sp.nblk + kFinalThreads - 1) / kFinalThreads;
        lay.n_final_c[cls] += (sp.nblk + kFinalThreads - 1) / kFinalThreads;
        lay.any_capture |= sp.cfg.capture_bytes != 0;
        const size_t tab = ((size_t) d[i].L * 8 + 15) & ~(size_t) 15;
        const size_t ss = sync_smem(d[i].L, kSyncThreads, sp.cfg.capture_bytes != 0);
        lay.smem_sync = std::max(lay.smem_sync, ss);
        lay.smem_sync_c[cls] = std::max(lay.smem_sync_c[cls], ss);
        const uint32_t tile_bytes = (sp.cfg.block_units + 4) * 4;
        const uint32_t tile_stride = tile_bytes + ((tile_bytes & 127) == 0 ? 16 : 0);
        const size_t sf = tab + (size_t) (kFinalThreads / 32) *
                                    ((size_t) 32 * tile_stride + 16 + sp.stage_cap + 16);
        lay.smem_final = std::max(lay.smem_final, sf);
        lay.smem_final_c[cls] = std::max(lay.smem_final_c[cls], sf);
        lay.smem_prep = std::max(lay.smem_prep, (size_t) d[i].L * 12);
    }
    lay.n_items = lay.n_sync + lay.n_scan + lay.n_final;   // merge walks: built on the device
    size_t o = 0;
    lay.status = o; o += align256((size_t) n * 4);
    lay.flags = o; o += align256(flag_words * 4);
    lay.ticket = o; o += 256;
    lay.params = o; o += align256((size_t) n * sizeof(DecodeParams));
    lay.items = o; o += align256(lay.n_items * sizeof(BatchItem));
    lay.walk_list = o; o += align256(lay.n_walk * 4);
    lay.data = o; o += data;
    lay.total = o;
    return MANS_OK;
}

}  // namespace mans

struct mans_batch {
    int device = 0;
    uint32_t n = 0;
    char* base = nullptr;        // device workspace (header, then the slices unless split)
    bool owns = false;
    std::vector<mans::BatchStreamPlan> plans;
    std::vector<char*> slice;    // per-stream data slice
    mans::BatchLayout lay{};
    // host images of the parameters and work items; kept until destroy so
    // an asynchronous upload never reads freed memory
    std::vector<mans::DecodeParams> ps;
    std::vector<mans::BatchItem> items;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t graph_stream = nullptr;
};

extern "C" {

int mans_batch_workspace_size(const mans_stream_desc* streams, uint32_t n, const mans_cfg* hint,
                              size_t* bytes) {
    if (!streams || !bytes || n == 0) return MANS_ERR_ARG;
    std::vector<BatchStreamPlan> plans;
    BatchLayout lay;
    int rc = plan_batch(streams, n, hint, plans, lay);
    if (rc != MANS_OK) return rc;
    *bytes = lay.total;
    return MANS_OK;
}

int mans_batch_slice_size(const mans_stream_desc* stream, const mans_cfg* hint, size_t* bytes) {
    if (!stream || !bytes) return MANS_ERR_ARG;
    std::vector<BatchStreamPlan> plans;
    BatchLayout lay;
    int rc = plan_batch(stream, 1, hint, plans, lay);
    if (rc != MANS_OK) return rc;
    *bytes = lay.total - lay.data;
    return MANS_OK;
}

int mans_batch_header_size(const mans_stream_desc* streams, uint32_t n, const mans_cfg* hint,
                           size_t* bytes) {
    if (!streams || !bytes || n == 0) return MANS_ERR_ARG;
    std::vector<BatchStreamPlan> plans;
    BatchLayout lay;
    int rc = plan_batch(streams, n, hint, plans, lay);
    if (rc != MANS_OK) return rc;
    *bytes = lay.data;
    return MANS_OK;
}

}  // extern "C"

namespace {

// Plans the batch, places each stream's data slice (inside the workspace
// after the header, or at slices[i]) and uploads the parameters and work
// items: synchronously when `async` is false, else on `upload` with the
// host images kept alive in the batch object.
int batch_create(const mans_stream_desc* streams, uint32_t n, const mans_cfg* hint,
                 void* d_workspace, size_t workspace_bytes, void* const* slices,
                 cudaStream_t upload, bool async, mans_batch** out) {
    using namespace mans;
    if (!streams || !out || n == 0) return MANS_ERR_ARG;
    *out = nullptr;
    mans_batch* b = new mans_batch();
    b->n = n;
    cudaGetDevice(&b->device);
    int rc = plan_batch(streams, n, hint, b->plans, b->lay);
    if (rc != MANS_OK) { delete b; return rc; }
    const size_t need = slices ? b->lay.data : b->lay.total;
    if (d_workspace) {
        if (workspace_bytes < need) { delete b; return MANS_ERR_AUX_SMALL; }
        b->base = (char*) d_workspace;
    } else {
        if (cudaMalloc(&b->base, need) != cudaSuccess) { delete b; return MANS_ERR_NOMEM; }
        b->owns = true;
    }
    b->slice.assign(n, nullptr);
    b->ps.assign(n, DecodeParams{});
    b->items.assign(b->lay.n_items, BatchItem{});
    size_t is = 0, ic = b->lay.n_sync, iff = ic + b->lay.n_scan;
    for (uint32_t i = 0; i < n; ++i) {
        const BatchStreamPlan& sp = b->plans[i];
        DecodeParams& p = b->ps[i];
        std::memset(&p, 0, sizeof(p));
        p.status = (uint32_t*) (b->base + b->lay.status) + i;
        if (!sp.active) continue;
        const mans_stream_desc& d = streams[i];
        const AuxLayout a = layout_for(sp.nblk, sp.nreg, sp.cfg.walk_slots, sp.cfg.capture_bytes, false);
        char* slice = slices ? (char*) slices[i] : b->base + b->lay.data + sp.data_off;
        if (!slice || ((uintptr_t) slice & 255) != 0) { mans_batch_destroy(b); return MANS_ERR_ARG; }
        b->slice[i] = slice;
        p.units = d.d_units;
        p.out = d.d_out;
        p.table = d.d_table;
        p.tab_sync = (uint2*) (slice + a.tab_sync);
        p.tab_sym = (uint2*) (slice + a.tab_sym);
        p.rec_g = (uint2*) (slice + a.rec_g);
        p.rec_w = (uint2*) (slice + a.rec_w);
        p.m = (unsigned long long*) (slice + a.m);
        p.delta = (long long*) (slice + a.delta);
        p.Mpre = (unsigned long long*) (slice + a.Mpre);
        p.Dpre = (long long*) (slice + a.Dpre);
        p.scan_tiles = (ScanTile*) (slice + a.scan_tiles);
        p.scan_flags = (uint32_t*) (b->base + b->lay.flags) + sp.flags_off;
        p.walk_jobs = (WJob*) (slice + a.walk_jobs);
        p.n_out = d.n_out;
        p.n_units = (uint32_t) d.n_units;
        p.L = d.L;
        p.first_idx = d.first_state - d.L;
        p.first_pos = start_pos(d.first_bit, d.flags);
        p.B = sp.cfg.block_units;
        p.nb = sp.cfg.region_blocks;
        p.dmax = sp.cfg.walk_slots;
        p.nblk = (uint32_t) sp.nblk;
        p.nreg = (uint32_t) sp.nreg;
        p.stage_cap = sp.stage_cap;
        p.wcap = walk_cap(sp.cfg);
        p.flags = d.flags & MANS_DECODE_SOURCE_ORDER;
        p.cap_bytes = sp.cfg.capture_bytes;
        p.cap = sp.cfg.capture_bytes ? (uint8_t*) (slice + a.cap) : nullptr;
        p.cap_valid = sp.cfg.capture_bytes ? (uint32_t*) (slice + a.cap_valid) : nullptr;
        p.fb_list = sp.cfg.capture_bytes ? (uint32_t*) (slice + a.fb_list) : nullptr;
        for (size_t t = 0; t < sp.ntiles; ++t) b->items[ic++] = {i, (uint32_t) t, 0, 0};
    }
    // G-pass and final-pass items, heaviest first: a batch's CTAs run in
    // several waves (every stream has at least one CTA), and with the long
    // ones issued first the short ones fill in behind them instead of a
    // late long CTA setting the launch's end (longest-processing-time order)
    std::vector<uint32_t> order;
    for (uint32_t i = 0; i < n; ++i)
        if (b->plans[i].active) order.push_back(i);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
        const int cx = batch_class(streams[x].L), cy = batch_class(streams[y].L);
        if (cx != cy) return cx < cy;   // one launch per table class
        return (double) streams[x].n_out / (double) b->plans[x].nreg >
               (double) streams[y].n_out / (double) b->plans[y].nreg;   // symbols per region
    });
    for (const uint32_t i : order)
        for (size_t r = 0; r < b->plans[i].nreg; r += kSyncThreads)
            b->items[is++] = {i, (uint32_t) r, 0, 0};
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
        const int cx = batch_class(streams[x].L), cy = batch_class(streams[y].L);
        if (cx != cy) return cx < cy;
        return streams[x].n_out > streams[y].n_out;
    });
    for (const uint32_t i : order) {
        const uint32_t nctas = (uint32_t) ((b->plans[i].nblk + kFinalThreads - 1) / kFinalThreads);
        for (uint32_t c = 0; c < nctas; ++c) b->items[iff++] = {i, c, nctas, 0};
    }
    const size_t pbytes = n * sizeof(DecodeParams), ibytes = b->items.size() * sizeof(BatchItem);
    bool ok;
    if (async) {
        ok = cudaMemcpyAsync(b->base + b->lay.params, b->ps.data(), pbytes,
                             cudaMemcpyHostToDevice, upload) == cudaSuccess &&
             (!ibytes || cudaMemcpyAsync(b->base + b->lay.items, b->items.data(), ibytes,
                                         cudaMemcpyHostToDevice, upload) == cudaSuccess);
    } else {
        ok = cudaMemcpy(b->base + b->lay.params, b->ps.data(), pbytes, cudaMemcpyHostToDevice) ==
                 cudaSuccess &&
             (!ibytes || cudaMemcpy(b->base + b->lay.items, b->items.data(), ibytes,
                                    cudaMemcpyHostToDevice) == cudaSuccess);
    }
    if (!ok) {
        mans_batch_destroy(b);
        return MANS_ERR_CUDA;
    }
    set_kernel_attributes();
    if (b->lay.n_walk) {
        // the persistent merge-walk grid: as many CTAs as stay resident
        int per_sm = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wwalk_batch, kWalkThreads,
                                                          b->lay.smem_walk) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device) !=
                cudaSuccess) {
            mans_batch_destroy(b);
            return MANS_ERR_CUDA;
        }
        b->lay.walk_grid = (uint32_t) std::min<size_t>(
            b->lay.n_walk, (size_t) std::max(per_sm, 1) * (size_t) std::max(sms, 1));
    }
    *out = b;
    return MANS_OK;
}

}  // namespace

extern "C" {

int mans_batch_create(const mans_stream_desc* streams, uint32_t n, const mans_cfg* hint,
                      void* d_workspace, size_t workspace_bytes, mans_batch** out) {
    return batch_create(streams, n, hint, d_workspace, workspace_bytes, nullptr, nullptr, false,
                        out);
}

int mans_batch_create_split(const mans_stream_desc* streams, uint32_t n, const mans_cfg* hint,
                            void* d_header, size_t header_bytes, void* const* d_slices,
                            void* stream, mans_batch** out) {
    if (!d_header || !d_slices) return MANS_ERR_ARG;
    return batch_create(streams, n, hint, d_header, header_bytes, d_slices,
                        (cudaStream_t) stream, true, out);
}

int mans_batch_decode(mans_batch* b, void* stream) {
    if (!b) return MANS_ERR_ARG;
    cudaStream_t st = (cudaStream_t) stream;
    const BatchLayout& L = b->lay;
    if (cudaMemsetAsync(b->base, 0, L.params, st) != cudaSuccess) return MANS_ERR_CUDA;
    if (L.n_items == 0) return MANS_OK;
    const DecodeParams* ps = (const DecodeParams*) (b->base + L.params);
    const BatchItem* items = (const BatchItem*) (b->base + L.items);
    timing_mark(0, st);
    k_prep_batch<<<b->n, 1024, L.smem_prep, st>>>(ps);
    timing_mark(1, st);
    for (int c = 0, at = 0; c < 2; at += (int) L.n_sync_c[c], ++c)
        if (L.n_sync_c[c])
            k_gwalk_batch<<<(unsigned) L.n_sync_c[c], kSyncThreads, L.smem_sync_c[c], st>>>(
                ps, items + at);
    timing_mark(2, st);
    if (L.n_walk) {
        // ticket words: 0 scan tiles, 1 merge-walk items, 2 next item
        uint32_t* const count = (uint32_t*) (b->base + L.ticket) + 1;
        uint32_t* const list = (uint32_t*) (b->base + L.walk_list);
        k_walk_items<<<(b->n + 255) / 256, 256, 0, st>>>(ps, b->n, list, count);
        k_wwalk_batch<<<L.walk_grid, kWalkThreads, L.smem_walk, st>>>(ps, list, count);
    }
    timing_mark(3, st);
    if (L.n_scan)
        k_scan_batch<<<(unsigned) L.n_scan, kScanThreads, 0, st>>>(
            ps, items + L.n_sync, (uint32_t*) (b->base + L.ticket));
    timing_mark(4, st);
    if (L.n_final && L.any_capture)
        k_copy_batch<<<(unsigned) L.n_final, kCopyThreads, 0, st>>>(
            ps, items + L.n_sync + L.n_scan);
    for (int c = 0, at = 0; c < 2; at += (int) L.n_final_c[c], ++c)
        if (L.n_final_c[c])
            k_final_batch<<<(unsigned) L.n_final_c[c], kFinalThreads, L.smem_final_c[c], st>>>(
                ps, items + L.n_sync + L.n_scan + at);
    timing_mark(5, st);
    if (g_timing.on && g_timing.used < g_timing.cap) ++g_timing.used;
    g_last_launches = 1 + (L.n_sync_c[0] ? 1 : 0) + (L.n_sync_c[1] ? 1 : 0) +
                      (L.n_walk ? 2 : 0) + (L.n_scan ? 1 : 0) + (L.n_final_c[0] ? 1 : 0) +
                      (L.n_final_c[1] ? 1 : 0) + (L.n_final && L.any_capture ? 1 : 0);
    return cudaGetLastError() == cudaSuccess ? MANS_OK : MANS_ERR_CUDA;
}

int mans_batch_graph_decode(mans_batch* b, void* stream) {
    if (!b) return MANS_ERR_ARG;
    if (!b->exec) {
        // capture on a private stream, replay on the caller's (NULL works)
        if (!b->graph_stream &&
            cudaStreamCreateWithFlags(&b->graph_stream, cudaStreamNonBlocking) != cudaSuccess)
            return MANS_ERR_CUDA;
        if (cudaStreamBeginCapture(b->graph_stream, cudaStreamCaptureModeThreadLocal) !=
            cudaSuccess)
            return MANS_ERR_CUDA;
        const int rc = mans_batch_decode(b, b->graph_stream);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(b->graph_stream, &g);
        if (rc != MANS_OK || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return rc != MANS_OK ? rc : MANS_ERR_CUDA;
        }
        if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) {
            cudaGraphDestroy(g);
            b->exec = nullptr;
            return MANS_ERR_CUDA;
        }
        b->graph = g;
    }
    return cudaGraphLaunch(b->exec, (cudaStream_t) stream) == cudaSuccess ? MANS_OK : MANS_ERR_CUDA;
}

int mans_batch_fixup(mans_batch* b, void* stream, uint32_t* n_redone) {
    if (!b) return MANS_ERR_ARG;
    if (n_redone) *n_redone = 0;
    cudaStream_t st = (cudaStream_t) stream;
    std::vector<uint32_t> v(b->n);
    if (cudaMemcpyAsync(v.data(), b->base + b->lay.status, b->n * 4, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return MANS_ERR_CUDA;
    const DecodeParams* dps = (const DecodeParams*) (b->base + b->lay.params);
    for (uint32_t i = 0; i < b->n; ++i) {
        if (!(v[i] & MANS_DEV_SYNC_OVERFLOW) || !b->plans[i].active) continue;
        DecodeParams p;
        if (cudaMemcpy(&p, dps + i, sizeof(p), cudaMemcpyDeviceToHost) != cudaSuccess)
            return MANS_ERR_CUDA;
        const BatchStreamPlan& sp = b->plans[i];
        char* slice = b->slice[i];
        const size_t slice_bytes = stream_data_bytes(sp);
        mans_cfg hint = sp.cfg;
        hint.region_blocks = sp.cfg.region_blocks * 4;   // longer regions, same slots
        uint32_t dev_status = 0;
        const int rc = mans_decode_sync(p.units, p.n_units, p.out, p.n_out, p.table, p.L,
                                        p.first_idx + p.L,
                                        (sp.cfg.flags & MANS_DECODE_START_OFFSET)
                                            ? p.first_pos : 32 - p.first_pos,
                                        slice, slice_bytes,
                                        &hint, stream, &dev_status);
        if (rc != MANS_OK && rc != MANS_ERR_SYNC) return rc;
        if (cudaMemcpyAsync(b->base + b->lay.status + 4ull * i, &dev_status, 4,
                            cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return MANS_ERR_CUDA;
        if (n_redone) ++*n_redone;
    }
    return MANS_OK;
}

int mans_decode_batch(const mans_stream_desc* streams, uint32_t n, const mans_cfg* hint,
                      void* d_workspace, size_t workspace_bytes, void* stream,
                      uint32_t* or_status, uint32_t* per_stream) {
    if (or_status) *or_status = 0;
    mans_batch* b = nullptr;
    int rc = mans_batch_create(streams, n, hint, d_workspace, workspace_bytes, &b);
    if (rc != MANS_OK) return rc;
    uint32_t acc = 0, redone = 0;
    rc = mans_batch_decode(b, stream);
    if (rc == MANS_OK) rc = mans_batch_status(b, stream, &acc, nullptr);
    if (rc == MANS_OK && (acc & MANS_DEV_SYNC_OVERFLOW)) rc = mans_batch_fixup(b, stream, &redone);
    if (rc == MANS_OK) rc = mans_batch_status(b, stream, &acc, per_stream);
    mans_batch_destroy(b);
    if (rc != MANS_OK) return rc;
    if (or_status) *or_status = acc;
    return mans_status_code(acc & ~MANS_DEV_DEGENERATE);
}

int mans_batch_status(mans_batch* b, void* stream, uint32_t* or_status, uint32_t* per_stream) {
    if (!b) return MANS_ERR_ARG;
    std::vector<uint32_t> v(b->n);
    cudaStream_t st = (cudaStream_t) stream;
    if (cudaMemcpyAsync(v.data(), b->base + b->lay.status, b->n * 4, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return MANS_ERR_CUDA;
    uint32_t acc = 0;
    for (uint32_t i = 0; i < b->n; ++i) acc |= v[i];
    if (or_status) *or_status = acc;
    if (per_stream) std::memcpy(per_stream, v.data(), b->n * 4);
    return MANS_OK;
}

int mans_batch_destroy(mans_batch* b) {
    if (!b) return MANS_OK;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->graph_stream) cudaStreamDestroy(b->graph_stream);
    if (b->owns && b->base) cudaFree(b->base);
    delete b;
    return MANS_OK;
}

}  // extern "C"
