// GPU tANS encoder producing the reference encoder's exact stream
// (src/ans_encoder.cc:13-72: one raw single-state stream, codes packed
// MSB-first into 32-bit units, units then reversed with four zero units of
// padding as CUHDInputBuffer holds them, src/multians_input_buffer.cc:15-30).
//
// Encoding is sequential in the state: x' = next(s, x >> k(s, x)), and the
// code of each byte is the k low bits of x.  But two encodes of the same
// bytes from different states meet after a while and agree from there on,
// so the decoder's method carries over with symbol positions in place of
// bit positions:
//
//  k_enc_g     one lane per chunk of Cs bytes encodes it from the initial
//              state (the guess), recording at every block of Bs bytes the
//              state and the code bits so far (rec_g), and its end record.
//  k_enc_w     one lane per chunk k walks Gamma_k past its chunk end and
//              compares it at every block start with Gamma_{k+1} (its
//              records inside chunk k+1, a second cursor beyond) until the
//              states agree: merge point m_k, bit difference delta_k.
//  k_scan      M_k = max m_0..m_{k-1}, D_k = sum delta_0..delta_{k-1}
//              (the decoder's scan).
//  k_enc_total the owner of the stream end gives the total bit count T,
//              n_units = floor(T / 32) + 1 and first_bit = T mod 32.
//  k_enc_final one lane per block: its owner's record gives the true state
//              and bit offset; it encodes the block again and writes the
//              codes at that offset (units shared with a neighbour by
//              atomicOr), in reversed unit order.
//  k_enc_tail  the reference's flush puts more code bits below the last
//              unit's valid bits (the last byte's code again when it fitted
//              its unit, else the code of byte value 0 past the end); they
//              are reproduced so the units match bit for bit.
//
// Tables: the compact encoder table built on the host from the byte
// histogram (mans_host_encode_tables), loaded into shared memory per CTA:
// per byte {delta, base} and the L next states (uint16).  L is a power of
// two <= 8192.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

#include "mans_scan.cuh"
#include "multians_gb300.h"

namespace mans {
namespace {

constexpr uint32_t kEncThreads = 128;
constexpr uint32_t kEncBlock = 256;        // bytes per block (records, final-pass lanes)
constexpr uint32_t kEncSlots = 8;          // chunks a walk may cross

struct EncResult {
    unsigned long long total_bits;
    unsigned long long n_units;
    uint32_t first_bit, first_state;
    uint32_t last_code, last_len;          // the last byte's code
    uint32_t owner_end;                    // chunk whose trajectory owns the end
    uint32_t pad;
};

struct EncParams {
    const uint8_t* sym;
    unsigned long long n;
    const uint32_t* blob;                  // global compact table
    uint32_t L, Cs, nb, nchunk, nblk, dmax;
    uint2* rec_g;                          // [nblk] {state, bits since chunk start}
    uint2* rec_w;                          // [nblk * dmax]
    uint4* end_rec;                        // [nchunk] {state, bits lo, last code, last len}
    unsigned long long* m;
    long long* delta;
    unsigned long long* Mpre;
    long long* Dpre;
    ScanTile* scan_tiles;
    uint32_t* scan_flags;
    uint32_t* status;
    uint32_t nreg;                         // = nchunk (scan)
    EncResult* result;
    uint32_t* units;
    unsigned long long cap;                // units capacity (words)
};

// Shared tables: 256 x uint2 {delta, base}, then L uint16 next states.
__device__ __forceinline__ void load_enc_tables(uint2* s_sym, uint16_t* s_next,
                                                const uint32_t* __restrict__ blob, uint32_t L) {
    for (uint32_t v = threadIdx.x; v < 256; v += blockDim.x)
        s_sym[v] = make_uint2(__ldg(blob + 2 * v), __ldg(blob + 2 * v + 1));
    const uint32_t* nx = blob + 512;
    uint32_t* s32 = reinterpret_cast<uint32_t*>(s_next);
    for (uint32_t i = threadIdx.x; i < L / 2; i += blockDim.x) s32[i] = __ldg(nx + i);
    __syncthreads();
}

// One encode step of byte s from state x: returns k (the code length) and
// the code; x becomes the next state.  Bytes absent from the table never
// occur in the data the table was built from.
__device__ __forceinline__ uint32_t enc_step(uint32_t& x, uint32_t s, const uint2* s_sym,
                                             const uint16_t* s_next, uint32_t L,
                                             uint32_t& code) {
    const uint2 q = s_sym[s];
    const uint32_t k = (x + q.x) >> 16;
    code = x & ((1u << k) - 1u);
    const uint32_t idx = min(q.y + (x >> k), L - 1);   // clamped: absent bytes stay in range
    x = s_next[idx];
    return k;
}

// A lane's bytes [start, end), read 16 at a time (start is 16-byte aligned;
// the group that crosses `end` is read byte by byte, so nothing past the
// buffer is touched).
struct ByteReader {
    const uint8_t* p;
    unsigned long long g, n;   // next 16-byte group, end
    uint4 cur;
    uint32_t pos;              // next byte within cur; 16 = empty
    __device__ __forceinline__ void init(const uint8_t* base, unsigned long long start,
                                         unsigned long long end) {
        p = base;
        g = start;
        n = end;
        pos = 16;
    }
    __device__ __forceinline__ uint32_t next() {
        if (pos == 16) {
            if (g + 16 <= n) {
                cur = __ldg(reinterpret_cast<const uint4*>(p + g));
            } else {
                uint32_t w[4] = {0, 0, 0, 0};
                for (uint32_t t = 0; t < 16; ++t)
                    if (g + t < n) w[t >> 2] |= (uint32_t) p[g + t] << (8 * (t & 3));
                cur = make_uint4(w[0], w[1], w[2], w[3]);
            }
            g += 16;
            pos = 0;
        }
        const uint32_t w = pos < 8 ? (pos < 4 ? cur.x : cur.y) : (pos < 12 ? cur.z : cur.w);
        const uint32_t b = (w >> (8 * (pos & 3))) & 0xffu;
        ++pos;
        return b;
    }
};

__device__ __forceinline__ uint2 rec(uint32_t state, uint32_t bits) {
    return make_uint2(state, bits);
}

// G pass: chunk k from the initial state L.
__global__ void __launch_bounds__(kEncThreads) k_enc_g(EncParams p) {
    extern __shared__ __align__(16) uint2 s_sym[];
    uint16_t* s_next = reinterpret_cast<uint16_t*>(s_sym + 256);
    load_enc_tables(s_sym, s_next, p.blob, p.L);
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= p.nchunk) return;
    const unsigned long long s0 = (unsigned long long) k * p.Cs;
    const unsigned long long s1 = min(s0 + p.Cs, p.n);
    uint32_t x = p.L, bits = 0, code = 0, len = 0;
    ByteReader rd;
    rd.init(p.sym, s0, s1);
    uint32_t b = k * p.nb;
    for (unsigned long long i = s0; i < s1; i += kEncBlock, ++b) {
        p.rec_g[b] = rec(x, bits);
        const unsigned long long e = min(i + kEncBlock, s1);
        for (unsigned long long j = i; j < e; ++j) {
            len = enc_step(x, rd.next(), s_sym, s_next, p.L, code);
            bits += len;
        }
    }
    if (k + 1 < p.nchunk) {
        p.rec_w[(size_t) (k + 1) * p.nb * p.dmax] = rec(x, bits);   // Gamma_k at chunk k+1
    } else {
        p.m[k] = ~0ull;
        p.delta[k] = 0;
        p.end_rec[k] = make_uint4(x, bits, code, len);
    }
}

// Merge walk of chunk k (k + 1 < nchunk), one lane each.
__global__ void __launch_bounds__(kEncThreads) k_enc_w(EncParams p) {
    extern __shared__ __align__(16) uint2 s_sym[];
    uint16_t* s_next = reinterpret_cast<uint16_t*>(s_sym + 256);
    load_enc_tables(s_sym, s_next, p.blob, p.L);
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k + 1 >= p.nchunk) return;
    uint32_t b = (k + 1) * p.nb;                        // block the cursors stand at
    const uint2 r0 = p.rec_w[(size_t) b * p.dmax];
    uint32_t xa = r0.x, ca = r0.y;                      // Gamma_k
    uint32_t xg = 0, cg = 0;                            // Gamma_{k+1} past its chunk
    bool g_on = false;
    uint32_t code = 0, len = 0;
    ByteReader rd;
    rd.init(p.sym, (unsigned long long) b * kEncBlock, p.n);
    for (;;) {
        const uint32_t d = b / p.nb - k;
        if (d > p.dmax) {
            atomicOr(p.status, MANS_DEV_SYNC_OVERFLOW);
            p.m[k] = ~0ull;
            p.delta[k] = 0;
            return;
        }
        if (d >= 1 && b != (k + 1) * p.nb) p.rec_w[(size_t) b * p.dmax + (d - 1)] = rec(xa, ca);
        uint32_t gx, gc;
        if (d == 1) {
            const uint2 rg = p.rec_g[b];
            gx = rg.x;
            gc = rg.y;
        } else {
            if (!g_on) {
                const uint2 r1 = p.rec_w[(size_t) b * p.dmax];   // Gamma_{k+1} entering chunk k+2
                xg = r1.x;
                cg = r1.y;
                g_on = true;
            }
            gx = xg;
            gc = cg;
        }
        if (xa == gx) {
            p.m[k] = (unsigned long long) b * kEncBlock;
            p.delta[k] = (long long) ca - (long long) gc;
            return;
        }
        const unsigned long long i0 = (unsigned long long) b * kEncBlock;
        const unsigned long long i1 = min(i0 + kEncBlock, p.n);
        for (unsigned long long j = i0; j < i1; ++j) {
            const uint32_t s = rd.next();
            len = enc_step(xa, s, s_sym, s_next, p.L, code);
            ca += len;
            if (g_on) {
                uint32_t c2;
                cg += enc_step(xg, s, s_sym, s_next, p.L, c2);
            }
        }
        ++b;
        if (b >= p.nblk) {
            // the stream ends before the trajectories agree
            p.m[k] = ~0ull;
            p.delta[k] = 0;
            p.end_rec[k] = make_uint4(xa, ca, code, len);
            return;
        }
    }
}

__global__ void __launch_bounds__(kScanThreads) k_enc_scan(EncParams p) {
    __shared__ uint32_t s_tile;
    if (threadIdx.x == 0)
        s_tile = atomicAdd(p.scan_flags + (p.nreg + kScanTile - 1) / kScanTile, 1u);
    __syncthreads();
    scan_body(p, s_tile);
}

// Owner of symbol position i: the largest chunk k <= chunk(i) with
// M_k <= i; d = chunk(i) - k.
__device__ __forceinline__ bool enc_owner(const EncParams& p, unsigned long long i, uint32_t c,
                                          uint32_t& k, uint32_t& d) {
    for (d = 0;; ++d) {
        if (d > c || d > p.dmax) return false;
        if (p.Mpre[c - d] <= i) break;
    }
    k = c - d;
    return true;
}

__global__ void k_enc_total(EncParams p) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t k = 0, d = 0;
    const uint32_t c = p.nchunk - 1;
    if (!enc_owner(p, p.n, c, k, d)) {
        atomicOr(p.status, MANS_DEV_SYNC_OVERFLOW);
        return;
    }
    const uint4 e = p.end_rec[k];
    const unsigned long long T = (unsigned long long) (p.Dpre[k] + (long long) e.y);
    EncResult* r = p.result;
    r->total_bits = T;
    r->n_units = T / 32 + 1;
    r->first_bit = (uint32_t) (T & 31);
    r->first_state = e.x;
    r->last_code = e.z;
    r->last_len = e.w;
    r->owner_end = k;
    if (T / 32 + 1 + 4 > p.cap) atomicOr(p.status, MANS_DEV_COUNT_MISMATCH);
}

// Unit u of the forward stream lives at units[n_units - 1 - u].
__device__ __forceinline__ void put_unit(uint32_t* units, unsigned long long n_units,
                                         unsigned long long u, uint32_t w, bool shared) {
    if (u >= n_units) return;
    uint32_t* a = units + (n_units - 1 - u);
    if (shared) atomicOr(a, w);
    else *a = w;
}

__global__ void __launch_bounds__(kEncThreads) k_enc_final(EncParams p) {
    extern __shared__ __align__(16) uint2 s_sym[];
    uint16_t* s_next = reinterpret_cast<uint16_t*>(s_sym + 256);
    load_enc_tables(s_sym, s_next, p.blob, p.L);
    if (*(volatile uint32_t*) p.status & (MANS_DEV_SYNC_OVERFLOW | MANS_DEV_SCAN_TIMEOUT |
                                          MANS_DEV_COUNT_MISMATCH))
        return;
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p.nblk) return;
    const unsigned long long n_units = p.result->n_units;
    const unsigned long long i0 = (unsigned long long) b * kEncBlock;
    const unsigned long long i1 = min(i0 + kEncBlock, p.n);
    uint32_t k = 0, d = 0;
    if (!enc_owner(p, i0, b / p.nb, k, d)) {
        atomicOr(p.status, MANS_DEV_SYNC_OVERFLOW);
        return;
    }
    const uint2 r = d == 0 ? p.rec_g[b] : p.rec_w[(size_t) b * p.dmax + (d - 1)];
    const unsigned long long o = (unsigned long long) (p.Dpre[k] + (long long) r.y);
    uint32_t x = min(max(r.x, p.L), 2 * p.L - 1);
    // codes MSB-first from bit o: acc holds the pending bits of unit u
    unsigned long long acc = 0;
    uint32_t nbits = (uint32_t) (o & 31);
    unsigned long long u = o >> 5;
    bool first = true;
    uint32_t code = 0, len = 0;
    ByteReader rd;
    rd.init(p.sym, i0, i1);
    for (unsigned long long j = i0; j < i1; ++j) {
        len = enc_step(x, rd.next(), s_sym, s_next, p.L, code);
        acc = (acc << len) | code;
        nbits += len;
        if (nbits >= 32) {
            nbits -= 32;
            put_unit(p.units, n_units, u, (uint32_t) (acc >> nbits), first);
            acc &= (1ull << nbits) - 1ull;
            first = false;
            ++u;
        }
    }
    if (nbits > 0) put_unit(p.units, n_units, u, (uint32_t) (acc << (32 - nbits)), true);
}

// The flush of the reference encoder (src/ans_encoder.cc:40-66): below the
// last unit's at = T mod 32 valid bits it adds the high bits of one more
// code when that code reaches 32 - at bits: the last byte's code again when
// the last byte's code fitted its unit (at the unit loop's exit it is still
// the current entry), else the code of byte value 0 (the byte past the end)
// from the final state.
__global__ void k_enc_tail(EncParams p) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (*(volatile uint32_t*) p.status & (MANS_DEV_SYNC_OVERFLOW | MANS_DEV_SCAN_TIMEOUT |
                                          MANS_DEV_COUNT_MISMATCH))
        return;
    const EncResult r = *p.result;
    const uint32_t at = (uint32_t) (r.total_bits & 31);
    const unsigned long long P = r.total_bits - r.last_len;   // start of the last code
    uint32_t code, len;
    if ((uint32_t) (P & 31) + r.last_len < 32) {
        code = r.last_code;
        len = r.last_len;
    } else {
        const uint32_t dq = __ldg(p.blob + 0), bq = __ldg(p.blob + 1);
        if (bq == ~0u) return;                              // byte 0 absent: zero entry
        const uint32_t x = r.first_state;
        len = (x + dq) >> 16;
        code = x & ((1u << len) - 1u);
    }
    if (at + len >= 32) {
        const uint32_t spill = at + len - 32;
        p.units[0] |= code >> spill;                        // forward unit n_units - 1
    }
}

// Byte histogram: per-CTA counts in shared memory (one copy per warp, so
// lanes of different warps do not contend), merged into 64-bit totals.
__global__ void __launch_bounds__(256) k_hist(const uint8_t* __restrict__ sym,
                                             unsigned long long n,
                                             unsigned long long* __restrict__ hist) {
    __shared__ uint32_t h[8][256];
    for (uint32_t i = threadIdx.x; i < 8 * 256; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    uint32_t* mine = h[threadIdx.x >> 5];
    const unsigned long long n16 = n / 16;
    const uint4* v = reinterpret_cast<const uint4*>(sym);
    const bool aligned = ((uintptr_t) sym & 15) == 0;
    const unsigned long long stride = (unsigned long long) gridDim.x * blockDim.x;
    if (aligned) {
        for (unsigned long long i = (unsigned long long) blockIdx.x * blockDim.x + threadIdx.x;
             i < n16; i += stride) {
            const uint4 q = __ldg(v + i);
            const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int t = 0; t < 16; ++t) atomicAdd(&mine[(w[t >> 2] >> (8 * (t & 3))) & 0xffu], 1u);
        }
    }
    for (unsigned long long i = (aligned ? n16 * 16 : 0) + (unsigned long long) blockIdx.x * blockDim.x +
                                threadIdx.x;
         i < n; i += stride)
        atomicAdd(&mine[sym[i]], 1u);
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < 256; b += blockDim.x) {
        uint32_t c = 0;
        for (int w = 0; w < 8; ++w) c += h[w][b];
        if (c) atomicAdd(hist + b, (unsigned long long) c);
    }
}

struct EncLayout {
    size_t status, result, rec_g, rec_w, end_rec, m, delta, Mpre, Dpre, tiles, flags, total;
};

size_t al256(size_t x) { return (x + 255) & ~(size_t) 255; }

EncLayout enc_layout(size_t nchunk, size_t nblk, size_t dmax) {
    EncLayout a;
    size_t o = 0;
    a.status = o; o += 256;
    a.result = o; o += 256;
    a.rec_g = o; o += al256(nblk * 8);
    a.rec_w = o; o += al256(nblk * dmax * 8);
    a.end_rec = o; o += al256(nchunk * 16);
    a.m = o; o += al256(nchunk * 8);
    a.delta = o; o += al256(nchunk * 8);
    a.Mpre = o; o += al256(nchunk * 8);
    a.Dpre = o; o += al256(nchunk * 8);
    const size_t ntiles = (nchunk + kScanTile - 1) / kScanTile;
    a.tiles = o; o += al256(ntiles * sizeof(ScanTile));
    a.flags = o; o += al256((ntiles + 1) * 4);
    a.total = o;
    return a;
}

// Chunk length: about 78 k chunks when the stream is long enough, at least
// 2048 bytes, a multiple of the block.
uint32_t enc_chunk(unsigned long long n, uint32_t hint) {
    if (hint) return std::max<uint32_t>(kEncBlock, std::min<uint32_t>(hint, 1u << 30) / kEncBlock * kEncBlock);
    unsigned long long c = (n + 78000 - 1) / 78000;
    c = std::max<unsigned long long>(c, 2048);
    c = std::min<unsigned long long>(c, 1u << 20);
    return (uint32_t) ((c + kEncBlock - 1) / kEncBlock * kEncBlock);
}

}  // namespace
}  // namespace mans

using namespace mans;

extern "C" {

size_t mans_encode_blob_words(uint32_t L) { return 512 + (size_t) (L + 1) / 2; }

size_t mans_encode_max_units(size_t n, uint32_t L) {
    uint32_t lg = 0;
    while ((1u << lg) < L && lg < 31) ++lg;
    return (size_t) ((n * (unsigned long long) lg) / 32) + 6;
}

size_t mans_encode_aux_size(size_t n, uint32_t chunk_hint) {
    if (n == 0) return 0;
    const uint32_t Cs = enc_chunk(n, chunk_hint);
    const size_t nchunk = (n + Cs - 1) / Cs;
    const size_t nblk = (n + kEncBlock - 1) / kEncBlock;
    return enc_layout(nchunk, nblk, kEncSlots).total;
}

int mans_encode(const uint8_t* d_sym, size_t n, const uint32_t* d_enc_blob, uint32_t L,
                uint32_t* d_units, size_t cap_units, void* d_aux, size_t aux_bytes,
                uint32_t chunk_hint, void* stream) {
    if (!d_sym || !d_enc_blob || !d_units || !d_aux || n == 0 || L < 2 || L > 8192 ||
        (L & (L - 1)) != 0 || ((uintptr_t) d_sym & 15) != 0 || ((uintptr_t) d_enc_blob & 3) != 0)
        return MANS_ERR_ARG;
    const uint32_t Cs = enc_chunk(n, chunk_hint);
    const size_t nchunk = (n + Cs - 1) / Cs;
    const size_t nblk = (n + kEncBlock - 1) / kEncBlock;
    if (nchunk > 0x7fffffffull || nblk > 0x7fffffffull) return MANS_ERR_ARG;
    const EncLayout lay = enc_layout(nchunk, nblk, kEncSlots);
    if (aux_bytes < lay.total) return MANS_ERR_AUX_SMALL;
    if (cap_units < mans_encode_max_units(n, L)) return MANS_ERR_AUX_SMALL;
    cudaStream_t st = (cudaStream_t) stream;
    char* base = (char*) d_aux;
    EncParams p;
    std::memset(&p, 0, sizeof(p));
    p.sym = d_sym;
    p.n = n;
    p.blob = d_enc_blob;
    p.L = L;
    p.Cs = Cs;
    p.nb = Cs / kEncBlock;
    p.nchunk = (uint32_t) nchunk;
    p.nblk = (uint32_t) nblk;
    p.dmax = kEncSlots;
    p.rec_g = (uint2*) (base + lay.rec_g);
    p.rec_w = (uint2*) (base + lay.rec_w);
    p.end_rec = (uint4*) (base + lay.end_rec);
    p.m = (unsigned long long*) (base + lay.m);
    p.delta = (long long*) (base + lay.delta);
    p.Mpre = (unsigned long long*) (base + lay.Mpre);
    p.Dpre = (long long*) (base + lay.Dpre);
    p.scan_tiles = (ScanTile*) (base + lay.tiles);
    p.scan_flags = (uint32_t*) (base + lay.flags);
    p.status = (uint32_t*) (base + lay.status);
    p.nreg = (uint32_t) nchunk;
    p.result = (EncResult*) (base + lay.result);
    p.units = d_units;
    p.cap = cap_units;
    const size_t ntiles = (nchunk + kScanTile - 1) / kScanTile;
    if (cudaMemsetAsync(base, 0, 512, st) != cudaSuccess ||
        cudaMemsetAsync(base + lay.flags, 0, (ntiles + 1) * 4, st) != cudaSuccess ||
        cudaMemsetAsync(d_units, 0, cap_units * 4, st) != cudaSuccess)
        return MANS_ERR_CUDA;
    const size_t smem = 256 * sizeof(uint2) + (size_t) L * 2;
    const unsigned gc = (unsigned) ((nchunk + kEncThreads - 1) / kEncThreads);
    k_enc_g<<<gc, kEncThreads, smem, st>>>(p);
    if (nchunk > 1) k_enc_w<<<gc, kEncThreads, smem, st>>>(p);
    k_enc_scan<<<(unsigned) ntiles, kScanThreads, 0, st>>>(p);
    k_enc_total<<<1, 32, 0, st>>>(p);
    k_enc_final<<<(unsigned) ((nblk + kEncThreads - 1) / kEncThreads), kEncThreads, smem, st>>>(p);
    k_enc_tail<<<1, 32, 0, st>>>(p);
    return cudaGetLastError() == cudaSuccess ? MANS_OK : MANS_ERR_CUDA;
}

int mans_encode_result(const void* d_aux, void* stream, uint64_t* n_units, uint32_t* first_bit,
                       uint32_t* first_state, uint32_t* dev_status) {
    if (!d_aux) return MANS_ERR_ARG;
    cudaStream_t st = (cudaStream_t) stream;
    uint32_t status = 0;
    EncResult r;
    const char* base = (const char*) d_aux;
    if (cudaMemcpyAsync(&status, base, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&r, base + 256, sizeof(r), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return MANS_ERR_CUDA;
    if (dev_status) *dev_status = status;
    if (n_units) *n_units = r.n_units;
    if (first_bit) *first_bit = r.first_bit;
    if (first_state) *first_state = r.first_state;
    if (status & MANS_DEV_SYNC_OVERFLOW) return MANS_ERR_SYNC;
    if (status & (MANS_DEV_SCAN_TIMEOUT)) return MANS_ERR_CUDA;
    if (status & MANS_DEV_COUNT_MISMATCH) return MANS_ERR_AUX_SMALL;
    return MANS_OK;
}

int mans_encode_sync(const uint8_t* d_sym, size_t n, const uint32_t* d_enc_blob, uint32_t L,
                     uint32_t* d_units, size_t cap_units, void* d_aux, size_t aux_bytes,
                     void* stream, uint64_t* n_units, uint32_t* first_bit,
                     uint32_t* first_state) {
    // merges that outrun their slots: the same workspace holds 4x longer
    // chunks (fewer of them), so re-plan until the walks fit
    uint32_t chunk = 0;
    for (int attempt = 0; attempt < 8; ++attempt) {
        int rc = mans_encode(d_sym, n, d_enc_blob, L, d_units, cap_units, d_aux, aux_bytes, chunk,
                             stream);
        if (rc != MANS_OK) return rc;
        uint32_t dev = 0;
        rc = mans_encode_result(d_aux, stream, n_units, first_bit, first_state, &dev);
        if (rc != MANS_ERR_SYNC) return rc;
        const uint32_t cur = enc_chunk(n, chunk);
        if ((uint64_t) cur >= n) return rc;
        chunk = (uint32_t) std::min<uint64_t>((uint64_t) cur * 4, 1u << 30);
    }
    return MANS_ERR_SYNC;
}

int mans_histogram(const uint8_t* d_sym, size_t n, uint64_t* d_hist, void* stream) {
    if (!d_sym || !d_hist) return MANS_ERR_ARG;
    cudaStream_t st = (cudaStream_t) stream;
    if (cudaMemsetAsync(d_hist, 0, 256 * sizeof(uint64_t), st) != cudaSuccess) return MANS_ERR_CUDA;
    if (n == 0) return MANS_OK;
    const unsigned grid = (unsigned) std::min<size_t>((n + 256 * 1024 - 1) / (256 * 1024), 152 * 8);
    k_hist<<<grid, 256, 0, st>>>(d_sym, n, (unsigned long long*) d_hist);
    return cudaGetLastError() == cudaSuccess ? MANS_OK : MANS_ERR_CUDA;
}

}  // extern "C"
