// Plain single-stream decode: the reference's four phases (guessed-state
// decode, sync extension, exclusive prefix sum, final write pass) rebuilt
// as three sm_103a kernels that never stop for the host.
//
// Geometry.  The stream is cut into blocks of B units (final-pass work
// items) and regions of nb blocks (sync work items, R = nb * B units).
//
//  k_sync   one thread per region k.  It decodes region k from a guessed
//           start (bit 0 of the region, state = the stream's first state;
//           region 0 starts from the true start), the trajectory Gamma_k,
//           and records for every block of the region the first codeword
//           at or after the block start and Gamma_k's symbol count before
//           it.  It then keeps walking Gamma_k past the region end while
//           replaying Gamma_{k+1} (region k+1 from its guessed start) until
//           the two trajectories meet at the same bit position in the same
//           state: the merge point m_k.  Gamma_k's count minus
//           Gamma_{k+1}'s count at m_k is delta_k.  Blocks the walk crosses
//           before m_k get Gamma_k's records in walk slot (region - k).
//           This is the reference's sync extension
//           (src/multians_gpu_decoder.cu:251-261, 363-466) with the check
//           made at every codeword instead of at subsequence ends.
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
//
// No pass waits on another thread: correctness needs only that every walk
// ends inside its slots, which the host checks and cures by re-planning.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>

#include "mans_device.cuh"
#include "multians_gb300.h"

namespace mans {

struct DecodeParams {
    const uint32_t* units;
    uint8_t* out;
    const uint32_t* table;
    uint2* rec_g;          // [nblk]       Gamma_region records
    uint2* rec_w;          // [nblk*dmax]  walk records, slot d-1 = Gamma_{r-d}
    unsigned long long* m;      // [nreg] merge bit position (~0 = none)
    long long* delta;           // [nreg]
    unsigned long long* Mpre;   // [nreg] prefix max of m
    long long* Dpre;            // [nreg] prefix sum of delta
    uint32_t* status;
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
};

// record: x = bit offset from the block start | state index << 8; y = count
__device__ __forceinline__ uint2 make_rec(uint64_t pos, uint64_t bstart,
                                          uint32_t idx, uint32_t cnt) {
    return make_uint2((uint32_t) (pos - bstart) | (idx << 8), cnt);
}

__global__ void k_sync(DecodeParams p) {
    extern __shared__ uint32_t s_tbl[];
    int any_bad, all_loop;
    load_table(s_tbl, p.table, p.L, any_bad, all_loop);
    if (any_bad) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            atomicOr(p.status, all_loop ? MANS_DEV_DEGENERATE : MANS_DEV_BAD_TABLE);
        return;
    }
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= p.nreg) return;

    const uint64_t blk_bits = (uint64_t) p.B * 32;
    const uint32_t b0 = k * p.nb;
    const uint32_t b1 = min(b0 + p.nb, p.nblk);
    const uint64_t end_bits = (uint64_t) p.nblk * blk_bits;

    // Gamma_k inside region k
    BitCursor a;
    uint32_t ia;
    if (k == 0) {
        a.init(p.units, p.n_units, p.first_pos);
        ia = p.first_idx;
    } else {
        a.init(p.units, p.n_units, (uint64_t) b0 * blk_bits);
        ia = p.first_idx;
    }
    uint32_t ca = 0;
    for (uint32_t b = b0; b < b1; ++b) {
        const uint64_t bs = (uint64_t) b * blk_bits;
        const uint64_t be = bs + blk_bits;
        p.rec_g[b] = make_rec(a.pos, bs, ia, ca);
        while (a.pos < be) {
            a.step(s_tbl, ia);
            ++ca;
        }
    }
    if (k + 1 >= p.nreg) {
        p.m[k] = ~0ull;
        p.delta[k] = 0;
        return;
    }

    // walk: Gamma_k (cursor a) against a replay of Gamma_{k+1} (cursor g)
    BitCursor g;
    uint32_t ig = p.first_idx;
    g.init(p.units, p.n_units, (uint64_t) b1 * blk_bits);
    uint32_t cg = 0;
    uint32_t bn = b1;  // next block whose start cursor a has to record
    for (;;) {
        while (bn < p.nblk && a.pos >= (uint64_t) bn * blk_bits) {
            const uint32_t d = bn / p.nb - k;
            if (d > p.dmax) {
                atomicOr(p.status, MANS_DEV_SYNC_OVERFLOW);
                p.m[k] = ~0ull;
                p.delta[k] = 0;
                return;
            }
            p.rec_w[(size_t) bn * p.dmax + (d - 1)] =
                make_rec(a.pos, (uint64_t) bn * blk_bits, ia, ca);
            ++bn;
        }
        if (a.pos >= end_bits && g.pos >= end_bits) {
            // no merge before the stream end
            p.m[k] = ~0ull;
            p.delta[k] = 0;
            return;
        }
        if (a.pos == g.pos) {
            if (ia == ig) {
                p.m[k] = a.pos;
                p.delta[k] = (long long) ca - (long long) cg;
                return;
            }
            a.step(s_tbl, ia);
            ++ca;
            g.step(s_tbl, ig);
            ++cg;
        } else if (a.pos < g.pos) {
            a.step(s_tbl, ia);
            ++ca;
        } else {
            g.step(s_tbl, ig);
            ++cg;
        }
    }
}

// Exclusive prefix max of m (identity 0) and prefix sum of delta; one CTA.
__global__ void k_scan(DecodeParams p) {
    __shared__ unsigned long long s_max[1024];
    __shared__ long long s_sum[1024];
    const uint32_t T = blockDim.x, t = threadIdx.x;
    const uint32_t n = p.nreg;
    const uint32_t chunk = (n + T - 1) / T;
    const uint32_t lo = min(t * chunk, n), hi = min(lo + chunk, n);
    unsigned long long mx = 0;
    long long sm = 0;
    for (uint32_t i = lo; i < hi; ++i) {
        mx = max(mx, p.m[i]);
        sm += p.delta[i];
    }
    s_max[t] = mx;
    s_sum[t] = sm;
    __syncthreads();
    for (uint32_t off = 1; off < T; off <<= 1) {
        unsigned long long vm = 0;
        long long vs = 0;
        if (t >= off) {
            vm = s_max[t - off];
            vs = s_sum[t - off];
        }
        __syncthreads();
        if (t >= off) {
            s_max[t] = max(s_max[t], vm);
            s_sum[t] += vs;
        }
        __syncthreads();
    }
    unsigned long long run_m = t ? s_max[t - 1] : 0ull;
    long long run_s = t ? s_sum[t - 1] : 0ll;
    for (uint32_t i = lo; i < hi; ++i) {
        p.Mpre[i] = run_m;
        p.Dpre[i] = run_s;
        run_m = max(run_m, p.m[i]);
        run_s += p.delta[i];
    }
}

__global__ void k_final(DecodeParams p) {
    extern __shared__ uint32_t s_tbl[];
    int any_bad, all_loop;
    load_table(s_tbl, p.table, p.L, any_bad, all_loop);
    if (any_bad) {
        if (all_loop) {
            // single-symbol table: every state decodes that symbol
            const uint8_t sym = (uint8_t) (__ldg(p.table) >> 16);
            const unsigned long long stride = (unsigned long long) gridDim.x * blockDim.x;
            for (unsigned long long i = (unsigned long long) blockIdx.x * blockDim.x + threadIdx.x;
                 i < p.n_out; i += stride)
                p.out[i] = sym;
        }
        return;
    }
    if (*(volatile uint32_t*) p.status & MANS_DEV_SYNC_OVERFLOW) return;
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= p.nblk) return;

    const uint64_t blk_bits = (uint64_t) p.B * 32;
    const uint64_t bs = (uint64_t) b * blk_bits;
    const uint64_t be = bs + blk_bits;
    const uint32_t r = b / p.nb;
    uint32_t d = 0;
    for (;; ++d) {
        if (d > r || d > p.dmax) {
            atomicOr(p.status, MANS_DEV_SYNC_OVERFLOW);
            return;
        }
        if (p.Mpre[r - d] <= bs) break;
    }
    const uint32_t k = r - d;
    const uint2 rec = d == 0 ? p.rec_g[b] : p.rec_w[(size_t) b * p.dmax + (d - 1)];
    unsigned long long off = (unsigned long long) (p.Dpre[k] + (long long) rec.y);
    uint32_t idx = rec.x >> 8;
    BitCursor c;
    c.init(p.units, p.n_units, bs + (rec.x & 0xffu));
    while (c.pos < be) {
        const uint32_t e = c.step(s_tbl, idx);
        if (off < p.n_out) p.out[off] = (uint8_t) (e >> 24);
        ++off;
    }
}

// ---------------------------------------------------------------------------
// host side

struct AuxLayout {
    size_t rec_g, rec_w, m, delta, Mpre, Dpre, status, total;
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t) 255; }

static AuxLayout layout_for(size_t nblk, size_t nreg, size_t dmax) {
    AuxLayout a;
    size_t o = 0;
    a.status = o; o += 256;
    a.rec_g = o; o += align256(nblk * sizeof(uint2));
    a.rec_w = o; o += align256(nblk * dmax * sizeof(uint2));
    a.m = o; o += align256(nreg * 8);
    a.delta = o; o += align256(nreg * 8);
    a.Mpre = o; o += align256(nreg * 8);
    a.Dpre = o; o += align256(nreg * 8);
    a.total = o;
    return a;
}

static uint32_t pow2_floor(uint64_t x) {
    uint32_t r = 1;
    while ((uint64_t) r * 2 <= x && r < (1u << 30)) r *= 2;
    return r;
}

static thread_local uint32_t g_last_launches = 0;

}  // namespace mans

using namespace mans;

extern "C" {

const char* mans_version(void) { return "multians_gb300 0.1"; }

uint32_t mans_last_launch_count(void) { return g_last_launches; }

int mans_plan(size_t n_units, size_t n_out, uint32_t L, const mans_cfg* hint,
              mans_cfg* out) {
    if (!out || n_units == 0 || L < 2 || L > 32768) return MANS_ERR_ARG;
    mans_cfg c = {0, 0, 0, 0};
    if (hint) c = *hint;
    const double sym_per_unit = n_out ? (double) n_out / (double) n_units : 1.0;
    if (c.block_units == 0) {
        // about 128 symbols per block
        uint64_t b = (uint64_t) (128.0 / std::max(sym_per_unit, 1e-3));
        c.block_units = std::min<uint32_t>(std::max<uint32_t>(pow2_floor(std::max<uint64_t>(b, 1)), 4), 256);
    }
    if (c.region_blocks == 0) {
        uint64_t R = L <= 1024 ? 512 : 2048;  // units per sync region
        // keep at least ~4 regions per SM when the stream is small
        const uint64_t want_regions = 152ull * 4;
        while (R > 64 && n_units / R < want_regions) R /= 2;
        c.region_blocks = (uint32_t) std::max<uint64_t>(1, R / c.block_units);
    }
    if (c.walk_slots == 0) c.walk_slots = 4;
    if (c.threads == 0) c.threads = 128;
    *out = c;
    return MANS_OK;
}

size_t mans_aux_size(size_t n_units, const mans_cfg* cfg) {
    if (!cfg || cfg->block_units == 0 || cfg->region_blocks == 0 || cfg->walk_slots == 0)
        return 0;
    const size_t nblk = (n_units + cfg->block_units - 1) / cfg->block_units;
    const size_t nreg = (nblk + cfg->region_blocks - 1) / cfg->region_blocks;
    return layout_for(nblk, nreg, cfg->walk_slots).total;
}

size_t mans_aux_size_max(size_t n_units) {
    // smallest blocks (4 units), smallest regions (64 units), 8 slots
    mans_cfg c = {4, 16, 8, 128};
    return mans_aux_size(n_units, &c);
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

int mans_decode(const uint32_t* d_units, size_t n_units, uint8_t* d_out,
                size_t n_out, const uint32_t* d_table, uint32_t L,
                uint32_t first_state, uint32_t first_bit, void* d_aux,
                size_t aux_bytes, const mans_cfg* cfg_in, void* stream) {
    g_last_launches = 0;
    if (n_out == 0) return MANS_OK;
    if (!d_units || !d_out || !d_table || !d_aux || n_units == 0 ||
        n_units > 0xffffffffull || L < 2 || L > 32768 || first_state < L ||
        first_state >= 2 * L || first_bit > 32)
        return MANS_ERR_ARG;
    mans_cfg cfg;
    int rc = mans_plan(n_units, n_out, L, cfg_in, &cfg);
    if (rc != MANS_OK) return rc;
    const size_t nblk = (n_units + cfg.block_units - 1) / cfg.block_units;
    const size_t nreg = (nblk + cfg.region_blocks - 1) / cfg.region_blocks;
    const AuxLayout lay = layout_for(nblk, nreg, cfg.walk_slots);
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
    p.n_out = n_out;
    p.n_units = (uint32_t) n_units;
    p.L = L;
    p.first_idx = first_state - L;
    p.first_pos = 32 - first_bit;
    p.B = cfg.block_units;
    p.nb = cfg.region_blocks;
    p.dmax = cfg.walk_slots;
    p.nblk = (uint32_t) nblk;
    p.nreg = (uint32_t) nreg;

    if (cudaMemsetAsync(p.status, 0, sizeof(uint32_t), st) != cudaSuccess)
        return MANS_ERR_CUDA;
    const size_t smem = (size_t) L * sizeof(uint32_t);
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_sync, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
        cudaFuncSetAttribute(k_final, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
        attr_set = true;
    }
    const uint32_t T = cfg.threads;
    k_sync<<<(unsigned) ((nreg + T - 1) / T), T, smem, st>>>(p);
    k_scan<<<1, 1024, 0, st>>>(p);
    k_final<<<(unsigned) ((nblk + T - 1) / T), T, smem, st>>>(p);
    g_last_launches = 3;
    if (cudaGetLastError() != cudaSuccess) return MANS_ERR_CUDA;
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

int mans_decode_sync(const uint32_t* d_units, size_t n_units, uint8_t* d_out,
                     size_t n_out, const uint32_t* d_table, uint32_t L,
                     uint32_t first_state, uint32_t first_bit, void* d_aux,
                     size_t aux_bytes, const mans_cfg* hint, void* stream,
                     uint32_t* status_out) {
    mans_cfg c = {0, 0, 0, 0};
    if (hint) c = *hint;
    mans_cfg plan;
    uint32_t st = 0;
    for (int attempt = 0; attempt < 6; ++attempt) {
        int rc = mans_plan(n_units, n_out, L, &c, &plan);
        if (rc != MANS_OK) return rc;
        if (mans_aux_size(n_units, &plan) > aux_bytes) {
            // fewer slots fit in the same memory
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
        // a walk outran its slots: longer regions, same slot count
        c = plan;
        c.region_blocks = plan.region_blocks * 4;
    }
    if (status_out) *status_out = st;
    if (st & MANS_DEV_BAD_TABLE) return MANS_ERR_TABLE;
    if (st & MANS_DEV_SYNC_OVERFLOW) return MANS_ERR_SYNC;
    return MANS_OK;
}

}  // extern "C"
