/*
 * CPU oracle for the MULTIANS tANS decode path -- TEST INFRASTRUCTURE ONLY.
 * See mans_oracle.h for the formats and for who may load this file.
 *
 * Every function restates a reference algorithm and cites it (paths are
 * relative to the reference project root).  Where the reference relies on
 * undefined behaviour (32-bit shifts by >= 32 in the encoder flush and the
 * multicore decoder's start shift) this file spells out what x86-64 and
 * AArch64 hardware do for a variable shift: the count is taken modulo 32.
 * That is what the reference's compiled code does on x86 and Arm, and the
 * restated encoder is checked bit for bit against it.
 */
#include "mans_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------------- */
/* Hardware-style 32-bit shifts (count modulo 32).                         */

static inline uint32_t hshl(uint32_t x, uint64_t n) { return x << (n & 31u); }
static inline uint32_t hshr(uint32_t x, uint64_t n) { return x >> (n & 31u); }

/* Segment of source symbol i (segments in order; seg: the last answer, as
 * i only grows); past the end, the last segment. */
static inline size_t seg_of(const size_t* seg_end, size_t n_seg, size_t seg, uint64_t i) {
    while (seg + 1 < n_seg && i >= seg_end[seg]) ++seg;
    return seg;
}

/* ---------------------------------------------------------------------- */
/* Mersenne Twister generators (Matsumoto & Nishimura 1998; the 64-bit    */
/* variant of 2004), as std::mt19937 / std::mt19937_64 define them.       */

typedef struct { uint32_t mt[624]; int idx; } mt32_t;

static void mt32_seed(mt32_t* g, uint32_t s) {
    g->mt[0] = s;
    for (int i = 1; i < 624; ++i)
        g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t) i;
    g->idx = 624;
}

static uint32_t mt32_next(mt32_t* g) {
    if (g->idx >= 624) {
        for (int i = 0; i < 624; ++i) {
            uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
            uint32_t v = g->mt[(i + 397) % 624] ^ (y >> 1);
            if (y & 1u) v ^= 0x9908b0dfu;
            g->mt[i] = v;
        }
        g->idx = 0;
    }
    uint32_t y = g->mt[g->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

/* generate_canonical<double, 53> over a 32-bit engine, as the C++ standard
 * defines it ([rand.util.canonical]: k = 2 draws, S = g0 + g1 * 2^32,
 * result S / 2^64), with libstdc++'s clamp of a rounded-up 1.0 to the
 * largest double below 1.  This is what uniform_real_distribution<double>
 * (0, 1) returns in ans_table_generator.cc:106-119. */
static double mt32_canonical(mt32_t* g) {
    double sum = 0.0, tmp = 1.0;
    for (int i = 0; i < 2; ++i) {
        sum += (double) mt32_next(g) * tmp;
        tmp *= 4294967296.0;
    }
    double r = sum / tmp;
    if (r >= 1.0) r = nextafter(1.0, 0.0);
    return r;
}

typedef struct { uint64_t mt[312]; int idx; } mt64_t;

static void mt64_seed(mt64_t* g, uint64_t s) {
    g->mt[0] = s;
    for (int i = 1; i < 312; ++i)
        g->mt[i] = 6364136223846793005ull * (g->mt[i - 1] ^ (g->mt[i - 1] >> 62)) + (uint64_t) i;
    g->idx = 312;
}

static uint64_t mt64_next(mt64_t* g) {
    if (g->idx >= 312) {
        for (int i = 0; i < 312; ++i) {
            uint64_t y = (g->mt[i] & 0xffffffff80000000ull) | (g->mt[(i + 1) % 312] & 0x7fffffffull);
            uint64_t v = g->mt[(i + 156) % 312] ^ (y >> 1);
            if (y & 1u) v ^= 0xb5026f5aa96619e9ull;
            g->mt[i] = v;
        }
        g->idx = 0;
    }
    uint64_t y = g->mt[g->idx++];
    y ^= (y >> 29) & 0x5555555555555555ull;
    y ^= (y << 17) & 0x71d67fffeda60000ull;
    y ^= (y << 37) & 0xfff7eee000000000ull;
    y ^= y >> 43;
    return y;
}

/* The benchmark workloads' symbol generator: mt19937_64(seed), U = ((x >> 11)
 * + 1) * 2^-53 in (0, 1], symbol min(255, floor(-ln U / lambda)), an
 * exponential distribution of rate lambda like the reference demo's
 * (src/main.cc:46-61, which draws through generate_distribution and
 * generate_test_data instead; this portable form fixes the bytes for any
 * standard library). */
void mo_gen_symbols(uint64_t seed, double lambda, uint8_t* out, size_t n) {
    mt64_t g;
    mt64_seed(&g, seed);
    for (size_t i = 0; i < n; ++i) {
        uint64_t x = mt64_next(&g);
        double u = (double) ((x >> 11) + 1) * 0x1.0p-53;
        double v = -log(u) / lambda;
        out[i] = (v >= 255.0) ? 255 : (uint8_t) floor(v);
    }
}

/* ---------------------------------------------------------------------- */
/* Table generation.                                                       */

static int cmp_desc(const void* a, const void* b) {
    size_t x = *(const size_t*) a, y = *(const size_t*) b;
    return (x < y) - (x > y);
}

/* generate_distribution_from_buffer (ans_table_generator.cc:61-131).
 * Counts are sorted descending while the symbol list stays ascending, so
 * the i-th largest count pairs with the i-th smallest present byte
 * (ans_table_generator.cc:84-85); the float accumulators of lines 92 and
 * 99 are kept. */
static size_t distribution_from_buffer(uint32_t seed, size_t N,
                                       const uint8_t* in, size_t size,
                                       double* prob, size_t* counts,
                                       uint8_t* symbols) {
    uint32_t freq[256];
    memset(freq, 0, sizeof(freq));
    for (size_t i = 0; i < size; ++i) ++freq[in[i]];

    size_t K = 0;
    for (size_t i = 0; i < 256; ++i) {
        if (freq[i] != 0) {
            counts[K] = freq[i];
            symbols[K] = (uint8_t) i;
            ++K;
        }
    }
    qsort(counts, K, sizeof(size_t), cmp_desc);

    double prob_a[256];
    float acc = 0.0f;
    for (size_t i = 0; i < K; ++i) acc = acc + (float) counts[i];
    double sum_a = acc;
    for (size_t i = 0; i < K; ++i) prob_a[i] = (double) counts[i] / sum_a;
    for (size_t i = 0; i < K; ++i)
        if (prob_a[i] < 0.001) prob_a[i] += 0.001;
    acc = 0.0f;
    for (size_t i = 0; i < K; ++i) acc = (float) ((double) acc + prob_a[i]);
    sum_a = acc;
    for (size_t i = 0; i < K; ++i) prob[i] = prob_a[i] / sum_a;
    for (size_t i = 0; i < K; ++i) counts[i] = (size_t) ceil(prob[i] * (double) N);

    mt32_t g;
    mt32_seed(&g, seed);
    int isum = 0;   /* std::accumulate with an int initial value */
    for (size_t i = 0; i < K; ++i) isum = (int) ((size_t) isum + counts[i]);
    size_t del = (size_t) (long) isum - N;
    while (del > 0) {
        size_t idx = (size_t) floor(mt32_canonical(&g) * (double) K);
        mt32_canonical(&g);
        while (counts[idx] == 1) {
            idx = (size_t) floor(mt32_canonical(&g) * (double) K);
            mt32_canonical(&g);
        }
        --counts[idx];
        --del;
    }
    for (size_t i = 0; i < K; ++i) prob[i] = (double) counts[i] / (double) N;
    return K;
}

/* generate_table, symbols != nullptr branch (ans_table_generator.cc:164-259)
 * followed by generate_encoder_table (ans_table_generator.cc:290-314).
 * enc: 256 rows x L states x {next_state, code_sequence, code_length,
 * symbol}; rows of absent symbols stay zero. */
static void build_encoder_table(const double* P, const size_t* Ls,
                                const uint8_t* symbols, size_t K, uint32_t L,
                                uint32_t* enc) {
    double qp[256];
    uint8_t qs[256];
    uint32_t X[256];
    for (size_t i = 0; i < K; ++i) {
        qp[i] = 0.5 / P[i];
        qs[i] = symbols[i];
        X[i] = (uint32_t) Ls[i];
    }
    uint8_t* pre_s = (uint8_t*) malloc(L);
    uint32_t* pre_x = (uint32_t*) malloc(L * sizeof(uint32_t));
    for (uint32_t i = L; i < 2 * L; ++i) {
        size_t idx = 0;   /* std::min_element: first smallest */
        for (size_t j = 1; j < K; ++j)
            if (qp[j] < qp[idx]) idx = j;
        double v = qp[idx];
        qp[idx] = v + (1 / P[idx]);
        pre_s[i - L] = qs[idx];
        pre_x[i - L] = X[idx];
        X[idx] = X[idx] + 1;
    }
    memset(enc, 0, (size_t) 256 * L * 4 * sizeof(uint32_t));
    for (uint32_t i = L; i < 2 * L; ++i) {
        uint8_t symbol = pre_s[i - L];
        uint32_t slide = pre_x[i - L];
        uint32_t shift = 0;
        for (; slide < 2 * L; slide = slide * 2) {
            for (uint32_t rem = 0; rem < (1u << shift); ++rem) {
                if (L <= slide + rem && slide + rem < 2 * L) {
                    uint32_t* e = enc + ((size_t) symbol * L + (slide + rem - L)) * 4;
                    e[0] = i;
                    e[1] = rem;
                    e[2] = shift;
                    e[3] = symbol;
                }
            }
            ++shift;
        }
    }
    free(pre_s);
    free(pre_x);
}

/* get_decoder_table (ans_table_generator.cc:261-288) over the rows of the
 * present symbols only (the walk over absent all-zero rows at lines 270-283
 * indexes far out of bounds).  Returns -1 on an out-of-range entry. */
static int build_decoder_table(const uint32_t* enc, const uint8_t* present,
                               uint32_t L, uint32_t* dec) {
    memset(dec, 0, L * sizeof(uint32_t));
    for (size_t s = 0; s < 256; ++s) {
        if (!present[s]) continue;
        for (uint32_t j = 0; j < L; ++j) {
            const uint32_t* e = enc + (s * L + j) * 4;
            uint32_t prev = e[0] - L;
            uint32_t len = e[2];
            if (prev >= L) return -1;
            uint32_t next_state = (uint16_t) ((L + j) >> len);
            uint32_t old_bits = dec[prev] >> 24;
            uint32_t bits = (old_bits == 0 && len > 0) ? len : old_bits;
            dec[prev] = next_state | ((e[3] & 0xffu) << 16) | ((bits & 0xffu) << 24);
        }
    }
    return 0;
}

int mo_build_tables(const uint8_t* sym, size_t n, uint32_t L, uint32_t seed,
                    uint32_t* enc, uint32_t* dec, uint32_t* max_len) {
    if (L < 2 || L > 65536 || (L & (L - 1)) != 0 || n == 0) return -1;
    double prob[256];
    size_t counts[256];
    uint8_t symbols[256];
    size_t K = distribution_from_buffer(seed, L, sym, n, prob, counts, symbols);
    if (K > L) return -1;
    build_encoder_table(prob, counts, symbols, K, L, enc);
    uint8_t present[256];
    memset(present, 0, sizeof(present));
    for (size_t i = 0; i < K; ++i) present[symbols[i]] = 1;
    if (build_decoder_table(enc, present, L, dec) != 0) return -1;
    /* get_max_compressed_size reads row 255 at state L-1
     * (ans_table_generator.cc:323-324); an absent row 255 is replaced by
     * the present row with the longest code there. */
    uint32_t ml = 0;
    if (present[255]) {
        ml = enc[((size_t) 255 * L + (L - 1)) * 4 + 2];
    } else {
        for (size_t s = 0; s < 256; ++s)
            if (present[s]) {
                uint32_t len = enc[(s * L + (L - 1)) * 4 + 2];
                if (len >= ml) ml = len;
            }
    }
    *max_len = ml;
    return (int) K;
}

/* get_max_compressed_size (ans_table_generator.cc:316-333). */
size_t mo_max_units(uint32_t max_len, size_t n) {
    size_t size = ((size_t) max_len * n) / 8 + 1;
    return size % 4 == 0 ? size / 4 : size / 4 + 1;
}

/* ANSEncoder::encode_memory (ans_encoder.cc:13-72) into a zeroed buffer of
 * mo_max_units words, then the CUHDInputBuffer layout: units reversed and
 * four zero units appended (multians_input_buffer.cc:15-30). */
size_t mo_encode(const uint32_t* enc, uint32_t L, uint32_t max_len,
                 const uint8_t* in, size_t size_in, uint32_t* units,
                 size_t cap, uint32_t* first_bit, uint32_t* first_state) {
    const size_t size_out = mo_max_units(max_len, size_in);
    uint32_t* out = (uint32_t*) calloc(size_out ? size_out : 1, sizeof(uint32_t));
    if (!out) return 0;
    const uint64_t max_bits = 32;
    (void) L;

    uint32_t window = 0, state = 0, final_state = 0;
    uint64_t final_bit = 0, final_size = 0, at = 0, in_unit = 0;

    for (size_t i = 0; i < size_out && in_unit < size_in + 1; ++i) {
        const uint32_t* e = enc + ((size_t) in[in_unit] * L + state) * 4;
        state = e[0] - L;
        uint32_t rem = e[1];
        uint64_t shift = e[2];
        while (at + shift < max_bits && in_unit < size_in) {
            window = hshl(window, shift);
            window += rem;
            at += shift;
            ++in_unit;
            if (in_unit < size_in) {
                e = enc + ((size_t) in[in_unit] * L + state) * 4;
                state = e[0] - L;
                rem = e[1];
                shift = e[2];
            }
            final_state = e[0];
        }
        const uint64_t diff = at + shift - max_bits;   /* wraps at the end */
        final_bit = at;
        final_size = i;
        window = hshl(window, shift - diff);
        window += hshr(rem, diff);
        out[i] = window;
        window = rem & ~hshl(~0u, diff);
        at = diff;
        ++in_unit;
    }

    const size_t size = (size_t) final_size + 1;
    if (size + 4 > cap) { free(out); return 0; }
    for (size_t i = 0; i < size; ++i) units[i] = out[size - 1 - i];
    for (size_t i = 0; i < 4; ++i) units[size + i] = 0;
    *first_bit = (uint32_t) final_bit;
    *first_state = final_state;
    free(out);
    return size;
}

/* Multi-table streams (the reference names multi-table decoding as future
 * work, README.md:11, and defines no format for it).  The encoder above
 * with the encoder table chosen per source symbol by the segment the symbol
 * belongs to: segment j holds source symbols [seg_end[j-1], seg_end[j]),
 * all tables have L states, and the state carries over from one segment to
 * the next, so the stream is one bitstream with one first state and bit.
 * The look-ahead byte past the end is encoded with the last segment's
 * table. */
size_t mo_encode_segments(const uint32_t* const* encs, const size_t* seg_end, size_t n_seg,
                          uint32_t L, uint32_t max_len, const uint8_t* in, size_t size_in,
                          uint32_t* units, size_t cap, uint32_t* first_bit,
                          uint32_t* first_state) {
    if (n_seg == 0 || seg_end[n_seg - 1] != size_in) return 0;
    const size_t size_out = mo_max_units(max_len, size_in);
    uint32_t* out = (uint32_t*) calloc(size_out ? size_out : 1, sizeof(uint32_t));
    if (!out) return 0;
    const uint64_t max_bits = 32;
    size_t seg = 0;
#define SEG_ENC(i) (encs[(seg = seg_of(seg_end, n_seg, seg, (i)))])
    uint32_t window = 0, state = 0, final_state = 0;
    uint64_t final_bit = 0, final_size = 0, at = 0, in_unit = 0;

    for (size_t i = 0; i < size_out && in_unit < size_in + 1; ++i) {
        const uint32_t* e = SEG_ENC(in_unit) + ((size_t) in[in_unit] * L + state) * 4;
        state = e[0] - L;
        uint32_t rem = e[1];
        uint64_t shift = e[2];
        while (at + shift < max_bits && in_unit < size_in) {
            window = hshl(window, shift);
            window += rem;
            at += shift;
            ++in_unit;
            if (in_unit < size_in) {
                e = SEG_ENC(in_unit) + ((size_t) in[in_unit] * L + state) * 4;
                state = e[0] - L;
                rem = e[1];
                shift = e[2];
            }
            final_state = e[0];
        }
        const uint64_t diff = at + shift - max_bits;
        final_bit = at;
        final_size = i;
        window = hshl(window, shift - diff);
        window += hshr(rem, diff);
        out[i] = window;
        window = rem & ~hshl(~0u, diff);
        at = diff;
        ++in_unit;
    }
#undef SEG_ENC
    const size_t size = (size_t) final_size + 1;
    if (size + 4 > cap) { free(out); return 0; }
    for (size_t i = 0; i < size; ++i) units[i] = out[size - 1 - i];
    for (size_t i = 0; i < 4; ++i) units[size + i] = 0;
    *first_bit = (uint32_t) final_bit;
    *first_state = final_state;
    free(out);
    return size;
}

/* CUHDOutputBuffer::reverse (src/multians_output_buffer.cc:27-29): the
 * decoder writes symbols newest first. */
void mo_reverse_bytes(uint8_t* buf, size_t n) {
    for (size_t i = 0, j = n ? n - 1 : 0; i < j; ++i, --j) {
        uint8_t t = buf[i];
        buf[i] = buf[j];
        buf[j] = t;
    }
}

/* ---------------------------------------------------------------------- */
/* Sequential decode (the per-symbol step of decode_subsequence,           */
/* src/multians_gpu_decoder.cu:127-169, run from the stream start).        */

static inline uint32_t unit_at(const uint32_t* u, size_t n, uint64_t i) {
    return i < n ? u[i] : 0u;
}

/* k (<= 32) stream bits starting at bit position p, LSB first. */
static inline uint32_t read_bits(const uint32_t* u, size_t n, uint64_t p, uint32_t k) {
    uint64_t w = (uint64_t) unit_at(u, n, p >> 5) | ((uint64_t) unit_at(u, n, (p >> 5) + 1) << 32);
    w >>= (p & 31);
    return k == 0 ? 0u : (uint32_t) (w & (0xffffffffull >> (32 - k)));
}

/* One decode step from state x at bit position *p: returns the table word
 * of x and advances x and *p. */
static inline uint32_t step(const uint32_t* u, size_t n, const uint32_t* dec,
                            uint32_t L, uint32_t* x, uint64_t* p) {
    const uint32_t hit = dec[*x - L];
    uint32_t k = hit >> 24;
    uint32_t s = ((hit & 0xffffu) << k) | read_bits(u, n, *p, k);
    while (s < L) {   /* never taken for tables from the generator */
        s = (s << 1) | read_bits(u, n, *p + k, 1);
        ++k;
    }
    *x = s;
    *p += k;
    return hit;
}

int mo_decode_seq(const uint32_t* units, size_t n_units, uint32_t first_bit,
                  uint32_t first_state, const uint32_t* dec, uint32_t L,
                  uint8_t* out, size_t n_out) {
    uint32_t x = first_state;
    uint64_t p = 32 - (uint64_t) first_bit;
    uint64_t last_p = p, zero_run = 0;
    if (x < L || x >= 2 * L) return -1;
    for (size_t i = 0; i < n_out; ++i) {
        uint32_t hit = step(units, n_units, dec, L, &x, &p);
        out[i] = (uint8_t) (hit >> 16);
        if (p == last_p) {
            if (++zero_run > L) return -1;
        } else {
            zero_run = 0;
            last_p = p;
        }
        if (x < L || x >= 2 * L) return -1;
    }
    return 0;
}

/* Sequential decode of a multi-table stream: counts[j] symbols with
 * decs[j] for the segments in decode order (the source's last segment
 * first), the state carried across; starts[j] receives the bit position of
 * segment j's first codeword. */
int mo_decode_segments(const uint32_t* units, size_t n_units, uint32_t first_bit,
                       uint32_t first_state, const uint32_t* const* decs, const size_t* counts,
                       size_t n_seg, uint32_t L, uint8_t* out, uint64_t* starts) {
    uint32_t x = first_state;
    uint64_t p = 32 - (uint64_t) first_bit;
    size_t o = 0;
    if (x < L || x >= 2 * L) return -1;
    for (size_t j = 0; j < n_seg; ++j) {
        starts[j] = p;
        uint64_t last_p = p, zero_run = 0;
        for (size_t i = 0; i < counts[j]; ++i) {
            uint32_t hit = step(units, n_units, decs[j], L, &x, &p);
            out[o++] = (uint8_t) (hit >> 16);
            if (p == last_p) {
                if (++zero_run > L) return -1;
            } else {
                zero_run = 0;
                last_p = p;
            }
            if (x < L || x >= 2 * L) return -1;
        }
    }
    return 0;
}

int mo_sync_points(size_t S, const uint32_t* units, size_t n_units,
                   uint32_t first_bit, uint32_t first_state,
                   const uint32_t* dec, uint32_t L, uint32_t* sp) {
    if (S == 0 || n_units == 0) return -1;
    const size_t nsub = (n_units + S - 1) / S;
    const uint64_t end_bit = (uint64_t) nsub * S * 32;
    uint32_t x = first_state;
    uint64_t p = 32 - (uint64_t) first_bit;
    uint64_t last_p = p, zero_run = 0;
    if (x < L || x >= 2 * L) return -1;
    memset(sp, 0, nsub * 4 * sizeof(uint32_t));
    while (p < end_bit) {
        const uint64_t u = p >> 5;
        const size_t i = (size_t) (u / S);
        sp[4 * i + 0] = (uint32_t) (u - (uint64_t) i * S);
        sp[4 * i + 1] = (uint32_t) (p & 31);
        sp[4 * i + 3] = x;
        sp[4 * i + 2] += 1;
        step(units, n_units, dec, L, &x, &p);
        if (p == last_p) {
            if (++zero_run > L) return -1;
        } else {
            zero_run = 0;
            last_p = p;
        }
        if (x < L || x >= 2 * L) return -1;
    }
    uint32_t run = 0;   /* exclusive prefix, 32-bit like the reference */
    for (size_t i = 0; i < nsub; ++i) {
        uint32_t c = sp[4 * i + 2];
        sp[4 * i + 2] = run;
        run += c;
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* Multicore decoder (src/multicore_decoder.cc).                           */

typedef struct { uint32_t state, bit, unit, num_symbols; } mc_sync_t;

typedef struct {
    size_t thread_id, begin, end, subsequence, subsequence_size, num_units,
        num_threads;
    size_t* out_positions;
    uint8_t* out;
    size_t size_out;
    const uint32_t* in;
    size_t in_len;           /* readable units: data + 4 padding */
    uint32_t first_bit, first_state;
    const uint32_t* table;
    uint32_t number_of_states;
    mc_sync_t* sync;
    volatile uint8_t* thread_synced;
    volatile int* stuck;     /* set when a zero-bit run exceeds L steps */
    int overflow, write;
} mc_args_t;

/* A run of more than L zero-bit steps can only come from a zero-bit cycle
 * (a single-symbol table); the reference loops forever there, the port
 * stops the thread and reports it. */
static inline int taken_guard(uint32_t* zero_run, uint32_t L, volatile int* stuck) {
    if (*zero_run > L) {
        *stuck = 1;
        return 1;
    }
    return 0;
}

/* MulticoreDecoder::decode_phase1 (multicore_decoder.cc:92-273). */
static void* mc_decode_phase1(void* arg) {
    const mc_args_t* a = (const mc_args_t*) arg;
    const size_t thread_id = a->thread_id;
    if (a->overflow && a->thread_synced[thread_id]) return NULL;

    uint8_t* out_ptr = a->out;
    const uint32_t* in = a->in;
    const size_t in_len = a->in_len;
    const uint32_t* table = a->table;
    mc_sync_t* sync = a->sync;
    const uint32_t L = a->number_of_states;
    const uint32_t bits_in_unit = 32;
    const size_t S = a->subsequence_size;

    uint32_t current_state = a->first_state;
    uint32_t at = (thread_id == 0) ? bits_in_unit - a->first_bit : 0;
    size_t in_pos = a->begin;
    size_t out_pos = 0, out_size = 0;
    size_t current_subsequence = a->subsequence;
    uint32_t current_unit = 0;

    if (a->overflow || (a->write && thread_id > 0)) {
        mc_sync_t sp = sync[current_subsequence - 1];
        current_state = sp.state;
        at = sp.bit;
        in_pos -= S;
        in_pos += sp.unit;
        current_unit = sp.unit;
    }
    if (a->write) {
        out_pos = a->out_positions[thread_id];
        out_size = (thread_id < a->num_threads - 1)
            ? a->out_positions[thread_id + 1] : a->size_out;
    }

    uint32_t window = unit_at(in, in_len, in_pos);
    uint32_t next = unit_at(in, in_len, in_pos + 1);
    const uint32_t mask = ~0u;
    uint32_t last_state = 0, last_bit = 0;
    int reset = a->write && thread_id == 0;

    uint32_t copy_next = next;
    copy_next = hshl(copy_next, bits_in_unit - at);
    next = hshr(next, at);
    window = hshr(window, at);
    window += copy_next;

    uint32_t num_symbols = 0;
    uint32_t zero_run = 0;   /* termination guard, not in the reference */
    while (in_pos < a->end) {
        while (at < bits_in_unit) {
            if (taken_guard(&zero_run, L, a->stuck)) return NULL;
            last_state = current_state;
            const uint32_t hit = table[current_state - L];
            const uint32_t next_state = hit & 0xffffu;
            uint32_t taken = hit >> 24;
            ++num_symbols;
            uint32_t reversed = ~hshl(mask, taken) & window;
            current_state = hshl(next_state, taken) + reversed;
            while (current_state < L) {
                const uint32_t sh = hshr(window, taken);
                ++taken;
                current_state = (current_state << 1) + (1u & sh);
            }
            if (a->write && reset && out_pos < out_size) {
                out_ptr[out_pos] = (uint8_t) (hit >> 16);
                ++out_pos;
            }
            copy_next = taken > 0 ? hshl(next, bits_in_unit - taken) : 0u;
            last_bit = at;
            next = hshr(next, taken);
            window = hshr(window, taken);
            at += taken;
            window += copy_next;
            zero_run = taken ? 0 : zero_run + 1;
        }
        ++in_pos;
        ++current_unit;
        if (current_unit == S) {
            if (a->overflow && reset) {
                mc_sync_t sp = sync[current_subsequence];
                if (sp.state == last_state && sp.bit == last_bit &&
                    sp.unit == current_unit - 1) {
                    sync[current_subsequence].num_symbols = num_symbols;
                    a->thread_synced[thread_id] = 1;
                    return NULL;
                }
            }
            if (!a->overflow || reset) {
                if (!a->write) {
                    mc_sync_t v = {last_state, last_bit, current_unit - 1, num_symbols};
                    sync[current_subsequence] = v;
                }
                ++current_subsequence;
            }
            if (a->overflow && in_pos > a->num_units) a->thread_synced[thread_id] = 1;
            reset = 1;
            current_unit = 0;
            num_symbols = 0;
        }
        window = unit_at(in, in_len, in_pos);
        next = unit_at(in, in_len, in_pos + 1);
        if (at == bits_in_unit) {
            at = 0;
        } else {
            at -= bits_in_unit;
            window = hshr(window, at);
            next = hshr(next, at);
            uint32_t cn = unit_at(in, in_len, in_pos + 1);
            cn = hshl(cn, bits_in_unit - at);
            window += cn;
        }
    }
    return NULL;
}

int mo_multicore_decode(size_t S, size_t T, const uint32_t* units,
                        size_t n_units, uint32_t first_bit,
                        uint32_t first_state, const uint32_t* dec, uint32_t L,
                        uint8_t* out, size_t n_out) {
    if (S == 0 || T == 0 || n_units == 0) return -1;
    /* get_decoder_intervals (multicore_decoder.cc:275-303) */
    size_t nsub = n_units / S;
    size_t rem = n_units % S;
    if (rem != 0) ++nsub;
    if (nsub < T) return -1;
    const size_t spt = nsub / T;
    const size_t remaining_subs = nsub % T;

    volatile int stuck = 0;
    mc_sync_t* sync = (mc_sync_t*) calloc(nsub, sizeof(mc_sync_t));
    size_t* out_positions = (size_t*) calloc(T, sizeof(size_t));
    uint8_t* synced = (uint8_t*) calloc(T, 1);
    mc_args_t* args = (mc_args_t*) calloc(T, sizeof(mc_args_t));
    pthread_t* th = (pthread_t*) calloc(T, sizeof(pthread_t));
    if (!sync || !out_positions || !synced || !args || !th) {
        free(sync); free(out_positions); free(synced); free(args); free(th);
        return -1;
    }
    size_t at = 0;
    for (size_t i = 0; i < T; ++i) {
        mc_args_t* a = &args[i];
        a->thread_id = i;
        a->begin = at;
        a->end = spt * S + at;
        a->subsequence = spt * i;
        at += spt * S;
        a->subsequence_size = S;
        a->num_units = n_units;
        a->num_threads = T;
        a->out_positions = out_positions;
        a->out = out;
        a->size_out = n_out;
        a->in = units;
        a->in_len = n_units;   /* units past the data read as the zero padding */
        a->first_bit = first_bit;
        a->first_state = first_state;
        a->table = dec;
        a->number_of_states = L;
        a->sync = sync;
        a->thread_synced = synced;
        a->stuck = &stuck;
    }
    args[T - 1].end += remaining_subs * S;

    /* pass 1: guessed-state decode of every interval (lines 43-53) */
    for (size_t i = 0; i < T; ++i) {
        args[i].overflow = 0; args[i].write = 0;
        pthread_create(&th[i], NULL, mc_decode_phase1, &args[i]);
    }
    for (size_t i = 0; i < T; ++i) pthread_join(th[i], NULL);

    /* seam repair until every seam is synchronised (lines 55-75) */
    int passes = 0;
    int synchronized = 0;
    while (!synchronized) {
        ++passes;
        for (size_t i = 1; i < T; ++i) {
            args[i].overflow = 1; args[i].write = 0;
            pthread_create(&th[i], NULL, mc_decode_phase1, &args[i]);
        }
        for (size_t i = 1; i < T; ++i) pthread_join(th[i], NULL);
        synchronized = 1;
        for (size_t i = 1; i < T; ++i)
            if (!synced[i]) synchronized = 0;
        if (stuck || passes > (int) T + 1) break;   /* cannot happen on valid input */
    }

    /* prefix_sum (lines 305-333) */
    {
        size_t pos = 0, nxt = spt;
        uint32_t sum = 0;
        out_positions[0] = 0;
        for (size_t i = 1; i < T; ++i) {
            for (; pos < nxt; ++pos) sum += sync[pos].num_symbols;
            out_positions[i] = sum;
            pos = nxt;
            nxt += spt;
        }
    }

    /* write pass (lines 79-89) */
    for (size_t i = 0; i < T; ++i) {
        args[i].overflow = 0; args[i].write = 1;
        pthread_create(&th[i], NULL, mc_decode_phase1, &args[i]);
    }
    for (size_t i = 0; i < T; ++i) pthread_join(th[i], NULL);

    free(sync); free(out_positions); free(synced); free(args); free(th);
    return stuck ? -2 : passes;
}
