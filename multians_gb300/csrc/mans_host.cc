// Host side of the reference API: data model (CUHDCodetable,
// CUHDInputBuffer, CUHDOutputBuffer), tANS table generation
// (ANSTableGenerator), the single-state encoder (ANSEncoder), CUHDUtil, and
// the C entry points that expose encoding to non-C++ callers.
//
// Results are bit-identical to the reference's on every input the reference
// handles (checked against the reference build by the test suite); the
// float accumulators, the normalisation draws and the encoder's flush are
// kept as the reference has them because they decide the table and the
// stream bits.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <functional>
#include <iostream>
#include <numeric>
#include <random>
#include <vector>

#include <cuda_runtime.h>

#include "ans_encoder.h"
#include "ans_table_generator.h"
#include "cuhd_codetable.h"
#include "cuhd_input_buffer.h"
#include "cuhd_output_buffer.h"
#include "cuhd_util.h"
#include "multians_gb300.h"

// ---------------------------------------------------------------------------
// data model (src/multians_codetable.cc, multians_input_buffer.cc,
// multians_output_buffer.cc)

CUHDCodetable::CUHDCodetable(size_t num_entries)
    : size_(num_entries), num_entries_(num_entries),
      table_(new CUHDCodetableItem[num_entries]()) {}

size_t CUHDCodetable::get_size() { return size_; }
size_t CUHDCodetable::get_num_entries() { return num_entries_; }
size_t CUHDCodetable::get_max_codeword_length() { return MAX_CODEWORD_LENGTH; }
CUHDCodetableItem* CUHDCodetable::get() { return table_.get(); }

CUHDInputBuffer::CUHDInputBuffer(UNIT_TYPE* buffer, size_t size, size_t first_bit,
                                 size_t first_state)
    : first_bit_(first_bit), first_state_(first_state), compressed_size_(size),
      buffer_(new UNIT_TYPE[size + 4]()) {
    // units in reverse order, then four zero units the decoder may read
    std::reverse_copy(buffer, buffer + size, buffer_.get());
}

UNIT_TYPE* CUHDInputBuffer::get_compressed_data() { return buffer_.get(); }
size_t CUHDInputBuffer::get_first_bit() { return first_bit_; }
size_t CUHDInputBuffer::get_first_state() { return first_state_; }
size_t CUHDInputBuffer::get_compressed_size() { return compressed_size_; }
size_t CUHDInputBuffer::get_unit_size() { return unit_size_; }

CUHDOutputBuffer::CUHDOutputBuffer(size_t size)
    : uncompressed_size_(size), buffer_(new SYMBOL_TYPE[size]()) {}

std::shared_ptr<SYMBOL_TYPE[]>& CUHDOutputBuffer::get_decompressed_data() { return buffer_; }
void CUHDOutputBuffer::reverse() {
    std::reverse(buffer_.get(), buffer_.get() + uncompressed_size_);
}
size_t CUHDOutputBuffer::get_uncompressed_size() { return uncompressed_size_; }
size_t CUHDOutputBuffer::get_symbol_size() { return symbol_size_; }

// ---------------------------------------------------------------------------
// CUHDUtil (src/multians_util.cc)

std::pair<std::string, size_t> cuhd::CUHDUtil::time(std::string s, std::function<void()> f) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a);
    f();
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return {s, (size_t) (ms * 1000.0f)};
}

bool cuhd::CUHDUtil::equals(SYMBOL_TYPE* a, SYMBOL_TYPE* b, size_t size) {
    for (size_t i = 0; i < size; ++i) {
        if (a[i] != b[i]) {
            std::cout << "mismatch at: " << i << std::endl;
            return false;
        }
    }
    return true;
}

size_t cuhd::CUHDUtil::optimal_subsequence_size(size_t input_size, size_t output_size,
                                                size_t pref, size_t device_pref) {
    // halve the preferred size while subsequences per output symbol stay
    // below 1 / device_pref (src/multians_util.cc:74-86)
    const float device = 1.0f / (float) device_pref;
    size_t cur = pref;
    while (cur > 1 &&
           (float) SDIV(SDIV(input_size, 4), cur) / (float) SDIV(output_size, 4) < device)
        cur = SDIV(cur, 2);
    return cur;
}

// ---------------------------------------------------------------------------
// table generation (src/ans_table_generator.cc)

namespace {

// Brings the quantised counts down to exactly N by random unit decrements
// of counts above one (ans_table_generator.cc:39-52, 106-123).
void normalise_counts(std::vector<size_t>& counts, size_t N, size_t seed) {
    std::mt19937 engine(seed);
    std::uniform_real_distribution<double> draw(0.0, 1.0);
    const size_t K = counts.size();
    int total = 0;   // the reference sums with an int accumulator
    for (size_t c : counts) total = (int) (total + c);
    size_t excess = (size_t) total - N;
    auto pick = [&]() {
        size_t i = (size_t) std::floor(draw(engine) * (double) K);
        draw(engine);   // every pick consumes two draws
        return i;
    };
    while (excess > 0) {
        size_t i = pick();
        while (counts.at(i) == 1) i = pick();
        --counts.at(i);
        --excess;
    }
}

}  // namespace

Distribution ANSTableGenerator::generate_distribution(size_t seed, size_t n, size_t N,
                                                      std::function<double(double)> fun) {
    std::vector<double> prob(n);
    for (size_t i = 0; i < n; ++i) {
        double x = fun((double) i);
        prob[i] = x < 0.001 ? x + 0.001 : x;
    }
    float total = 0.0f;
    for (double x : prob) total = (float) ((double) total + x);
    for (double& x : prob) x = x / (double) total;
    std::vector<size_t> counts(n);
    for (size_t i = 0; i < n; ++i) counts[i] = (size_t) std::ceil(prob[i] * (double) N);
    normalise_counts(counts, N, seed);
    std::vector<double> prob_ans(n);
    for (size_t i = 0; i < n; ++i) prob_ans[i] = (double) counts[i] / (double) N;
    return {std::make_shared<std::vector<double>>(std::move(prob_ans)),
            std::make_shared<std::vector<size_t>>(std::move(counts)), nullptr};
}

Distribution ANSTableGenerator::generate_distribution_from_buffer(size_t seed, size_t N,
                                                                  std::uint8_t* in,
                                                                  size_t size) {
    std::array<std::uint64_t, 256> hist{};
    for (size_t i = 0; i < size; ++i) ++hist[in[i]];
    return generate_distribution_from_histogram(seed, N, hist.data());
}

// The distribution depends on the buffer only through its byte histogram
// (src/ans_table_generator.cc:61-100 counts, then normalises), so a
// histogram taken elsewhere (on the GPU) gives the same table.
Distribution ANSTableGenerator::generate_distribution_from_histogram(size_t seed, size_t N,
                                                                     const std::uint64_t* hist) {
    std::vector<size_t> counts;
    std::vector<SYMBOL_TYPE> symbols;
    for (size_t v = 0; v < 256; ++v) {
        if (hist[v]) {
            counts.push_back(hist[v]);
            symbols.push_back((SYMBOL_TYPE) v);
        }
    }
    // Only the counts are sorted: the i-th largest count goes with the i-th
    // smallest occurring byte, as in the reference (lines 84-85).
    std::sort(counts.begin(), counts.end(), std::greater<size_t>());
    const size_t K = counts.size();

    float total = 0.0f;
    for (size_t c : counts) total = total + (float) c;
    std::vector<double> prob(K);
    for (size_t i = 0; i < K; ++i) {
        double x = (double) counts[i] / (double) total;
        prob[i] = x < 0.001 ? x + 0.001 : x;
    }
    float total2 = 0.0f;
    for (double x : prob) total2 = (float) ((double) total2 + x);
    for (double& x : prob) x = x / (double) total2;
    for (size_t i = 0; i < K; ++i) counts[i] = (size_t) std::ceil(prob[i] * (double) N);
    normalise_counts(counts, N, seed);
    for (size_t i = 0; i < K; ++i) prob[i] = (double) counts[i] / (double) N;
    return {std::make_shared<std::vector<double>>(std::move(prob)),
            std::make_shared<std::vector<size_t>>(std::move(counts)),
            std::make_shared<std::vector<SYMBOL_TYPE>>(std::move(symbols))};
}

std::shared_ptr<std::vector<SYMBOL_TYPE>> ANSTableGenerator::generate_test_data(
    std::shared_ptr<std::vector<size_t>> distr, size_t size, size_t num_states, size_t seed) {
    // symbol i fills distr[i] of the num_states slots; draws pick slots
    std::vector<SYMBOL_TYPE> slots;
    slots.reserve(num_states);
    for (size_t i = 0; i < distr->size(); ++i)
        slots.insert(slots.end(), distr->at(i), (SYMBOL_TYPE) i);
    slots.resize(num_states, 0);
    std::vector<SYMBOL_TYPE> out(size + 8, 0);
    std::mt19937 engine(seed);
    std::uniform_int_distribution<size_t> draw(0, num_states - 1);
    for (size_t i = 0; i < size; ++i) {
        out[i] = slots[draw(engine)];
        draw(engine);
    }
    return std::make_shared<std::vector<SYMBOL_TYPE>>(std::move(out));
}

std::shared_ptr<std::vector<std::vector<Encoder_Table_Entry>>> ANSTableGenerator::generate_table(
    std::shared_ptr<std::vector<double>> P_s, std::shared_ptr<std::vector<size_t>> L_s,
    std::shared_ptr<std::vector<SYMBOL_TYPE>> symbols, size_t num_symbols, size_t num_states) {
    const size_t L = num_states;
    // Spread: state L + i goes to the queue entry with the smallest key
    // (first one on ties); an entry's key starts at 0.5 / p and grows by
    // 1 / p per state it takes, so each symbol gets exactly its count
    // (ans_table_generator.cc:170-234).
    std::vector<double> key(num_symbols);
    std::vector<SYMBOL_TYPE> sym_of(num_symbols);
    std::vector<std::uint32_t> x_next(num_symbols);
    for (size_t i = 0; i < num_symbols; ++i) {
        key[i] = 0.5 / P_s->at(i);
        sym_of[i] = symbols ? symbols->at(i) : (SYMBOL_TYPE) i;
        x_next[i] = (std::uint32_t) L_s->at(i);
    }
    std::vector<XS_pair> spread(L);
    for (size_t i = 0; i < L; ++i) {
        size_t q = (size_t) (std::min_element(key.begin(), key.end()) - key.begin());
        // in the symbol-less branch the reference steps the symbol's own
        // key, which is the same queue entry
        key[q] = key[q] + 1.0 / P_s->at(symbols ? q : sym_of[q]);
        spread[i] = {sym_of[q], x_next[q]++};
    }
    const size_t rows = symbols ? (size_t) 1 << (8 * sizeof(SYMBOL_TYPE)) : num_symbols;
    std::vector<std::vector<Encoder_Table_Entry>> table(rows,
                                                        std::vector<Encoder_Table_Entry>(L));
    // Encoding symbol s from state X in [L, 2L) shifts out the k low bits
    // with X >> k == x_s (the spread position's count index) and moves to
    // that spread state (ans_table_generator.cc:236-255).
    for (std::uint32_t i = 0; i < L; ++i) {
        const SYMBOL_TYPE s = spread[i].s;
        std::uint32_t shift = 0;
        for (std::uint64_t slide = spread[i].next_state; slide < 2 * L; slide *= 2, ++shift) {
            const std::uint64_t lo = std::max<std::uint64_t>(slide, L);
            const std::uint64_t hi = std::min<std::uint64_t>(slide + (1ull << shift), 2 * L);
            for (std::uint64_t X = lo; X < hi; ++X)
                table.at(s).at(X - L) = {(std::uint32_t) (L + i), (std::uint32_t) (X - slide),
                                         shift, s};
        }
    }
    return std::make_shared<std::vector<std::vector<Encoder_Table_Entry>>>(std::move(table));
}

std::shared_ptr<ANSEncoderTable> ANSTableGenerator::generate_encoder_table(
    std::shared_ptr<std::vector<std::vector<Encoder_Table_Entry>>> tab) {
    auto enc = std::make_shared<ANSEncoderTable>();
    enc->number_of_states = tab->at(0).size();
    enc->max_number_of_symbols = (size_t) 1 << (8 * sizeof(SYMBOL_TYPE));
    enc->number_of_symbols = tab->size();
    enc->table.resize(tab->size());
    for (size_t s = 0; s < tab->size(); ++s) {
        enc->table[s].reserve(enc->number_of_states);
        for (const Encoder_Table_Entry& e : tab->at(s))
            enc->table[s].push_back({e.x, e.rem, e.shift, e.symbol});
    }
    return enc;
}

namespace {
// A row is in use iff its entries point into [L, 2L); rows of absent byte
// values are all zero.
bool row_in_use(const std::vector<ANSEncoderTable::ANSEncoderTableItem>& row, size_t L) {
    return !row.empty() && row[0].next_state >= L;
}
}  // namespace

std::shared_ptr<CUHDCodetable> ANSTableGenerator::get_decoder_table(
    std::shared_ptr<ANSEncoderTable> enc_table) {
    const size_t L = enc_table->number_of_states;
    auto dec = std::make_shared<CUHDCodetable>(L);
    CUHDCodetableItem* t = dec->get();
    // The decoder entry of spread state X' = next_state undoes the encoder
    // step: symbol, next_state = X >> k and k (ans_table_generator.cc:261-288).
    for (const auto& row : enc_table->table) {
        if (!row_in_use(row, L)) continue;
        for (size_t j = 0; j < L; ++j) {
            const auto& e = row[j];
            const size_t prev = e.next_state - L;
            CUHDCodetableItem& item = t[prev];
            const std::uint8_t bits =
                item.min_num_bits == 0 && e.code_length > 0 ? (std::uint8_t) e.code_length
                                                            : item.min_num_bits;
            item.next_state = (std::uint16_t) ((L + j) >> e.code_length);
            item.symbol = e.symbol;
            item.min_num_bits = bits;
        }
    }
    return dec;
}

size_t ANSTableGenerator::get_max_compressed_size(std::shared_ptr<ANSEncoderTable> encoder_table,
                                                  size_t input_size) {
    const size_t L = encoder_table->table.at(0).size();
    size_t longest = 0;
    for (const auto& row : encoder_table->table)
        if (row_in_use(row, L)) longest = std::max<size_t>(longest, row[L - 1].code_length);
    const size_t bytes = (longest * input_size) / 8 + 1;
    return SDIV(bytes, sizeof(UNIT_TYPE));
}

// ---------------------------------------------------------------------------
// encoder (src/ans_encoder.cc)

namespace {
// A 32-bit shift whose count is taken modulo 32, what both x86-64 and
// AArch64 do for a variable shift; the reference's final flush relies on it
// (ans_encoder.cc:54-63) for bits that land in the first unit's padding.
inline std::uint32_t shl32(std::uint32_t x, std::uint64_t n) { return x << (n & 31u); }
inline std::uint32_t shr32(std::uint32_t x, std::uint64_t n) { return x >> (n & 31u); }
}  // namespace

void ANSEncoder::encode_memory(UNIT_TYPE* out, size_t size_out, SYMBOL_TYPE* in, size_t size_in,
                               std::shared_ptr<ANSEncoderTable> encoder_table,
                               std::shared_ptr<Decoder_Info> decoder_info) {
    const auto& tab = encoder_table->table;
    const std::uint32_t L = (std::uint32_t) tab.at(0).size();
    // Codes are appended below the bits already in `window`; a unit is
    // written when the next code no longer fits, its low part starting the
    // following unit.  The last iteration flushes a partial unit (and reads
    // the symbol past the end, whose code only reaches the padding bits).
    std::uint32_t window = 0, idx = 0, final_state = 0;
    std::uint64_t at = 0, final_bit = 0, last_unit = 0;
    size_t pos = 0;
    for (size_t u = 0; u < size_out && pos < size_in + 1; ++u) {
        auto e = &tab[in[pos]][idx];
        idx = e->next_state - L;
        while (at + e->code_length < 32 && pos < size_in) {
            window = (window << e->code_length) + e->code_sequence;
            at += e->code_length;
            ++pos;
            if (pos < size_in) {
                e = &tab[in[pos]][idx];
                idx = e->next_state - L;
            }
            // taken after the look-ahead, as the reference does: when the
            // last symbol does not fit it is still the one recorded
            final_state = e->next_state;
        }
        const std::uint64_t spill = at + e->code_length - 32;   // wraps on the flush
        final_bit = at;
        last_unit = u;
        window = shl32(window, e->code_length - spill);
        window += shr32(e->code_sequence, spill);
        out[u] = window;
        window = e->code_sequence & ~shl32(~0u, spill);
        at = spill;
        ++pos;
    }
    decoder_info->state = final_state;
    decoder_info->bit = final_bit;
    decoder_info->size = last_unit + 1;
}

std::shared_ptr<CUHDInputBuffer> ANSEncoder::encode(SYMBOL_TYPE* in, size_t size_in,
                                                    std::shared_ptr<ANSEncoderTable> encoder_table) {
    const size_t cap = ANSTableGenerator::get_max_compressed_size(encoder_table, size_in);
    std::vector<UNIT_TYPE> buf(cap, 0);
    auto info = std::make_shared<Decoder_Info>();
    encode_memory(buf.data(), cap, in, size_in, encoder_table, info);
    return std::make_shared<CUHDInputBuffer>(buf.data(), info->size, info->bit, info->state);
}

// ---------------------------------------------------------------------------
// C entry points

extern "C" {

int mans_host_gen_symbols(uint64_t seed, double lambda, uint8_t* out, size_t n) {
    if (!out || !(lambda > 0)) return MANS_ERR_ARG;
    std::mt19937_64 g(seed);
    for (size_t i = 0; i < n; ++i) {
        const double u = (double) ((g() >> 11) + 1) * 0x1.0p-53;   // (0, 1]
        const double v = -std::log(u) / lambda;
        out[i] = v >= 255.0 ? 255 : (uint8_t) std::floor(v);
    }
    return MANS_OK;
}

namespace {
std::shared_ptr<ANSEncoderTable> tables_for(const uint8_t* sym, size_t n, uint32_t L,
                                            uint32_t seed) {
    auto d = ANSTableGenerator::generate_distribution_from_buffer(
        seed, L, const_cast<uint8_t*>(sym), n);
    auto t = ANSTableGenerator::generate_table(d.prob, d.dist, d.symbols, d.symbols->size(), L);
    return ANSTableGenerator::generate_encoder_table(t);
}
}  // namespace

size_t mans_host_max_units(const uint8_t* sym, size_t n, uint32_t L, uint32_t table_seed) {
    if (!sym || n == 0 || L < 2) return 0;
    return ANSTableGenerator::get_max_compressed_size(tables_for(sym, n, L, table_seed), n) + 4;
}

int mans_host_encode_tables(const uint64_t* hist, uint32_t L, uint32_t table_seed,
                            uint32_t* dec_table, uint32_t* enc_blob) {
    if (!hist || !dec_table || !enc_blob || L < 2 || L > 8192 || (L & (L - 1)) != 0)
        return MANS_ERR_ARG;
    uint64_t n = 0;
    for (int v = 0; v < 256; ++v) n += hist[v];
    if (n == 0) return MANS_ERR_ARG;
    auto d = ANSTableGenerator::generate_distribution_from_histogram(table_seed, L, hist);
    auto t = ANSTableGenerator::generate_table(d.prob, d.dist, d.symbols, d.symbols->size(), L);
    auto enc = ANSTableGenerator::generate_encoder_table(t);
    auto dec = ANSTableGenerator::get_decoder_table(enc);
    std::memcpy(dec_table, dec->get(), (size_t) L * sizeof(uint32_t));
    // Compact encoder table (the encoder kernels' format).  Encoding byte s
    // from state X in [L, 2L) shifts out k low bits with (X >> k) in
    // [f, 2f) (f = the byte's normalised count) and moves to the spread
    // state of (s, X >> k).  With L = 2^R and m = R + 1 - bitlength(f - 1),
    // k = (X + delta) >> 16 for delta = (m << 16) - (f << m); the next state
    // is next[base + (X >> k)] with base = (first slot of s) - f.
    //   words 0..511: per byte {delta, base} (base = ~0: byte absent)
    //   then L / 2 words: next states as uint16 (L + spread index)
    const size_t K = d.symbols->size();
    uint32_t lg = 0;
    while ((1u << lg) < L) ++lg;
    std::vector<uint32_t> first(256, 0), cnt(256, 0);
    uint32_t slot = 0;
    for (size_t i = 0; i < K; ++i) {
        const SYMBOL_TYPE sv = d.symbols->at(i);
        cnt[sv] = (uint32_t) d.dist->at(i);
        first[sv] = slot;
        slot += cnt[sv];
    }
    if (slot != L) return MANS_ERR_TABLE;
    for (int v = 0; v < 256; ++v) {
        if (cnt[v] == 0) {
            enc_blob[2 * v] = 0;
            enc_blob[2 * v + 1] = ~0u;
            continue;
        }
        uint32_t bl = 0;
        while (bl < 32 && ((cnt[v] - 1) >> bl) != 0) ++bl;
        const uint32_t m = lg + 1 - bl;
        enc_blob[2 * v] = (m << 16) - (cnt[v] << m);
        enc_blob[2 * v + 1] = first[v] - cnt[v];
    }
    uint16_t* next = reinterpret_cast<uint16_t*>(enc_blob + 512);
    for (int v = 0; v < 256; ++v) {
        if (cnt[v] == 0) continue;
        const auto& row = enc->table[v];
        for (uint32_t X = L; X < 2 * L; ++X) {
            const auto& e = row[X - L];
            const uint32_t xs = X >> e.code_length;
            next[first[v] + xs - cnt[v]] = (uint16_t) e.next_state;
        }
    }
    return MANS_OK;
}

int mans_host_encode(const uint8_t* sym, size_t n, uint32_t L, uint32_t table_seed,
                     uint32_t* dec_table, uint32_t* units, size_t cap, size_t* n_units,
                     uint32_t* first_bit, uint32_t* first_state) {
    if (!sym || n == 0 || L < 2 || L > 32768 || !dec_table || !units || !n_units ||
        !first_bit || !first_state)
        return MANS_ERR_ARG;
    auto enc = tables_for(sym, n, L, table_seed);
    if (enc->table.size() == 0) return MANS_ERR_ARG;
    auto dec = ANSTableGenerator::get_decoder_table(enc);
    std::memcpy(dec_table, dec->get(), (size_t) L * sizeof(uint32_t));
    auto in = ANSEncoder::encode(const_cast<uint8_t*>(sym), n, enc);
    const size_t nu = in->get_compressed_size();
    if (nu + 4 > cap) return MANS_ERR_ARG;
    std::memcpy(units, in->get_compressed_data(), (nu + 4) * sizeof(uint32_t));
    *n_units = nu;
    *first_bit = (uint32_t) in->get_first_bit();
    *first_state = (uint32_t) in->get_first_state();
    return MANS_OK;
}

}  // extern "C"
