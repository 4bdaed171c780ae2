// Test infrastructure only: a C-callable wrapper around the reference
// implementation's own host code (table generator, encoder, multicore CPU
// decoder), compiled from the reference sources by oracle/Makefile into
// oracle/_ref/libmans_ref.so.  Nothing in the product links this file.
//
// Two shims make the reference's buffer-driven data path usable; both leave
// the arithmetic untouched:
//   shim 1  ANSTableGenerator::get_decoder_table walks all 256 encoder rows
//           (ans_table_generator.cc:270-283); rows of byte values absent
//           from the data are all-zero and make `prev` wrap to a huge index.
//           It is handed a copy of the encoder table that keeps only the
//           rows of present symbols (each item's symbol comes from the
//           entry, ans_table_generator.cc:278, so the result is the same).
//   shim 2  ANSTableGenerator::get_max_compressed_size reads the code length
//           of row 255 at state L-1 (ans_table_generator.cc:323-324), which
//           is 0 when byte 255 is absent and truncates the encoder buffer.
//           ANSEncoder::encode is handed a copy whose row 255, when absent,
//           is replaced by the present row with the longest code at L-1.
//           Row 255 is never encoded when the byte is absent, so only the
//           buffer size changes.

#include <cstdint>
#include <cstring>
#include <numeric>
#include <memory>
#include <vector>
#include <algorithm>

#include "ans_table_generator.h"
#include "ans_encoder.h"
#include "cuhd_input_buffer.h"
#include "cuhd_output_buffer.h"
#include "cuhd_codetable.h"
#include "multicore_decoder.h"

namespace {

struct RefTables {
    std::shared_ptr<ANSEncoderTable> enc_full;   // 256 rows, as generated
    std::shared_ptr<ANSEncoderTable> enc_sized;  // shim 2 copy for encode()
    std::shared_ptr<CUHDCodetable> dec;
    std::vector<bool> present;
};

RefTables build_tables(const std::uint8_t* sym, size_t n, std::uint32_t L,
                       std::uint32_t seed) {
    RefTables t;
    auto dist = ANSTableGenerator::generate_distribution_from_buffer(
        seed, L, const_cast<std::uint8_t*>(sym), n);
    const size_t K = dist.symbols->size();
    auto table = ANSTableGenerator::generate_table(
        dist.prob, dist.dist, dist.symbols, K, L);
    t.enc_full = ANSTableGenerator::generate_encoder_table(table);

    t.present.assign(256, false);
    for (auto s : *dist.symbols) t.present[s] = true;

    // shim 1: only the rows of present symbols
    auto compact = std::make_shared<ANSEncoderTable>(*t.enc_full);
    compact->table.clear();
    for (size_t s = 0; s < 256; ++s)
        if (t.present[s]) compact->table.push_back(t.enc_full->table[s]);
    compact->number_of_symbols = compact->table.size();
    t.dec = ANSTableGenerator::get_decoder_table(compact);

    // shim 2: row 255 carries the longest code at state L-1 when absent
    t.enc_sized = std::make_shared<ANSEncoderTable>(*t.enc_full);
    if (!t.present[255]) {
        size_t best = 0;
        std::uint32_t best_len = 0;
        for (size_t s = 0; s < 256; ++s) {
            if (!t.present[s]) continue;
            std::uint32_t len = t.enc_full->table[s][L - 1].code_length;
            if (len >= best_len) { best_len = len; best = s; }
        }
        t.enc_sized->table[255] = t.enc_full->table[best];
    }
    return t;
}

}  // namespace

extern "C" {

// Builds the decoder table (L packed CUHDCodetableItem words) for `sym`.
int mref_decoder_table(const std::uint8_t* sym, size_t n, std::uint32_t L,
                       std::uint32_t seed, std::uint32_t* dec_out) {
    RefTables t = build_tables(sym, n, L, seed);
    std::memcpy(dec_out, t.dec->get(), L * sizeof(std::uint32_t));
    return 0;
}

// Upper bound on the unit count the encoder may write (shimmed sizing).
size_t mref_max_units(const std::uint8_t* sym, size_t n, std::uint32_t L,
                      std::uint32_t seed) {
    RefTables t = build_tables(sym, n, L, seed);
    return ANSTableGenerator::get_max_compressed_size(t.enc_sized, n);
}

// Encodes `sym` (n symbols; sym[n] must be readable, the encoder reads one
// symbol past the end).  Writes the units in CUHDInputBuffer order (reversed,
// multians_input_buffer.cc:29) plus 4 zero padding units; returns the unit
// count without padding.
size_t mref_encode(const std::uint8_t* sym, size_t n, std::uint32_t L,
                   std::uint32_t seed, std::uint32_t* dec_out,
                   std::uint32_t* units_out, size_t cap,
                   std::uint32_t* first_bit, std::uint32_t* first_state) {
    RefTables t = build_tables(sym, n, L, seed);
    std::memcpy(dec_out, t.dec->get(), L * sizeof(std::uint32_t));
    auto in = ANSEncoder::encode(const_cast<std::uint8_t*>(sym), n,
                                 t.enc_sized);
    size_t units = in->get_compressed_size();
    if (units + 4 > cap) return 0;
    std::memcpy(units_out, in->get_compressed_data(),
                (units + 4) * sizeof(std::uint32_t));
    *first_bit = (std::uint32_t) in->get_first_bit();
    *first_state = (std::uint32_t) in->get_first_state();
    return units;
}

// Runs MulticoreDecoder::decode (multicore_decoder.cc:17-90) on a stream in
// CUHDInputBuffer order and writes the decoded symbols in the decoder's own
// (reversed) order, i.e. before CUHDOutputBuffer::reverse.
int mref_multicore_decode(size_t subseq, size_t threads,
                          const std::uint32_t* units, size_t n_units,
                          std::uint32_t first_bit, std::uint32_t first_state,
                          const std::uint32_t* dec, std::uint32_t L,
                          std::uint8_t* out, size_t n_out) {
    // CUHDInputBuffer reverses what it is given; hand it the encoder order.
    std::vector<std::uint32_t> enc_order(units, units + n_units);
    std::reverse(enc_order.begin(), enc_order.end());
    auto in = std::make_shared<CUHDInputBuffer>(enc_order.data(), n_units,
                                                first_bit, first_state);
    auto tab = std::make_shared<CUHDCodetable>(L);
    std::memcpy(tab->get(), dec, L * sizeof(std::uint32_t));
    auto ob = std::make_shared<CUHDOutputBuffer>(n_out);
    MulticoreDecoder::decode(subseq, threads, n_units, ob, in, tab);
    std::memcpy(out, ob->get_decompressed_data().get(), n_out);
    return 0;
}

}  // extern "C"
