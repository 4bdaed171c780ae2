/*
 * CPU oracle for the MULTIANS tANS decode path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's host algorithms (table generator,
 * encoder, multicore decoder) that the CUDA decoder's output is compared
 * against, and the timed CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it.  The product (multians_gb300/) never does.
 *
 * Each function cites the reference file:line it follows (paths relative to
 * the reference project root).  Pinning: the restatement is checked bit for
 * bit against the reference's own host code compiled from its sources
 * (oracle/_ref, see oracle/Makefile) and against committed golden fixtures
 * under tests/golden/.
 *
 * Formats (all little-endian, as the reference lays them out):
 *   decoder table  L words; word = next_state | symbol << 16 | bits << 24
 *                  (CUHDCodetableItem, include/cuhd_codetable.h:20-24)
 *   stream         units in CUHDInputBuffer order: the encoder's units
 *                  reversed (src/multians_input_buffer.cc:29), followed by
 *                  4 zero padding units (src/multians_input_buffer.cc:23)
 *   sync point     4 words: unit-in-subsequence of the last codeword, its
 *                  start bit, symbol count (then exclusive offset), state
 *                  before it (include/cuhd_subsequence_sync_point.h:17-22)
 */
#ifndef MANS_ORACLE_H_
#define MANS_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Seeded synthetic symbols: sym = min(255, floor(-ln(U) / lambda)) with
 * U = ((x >> 11) + 1) * 2^-53 and x from mt19937_64(seed). */
void mo_gen_symbols(uint64_t seed, double lambda, uint8_t* out, size_t n);

/* Encoder + decoder tables for the symbols in `sym` with L states.
 * enc: 256 * L * 4 words {next_state, code_sequence, code_length, symbol}.
 * dec: L packed decoder words.  *max_len: code length used for sizing.
 * Returns the number of distinct symbols K, or -1 on bad arguments. */
int mo_build_tables(const uint8_t* sym, size_t n, uint32_t L, uint32_t seed,
                    uint32_t* enc, uint32_t* dec, uint32_t* max_len);

/* Encoder buffer size in units (ans_table_generator.cc:316-333). */
size_t mo_max_units(uint32_t max_len, size_t n);

/* Encodes n symbols (sym[n] must be readable: the encoder reads one symbol
 * past the end).  units must hold mo_max_units(..) + 4 words.  Returns the
 * unit count (without padding); 0 if cap is too small. */
size_t mo_encode(const uint32_t* enc, uint32_t L, uint32_t max_len,
                 const uint8_t* sym, size_t n, uint32_t* units, size_t cap,
                 uint32_t* first_bit, uint32_t* first_state);

/* Sequential decode from the stream start; writes n_out symbols in decode
 * (reversed) order.  Units at index >= n_units read as zero.
 * Returns 0, or -1 if the table is degenerate (a zero-bit cycle). */
int mo_decode_seq(const uint32_t* units, size_t n_units, uint32_t first_bit,
                  uint32_t first_state, const uint32_t* dec, uint32_t L,
                  uint8_t* out, size_t n_out);

/* True sync points for subsequences of S units (nsub = ceil(n_units / S)):
 * sp[4*i .. 4*i+3] = {unit, bit, exclusive symbol offset, state}.  The last
 * subsequence is decoded to its end, padding included. Returns 0 / -1. */
size_t mo_encode_segments(const uint32_t* const* encs, const size_t* seg_end, size_t n_seg,
                          uint32_t L, uint32_t max_len, const uint8_t* in, size_t size_in,
                          uint32_t* units, size_t cap, uint32_t* first_bit,
                          uint32_t* first_state);
int mo_decode_segments(const uint32_t* units, size_t n_units, uint32_t first_bit,
                       uint32_t first_state, const uint32_t* const* decs, const size_t* counts,
                       size_t n_seg, uint32_t L, uint8_t* out, uint64_t* starts);
int mo_sync_points(size_t S, const uint32_t* units, size_t n_units,
                   uint32_t first_bit, uint32_t first_state,
                   const uint32_t* dec, uint32_t L, uint32_t* sp);

/* The reference's multicore method (multicore_decoder.cc:17-90) on T POSIX
 * threads: guessed-state pass, seam repair passes, prefix sum, write pass.
 * Output in decode (reversed) order.  Returns the number of repair passes,
 * -1 on bad arguments (fewer subsequences than threads), or -2 when a
 * thread met a zero-bit cycle (single-symbol table), where the reference
 * itself never returns. */
int mo_multicore_decode(size_t S, size_t T, const uint32_t* units,
                        size_t n_units, uint32_t first_bit,
                        uint32_t first_state, const uint32_t* dec, uint32_t L,
                        uint8_t* out, size_t n_out);

/* Reverses n bytes in place (CUHDOutputBuffer::reverse,
 * multians_output_buffer.cc:27-29). */
void mo_reverse_bytes(uint8_t* buf, size_t n);

#ifdef __cplusplus
}
#endif

#endif /* MANS_ORACLE_H_ */
