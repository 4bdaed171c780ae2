// Container for one encoded stream: everything a decode needs in one
// buffer, for storage or the wire.  The reference passes these pieces as
// separate arguments (src/main.cc:111-116) and defines no format.
//
//   offset  size            field
//   0       8               magic "MANSGB\0\1"
//   8       4               header bytes (64)
//   12      4               flags (0)
//   16      8               n_symbols (the decoded size)
//   24      8               n_units (compressed units, padding not stored)
//   32      4               L (table words)
//   36      4               first_state
//   40      4               first_bit
//   44      4               reserved (0)
//   48      8               FNV-1a 64 of bytes 0..47
//   56      8               reserved (0)
//   64      4 L             decoder table (CUHDCodetableItem words)
//   64+4L   4 n_units       units in CUHDInputBuffer order
// Little-endian throughout; the units start 16-byte aligned when L is a
// multiple of 4.
#include <cstdint>
#include <cstring>

#include "multians_gb300.h"

namespace {

constexpr unsigned char kMagic[8] = {'M', 'A', 'N', 'S', 'G', 'B', 0, 1};
constexpr uint32_t kHeader = 64;

uint64_t fnv1a(const unsigned char* p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

void put32(unsigned char* p, uint32_t v) {
    for (int i = 0; i < 4; ++i) p[i] = (unsigned char) (v >> (8 * i));
}
void put64(unsigned char* p, uint64_t v) {
    for (int i = 0; i < 8; ++i) p[i] = (unsigned char) (v >> (8 * i));
}
uint32_t get32(const unsigned char* p) {
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i) v |= (uint32_t) p[i] << (8 * i);
    return v;
}
uint64_t get64(const unsigned char* p) {
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t) p[i] << (8 * i);
    return v;
}

}  // namespace

extern "C" {

size_t mans_container_size(uint64_t n_units, uint32_t L) {
    return kHeader + (size_t) L * 4 + (size_t) n_units * 4;
}

int mans_container_write(void* buf, size_t cap, const uint32_t* units, uint64_t n_units,
                         uint64_t n_symbols, const uint32_t* table, uint32_t L,
                         uint32_t first_state, uint32_t first_bit, size_t* size) {
    // the same limits parse enforces (n_units also keeps the size from wrapping)
    if (!buf || !units || !table || L < 2 || L > 8192 || first_state < L ||
        first_state >= 2 * L || first_bit > 32 || n_units > 0xffffffffull)
        return MANS_ERR_ARG;
    const size_t need = mans_container_size(n_units, L);
    if (cap < need) return MANS_ERR_AUX_SMALL;
    unsigned char* p = (unsigned char*) buf;
    std::memset(p, 0, kHeader);
    std::memcpy(p, kMagic, 8);
    put32(p + 8, kHeader);
    put32(p + 12, 0);
    put64(p + 16, n_symbols);
    put64(p + 24, n_units);
    put32(p + 32, L);
    put32(p + 36, first_state);
    put32(p + 40, first_bit);
    put64(p + 48, fnv1a(p, 48));
    for (uint32_t j = 0; j < L; ++j) put32(p + kHeader + 4 * j, table[j]);
    std::memcpy(p + kHeader + (size_t) L * 4, units, (size_t) n_units * 4);
    if (size) *size = need;
    return MANS_OK;
}

int mans_container_parse(const void* buf, size_t size, mans_container_info* info) {
    if (!buf || !info || size < kHeader) return MANS_ERR_ARG;
    const unsigned char* p = (const unsigned char*) buf;
    if (std::memcmp(p, kMagic, 8) != 0 || get32(p + 8) != kHeader || get32(p + 12) != 0)
        return MANS_ERR_ARG;
    if (get64(p + 48) != fnv1a(p, 48)) return MANS_ERR_ARG;
    mans_container_info v;
    v.n_symbols = get64(p + 16);
    v.n_units = get64(p + 24);
    v.L = get32(p + 32);
    v.first_state = get32(p + 36);
    v.first_bit = get32(p + 40);
    v.table_offset = kHeader;
    v.units_offset = kHeader + (uint64_t) v.L * 4;
    if (v.L < 2 || v.L > 8192 || v.first_state < v.L || v.first_state >= 2 * v.L ||
        v.first_bit > 32 || v.n_units > 0xffffffffull ||
        mans_container_size(v.n_units, v.L) > size)
        return MANS_ERR_ARG;
    *info = v;
    return MANS_OK;
}

}  // extern "C"
