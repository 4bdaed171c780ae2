// Randomised check of the serving loop's device-range allocator
// (multians_gb300/csrc/mans_arena.h) against a brute-force first-fit model
// over a bitmap of 256-byte granules.  Prints "ok <ops>" or the first
// disagreement.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "mans_arena.h"

int main(int argc, char** argv) {
    const uint64_t seed = argc > 1 ? strtoull(argv[1], nullptr, 10) : 1;
    const int ops = argc > 2 ? atoi(argv[2]) : 20000;
    const uint64_t G = 256, granules = 1024;
    mans::Arena a(granules * G, G);
    std::vector<int> owner(granules, -1);   // model: granule -> block id
    struct Blk { uint64_t off, n; };
    std::vector<Blk> live;
    std::mt19937_64 rng(seed);
    int next_id = 0;
    for (int i = 0; i < ops; ++i) {
        const bool do_alloc = live.empty() || (rng() % 100) < 55;
        if (do_alloc) {
            // sizes 1 byte .. 40 granules, skewed small
            const uint64_t bytes = 1 + rng() % ((rng() % 4 == 0 ? 40 : 4) * G);
            const uint64_t need = (bytes + G - 1) / G;
            // model: lowest run of `need` free granules
            int64_t want = -1;
            for (uint64_t s = 0, run = 0; s < granules; ++s) {
                run = owner[s] < 0 ? run + 1 : 0;
                if (run == need) { want = (int64_t) (s + 1 - need); break; }
            }
            uint64_t off = 0;
            const bool ok = a.alloc(bytes, &off);
            if (ok != (want >= 0) || (ok && off != (uint64_t) want * G)) {
                printf("mismatch op %d alloc %llu: arena %d/%llu model %lld\n", i,
                       (unsigned long long) bytes, ok, (unsigned long long) off,
                       (long long) want);
                return 1;
            }
            if (ok) {
                for (uint64_t g = 0; g < need; ++g) owner[want + g] = next_id;
                ++next_id;
                live.push_back({off, need});
            }
        } else {
            const size_t k = rng() % live.size();
            const Blk b = live[k];
            live[k] = live.back();
            live.pop_back();
            if (!a.release(b.off)) { printf("release failed op %d\n", i); return 1; }
            for (uint64_t g = 0; g < b.n; ++g) owner[b.off / G + g] = -1;
        }
        uint64_t used = 0;
        for (const Blk& b : live) used += b.n * G;
        if (!a.check() || a.in_use() != used) { printf("invariant broken op %d\n", i); return 1; }
    }
    if (a.release(12345)) { printf("released an unknown offset\n"); return 1; }
    for (const Blk& b : live) a.release(b.off);
    if (a.in_use() != 0 || a.largest_free() != granules * G || !a.check()) {
        printf("not whole after releasing everything\n");
        return 1;
    }
    printf("ok %d\n", ops);
    return 0;
}
