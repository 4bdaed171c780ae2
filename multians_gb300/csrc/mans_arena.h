// First-fit allocator over one contiguous device range, host bookkeeping
// only (offsets, never touches the memory).  The serving loop carves every
// request's device memory (compressed units, output, decode workspace) and
// every resident table out of one range allocated at start-up, so admission
// is a host-side decision that needs no cudaMalloc/cudaFree on the request
// path.  Free blocks are kept ordered by offset and merged with their
// neighbours on release; allocation takes the lowest-addressed block that
// fits, which keeps long-lived tables and early requests at the bottom and
// the free space in a few large pieces.
#pragma once

#include <cstdint>
#include <iterator>
#include <map>
#include <unordered_map>

namespace mans {

class Arena {
  public:
    explicit Arena(uint64_t size = 0, uint64_t align = 256) { reset(size, align); }

    void reset(uint64_t size, uint64_t align = 256) {
        align_ = align ? align : 1;
        size_ = size / align_ * align_;
        free_.clear();
        used_.clear();
        if (size_) free_[0] = size_;
        in_use_ = peak_ = 0;
    }

    // Rounds `bytes` up to the alignment; false if no free block fits.
    bool alloc(uint64_t bytes, uint64_t* off) {
        const uint64_t need = round(bytes ? bytes : 1);
        if (need == 0 || need > size_) return false;   // 0: the rounding overflowed
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < need) continue;
            const uint64_t o = it->first, rest = it->second - need;
            free_.erase(it);
            if (rest) free_[o + need] = rest;
            used_[o] = need;
            in_use_ += need;
            if (in_use_ > peak_) peak_ = in_use_;
            *off = o;
            return true;
        }
        return false;
    }

    // Releases a block returned by alloc; false for an unknown offset.
    bool release(uint64_t off) {
        auto u = used_.find(off);
        if (u == used_.end()) return false;
        uint64_t o = off, n = u->second;
        used_.erase(u);
        in_use_ -= n;
        auto next = free_.lower_bound(o);
        if (next != free_.end() && next->first == o + n) {
            n += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == o) {
                o = prev->first;
                n += prev->second;
                free_.erase(prev);
            }
        }
        free_[o] = n;
        return true;
    }

    // Would `bytes` fit in an empty arena?
    bool ever_fits(uint64_t bytes) const {
        const uint64_t need = round(bytes ? bytes : 1);
        return need != 0 && need <= size_;
    }

    uint64_t size() const { return size_; }
    uint64_t in_use() const { return in_use_; }
    uint64_t peak() const { return peak_; }
    size_t blocks() const { return used_.size(); }
    uint64_t largest_free() const {
        uint64_t m = 0;
        for (const auto& f : free_) m = f.second > m ? f.second : m;
        return m;
    }

    // Invariants: free and used blocks tile [0, size) without overlap, no
    // two free blocks are adjacent, in_use equals the used total.
    bool check() const {
        std::map<uint64_t, std::pair<uint64_t, bool>> all;
        for (const auto& f : free_) all[f.first] = {f.second, true};
        for (const auto& u : used_) {
            if (all.count(u.first)) return false;
            all[u.first] = {u.second, false};
        }
        uint64_t pos = 0, used = 0;
        bool prev_free = false;
        for (const auto& b : all) {
            if (b.first != pos || b.second.first == 0 || b.second.first % align_) return false;
            if (b.second.second && prev_free) return false;
            prev_free = b.second.second;
            if (!b.second.second) used += b.second.first;
            pos += b.second.first;
        }
        return pos == size_ && used == in_use_;
    }

  private:
    uint64_t round(uint64_t b) const { return (b + align_ - 1) / align_ * align_; }

    uint64_t size_ = 0, align_ = 256, in_use_ = 0, peak_ = 0;
    std::map<uint64_t, uint64_t> free_;             // offset -> bytes
    std::unordered_map<uint64_t, uint64_t> used_;   // offset -> bytes
};

}  // namespace mans
