// First-fit allocator over one fixed range (the serving loop's HBM budget).
// Offsets only: the caller owns the memory the range describes.  Free blocks
// coalesce with their neighbours.  Not thread-safe (one scheduler thread
// owns it).  Header-only C++ so that host tests can compile it alone.
#pragma once

#include <stddef.h>

#include <iterator>
#include <map>

namespace cusat_internal {

class Arena {
public:
    explicit Arena(size_t size = 0, size_t align = 256) : size_(size), align_(align), used_(0), peak_(0)
    {
        if (size_)
            free_[0] = size_;
    }

    size_t size() const { return size_; }
    size_t used() const { return used_; }
    size_t peak() const { return peak_; }
    size_t round(size_t n) const { return (n + align_ - 1) / align_ * align_; }

    // Size of the largest free block (what one allocation can get now).
    size_t largest() const
    {
        size_t m = 0;
        for (const auto& kv : free_)
            if (kv.second > m)
                m = kv.second;
        return m;
    }

    // First fit; false when no free block holds round(n) bytes.
    bool alloc(size_t n, size_t* off)
    {
        n = round(n ? n : 1);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n)
                continue;
            *off = it->first;
            const size_t rest = it->second - n;
            const size_t at = it->first + n;
            free_.erase(it);
            if (rest)
                free_[at] = rest;
            used_ += n;
            if (used_ > peak_)
                peak_ = used_;
            return true;
        }
        return false;
    }

    void release(size_t off, size_t n)
    {
        n = round(n ? n : 1);
        used_ -= n;
        auto it = free_.emplace(off, n).first;
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
                it = prev;
            }
        }
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
    }

    // Number of free blocks (fragmentation measure, tests).
    size_t free_blocks() const { return free_.size(); }

private:
    size_t size_, align_, used_, peak_;
    std::map<size_t, size_t> free_;  // offset -> bytes
};

}  // namespace cusat_internal
