// Offset allocator over one pre-allocated range (device arena or pinned host
// staging of the serving loop).  Host-only: no CUDA calls, so it is tested on
// machines without a GPU through xk_arena_*.
//
// First fit over free ranges kept by offset; freeing merges a range with its
// free neighbours.  Every allocation is rounded up to XK_ARENA_ALIGN bytes, so
// offsets stay aligned for 128-bit and TMA accesses.
#pragma once

#include <stdint.h>

#include <iterator>
#include <map>

#define XK_ARENA_ALIGN 256

class XkArena {
public:
    explicit XkArena(int64_t capacity) : cap_(capacity / XK_ARENA_ALIGN * XK_ARENA_ALIGN)
    {
        if (cap_ > 0) free_[0] = cap_;
    }

    static int64_t round(int64_t bytes)
    {
        return (bytes + XK_ARENA_ALIGN - 1) / XK_ARENA_ALIGN * XK_ARENA_ALIGN;
    }

    // offset of a free range of `bytes` (rounded up), or -1
    int64_t alloc(int64_t bytes)
    {
        if (bytes <= 0) bytes = 1;
        const int64_t need = round(bytes);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < need) continue;
            const int64_t off = it->first, len = it->second;
            free_.erase(it);
            if (len > need) free_[off + need] = len - need;
            used_[off] = need;
            in_use_ += need;
            return off;
        }
        return -1;
    }

    // false if `off` is not the start of a live allocation
    bool release(int64_t off)
    {
        auto u = used_.find(off);
        if (u == used_.end()) return false;
        int64_t start = off, len = u->second;
        used_.erase(u);
        in_use_ -= len;
        auto next = free_.lower_bound(start);
        if (next != free_.end() && next->first == start + len) {
            len += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == start) {
                start = prev->first;
                len += prev->second;
                free_.erase(prev);
            }
        }
        free_[start] = len;
        return true;
    }

    int64_t capacity() const { return cap_; }
    int64_t in_use() const { return in_use_; }
    int64_t largest_free() const
    {
        int64_t m = 0;
        for (const auto &kv : free_) m = kv.second > m ? kv.second : m;
        return m;
    }
    int free_ranges() const { return (int)free_.size(); }

private:
    int64_t cap_;
    int64_t in_use_ = 0;
    std::map<int64_t, int64_t> free_;   // offset -> length
    std::map<int64_t, int64_t> used_;   // offset -> length
};
