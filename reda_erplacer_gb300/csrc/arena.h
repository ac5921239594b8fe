// The layout of a context's device arrays inside one allocation: each array at
// a 256-byte boundary, in the order added, at least one element long.  Host
// code only (the header compiles without CUDA, so that a host program can check
// the layout: tests/test_arena_layout.py).
#pragma once

#include <stddef.h>

#include <utility>
#include <vector>

namespace erp {

constexpr size_t kArenaAlign = 256;

struct ArenaPlan {
    std::vector<std::pair<void **, size_t>> items;   // (pointer to set, offset)
    size_t total = 0;
    template <typename T>
    void add(T **p, size_t count) {
        items.emplace_back(reinterpret_cast<void **>(p), total);
        total += (sizeof(T) * (count ? count : 1) + kArenaAlign - 1) & ~(kArenaAlign - 1);
    }
    // bytes to allocate (never zero)
    size_t bytes() const { return total ? total : kArenaAlign; }
    // point every added array into the allocation at base
    void place(void *base) const {
        for (const auto &it : items) *it.first = static_cast<char *>(base) + it.second;
    }
};

}  // namespace erp
