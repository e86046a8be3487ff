// Stand-in for parallel-hashmap's flat_hash_map, used by the reference sources
// only through find/insert/operator[]/reserve/clear/iteration/swap
// (pyci/include/pyci.h:156-157, pyci/src/enpt2.cpp:20-35).  Test
// infrastructure only: backed by std::unordered_map.
#pragma once

#include <cstddef>
#include <functional>
#include <unordered_map>
#include <utility>

namespace phmap {

struct PairHash {
    template<typename A, typename B>
    std::size_t operator()(const std::pair<A, B> &p) const noexcept {
        std::size_t h = std::hash<A>()(p.first);
        std::size_t g = std::hash<B>()(p.second);
        return h ^ (g + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2));
    }
};

template<class K, class V>
using flat_hash_map = std::unordered_map<K, V, PairHash>;

} // namespace phmap
