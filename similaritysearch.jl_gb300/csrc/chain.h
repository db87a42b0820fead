// Greedy chain order of the locality order's pivots (host code, no CUDA).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace ssg {

// place[p] = position of pivot p in a greedy chain over the P pivots.  `near`
// holds k_near entries per pivot: other pivots, nearest first (UINT32_MAX, or
// any value outside 0 .. P - 1, pads a short list and is skipped).  The chain
// starts at pivot 0; the next link is the first pivot not yet placed in the
// last link's list, else in the lists of up to `back` links before it (the
// latest first), else the lowest-numbered pivot not yet placed.  So every
// pivot is placed exactly once and `place` is a permutation of 0 .. P - 1,
// which the bucket sort that follows relies on (it counts rows per place).
inline void greedy_chain(const uint32_t *near, int P, int k_near, int back, uint32_t *place) {
    if (P <= 0) return;
    for (int p = 0; p < P; ++p) place[p] = UINT32_MAX;
    std::vector<uint32_t> chain;
    chain.reserve(static_cast<size_t>(P));
    place[0] = 0;
    chain.push_back(0);
    int lowest = 1;  // every pivot below it is placed
    for (int r = 1; r < P; ++r) {
        uint32_t next = UINT32_MAX;
        for (int b = 0; b <= back && b < r && next == UINT32_MAX; ++b) {
            const uint32_t *lst = near + static_cast<size_t>(chain[static_cast<size_t>(r - 1 - b)]) * k_near;
            for (int i = 0; i < k_near; ++i) {
                const uint32_t q = lst[i];
                if (q < static_cast<uint32_t>(P) && place[q] == UINT32_MAX) {
                    next = q;
                    break;
                }
            }
        }
        if (next == UINT32_MAX) {
            while (place[lowest] != UINT32_MAX) ++lowest;
            next = static_cast<uint32_t>(lowest);
        }
        place[next] = static_cast<uint32_t>(r);
        chain.push_back(next);
    }
}

}  // namespace ssg
