// First-fit allocator of contiguous slot ranges: the serving loop's arena of device query slots
// (gsx_server.cpp).  A group of requests takes one range; freed ranges merge with their
// neighbours.  Host-only and header-only, so that it can be tested on its own.
#pragma once

#include <algorithm>
#include <iterator>
#include <map>

namespace gsx {

struct Ranges {
    std::map<int, int> free_;  // start -> length
    void init(int n) {
        free_.clear();
        free_[0] = n;
    }
    int take(int n) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                const int s = it->first, len = it->second;
                free_.erase(it);
                if (len > n) free_[s + n] = len - n;
                return s;
            }
        }
        return -1;
    }
    int largest() const {
        int m = 0;
        for (const auto &kv : free_) m = std::max(m, kv.second);
        return m;
    }
    void give(int s, int n) {
        auto it = free_.emplace(s, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

}  // namespace gsx
