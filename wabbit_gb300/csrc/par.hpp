// par.hpp -- host-thread helpers of the planning code (neighbour search,
// patch tables, full-tree planning). Plain std::thread fork/join: the work
// items are independent per block, results are written to disjoint ranges.
#pragma once
#include <algorithm>
#include <thread>
#include <vector>

namespace wg {

// f(chunk, lo, hi) on contiguous chunks of [0, n), one host thread each;
// below min_n items one call on the calling thread
template <class F>
void par_chunks(int n, int nchunk, F f, int min_n = 8192) {
    if (nchunk <= 1 || n < min_n) {
        f(0, 0, n);
        return;
    }
    std::vector<std::thread> th;
    for (int c = 0; c < nchunk; c++) {
        const int lo = (int)((long long)n * c / nchunk), hi = (int)((long long)n * (c + 1) / nchunk);
        th.emplace_back([=, &f]() { f(c, lo, hi); });
    }
    for (auto &t : th) t.join();
}

// f(task) for task = 0..ntask-1, one host thread each
template <class F>
void par_tasks(int ntask, F f) {
    if (ntask <= 1) {
        if (ntask == 1) f(0);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < ntask; t++) th.emplace_back([=, &f]() { f(t); });
    for (auto &t : th) t.join();
}

inline int host_threads() {
    const unsigned h = std::thread::hardware_concurrency();
    return h ? (int)std::min(h, 32u) : 4;
}

}  // namespace wg
