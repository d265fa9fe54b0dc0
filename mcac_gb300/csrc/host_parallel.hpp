// A parallel loop over independent items on the host's cores.
#pragma once
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

namespace mcacg {

// Calls f(i) for i in [0, n) on up to hardware_concurrency() threads; items
// are handed out one at a time, so uneven items balance.
template <class F>
void parallel_for(int n, F &&f) {
    if (n <= 0) return;
    const unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), unsigned(n)));
    if (nt == 1) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    pool.reserve(nt);
    for (unsigned t = 0; t < nt; ++t)
        pool.emplace_back([&] {
            for (int i = next++; i < n; i = next++) f(i);
        });
    for (auto &th : pool) th.join();
}

}  // namespace mcacg
