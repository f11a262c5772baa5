// Loops over independent items on the host's cores.
#pragma once
#include <algorithm>
#include <cstdint>
#include <thread>
#include <vector>

namespace eqc {

// f(i) for i in [0, n), in contiguous chunks, one per thread (at most one thread per 16 items).
// Callers write disjoint outputs, so results do not depend on the thread count; f must not throw.
template <class F>
void parallel_for(int64_t n, F&& f) {
    const int64_t nt = std::max<int64_t>(1, std::min<int64_t>(std::thread::hardware_concurrency(), n / 16 + 1));
    if (nt <= 1) {
        for (int64_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::vector<std::thread> th;
    for (int64_t t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            for (int64_t i = n * t / nt; i < n * (t + 1) / nt; ++i) f(i);
        });
    for (std::thread& x : th) x.join();
}

}  // namespace eqc
