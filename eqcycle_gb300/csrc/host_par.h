// Loops over independent items on the host's cores.
#pragma once
#include <algorithm>
#include <cstdint>
#include <thread>
#include <vector>

namespace eqc {

// f(i) for i in [0, n), in contiguous ranges, one per thread, with at least `grain` items per
// thread (1 where every item is already a large chunk of work, e.g. 16K nodes).  Callers write
// disjoint outputs, so results do not depend on the thread count; f must not throw.
template <class F>
void parallel_for(int64_t n, F&& f, int64_t grain = 16) {
    const int64_t hw = std::max<int64_t>(1, (int64_t)std::thread::hardware_concurrency());
    const int64_t nt = std::max<int64_t>(1, std::min<int64_t>(hw, n / std::max<int64_t>(grain, 1)));
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
