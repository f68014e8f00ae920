// Host thread pool-free parallel loops for the mesh preprocessing (std::thread,
// static contiguous chunks: chunk k of T covers [k n / T, (k+1) n / T)).
#pragma once

#include <algorithm>
#include <cstdlib>
#include <thread>
#include <vector>

namespace sysu {

// Threads for host preprocessing: SYSU_THREADS if set, else the hardware count
// (at most 64).
inline int host_threads() {
    if (const char *e = std::getenv("SYSU_THREADS")) {
        int v = std::atoi(e);
        if (v >= 1) return std::min(v, 256);
    }
    unsigned h = std::thread::hardware_concurrency();
    return (int)std::max(1u, std::min(h, 64u));
}

// fn(begin, end, chunk) over T chunks of [0, n); runs inline when T == 1.
template <class F>
void parallel_chunks(long n, int T, F &&fn) {
    if (T <= 1 || n < 2) {
        fn(0L, n, 0);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(T - 1);
    for (int k = 1; k < T; ++k) th.emplace_back([&, k] { fn(n * k / T, n * (k + 1) / T, k); });
    fn(0L, n / T, 0);
    for (std::thread &t : th) t.join();
}

}  // namespace sysu
