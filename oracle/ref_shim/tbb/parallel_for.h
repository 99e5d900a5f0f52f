// tbb/parallel_for.h -- minimal stand-in for TBB's parallel_for(first, last, f),
// the only TBB call Lantern's integrator makes (integrator.cpp:38-40).
//
// TEST INFRASTRUCTURE ONLY (reference build for the CPU oracle / baseline).
// Items are handed out one at a time from an atomic counter to a fixed set of
// std::threads. Each tile of the reference owns its sampler, so the film does
// not depend on the schedule. Thread count: LT_REF_THREADS, else all cores.
#pragma once

#include <atomic>
#include <cstdlib>
#include <thread>
#include <vector>

namespace tbb {

inline unsigned lt_ref_thread_count() {
    const char *e = std::getenv("LT_REF_THREADS");
    if (e && std::atoi(e) > 0) return (unsigned)std::atoi(e);
    unsigned n = std::thread::hardware_concurrency();
    return n ? n : 1;
}

template <typename Index, typename Func>
void parallel_for(Index first, Index last, const Func &f) {
    if (last <= first) return;
    std::atomic<unsigned long long> next((unsigned long long)first);
    unsigned nt = lt_ref_thread_count();
    auto body = [&]() {
        for (;;) {
            unsigned long long i = next.fetch_add(1);
            if (i >= (unsigned long long)last) break;
            f((Index)i);
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t) pool.emplace_back(body);
    body();
    for (auto &t : pool) t.join();
}

}  // namespace tbb
