/*
 * Minimal stand-in for oneTBB's functional-form parallel_reduce, written for
 * this project on std::thread.
 *
 * TEST INFRASTRUCTURE: only the unmodified reference source compiled against
 * the shim uses it (mo_lradtopo_horayzon.cpp:686-761). Workers pull chunks of
 * the range from a shared counter, fold each chunk into a private value with
 * the body, and the private values are combined with the reduction. Thread
 * count: HZ_REF_THREADS if set, else std::thread::hardware_concurrency().
 */
#ifndef HZ_SHIM_TBB_PARALLEL_REDUCE_H
#define HZ_SHIM_TBB_PARALLEL_REDUCE_H
#include <atomic>
#include <cstdlib>
#include <mutex>
#include <thread>
#include <vector>

#include "blocked_range.h"

namespace tbb {
inline unsigned hz_shim_threads() {
    const char* env = std::getenv("HZ_REF_THREADS");
    if (env && std::atoi(env) > 0) return (unsigned)std::atoi(env);
    unsigned n = std::thread::hardware_concurrency();
    return n ? n : 1u;
}

template <typename Range, typename Value, typename RealBody, typename Reduction>
Value parallel_reduce(const Range& range, const Value& identity,
                      const RealBody& body, const Reduction& reduction) {
    using Index = decltype(range.begin());
    const Index b = range.begin(), e = range.end();
    const std::size_t n = range.size();
    const std::size_t chunk = 64;
    std::atomic<std::size_t> next(0);
    std::mutex mu;
    Value result = identity;
    auto worker = [&]() {
        Value acc = identity;
        for (;;) {
            std::size_t s = next.fetch_add(chunk);
            if (s >= n) break;
            std::size_t t = s + chunk < n ? s + chunk : n;
            acc = body(Range(Index(b + s), Index(b + t)), acc);
        }
        std::lock_guard<std::mutex> lock(mu);
        result = reduction(result, acc);
    };
    unsigned nth = hz_shim_threads();
    std::vector<std::thread> pool;
    for (unsigned k = 1; k < nth; k++) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
    (void)e;
    return result;
}
}  // namespace tbb
#endif
