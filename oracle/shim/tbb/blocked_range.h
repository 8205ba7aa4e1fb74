/*
 * Minimal stand-in for oneTBB's blocked_range, written for this project.
 * TEST INFRASTRUCTURE: only the unmodified reference source compiled against
 * the shim uses it (mo_lradtopo_horayzon.cpp:14-15, 686-761).
 */
#ifndef HZ_SHIM_TBB_BLOCKED_RANGE_H
#define HZ_SHIM_TBB_BLOCKED_RANGE_H
#include <cstddef>

namespace tbb {
template <typename Value>
class blocked_range {
public:
    blocked_range(Value begin, Value end, std::size_t grain = 1)
        : b_(begin), e_(end), grain_(grain) {}
    Value begin() const { return b_; }
    Value end() const { return e_; }
    std::size_t size() const { return std::size_t(e_ - b_); }
    std::size_t grainsize() const { return grain_; }
    bool empty() const { return !(b_ < e_); }
private:
    Value b_, e_;
    std::size_t grain_;
};
}  // namespace tbb
#endif
