// tbb::blocked_range for the project's TBB stand-in (see pdpd_pool.h): a half-open range
// [begin, end) that may be cut into pieces no larger than its grain size.
#pragma once

#include <cstddef>

namespace tbb {

struct split {};

template <typename Value>
class blocked_range {
public:
    using const_iterator = Value;
    using size_type = std::size_t;

    blocked_range() = default;
    blocked_range(Value begin, Value end, size_type grainsize = 1)
        : begin_(begin), end_(end), grain_(grainsize ? grainsize : 1) {}
    // Splitting constructor: takes the upper half of r, r keeps the lower half.
    blocked_range(blocked_range &r, split)
        : begin_(r.midpoint()), end_(r.end_), grain_(r.grain_) { r.end_ = begin_; }

    Value begin() const { return begin_; }
    Value end() const { return end_; }
    size_type size() const { return end_ > begin_ ? size_type(end_ - begin_) : 0; }
    size_type grainsize() const { return grain_; }
    bool empty() const { return !(begin_ < end_); }
    bool is_divisible() const { return size() > grain_; }

private:
    Value midpoint() const { return begin_ + (end_ - begin_) / 2; }
    Value begin_{}, end_{};
    size_type grain_ = 1;
};

}  // namespace tbb
