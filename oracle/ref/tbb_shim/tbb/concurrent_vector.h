// tbb::concurrent_vector for the project's TBB stand-in (see pdpd_pool.h): push_back may run
// on many threads at once (a spin lock guards it); iteration, size and clear are for when no
// push_back runs, as in the reference's engines.
#pragma once

#include <atomic>
#include <cstddef>
#include <vector>

namespace tbb {

template <typename T>
class concurrent_vector {
public:
    using value_type = T;
    using size_type = std::size_t;
    using iterator = typename std::vector<T>::iterator;
    using const_iterator = typename std::vector<T>::const_iterator;

    concurrent_vector() = default;
    concurrent_vector(const concurrent_vector &o) : v_(o.v_) {}
    concurrent_vector(concurrent_vector &&o) noexcept : v_(std::move(o.v_)) {}
    concurrent_vector &operator=(const concurrent_vector &o)
    {
        v_ = o.v_;
        return *this;
    }
    concurrent_vector &operator=(concurrent_vector &&o) noexcept
    {
        v_ = std::move(o.v_);
        return *this;
    }

    iterator push_back(const T &x)
    {
        while (lock_.test_and_set(std::memory_order_acquire)) {
        }
        v_.push_back(x);
        const size_type k = v_.size() - 1;
        lock_.clear(std::memory_order_release);
        return v_.begin() + k;
    }

    size_type size() const { return v_.size(); }
    bool empty() const { return v_.empty(); }
    void clear() { v_.clear(); }
    void reserve(size_type n) { v_.reserve(n); }
    T &operator[](size_type i) { return v_[i]; }
    const T &operator[](size_type i) const { return v_[i]; }
    iterator begin() { return v_.begin(); }
    iterator end() { return v_.end(); }
    const_iterator begin() const { return v_.begin(); }
    const_iterator end() const { return v_.end(); }

private:
    std::vector<T> v_;
    std::atomic_flag lock_ = ATOMIC_FLAG_INIT;
};

}  // namespace tbb
