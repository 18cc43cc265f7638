// tbb::global_control for the project's TBB stand-in (see pdpd_pool.h): while an object of
// max_allowed_parallelism lives, parallel loops use at most that many threads.
#pragma once

#include <cstddef>

#include "pdpd_pool.h"

namespace tbb {

class global_control {
public:
    enum parameter { max_allowed_parallelism, thread_stack_size };
    global_control(parameter p, std::size_t value) : p_(p)
    {
        if (p_ == max_allowed_parallelism) pdpd_tbb_shim::Pool::instance().set_limit((unsigned)value);
    }
    ~global_control()
    {
        if (p_ == max_allowed_parallelism) pdpd_tbb_shim::Pool::instance().set_limit(0);
    }
    static std::size_t active_value(parameter p)
    {
        return p == max_allowed_parallelism ? pdpd_tbb_shim::Pool::instance().threads() : 0;
    }

private:
    parameter p_;
};

}  // namespace tbb
