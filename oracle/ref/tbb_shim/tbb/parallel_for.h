// tbb::parallel_for for the project's TBB stand-in (see pdpd_pool.h): the range is cut into
// pieces by the partitioner's rule (partitioner.h), then the pool runs body(piece) for every
// piece.
#pragma once

#include <cstddef>
#include <deque>
#include <type_traits>
#include <vector>

#include "blocked_range.h"
#include "partitioner.h"
#include "pdpd_pool.h"

namespace tbb {
namespace shim_detail {

template <typename Range>
std::vector<Range> cut(const Range &range, std::size_t max_pieces)
{
    std::vector<Range> pieces{range};
    for (;;) {
        if (pieces.size() >= max_pieces) break;
        std::vector<Range> next;
        next.reserve(pieces.size() * 2);
        bool any = false;
        for (auto &p : pieces) {
            if (p.is_divisible() && pieces.size() + next.size() < 2 * max_pieces) {
                Range upper(p, split());
                next.push_back(p);
                next.push_back(upper);
                any = true;
            } else {
                next.push_back(p);
            }
        }
        pieces.swap(next);
        if (!any) break;
    }
    return pieces;
}

template <typename Range, typename Body>
void run_pieces(const std::vector<Range> &pieces, const Body &body)
{
    pdpd_tbb_shim::Pool::instance().run(pieces.size(), [&](std::size_t c) { body(pieces[c]); });
}

inline std::size_t threads() { return pdpd_tbb_shim::Pool::instance().threads(); }

}  // namespace shim_detail

template <typename Range, typename Body>
void parallel_for(const Range &range, const Body &body, const simple_partitioner &)
{
    if (range.empty()) return;
    shim_detail::run_pieces(shim_detail::cut(range, ~std::size_t(0) >> 1), body);
}

template <typename Range, typename Body>
void parallel_for(const Range &range, const Body &body, const auto_partitioner &)
{
    if (range.empty()) return;
    shim_detail::run_pieces(shim_detail::cut(range, 8 * shim_detail::threads()), body);
}

template <typename Range, typename Body>
void parallel_for(const Range &range, const Body &body, const static_partitioner &)
{
    if (range.empty()) return;
    shim_detail::run_pieces(shim_detail::cut(range, shim_detail::threads()), body);
}

template <typename Range, typename Body>
void parallel_for(const Range &range, const Body &body, affinity_partitioner &)
{
    parallel_for(range, body, auto_partitioner());
}

template <typename Range, typename Body>
void parallel_for(const Range &range, const Body &body)
{
    parallel_for(range, body, auto_partitioner());
}

// Index forms: f(i) for i in [first, last) (step 1 or the given step).
template <typename Index, typename Function,
          typename = std::enable_if_t<std::is_integral<Index>::value>>
void parallel_for(Index first, Index last, Index step, const Function &f)
{
    if (!(first < last) || step <= 0) return;
    const Index n = (last - first + step - 1) / step;
    parallel_for(blocked_range<Index>(0, n), [&](const blocked_range<Index> &r) {
        for (Index k = r.begin(); k < r.end(); k++) f(first + k * step);
    });
}

template <typename Index, typename Function,
          typename = std::enable_if_t<std::is_integral<Index>::value>>
void parallel_for(Index first, Index last, const Function &f)
{
    parallel_for(first, last, Index(1), f);
}

}  // namespace tbb
