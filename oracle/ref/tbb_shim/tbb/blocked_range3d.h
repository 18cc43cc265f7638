// tbb::blocked_range3d for the project's TBB stand-in (see pdpd_pool.h): pages x rows x cols,
// each a blocked_range; a split halves the dimension that is largest relative to its grain.
#pragma once

#include "blocked_range.h"

namespace tbb {

template <typename PageValue, typename RowValue = PageValue, typename ColValue = RowValue>
class blocked_range3d {
public:
    blocked_range3d(PageValue page_begin, PageValue page_end, std::size_t page_grain,
                    RowValue row_begin, RowValue row_end, std::size_t row_grain,
                    ColValue col_begin, ColValue col_end, std::size_t col_grain)
        : pages_(page_begin, page_end, page_grain), rows_(row_begin, row_end, row_grain),
          cols_(col_begin, col_end, col_grain) {}
    blocked_range3d(PageValue page_begin, PageValue page_end, RowValue row_begin,
                    RowValue row_end, ColValue col_begin, ColValue col_end)
        : pages_(page_begin, page_end), rows_(row_begin, row_end), cols_(col_begin, col_end) {}
    blocked_range3d(blocked_range3d &r, split)
        : pages_(r.pages_), rows_(r.rows_), cols_(r.cols_)
    {
        const double p = double(r.pages_.size()) / r.pages_.grainsize();
        const double w = double(r.rows_.size()) / r.rows_.grainsize();
        const double c = double(r.cols_.size()) / r.cols_.grainsize();
        if (p >= w && p >= c && r.pages_.is_divisible()) {
            pages_ = blocked_range<PageValue>(r.pages_, split());
        } else if (w >= c && r.rows_.is_divisible()) {
            rows_ = blocked_range<RowValue>(r.rows_, split());
        } else if (r.cols_.is_divisible()) {
            cols_ = blocked_range<ColValue>(r.cols_, split());
        } else if (r.rows_.is_divisible()) {
            rows_ = blocked_range<RowValue>(r.rows_, split());
        } else {
            pages_ = blocked_range<PageValue>(r.pages_, split());
        }
    }

    bool empty() const { return pages_.empty() || rows_.empty() || cols_.empty(); }
    bool is_divisible() const
    {
        return pages_.is_divisible() || rows_.is_divisible() || cols_.is_divisible();
    }
    std::size_t size() const { return pages_.size() * rows_.size() * cols_.size(); }
    const blocked_range<PageValue> &pages() const { return pages_; }
    const blocked_range<RowValue> &rows() const { return rows_; }
    const blocked_range<ColValue> &cols() const { return cols_; }

private:
    blocked_range<PageValue> pages_;
    blocked_range<RowValue> rows_;
    blocked_range<ColValue> cols_;
};

}  // namespace tbb
