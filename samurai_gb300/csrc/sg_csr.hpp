// LevelCellArray layout (level_cell_array.hpp:1005-1077) of one level of a
// cell set, built from its x-intervals: the intervals of every dimension and
// the offsets of the dimensions above x, as samurai stores them and as its
// restart files hold them (io/restart.hpp:90-155).  Host code, no CUDA.
#pragma once

#include <cstdint>
#include <vector>

namespace sg
{
    namespace csr
    {
        // samurai::Interval<int, long long> as stored (io/restart.hpp:31-47)
        struct IntervalRec
        {
            int32_t start, end, step, pad;
            int64_t index;
        };
        static_assert(sizeof(IntervalRec) == 24, "Interval record layout");

        // one level of the leaf CellArray: intervals per dimension and offsets
        struct LevelCSR
        {
            std::vector<IntervalRec> iv[3];
            std::vector<uint64_t> off[2];
        };

        // LevelCellArray built from the x-intervals of a level, given row by row in
        // for_each_interval order (z outer, y inner): the layout of
        // init_from_level_cell_list (level_cell_array.hpp:1005-1077).  Records of
        // `rows`: start, end, y[, z], index.
        inline void build_csr(int dim, const std::vector<long long>& rows, LevelCSR& out)
        {
            const int rec = dim + 2;
            const size_t n = rows.size() / static_cast<size_t>(rec);
            // working intervals of dimensions 1 and 2, invalid while end <= start
            IntervalRec cur_y{0, 0, 1, 0, 0}, cur_z{0, 0, 1, 0, 0};
            bool have_y = false, have_z = false;
            long long last_z = 0;
            bool any_row = false;
            auto close_y = [&]()
            {
                if (have_y)
                {
                    out.iv[1].push_back(cur_y);
                    have_y = false;
                }
            };
            for (size_t k = 0; k < n;)
            {
                const long long y = rows[k * rec + 2];
                const long long z = dim == 3 ? rows[k * rec + 3] : 0;
                if (dim == 3 && (!any_row || z != last_z))
                {
                    // a new z plane: its y-intervals start afresh
                    close_y();
                    const uint64_t prev = out.iv[1].size();
                    if (have_z && z == cur_z.end)
                    {
                        ++cur_z.end;
                    }
                    else
                    {
                        if (have_z)
                        {
                            out.iv[2].push_back(cur_z);
                        }
                        cur_z  = {static_cast<int32_t>(z), static_cast<int32_t>(z + 1), 1, 0, static_cast<int64_t>(out.off[1].size()) - z};
                        have_z = true;
                    }
                    out.off[1].push_back(prev);
                    last_z = z;
                }
                // the row (y, z): its x-intervals
                const uint64_t prev_x = out.iv[0].size();
                size_t e              = k;
                while (e < n && rows[e * rec + 2] == y && (dim == 2 || rows[e * rec + 3] == z))
                {
                    out.iv[0].push_back({static_cast<int32_t>(rows[e * rec]), static_cast<int32_t>(rows[e * rec + 1]), 1, 0,
                                         static_cast<int64_t>(rows[e * rec + dim + 1])});
                    ++e;
                }
                if (have_y && y == cur_y.end)
                {
                    ++cur_y.end;
                }
                else
                {
                    close_y();
                    cur_y  = {static_cast<int32_t>(y), static_cast<int32_t>(y + 1), 1, 0, static_cast<int64_t>(out.off[0].size()) - y};
                    have_y = true;
                }
                out.off[0].push_back(prev_x);
                any_row = true;
                k       = e;
            }
            close_y();
            if (have_z)
            {
                out.iv[2].push_back(cur_z);
            }
            if (any_row)
            {
                out.off[0].push_back(out.iv[0].size());
                if (dim == 3)
                {
                    out.off[1].push_back(out.iv[1].size());
                }
            }
        }
    } // namespace csr
} // namespace sg
