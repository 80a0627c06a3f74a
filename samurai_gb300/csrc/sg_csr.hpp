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

        enum class Decode
        {
            ok,
            outside,     // an interval leaves the level's box [0, 2^level)
            inconsistent // an offsets slot or range that the arrays do not hold
        };

        // The inverse of build_csr for a restart file's level: the cells of the layout in for_each_cell order
        // (z outer, y, x inner), appended to `coords` as x, y[, z].  The layout comes from a file, so every
        // interval is checked against the box (which also bounds the walk and keeps index + coordinate from
        // overflowing) and every offsets slot and range against the arrays, before it is used.  Offsets that
        // point many rows at the same intervals would make the walk emit the same cells again and again: a
        // layout that yields more than max_cells cells (at most the box's 2^(dim level) cells, fewer when the
        // caller knows a tighter bound) is inconsistent, and is refused before its cells are appended.
        inline Decode decode_csr(int dim, int level, const LevelCSR& c, std::vector<int>& coords, uint64_t max_cells = ~uint64_t(0))
        {
            const int64_t n = int64_t(1) << level;
            const uint64_t box = (dim * level >= 64) ? ~uint64_t(0) : uint64_t(1) << (dim * level);
            if (max_cells > box)
            {
                max_cells = box;
            }
            uint64_t emitted = 0;
            // in a layout built by build_csr every x-interval belongs to one row and every y-interval to one
            // plane, so the walk uses each once; a layout that sends two rows to the same intervals is refused
            std::vector<uint8_t> used_x(c.iv[0].size(), 0), used_y(c.iv[1].size(), 0);
            for (int d = 0; d < dim; ++d)
            {
                for (const auto& r : c.iv[d])
                {
                    if (r.start < 0 || r.start > r.end || r.end > n || r.index < -(int64_t(1) << 62) || r.index > (int64_t(1) << 62))
                    {
                        return Decode::outside;
                    }
                }
            }
            auto range = [&](int d, int64_t slot, uint64_t& b, uint64_t& e) -> bool
            {
                const auto& o = c.off[d - 1];
                if (slot < 0 || static_cast<uint64_t>(slot) + 1 >= o.size())
                {
                    return false;
                }
                b = o[static_cast<size_t>(slot)];
                e = o[static_cast<size_t>(slot) + 1];
                return b <= e && e <= c.iv[d - 1].size();
            };
            auto row = [&](uint64_t b, uint64_t e, int y, int z) -> bool
            {
                uint64_t cells = 0;
                for (uint64_t k = b; k < e; ++k)
                {
                    if (used_x[k])
                    {
                        return false;
                    }
                    used_x[k] = 1;
                    cells += static_cast<uint64_t>(c.iv[0][k].end - c.iv[0][k].start); // end >= start: checked above
                    if (cells > max_cells - emitted)
                    {
                        return false;
                    }
                }
                emitted += cells;
                for (uint64_t k = b; k < e; ++k)
                {
                    for (int x = c.iv[0][k].start; x < c.iv[0][k].end; ++x)
                    {
                        coords.push_back(x);
                        coords.push_back(y);
                        if (dim == 3)
                        {
                            coords.push_back(z);
                        }
                    }
                }
                return true;
            };
            auto plane = [&](uint64_t yb, uint64_t ye, int z) -> bool
            {
                for (uint64_t k = yb; k < ye; ++k)
                {
                    if (used_y[k])
                    {
                        return false;
                    }
                    used_y[k] = 1;
                    for (int y = c.iv[1][k].start; y < c.iv[1][k].end; ++y)
                    {
                        uint64_t b = 0, e = 0;
                        if (!range(1, c.iv[1][k].index + y, b, e) || !row(b, e, y, z))
                        {
                            return false;
                        }
                    }
                }
                return true;
            };
            if (dim == 2)
            {
                return plane(0, c.iv[1].size(), 0) ? Decode::ok : Decode::inconsistent;
            }
            for (const auto& rz : c.iv[2])
            {
                for (int z = rz.start; z < rz.end; ++z)
                {
                    uint64_t b = 0, e = 0;
                    if (!range(2, rz.index + z, b, e) || !plane(b, e, z))
                    {
                        return Decode::inconsistent;
                    }
                }
            }
            return Decode::ok;
        }
    } // namespace csr
} // namespace sg
