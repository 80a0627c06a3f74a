// CPU oracle: a plain C++20 restatement of samurai's multiresolution
// advection hot path (hpc-maths/samurai v0.33.0). TEST INFRASTRUCTURE ONLY.
//
// This file is the checker for the GPU product.  Only tests/, the smoke
// entry point and bench.py's cpu_baseline / reference arm may load it.  The
// product library never links or calls it.
//
// Representation: every set is "cells at one level", stored as rows keyed by
// the (y[,z]) coordinates, each row holding sorted, disjoint, non-touching
// half-open x-intervals.  This is the same information as samurai's
// LevelCellArray (level_cell_array.hpp:68-256) in a simpler container.  The
// set algebra follows the semantics of samurai's lazy subsets:
//   * n-ary operators are evaluated at the finest operand level, coarser
//     operands being refined (subset/nary_set_operator.hpp:102-113);
//   * .on(l) coarsens with start>>s, ((end-1)>>s)+1 and merges touching
//     intervals, or refines with start<<s, end<<s
//     (subset/traversers/utils.hpp:17-39,
//      subset/traversers/last_dim_projection_traverser.hpp:86-106);
//   * expand() is a box dilation (subset/expansion.hpp:181-192), contract()
//     a per-axis erosion (subset/contraction.hpp:124-146).
// All floating-point operators keep the reference's association order; the
// file must be compiled with -ffp-contract=off (as the reference is,
// CMakeLists.txt:16-20).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace oracle
{
    struct Iv
    {
        int s, e; // [s, e)
    };

    using Row = std::vector<Iv>; // sorted, disjoint, non-touching

    // ---------------------------------------------------------------- rows
    // Insert with merge of touching/overlapping intervals, as
    // ListOfIntervals::add_interval (list_of_intervals.hpp:170-215).
    inline void row_add(Row& r, Iv iv)
    {
        if (iv.s >= iv.e)
        {
            return;
        }
        if (r.empty() || r.back().e < iv.s)
        {
            r.push_back(iv);
            return;
        }
        // general insertion
        auto it = std::lower_bound(r.begin(), r.end(), iv.s, [](const Iv& a, int v) { return a.e < v; });
        if (it == r.end() || iv.e < it->s)
        {
            r.insert(it, iv);
            return;
        }
        it->s    = std::min(it->s, iv.s);
        it->e    = std::max(it->e, iv.e);
        auto nxt = it + 1;
        while (nxt != r.end() && nxt->s <= it->e)
        {
            it->e = std::max(it->e, nxt->e);
            ++nxt;
        }
        r.erase(it + 1, nxt);
    }

    inline Row row_union(const Row& a, const Row& b)
    {
        Row out;
        out.reserve(a.size() + b.size());
        std::size_t i = 0, j = 0;
        while (i < a.size() || j < b.size())
        {
            Iv nx;
            if (j >= b.size() || (i < a.size() && a[i].s <= b[j].s))
            {
                nx = a[i++];
            }
            else
            {
                nx = b[j++];
            }
            if (!out.empty() && nx.s <= out.back().e)
            {
                out.back().e = std::max(out.back().e, nx.e);
            }
            else
            {
                out.push_back(nx);
            }
        }
        return out;
    }

    inline Row row_inter(const Row& a, const Row& b)
    {
        Row out;
        std::size_t i = 0, j = 0;
        while (i < a.size() && j < b.size())
        {
            int s = std::max(a[i].s, b[j].s);
            int e = std::min(a[i].e, b[j].e);
            if (s < e)
            {
                out.push_back({s, e});
            }
            if (a[i].e < b[j].e)
            {
                ++i;
            }
            else
            {
                ++j;
            }
        }
        return out;
    }

    inline Row row_diff(const Row& a, const Row& b)
    {
        Row out;
        std::size_t j = 0;
        for (const auto& iv : a)
        {
            int s = iv.s;
            while (j < b.size() && b[j].e <= s)
            {
                ++j;
            }
            std::size_t k = j;
            while (k < b.size() && b[k].s < iv.e)
            {
                if (b[k].s > s)
                {
                    out.push_back({s, b[k].s});
                }
                s = std::max(s, b[k].e);
                if (s >= iv.e)
                {
                    break;
                }
                ++k;
            }
            if (s < iv.e)
            {
                out.push_back({s, iv.e});
            }
        }
        return out;
    }

    inline bool row_contains(const Row& r, int x)
    {
        auto it = std::upper_bound(r.begin(), r.end(), x, [](int v, const Iv& a) { return v < a.s; });
        if (it == r.begin())
        {
            return false;
        }
        --it;
        return x >= it->s && x < it->e;
    }

    // ---------------------------------------------------------------- keys
    template <std::size_t D>
    using Key = std::array<int, D - 1>;

    // rows are ordered with the last coordinate outermost, as samurai's
    // for_each_interval (algorithm.hpp:75-123)
    template <std::size_t D>
    struct KeyLess
    {
        bool operator()(const Key<D>& a, const Key<D>& b) const
        {
            for (int d = static_cast<int>(D) - 2; d >= 0; --d)
            {
                if (a[d] != b[d])
                {
                    return a[d] < b[d];
                }
            }
            return false;
        }
    };

    template <std::size_t D>
    using Coord = std::array<int, D>;

    template <std::size_t D>
    inline Key<D> key_of(const Coord<D>& c)
    {
        Key<D> k;
        for (int d = 0; d < static_cast<int>(D) - 1; ++d)
        {
            k[d] = c[d + 1];
        }
        return k;
    }

    // ---------------------------------------------------------------- sets
    template <std::size_t D>
    struct LSet
    {
        int level = 0;
        std::map<Key<D>, Row, KeyLess<D>> rows;

        LSet() = default;

        explicit LSet(int l)
            : level(l)
        {
        }

        bool empty() const
        {
            return rows.empty();
        }

        void add(const Key<D>& k, Iv iv)
        {
            if (iv.s >= iv.e)
            {
                return;
            }
            row_add(rows[k], iv);
        }

        void set_row(const Key<D>& k, Row r)
        {
            if (r.empty())
            {
                rows.erase(k);
            }
            else
            {
                rows[k] = std::move(r);
            }
        }

        bool contains(const Coord<D>& c) const
        {
            auto it = rows.find(key_of<D>(c));
            return it != rows.end() && row_contains(it->second, c[0]);
        }

        std::size_t count() const
        {
            std::size_t n = 0;
            for (const auto& [k, r] : rows)
            {
                for (const auto& iv : r)
                {
                    n += static_cast<std::size_t>(iv.e - iv.s);
                }
            }
            return n;
        }

        // visit every cell in for_each_cell order (rows ascending, x ascending)
        template <class F>
        void for_each_cell(F&& f) const
        {
            for (const auto& [k, r] : rows)
            {
                for (const auto& iv : r)
                {
                    for (int x = iv.s; x < iv.e; ++x)
                    {
                        Coord<D> c;
                        c[0] = x;
                        for (int d = 0; d < static_cast<int>(D) - 1; ++d)
                        {
                            c[d + 1] = k[d];
                        }
                        f(c);
                    }
                }
            }
        }
    };

    template <std::size_t D>
    inline bool operator==(const LSet<D>& a, const LSet<D>& b)
    {
        if (a.rows.size() != b.rows.size())
        {
            return false;
        }
        auto ia = a.rows.begin();
        auto ib = b.rows.begin();
        for (; ia != a.rows.end(); ++ia, ++ib)
        {
            if (ia->first != ib->first || ia->second.size() != ib->second.size())
            {
                return false;
            }
            for (std::size_t n = 0; n < ia->second.size(); ++n)
            {
                if (ia->second[n].s != ib->second[n].s || ia->second[n].e != ib->second[n].e)
                {
                    return false;
                }
            }
        }
        return true;
    }

    template <std::size_t D, class F>
    inline void for_each_offset(int lo, int hi, F&& f) // offsets in [lo,hi)^(D-1), first coordinate fastest
    {
        Key<D> k;
        if constexpr (D == 1)
        {
            f(k);
        }
        else if constexpr (D == 2)
        {
            for (k[0] = lo; k[0] < hi; ++k[0])
            {
                f(k);
            }
        }
        else
        {
            for (k[1] = lo; k[1] < hi; ++k[1])
            {
                for (k[0] = lo; k[0] < hi; ++k[0])
                {
                    f(k);
                }
            }
        }
    }

    // refine to a finer level: every cell becomes its 2^(D*s) descendants
    template <std::size_t D>
    LSet<D> refine(const LSet<D>& a, int s)
    {
        LSet<D> out(a.level + s);
        const int n = 1 << s;
        for (const auto& [k, r] : a.rows)
        {
            Row rr;
            rr.reserve(r.size());
            for (const auto& iv : r)
            {
                rr.push_back({iv.s << s, iv.e << s});
            }
            for_each_offset<D>(0, n,
                               [&](const Key<D>& o)
                               {
                                   Key<D> kk;
                                   for (int d = 0; d < static_cast<int>(D) - 1; ++d)
                                   {
                                       kk[d] = (k[d] << s) + o[d];
                                   }
                                   out.rows[kk] = rr;
                               });
        }
        return out;
    }

    // coarsen: parent of any member (traversers/utils.hpp:17-39)
    template <std::size_t D>
    LSet<D> coarsen(const LSet<D>& a, int s)
    {
        LSet<D> out(a.level - s);
        for (const auto& [k, r] : a.rows)
        {
            Key<D> kk;
            for (int d = 0; d < static_cast<int>(D) - 1; ++d)
            {
                kk[d] = k[d] >> s;
            }
            auto& dst = out.rows[kk];
            for (const auto& iv : r)
            {
                row_add(dst, {iv.s >> s, ((iv.e - 1) >> s) + 1});
            }
        }
        return out;
    }

    template <std::size_t D>
    LSet<D> on(const LSet<D>& a, int level)
    {
        if (level < a.level)
        {
            return coarsen(a, a.level - level);
        }
        if (level > a.level)
        {
            return refine(a, level - a.level);
        }
        return a;
    }

    enum class Op
    {
        Union,
        Inter,
        Diff
    };

    template <std::size_t D>
    LSet<D> binop(const LSet<D>& a0, const LSet<D>& b0, Op op)
    {
        const int L   = std::max(a0.level, b0.level);
        const auto& a = (a0.level == L) ? a0 : on(a0, L);
        LSet<D> btmp;
        const LSet<D>* bp = &b0;
        if (b0.level != L)
        {
            btmp = on(b0, L);
            bp   = &btmp;
        }
        const auto& b = *bp;
        LSet<D> out(L);
        if (op == Op::Union)
        {
            out.rows = a.rows;
            for (const auto& [k, r] : b.rows)
            {
                auto it = out.rows.find(k);
                if (it == out.rows.end())
                {
                    out.rows[k] = r;
                }
                else
                {
                    it->second = row_union(it->second, r);
                }
            }
        }
        else if (op == Op::Inter)
        {
            for (const auto& [k, r] : a.rows)
            {
                auto it = b.rows.find(k);
                if (it != b.rows.end())
                {
                    out.set_row(k, row_inter(r, it->second));
                }
            }
        }
        else
        {
            for (const auto& [k, r] : a.rows)
            {
                auto it = b.rows.find(k);
                if (it == b.rows.end())
                {
                    out.rows[k] = r;
                }
                else
                {
                    out.set_row(k, row_diff(r, it->second));
                }
            }
        }
        return out;
    }

    template <std::size_t D>
    LSet<D> uni(const LSet<D>& a, const LSet<D>& b)
    {
        return binop(a, b, Op::Union);
    }

    template <std::size_t D>
    LSet<D> inter(const LSet<D>& a, const LSet<D>& b)
    {
        return binop(a, b, Op::Inter);
    }

    template <std::size_t D>
    LSet<D> inter(const LSet<D>& a, const LSet<D>& b, const LSet<D>& c)
    {
        return binop(binop(a, b, Op::Inter), c, Op::Inter);
    }

    template <std::size_t D>
    LSet<D> diff(const LSet<D>& a, const LSet<D>& b)
    {
        return binop(a, b, Op::Diff);
    }

    template <std::size_t D>
    LSet<D> translate(const LSet<D>& a, const Coord<D>& t)
    {
        LSet<D> out(a.level);
        for (const auto& [k, r] : a.rows)
        {
            Key<D> kk;
            for (int d = 0; d < static_cast<int>(D) - 1; ++d)
            {
                kk[d] = k[d] + t[d + 1];
            }
            Row rr;
            rr.reserve(r.size());
            for (const auto& iv : r)
            {
                rr.push_back({iv.s + t[0], iv.e + t[0]});
            }
            out.rows[kk] = std::move(rr);
        }
        return out;
    }

    // box dilation by w (subset/expansion.hpp:181-192)
    template <std::size_t D>
    LSet<D> expand(const LSet<D>& a, int w)
    {
        if (w == 0)
        {
            return a;
        }
        LSet<D> out(a.level);
        for (const auto& [k, r] : a.rows)
        {
            Row rr;
            for (const auto& iv : r)
            {
                row_add(rr, {iv.s - w, iv.e + w});
            }
            for_each_offset<D>(-w, w + 1,
                               [&](const Key<D>& o)
                               {
                                   Key<D> kk;
                                   for (int d = 0; d < static_cast<int>(D) - 1; ++d)
                                   {
                                       kk[d] = k[d] + o[d];
                                   }
                                   auto it = out.rows.find(kk);
                                   if (it == out.rows.end())
                                   {
                                       out.rows[kk] = rr;
                                   }
                                   else
                                   {
                                       it->second = row_union(it->second, rr);
                                   }
                               });
        }
        return out;
    }

    // per-axis erosion (subset/contraction.hpp:124-146)
    template <std::size_t D>
    LSet<D> contract(const LSet<D>& a, int w)
    {
        LSet<D> out = a;
        for (int d = 0; d < static_cast<int>(D); ++d)
        {
            Coord<D> t{};
            t[d] = w;
            out  = inter(out, translate(a, t));
            t[d] = -w;
            out  = inter(out, translate(a, t));
        }
        return out;
    }

    template <std::size_t D>
    LSet<D> box_set(int level, int lo, int hi) // [lo,hi)^D
    {
        LSet<D> out(level);
        for_each_offset<D>(lo, hi,
                           [&](const Key<D>& k)
                           {
                               out.rows[k] = Row{{lo, hi}};
                           });
        return out;
    }

    template <std::size_t D>
    using Dir = Coord<D>;

    // static_nested_loop<dim,-1,2> order: first coordinate fastest
    // (static_algorithm.hpp:21-38)
    template <std::size_t D>
    std::vector<Dir<D>> all_directions()
    {
        std::vector<Dir<D>> out;
        Dir<D> d;
        if constexpr (D == 2)
        {
            for (d[1] = -1; d[1] <= 1; ++d[1])
            {
                for (d[0] = -1; d[0] <= 1; ++d[0])
                {
                    out.push_back(d);
                }
            }
        }
        else
        {
            for (d[2] = -1; d[2] <= 1; ++d[2])
            {
                for (d[1] = -1; d[1] <= 1; ++d[1])
                {
                    for (d[0] = -1; d[0] <= 1; ++d[0])
                    {
                        out.push_back(d);
                    }
                }
            }
        }
        return out;
    }

    template <std::size_t D>
    int n_nonzero(const Dir<D>& d)
    {
        int n = 0;
        for (int i = 0; i < static_cast<int>(D); ++i)
        {
            n += (d[i] != 0);
        }
        return n;
    }

    // for_each_diagonal_direction (stencil.hpp:338-349)
    template <std::size_t D>
    std::vector<Dir<D>> diagonal_directions()
    {
        std::vector<Dir<D>> out;
        for (auto& d : all_directions<D>())
        {
            if (n_nonzero<D>(d) > 1)
            {
                out.push_back(d);
            }
        }
        return out;
    }

    // for_each_cartesian_direction (stencil.hpp:301-317): +e0,-e0,+e1,-e1,...
    template <std::size_t D>
    std::vector<Dir<D>> cartesian_directions()
    {
        std::vector<Dir<D>> out;
        for (int d = 0; d < static_cast<int>(D); ++d)
        {
            Dir<D> v{};
            v[d] = 1;
            out.push_back(v);
            v[d] = -1;
            out.push_back(v);
        }
        return out;
    }

    template <std::size_t D>
    Coord<D> add(const Coord<D>& a, const Coord<D>& b, int k = 1)
    {
        Coord<D> c;
        for (int d = 0; d < static_cast<int>(D); ++d)
        {
            c[d] = a[d] + k * b[d];
        }
        return c;
    }

    template <std::size_t D>
    Dir<D> scale(const Dir<D>& a, int k)
    {
        Dir<D> c;
        for (int d = 0; d < static_cast<int>(D); ++d)
        {
            c[d] = k * a[d];
        }
        return c;
    }

    // ---------------------------------------------------------------- mesh
    struct MeshConfig
    {
        int min_level          = 0;
        int max_level          = 6;
        int max_stencil_radius = 1; // mesh_config.hpp:59-80
        int graduation_width   = 1;
        int prediction_radius  = 1; // config_t::prediction_stencil_radius
        int ghost_width        = 1; // max(max_stencil_radius, prediction_radius) after parse_args
        std::array<bool, 3> periodic{false, false, false}; // mesh_config::periodic (mesh_config.hpp)

        bool any_periodic() const
        {
            return periodic[0] || periodic[1] || periodic[2];
        }
    };

    // detail::get_periodic_directions (mesh.hpp:44-80, graduation.hpp:37-76):
    // every combination of {-n, +n, 0} over the periodic axes but the zero
    // one, n = 2^level the number of cells of the unit box per axis
    template <std::size_t D>
    std::vector<Coord<D>> periodic_shifts(const MeshConfig& cfg, int level)
    {
        std::vector<Coord<D>> out;
        const int n = 1 << level;
        Coord<D> cur{};
        std::function<void(int)> rec = [&](int d)
        {
            if (d == static_cast<int>(D))
            {
                out.push_back(cur);
                return;
            }
            if (cfg.periodic[d])
            {
                cur[d] = -n;
                rec(d + 1);
                cur[d] = n;
                rec(d + 1);
            }
            cur[d] = 0;
            rec(d + 1);
        };
        rec(0);
        out.pop_back(); // the zero shift
        return out;
    }

    constexpr int MAXL = 22; // levels 0..MAXL-1 stored (samurai's default max_level is 20)

    template <std::size_t D>
    struct Mesh
    {
        MeshConfig cfg;
        std::vector<LSet<D>> cells, cag, proj, uni, ref;
        std::vector<Dir<D>> corner_dirs;
        std::vector<LSet<D>> corners; // at max_level, mesh.hpp:914-990
        // reference numbering: per level, per row, (interval, offset) with index = offset + x
        struct RefIv
        {
            int s, e;
            long long off;
        };

        std::vector<std::map<Key<D>, std::vector<RefIv>, KeyLess<D>>> numbering;
        std::size_t nb_ref = 0;

        LSet<D> domain(int level) const
        {
            return box_set<D>(level, 0, 1 << level);
        }

        long long index(int level, const Coord<D>& c) const
        {
            if (level < 0 || level >= MAXL)
            {
                return -1;
            }
            const auto& rows = numbering[level];
            auto it          = rows.find(key_of<D>(c));
            if (it == rows.end())
            {
                return -1;
            }
            const auto& v = it->second;
            auto jt       = std::upper_bound(v.begin(), v.end(), c[0], [](int x, const RefIv& a) { return x < a.s; });
            if (jt == v.begin())
            {
                return -1;
            }
            --jt;
            if (c[0] >= jt->s && c[0] < jt->e)
            {
                return jt->off + c[0];
            }
            return -1;
        }

        long long idx(int level, const Coord<D>& c) const
        {
            long long i = index(level, c);
            if (i < 0)
            {
                throw std::out_of_range("oracle: cell not in the reference mesh");
            }
            return i;
        }
    };

    template <std::size_t D>
    void init_levels(std::vector<LSet<D>>& v)
    {
        v.assign(MAXL, LSet<D>());
        for (int l = 0; l < MAXL; ++l)
        {
            v[l].level = l;
        }
    }

    // Mesh_base::finalize_mesh (mesh.hpp:426-438) for the serial unit-box
    // case: construct_union, update_sub_mesh_impl (with its periodic parts),
    // construct_corners, renumbering.
    template <std::size_t D>
    void finalize_mesh(Mesh<D>& m)
    {
        const auto& cfg = m.cfg;
        const int maxl  = cfg.max_level;
        init_levels(m.cag);
        init_levels(m.proj);
        init_levels(m.uni);
        init_levels(m.ref);

        // construct_union (mesh.hpp:1231-1262)
        for (int level = maxl; level >= 1; --level)
        {
            m.uni[level - 1] = on(uni(m.cells[level], m.uni[level]), level - 1);
        }

        // MRMesh::update_sub_mesh_impl (mr/mesh.hpp:222-455)
        const int r = cfg.max_stencil_radius;
        const int p = cfg.prediction_radius;
        std::vector<LSet<D>> cl;
        init_levels(cl);
        for (int level = 0; level < MAXL; ++level)
        {
            if (!m.cells[level].empty())
            {
                cl[level] = expand(m.cells[level], r);
            }
        }
        m.cag = cl;
        // periodicity (mr/mesh.hpp:276-319): the cells translated across the
        // periodic axes, expanded by the stencil radius, within the expanded
        // domain -- added to the reference, not to cells_and_ghosts
        if (cfg.any_periodic())
        {
            for (int level = 0; level < MAXL; ++level)
            {
                if (m.cells[level].empty())
                {
                    continue;
                }
                for (const auto& t : periodic_shifts<D>(cfg, level))
                {
                    cl[level] = uni(cl[level], inter(expand(translate(m.cells[level], t), r), expand(m.domain(level), r)));
                }
            }
        }
        if (cfg.max_level != cfg.min_level)
        {
            for (int level = 0; level < MAXL; ++level)
            {
                if (m.cells[level].empty())
                {
                    continue;
                }
                if (level >= 1)
                {
                    auto sub_cag = inter(expand(on(m.cag[level], level - 1), p), expand(m.domain(level - 1), p));
                    cl[level - 1] = uni(cl[level - 1], sub_cag);
                }
                if (level - 1 > 0)
                {
                    auto sub_cells = expand(on(m.cells[level], level - 2), p);
                    cl[level - 2]  = uni(cl[level - 2], sub_cells);
                }
                // periodic part (mr/mesh.hpp:356-368): translated, projected,
                // expanded by the prediction radius, within the domain
                if (cfg.any_periodic())
                {
                    for (const auto& t : periodic_shifts<D>(cfg, level))
                    {
                        if (level >= 1)
                        {
                            auto pc = inter(expand(on(translate(m.cag[level], t), level - 1), p), m.domain(level - 1));
                            cl[level - 1] = uni(cl[level - 1], pc);
                        }
                        if (level - 1 > 0)
                        {
                            auto pc = inter(expand(on(translate(m.cells[level], t), level - 2), p), m.domain(level - 2));
                            cl[level - 2] = uni(cl[level - 2], pc);
                        }
                    }
                }
            }
            m.ref = cl;
            for (int level = 0; level + 1 < MAXL; ++level)
            {
                if (m.ref[level].empty())
                {
                    continue;
                }
                auto expr = inter(m.ref[level], m.uni[level]);
                LSet<D> lproj(level);
                for (const auto& [k, rr] : expr.rows)
                {
                    for (const auto& iv : rr)
                    {
                        for_each_offset<D>(0, 2,
                                           [&](const Key<D>& o)
                                           {
                                               Key<D> kk;
                                               for (int d = 0; d < static_cast<int>(D) - 1; ++d)
                                               {
                                                   kk[d] = 2 * k[d] + o[d];
                                               }
                                               cl[level + 1].add(kk, {iv.s << 1, iv.e << 1});
                                           });
                        lproj.add(k, iv);
                    }
                }
                m.ref[level + 1] = cl[level + 1];
                m.proj[level]    = lproj;
            }
        }
        m.ref = cl;
        for (int l = 0; l < MAXL; ++l)
        {
            m.ref[l].level = l;
            m.cag[l].level = l;
        }

        // construct_corners (mesh.hpp:914-990)
        m.corner_dirs.clear();
        m.corners.clear();
        auto dom = m.domain(maxl);
        for (const auto& d : diagonal_directions<D>())
        {
            LSet<D> u(maxl);
            for (int i = 0; i < static_cast<int>(D); ++i)
            {
                if (d[i] != 0)
                {
                    Coord<D> t{};
                    t[i] = -d[i];
                    u    = uni(u, translate(dom, t));
                }
            }
            m.corner_dirs.push_back(d);
            m.corners.push_back(diff(dom, u));
        }

        // renumbering (mesh.hpp:894-911, level_cell_array.hpp:775-784)
        m.numbering.assign(MAXL, {});
        long long acc = 0;
        for (int l = 0; l < MAXL; ++l)
        {
            for (const auto& [k, rr] : m.ref[l].rows)
            {
                auto& v = m.numbering[l][k];
                for (const auto& iv : rr)
                {
                    v.push_back({iv.s, iv.e, acc - iv.s});
                    acc += iv.e - iv.s;
                }
            }
        }
        m.nb_ref = static_cast<std::size_t>(acc);
    }

    // mra::make_mesh on the unit box: uniform at max_level (mr/mesh.hpp:511-518,
    // mesh.hpp:326-341).
    template <std::size_t D>
    Mesh<D> make_uniform_mesh(const MeshConfig& cfg)
    {
        Mesh<D> m;
        m.cfg = cfg;
        init_levels(m.cells);
        m.cells[cfg.max_level] = box_set<D>(cfg.max_level, 0, 1 << cfg.max_level);
        finalize_mesh(m);
        return m;
    }

    template <std::size_t D>
    Mesh<D> make_mesh_from_cells(const MeshConfig& cfg, const std::vector<LSet<D>>& cells)
    {
        Mesh<D> m;
        m.cfg = cfg;
        init_levels(m.cells);
        for (int l = 0; l < MAXL && l < static_cast<int>(cells.size()); ++l)
        {
            m.cells[l]       = cells[l];
            m.cells[l].level = l;
        }
        finalize_mesh(m);
        return m;
    }

    using Field = std::vector<double>;

    // ------------------------------------------------------------ operators
    // interp_coeffs<3> (numeric/prediction.hpp:32-36): even {1/8,1,-1/8}, odd {-1/8,1,1/8}
    inline double interp(int parity, int k, int order)
    {
        if (order == 0)
        {
            return 1.;
        }
        const double sign = parity ? -1. : 1.;
        const double c[3] = {sign / 8., 1, -sign / 8.};
        return c[k];
    }

    // prediction_op<order, false> for one fine cell (numeric/prediction.hpp:286-361)
    template <std::size_t D>
    double predict_one(const Mesh<D>& m, const Field& u, int level, const Coord<D>& fine, int order)
    {
        Coord<D> par;
        for (int d = 0; d < static_cast<int>(D); ++d)
        {
            par[d] = fine[d] >> 1;
        }
        if (order == 0)
        {
            return u[static_cast<std::size_t>(m.idx(level - 1, par))];
        }
        double acc = 0;
        Coord<D> st;
        auto body = [&]()
        {
            double coeff = 1.;
            Coord<D> c;
            for (int d = 0; d < static_cast<int>(D); ++d)
            {
                coeff *= interp(fine[d] & 1, st[d], 1);
                c[d] = par[d] + st[d] - 1;
            }
            acc += u[static_cast<std::size_t>(m.idx(level - 1, c))] * coeff;
        };
        if constexpr (D == 2)
        {
            for (st[1] = 0; st[1] < 3; ++st[1])
            {
                for (st[0] = 0; st[0] < 3; ++st[0])
                {
                    body();
                }
            }
        }
        else
        {
            for (st[2] = 0; st[2] < 3; ++st[2])
            {
                for (st[1] = 0; st[1] < 3; ++st[1])
                {
                    for (st[0] = 0; st[0] < 3; ++st[0])
                    {
                        body();
                    }
                }
            }
        }
        return acc;
    }

    // projection_op_ (numeric/projection.hpp:15-65): sum over child rows of
    // (left+right), then times 1/2^D.
    template <std::size_t D>
    double project_one(const Mesh<D>& msrc, const Field& u, int level_fine, const Coord<D>& coarse)
    {
        double sum = 0;
        auto body  = [&](const Key<D>& s)
        {
            Coord<D> c;
            c[0] = 2 * coarse[0];
            for (int d = 1; d < static_cast<int>(D); ++d)
            {
                c[d] = 2 * coarse[d] + s[d - 1];
            }
            Coord<D> c1 = c;
            c1[0] += 1;
            sum += u[static_cast<std::size_t>(msrc.idx(level_fine, c))] + u[static_cast<std::size_t>(msrc.idx(level_fine, c1))];
        };
        for_each_offset<D>(0, 2, body);
        constexpr double inv = 1.0 / static_cast<double>(1ULL << D);
        return sum * inv;
    }

    // ---------------------------------------------------------------- BCs
    struct BcConfig
    {
        double dirichlet_value = 0.; // make_bc<Dirichlet<1>>(u, value)
        int bc_stencil_size    = 2;  // DirichletImpl<1>: 2*order (bc/dirichlet.hpp:13)
    };

    // PolynomialExtrapolation value on the line stencil (bc/polynomial_extrapolation.hpp:22-92)
    template <std::size_t D>
    void apply_pe(const Mesh<D>& m, Field& u, int level, const Coord<D>& c, const Dir<D>& dir, int s)
    {
        auto at = [&](int k) { return static_cast<std::size_t>(m.idx(level, add<D>(c, dir, k))); };
        const int first = -s / 2 + 1; // line_stencil_from(-size/2+1)
        // cells[i] = c + (first+i)*dir, ghost = cells[s-1]
        auto cell = [&](int i) { return at(first + i); };
        if (s == 2)
        {
            u[cell(1)] = u[cell(0)];
        }
        else if (s == 4)
        {
            u[cell(3)] = u[cell(0)] - u[cell(1)] * 3.0 + u[cell(2)] * 3.0;
        }
        else if (s == 6)
        {
            u[cell(5)] = u[cell(0)] - u[cell(1)] * 5.0 + u[cell(2)] * 1.0E+1 - u[cell(3)] * 1.0E+1 + u[cell(4)] * 5.0;
        }
        else
        {
            throw std::runtime_error("oracle: polynomial extrapolation size not implemented");
        }
    }

    template <std::size_t D>
    const LSet<D>& corner_of(const Mesh<D>& m, const Dir<D>& d)
    {
        for (std::size_t i = 0; i < m.corner_dirs.size(); ++i)
        {
            if (m.corner_dirs[i] == d)
            {
                return m.corners[i];
            }
        }
        throw std::runtime_error("oracle: corner not found");
    }

    // apply_extrapolation_bc_cells (bc/apply_field_bc.hpp:115-137)
    template <std::size_t D>
    void extrapolation_bc_cells(const Mesh<D>& m, Field& u, int level, const Dir<D>& dir, const LSet<D>& bdry, int s)
    {
        LSet<D> cells;
        if (s == 2)
        {
            cells = on(inter(m.cells[level], bdry), level);
        }
        else
        {
            auto tr = translate(m.ref[level], scale<D>(dir, -(s / 2)));
            cells   = on(inter(tr, m.cells[level], bdry), level);
        }
        cells.for_each_cell([&](const Coord<D>& c) { apply_pe<D>(m, u, level, c, dir, s); });
    }

    // update_outer_corners_by_polynomial_extrapolation (bc/apply_field_bc.hpp:371-505)
    template <std::size_t D>
    void outer_corners(const Mesh<D>& m, Field& u, int level, const Dir<D>& dir)
    {
        const int gw           = m.cfg.ghost_width;
        const auto& corner_lca = corner_of(m, dir);
        for (int layer = 1; layer <= gw; ++layer)
        {
            const int s = 2 * layer;
            auto corner = on(corner_lca, level);
            extrapolation_bc_cells<D>(m, u, level, dir, corner, s);
        }
        // step 2: off-diagonal copies
        std::vector<int> nz;
        for (int d = 0; d < static_cast<int>(D); ++d)
        {
            if (dir[d] != 0)
            {
                nz.push_back(d);
            }
        }
        if (nz.size() < 2)
        {
            return;
        }
        auto corner_cells = on(inter(on(corner_lca, level), m.cells[level]), level);
        std::size_t num_combos = 1;
        for (std::size_t p = 1; p < nz.size(); ++p)
        {
            num_combos *= static_cast<std::size_t>(gw);
        }
        for (int k = 1; k <= gw; ++k)
        {
            auto src = translate(corner_cells, scale<D>(dir, k));
            for (std::size_t combo = 0; combo < num_combos; ++combo)
            {
                Dir<D> delta{};
                bool is_source  = true;
                std::size_t tmp = combo;
                for (std::size_t p = 1; p < nz.size(); ++p)
                {
                    int g = static_cast<int>(tmp % static_cast<std::size_t>(gw));
                    tmp /= static_cast<std::size_t>(gw);
                    int dp = g - (k - 1);
                    delta[nz[p]] += dp * dir[nz[p]];
                    if (dp != 0)
                    {
                        is_source = false;
                    }
                }
                if (is_source)
                {
                    continue;
                }
                src.for_each_cell(
                    [&](const Coord<D>& c)
                    {
                        u[static_cast<std::size_t>(m.idx(level, add<D>(c, delta)))] = u[static_cast<std::size_t>(m.idx(level, c))];
                    });
            }
        }
    }

    // project_corner_below (algorithm/update_outer_ghost.hpp:268-337)
    template <std::size_t D>
    void corner_below(const Mesh<D>& m, Field& u, int level, const Dir<D>& dir)
    {
        if (level == 0)
        {
            return;
        }
        for (int dl = 1; dl <= 2; ++dl)
        {
            int pl          = level - dl;
            auto fine_inner = on(corner_of(m, dir), level);
            auto fine_outer = inter(translate(fine_inner, dir), m.ref[level]);
            auto ghosts     = inter(on(fine_outer, pl), m.ref[pl]);
            ghosts.for_each_cell(
                [&](const Coord<D>& c)
                {
                    Coord<D> child;
                    for (int d = 0; d < static_cast<int>(D); ++d)
                    {
                        child[d] = (c[d] << dl) + (dir[d] == -1 ? ((1 << dl) - 1) : 0);
                    }
                    if (m.index(level, child) >= 0)
                    {
                        u[static_cast<std::size_t>(m.idx(pl, c))] = u[static_cast<std::size_t>(m.idx(level, child))];
                    }
                });
            if (pl == 0)
            {
                break;
            }
        }
    }

    // project_bc (algorithm/update_outer_ghost.hpp:20-155)
    template <std::size_t D>
    void project_bc(const Mesh<D>& m, Field& u, int level, const Dir<D>& dir, int layer)
    {
        auto dom      = m.domain(level);
        auto outside  = diff(translate(m.uni[level], scale<D>(dir, layer)), translate(dom, scale<D>(dir, layer - 1)));
        auto pghosts  = on(inter(outside, m.ref[level]), level);
        for (const auto& [k, rr] : pghosts.rows)
        {
            for (const auto& iv : rr)
            {
                for (int x = iv.s; x < iv.e; ++x)
                {
                    Coord<D> c;
                    c[0] = x;
                    for (int d = 1; d < static_cast<int>(D); ++d)
                    {
                        c[d] = k[d - 1];
                    }
                    u[static_cast<std::size_t>(m.idx(level, c))] = 0;
                }
            }
        }
        pghosts.for_each_cell(
            [&](const Coord<D>& c)
            {
                auto gi = static_cast<std::size_t>(m.idx(level, c));
                LSet<D> one(level);
                one.add(key_of<D>(c), {c[0], c[0] + 1});
                int n = 0;
                for (int cl = level + 1; cl <= level + 2; ++cl)
                {
                    auto children = inter(on(one, cl), m.ref[cl]);
                    children.for_each_cell(
                        [&](const Coord<D>& ch)
                        {
                            u[gi] += u[static_cast<std::size_t>(m.idx(cl, ch))];
                            ++n;
                        });
                    if (n > 0)
                    {
                        break;
                    }
                }
                if (n > 0)
                {
                    u[gi] /= n;
                }
            });
    }

    // apply_field_bc for Dirichlet<1> with the Everywhere region
    // (bc/apply_field_bc.hpp:53-101, bc/bc.hpp:324-362, bc/dirichlet.hpp:22-29)
    template <std::size_t D>
    void apply_dirichlet(const Mesh<D>& m, Field& u, int level, const Dir<D>& dir, const BcConfig& bc)
    {
        if (level < m.cfg.min_level)
        {
            return;
        }
        const int maxl = m.cfg.max_level;
        auto dom       = m.domain(maxl);
        auto region    = diff(dom, translate(dom, scale<D>(dir, -1)));
        auto bdry      = on(inter(m.cells[level], region), level);
        const double v = bc.dirichlet_value;
        bdry.for_each_cell(
            [&](const Coord<D>& c)
            {
                auto ic = static_cast<std::size_t>(m.idx(level, c));
                auto ig = static_cast<std::size_t>(m.idx(level, add<D>(c, dir)));
                u[ig]   = 2 * v - u[ic];
            });
    }

    // domain_boundary(mesh, level, direction) (boundary.hpp:26-36)
    template <std::size_t D>
    LSet<D> domain_boundary(const Mesh<D>& m, int level, const Dir<D>& dir)
    {
        return diff(m.cells[level], translate(m.domain(level), scale<D>(dir, -1)));
    }

    // predict_bc (algorithm/update_outer_ghost.hpp:195-266)
    template <std::size_t D>
    void predict_bc(const Mesh<D>& m, Field& u, int pred_level, const Dir<D>& dir, const BcConfig& bc)
    {
        const int nbc = bc.bc_stencil_size / 2;
        const int lv  = pred_level - 1;
        auto inner_b  = domain_boundary(m, lv, dir);
        auto dom      = m.domain(lv);
        LSet<D> bc_ghosts(lv);
        for (int layer = 1; layer <= nbc; ++layer)
        {
            bc_ghosts = uni(bc_ghosts, diff(translate(inner_b, scale<D>(dir, layer)), dom));
        }
        auto pg = on(inter(bc_ghosts, m.ref[pred_level]), pred_level);
        pg.for_each_cell(
            [&](const Coord<D>& c)
            {
                Coord<D> par;
                for (int d = 0; d < static_cast<int>(D); ++d)
                {
                    par[d] = c[d] >> 1;
                }
                u[static_cast<std::size_t>(m.idx(pred_level, c))] = u[static_cast<std::size_t>(m.idx(lv, par))];
            });
    }

    // update_further_ghosts_by_polynomial_extrapolation (bc/apply_field_bc.hpp:531-593)
    template <std::size_t D>
    void further_ghosts(const Mesh<D>& m, Field& u, int level, const Dir<D>& dir, const BcConfig& bc)
    {
        const int gw       = m.cfg.ghost_width;
        const int by_bc    = bc.bc_stencil_size / 2;
        for (int layer = by_bc + 1; layer <= gw; ++layer)
        {
            int s      = 2 * layer;
            auto bcell = domain_boundary(m, level, dir);
            extrapolation_bc_cells<D>(m, u, level, dir, bcell, s);
        }
        for (int layer = 2; layer <= gw; ++layer)
        {
            int s        = 2 * layer;
            auto dom2    = m.domain(level);
            auto bghosts = diff(dom2, translate(dom2, scale<D>(dir, -1)));
            // apply_extrapolation_bc_ghosts (bc/apply_field_bc.hpp:196-214)
            LSet<D> tr = translate(m.ref[level], scale<D>(dir, -1));
            for (int k = 2; k <= s / 2; ++k)
            {
                tr = inter(tr, translate(m.ref[level], scale<D>(dir, -k)));
            }
            auto pot   = on(inter(tr, bghosts), level);
            auto icg   = on(inter(pot, m.uni[level]), level);
            auto tgt   = on(diff(icg, m.cells[level]), level);
            tgt.for_each_cell([&](const Coord<D>& c) { apply_pe<D>(m, u, level, c, dir, s); });
        }
    }

    // a direction with a non-zero component along a periodic axis has no
    // boundary (update_outer_ghost.hpp:355-366, 379, 426; apply_field_bc.hpp:74-83)
    template <std::size_t D>
    bool crosses_periodic(const MeshConfig& cfg, const Dir<D>& d)
    {
        for (int i = 0; i < static_cast<int>(D); ++i)
        {
            if (d[i] != 0 && cfg.periodic[i])
            {
                return true;
            }
        }
        return false;
    }

    // update_outer_ghosts(level, field) (algorithm/update_outer_ghost.hpp:339-437)
    template <std::size_t D>
    void outer_ghosts(const Mesh<D>& m, Field& u, int level, const BcConfig& bc)
    {
        const int minl = m.cfg.min_level, maxl = m.cfg.max_level;
        if (D > 1 && level <= maxl && level >= minl)
        {
            for (const auto& d : diagonal_directions<D>())
            {
                if (crosses_periodic<D>(m.cfg, d))
                {
                    continue;
                }
                outer_corners<D>(m, u, level, d);
                corner_below<D>(m, u, level, d);
            }
        }
        for (const auto& d : cartesian_directions<D>())
        {
            if (crosses_periodic<D>(m.cfg, d))
            {
                continue;
            }
            if (level < maxl)
            {
                int nbc = bc.bc_stencil_size / 2;
                int mcl = nbc % 2 == 0 ? nbc / 2 : (nbc + 1) / 2;
                for (int layer = 1; layer <= mcl; ++layer)
                {
                    project_bc<D>(m, u, level, d, layer);
                }
            }
            if (level >= minl)
            {
                apply_dirichlet<D>(m, u, level, d, bc);
            }
            if (level < maxl && level >= minl)
            {
                predict_bc<D>(m, u, level + 1, d, bc);
            }
        }
        if (level >= minl)
        {
            for (const auto& d : cartesian_directions<D>())
            {
                if (!crosses_periodic<D>(m.cfg, d))
                {
                    further_ghosts<D>(m, u, level, d, bc);
                }
            }
        }
    }

    // [lo[d], hi[d]) per axis at a level
    template <std::size_t D>
    LSet<D> box_axes(int level, const Coord<D>& lo, const Coord<D>& hi)
    {
        LSet<D> out(level);
        if constexpr (D == 2)
        {
            for (int y = lo[1]; y < hi[1]; ++y)
            {
                out.rows[Key<D>{y}] = Row{{lo[0], hi[0]}};
            }
        }
        else
        {
            for (int z = lo[2]; z < hi[2]; ++z)
            {
                for (int y = lo[1]; y < hi[1]; ++y)
                {
                    out.rows[Key<D>{y, z}] = Row{{lo[0], hi[0]}};
                }
            }
        }
        return out;
    }

    // iterate_over_periodic_ghosts (algorithm/update_periodic.hpp:27-140), axis
    // by axis: the ghosts of [n, n + g) pair with [0, g) (shift -n) and then
    // those of [-g, 0) with [n - g, n) (shift +n), wherever both are
    // reference cells; the other axes span [-g, n + g).  f(ghost, inner).
    template <std::size_t D, class F>
    void periodic_pairs(const Mesh<D>& m, int level, F&& f)
    {
        const int g = m.cfg.ghost_width, n = 1 << level;
        for (int d = 0; d < static_cast<int>(D); ++d)
        {
            if (!m.cfg.periodic[d])
            {
                continue;
            }
            Coord<D> lo, hi;
            for (int k = 0; k < static_cast<int>(D); ++k)
            {
                lo[k] = -g;
                hi[k] = n + g;
            }
            for (int side = 0; side < 2; ++side)
            {
                lo[d]       = side == 0 ? n : -g;
                hi[d]       = side == 0 ? n + g : 0;
                const int t = side == 0 ? -n : n;
                inter(m.ref[level], box_axes<D>(level, lo, hi))
                    .for_each_cell(
                        [&](const Coord<D>& c)
                        {
                            Coord<D> q = c;
                            q[d] += t;
                            const long long iq = m.index(level, q);
                            if (iq >= 0)
                            {
                                f(static_cast<std::size_t>(m.idx(level, c)), static_cast<std::size_t>(iq));
                            }
                        });
            }
        }
    }

    // update_ghost_periodic(level, field) (algorithm/update_periodic.hpp:19-25)
    template <std::size_t D>
    void update_ghost_periodic(const Mesh<D>& m, Field& u, int level)
    {
        if (m.cfg.any_periodic())
        {
            periodic_pairs<D>(m, level, [&](std::size_t gi, std::size_t ii) { u[gi] = u[ii]; });
        }
    }

    // update_tag_periodic(level, tag) (algorithm/update_periodic.hpp:178-300)
    template <std::size_t D>
    void update_tag_periodic(const Mesh<D>& m, std::vector<std::uint8_t>& tag, int level)
    {
        if (m.cfg.any_periodic())
        {
            periodic_pairs<D>(m, level,
                              [&](std::size_t gi, std::size_t ii)
                              {
                                  tag[gi] |= tag[ii];
                                  tag[ii] |= tag[gi];
                              });
        }
    }

    // update_ghost_mr (algorithm/update_ghost_mr.hpp:195-237), serial: the
    // subdomain exchanges are empty
    template <std::size_t D>
    void update_ghost_mr(const Mesh<D>& m, Field& u, const BcConfig& bc)
    {
        const int maxl = m.cfg.max_level;
        for (int level = maxl; level >= 0; --level)
        {
            update_ghost_periodic<D>(m, u, level);
            outer_ghosts<D>(m, u, level, bc);
            update_ghost_periodic<D>(m, u, level);
            if (level > 0)
            {
                auto set = on(inter(m.ref[level], m.proj[level - 1]), level - 1);
                set.for_each_cell([&](const Coord<D>& c)
                                  { u[static_cast<std::size_t>(m.idx(level - 1, c))] = project_one<D>(m, u, level, c); });
            }
        }
        for (int level = 1; level <= maxl; ++level)
        {
            auto pred_ghosts = diff(m.ref[level], uni(m.cells[level], m.proj[level]));
            auto expr        = on(inter(pred_ghosts, m.domain(level), m.ref[level - 1]), level);
            expr.for_each_cell([&](const Coord<D>& c)
                               { u[static_cast<std::size_t>(m.idx(level, c))] = predict_one<D>(m, u, level, c, m.cfg.prediction_radius); });
            update_ghost_periodic<D>(m, u, level);
        }
    }

    // ------------------------------------------------------------ details
    // compute_detail_op (mr/operators.hpp:139-540) on one coarse cell
    template <std::size_t D>
    void detail_one(const Mesh<D>& m, const Field& u, Field& det, int level, const Coord<D>& c, int order)
    {
        constexpr int NC = 1 << D;
        std::array<std::size_t, NC> child_idx;
        for (int ch = 0; ch < NC; ++ch)
        {
            Coord<D> f;
            for (int d = 0; d < static_cast<int>(D); ++d)
            {
                f[d] = 2 * c[d] + ((ch >> d) & 1);
            }
            child_idx[ch] = static_cast<std::size_t>(m.idx(level + 1, f));
        }
        if (order == 0)
        {
            const double uc = u[static_cast<std::size_t>(m.idx(level, c))];
            for (int ch = 0; ch < NC; ++ch)
            {
                det[child_idx[ch]] = u[child_idx[ch]] - uc;
            }
            return;
        }
        std::array<double, NC> d;
        for (int ch = 0; ch < NC; ++ch)
        {
            d[ch] = u[child_idx[ch]];
        }
        Coord<D> st;
        auto body = [&]()
        {
            Coord<D> s;
            for (int dd = 0; dd < static_cast<int>(D); ++dd)
            {
                s[dd] = c[dd] + st[dd] - 1;
            }
            const double src = u[static_cast<std::size_t>(m.idx(level, s))];
            for (int ch = 0; ch < NC; ++ch)
            {
                // coefficient: product over dims, left-associated, x factor first
                double cf = interp((ch >> 0) & 1, st[0], 1) * interp((ch >> 1) & 1, st[1], 1);
                if constexpr (D == 3)
                {
                    cf = cf * interp((ch >> 2) & 1, st[2], 1);
                }
                d[ch] -= cf * src;
            }
        };
        if constexpr (D == 2)
        {
            for (st[1] = 0; st[1] < 3; ++st[1])
            {
                for (st[0] = 0; st[0] < 3; ++st[0])
                {
                    body();
                }
            }
        }
        else
        {
            for (st[2] = 0; st[2] < 3; ++st[2])
            {
                for (st[1] = 0; st[1] < 3; ++st[1])
                {
                    for (st[0] = 0; st[0] < 3; ++st[0])
                    {
                        body();
                    }
                }
            }
        }
        for (int ch = 0; ch < NC; ++ch)
        {
            det[child_idx[ch]] = d[ch];
        }
    }

    enum : std::uint8_t
    {
        FLAG_KEEP    = 1,
        FLAG_COARSEN = 2,
        FLAG_REFINE  = 4
    };

    struct AdaptStats
    {
        int harten_iterations = 0;
        int graduation_iterations = 0;
    };

    // make_graduation for the serial case with max_stencil_radius == 1
    // (algorithm/graduation.hpp:573-726, 245-330);
    // the contiguous-boundary pass is a no-op for a radius of 1
    // (algorithm/graduation.hpp:378-381).
    template <std::size_t D>
    int make_graduation(std::vector<LSet<D>>& ca, int grad_width, int max_stencil_radius, const MeshConfig* periodic_cfg = nullptr)
    {
        if (max_stencil_radius != 1 && max_stencil_radius != 2)
        {
            throw std::runtime_error("oracle: graduation implemented for max_stencil_radius 1 and 2");
        }
        int nit = 0;
        bool changed = true;
        while (changed)
        {
            ++nit;
            int minl = MAXL, maxl = -1;
            for (int l = 0; l < MAXL; ++l)
            {
                if (!ca[l].empty())
                {
                    minl = std::min(minl, l);
                    maxl = std::max(maxl, l);
                }
            }
            std::vector<LSet<D>> R;
            init_levels(R);
            if (maxl >= 0)
            {
                for (int fine = maxl + 1; fine >= minl + 2; --fine)
                {
                    if (fine >= MAXL || ca[fine].empty())
                    {
                        continue;
                    }
                    // with periodic axes the fine cells also act through their translates
                    // (graduation.hpp:309-318): the expansion and projection distribute over the union
                    LSet<D> src = ca[fine];
                    if (periodic_cfg && periodic_cfg->any_periodic())
                    {
                        for (const auto& t : periodic_shifts<D>(*periodic_cfg, fine))
                        {
                            src = uni(src, translate(ca[fine], t));
                        }
                    }
                    LSet<D> proj = on(expand(src, 2 * grad_width), fine - 2);
                    for (int cl = fine - 2;; --cl)
                    {
                        if (!proj.empty())
                        {
                            R[cl] = uni(R[cl], inter(proj, ca[cl]));
                        }
                        if (cl == minl || proj.empty())
                        {
                            break;
                        }
                        proj = on(proj, cl - 1);
                    }
                }
            }
            // list_interval_to_refine_for_contiguous_boundary_cells (graduation.hpp:370-497), radius 2: with
            // n = max(r, 2 (r - 2)) = 2 contiguous boundary cells, in each non-periodic Cartesian direction t, the
            // cells of level L - 1 that hold a boundary cell of level L (a cell outside the domain translated by -t)
            // translated by -2 t are refined, for L from the finest non-empty level down to the coarsest plus one;
            // the jump to L + 1 (radius > 2) does not apply
            if (max_stencil_radius == 2 && maxl >= 0)
            {
                for (int d = 0; d < static_cast<int>(D); ++d)
                {
                    if (periodic_cfg && periodic_cfg->periodic[d])
                    {
                        continue;
                    }
                    for (int sgn = 1; sgn >= -1; sgn -= 2)
                    {
                        Coord<D> t{};
                        t[d] = sgn;
                        for (int level = maxl; level != minl; --level)
                        {
                            LSet<D> dom(level);
                            dom = box_set<D>(level, 0, 1 << level);
                            auto bcells = on(diff(ca[level], translate(dom, scale<D>(t, -1))), level);
                            auto tb     = translate(bcells, scale<D>(t, -2));
                            auto sub    = on(inter(tb, ca[level - 1]), level - 1);
                            if (!sub.empty())
                            {
                                R[level - 1] = uni(R[level - 1], sub);
                            }
                        }
                    }
                }
            }
            bool any = false;
            for (int l = 0; l < MAXL; ++l)
            {
                any = any || !R[l].empty();
            }
            if (!any)
            {
                changed = false;
                continue;
            }
            std::vector<LSet<D>> nca;
            init_levels(nca);
            for (int l = 0; l < MAXL; ++l)
            {
                LSet<D> add(l);
                if (l >= 1 && !R[l - 1].empty())
                {
                    add = refine(R[l - 1], 1);
                }
                nca[l] = diff(uni(ca[l], add), R[l]);
                nca[l].level = l;
            }
            changed = false;
            for (int l = 0; l < MAXL; ++l)
            {
                if (!(nca[l] == ca[l]))
                {
                    changed = true;
                }
            }
            ca = nca;
        }
        return nit - 1;
    }

    struct MRConfig
    {
        double epsilon       = 1e-4; // mr/config.hpp:63-65
        double regularity    = 1.;
        bool relative_detail = false; // mr/config.hpp, mr/rel_detail.hpp
        bool refine_boundary = false; // args::refine_boundary (--refine-boundary, arguments.hpp:26, 67)
    };

    // compute_relative_detail (mr/rel_detail.hpp:75-111) for one scalar field:
    // the details divided by max |u| over the leaf cells (1 when that maximum is
    // below the machine epsilon), as a multiplication by its inverse
    template <std::size_t D>
    void relative_detail(const Mesh<D>& m, const Field& u, Field& det)
    {
        double mx = std::numeric_limits<double>::min();
        for (int l = 0; l < MAXL; ++l)
        {
            m.cells[l].for_each_cell([&](const Coord<D>& c) { mx = std::max(mx, std::abs(u[static_cast<std::size_t>(m.idx(l, c))])); });
        }
        if (mx < std::numeric_limits<double>::epsilon())
        {
            mx = 1.0;
        }
        const double inv = 1. / mx;
        for (auto& v : det)
        {
            v *= inv;
        }
    }

    // update_fields (algorithm/update_fields.hpp:27-127)
    template <std::size_t D>
    Field update_fields(const Mesh<D>& old_m, const Mesh<D>& new_m, const Field& u)
    {
        Field nu(new_m.nb_ref, 0.);
        const int minl = old_m.cfg.min_level, maxl = old_m.cfg.max_level;
        for (int level = minl; level <= maxl; ++level)
        {
            auto set = inter(old_m.ref[level], new_m.cells[level]);
            set.for_each_cell([&](const Coord<D>& c)
                              { nu[static_cast<std::size_t>(new_m.idx(level, c))] = u[static_cast<std::size_t>(old_m.idx(level, c))]; });
        }
        for (int level = minl + 1; level <= maxl; ++level)
        {
            auto set_coarsen = on(inter(old_m.cells[level], new_m.cells[level - 1]), level - 1);
            set_coarsen.for_each_cell([&](const Coord<D>& c)
                                      { nu[static_cast<std::size_t>(new_m.idx(level - 1, c))] = project_one<D>(old_m, u, level, c); });
            auto set_refine = on(inter(new_m.cells[level], old_m.cells[level - 1]), level - 1);
            const int order = old_m.cfg.prediction_radius;
            set_refine.for_each_cell(
                [&](const Coord<D>& c)
                {
                    // prediction<order, true>: every child from the same stencil
                    for (int ch = 0; ch < (1 << D); ++ch)
                    {
                        Coord<D> f;
                        for (int d = 0; d < static_cast<int>(D); ++d)
                        {
                            f[d] = 2 * c[d] + ((ch >> d) & 1);
                        }
                        nu[static_cast<std::size_t>(new_m.idx(level, f))] = predict_one<D>(old_m, u, level, f, order);
                    }
                });
        }
        return nu;
    }

    // Adapt<Fields...>::harten (mr/adapt.hpp:276-389), true at the fixed point, with the fields `fs`
    // driving the criteria (one detail component each: a cell is coarsened
    // when every component is small, refined when one is large,
    // mr/criteria.hpp:45-107) and the fields `others` carried to the new mesh
    // (ghost update, then update_fields: mr/adapt.hpp:383-385).
    template <std::size_t D>
    bool harten_fields(Mesh<D>& m, const std::vector<Field*>& fs, const std::vector<const BcConfig*>& bcs, int ite, const MRConfig& mr,
                       const std::vector<Field*>& others, const std::vector<const BcConfig*>& other_bcs, Field* det_out = nullptr,
                       std::vector<std::uint8_t>* tag_out = nullptr, int* grad_iters = nullptr)
    {
        const int minl = m.cfg.min_level, maxl = m.cfg.max_level;
        const std::size_t nf = fs.size();
        std::vector<Field> dets(nf, Field(m.nb_ref, 0.));
        std::vector<std::uint8_t> tag(m.nb_ref, 0);
        for (int l = 0; l < MAXL; ++l)
        {
            m.cells[l].for_each_cell([&](const Coord<D>& c) { tag[static_cast<std::size_t>(m.idx(l, c))] = FLAG_KEEP; });
        }
        for (std::size_t k = 0; k < nf; ++k)
        {
            update_ghost_mr<D>(m, *fs[k], *bcs[k]);
        }

        for (int level = (minl > 0 ? minl - 1 : 0); level < maxl - ite; ++level)
        {
            auto gbc = on(inter(m.ref[level], uni(m.cells[level + 1], m.cells[level + 2])), level);
            gbc.for_each_cell(
                [&](const Coord<D>& c)
                {
                    for (std::size_t k = 0; k < nf; ++k)
                    {
                        detail_one<D>(m, *fs[k], dets[k], level, c, m.cfg.prediction_radius);
                    }
                });
        }
        if (mr.relative_detail)
        {
            for (std::size_t k = 0; k < nf; ++k)
            {
                relative_detail<D>(m, *fs[k], dets[k]);
            }
        }
        // |detail| over the components
        auto above = [&](std::size_t o, double thr)
        {
            for (std::size_t k = 0; k < nf; ++k)
            {
                if (std::abs(dets[k][o]) > thr)
                {
                    return true;
                }
            }
            return false;
        };

        for (int level = minl; level <= maxl - ite; ++level)
        {
            const int exponent     = D * (maxl - level);
            const double eps_l     = mr.epsilon / (1 << exponent);
            const double reg       = mr.regularity + D;
            const double fine_eps  = std::pow(2.0, reg) * eps_l;
            const double coarse_eps = fine_eps / (1 << D);
            auto subset            = on(inter(m.cells[level], m.ref[level - 1]), level - 1);
            // mr_criteria_op (mr/criteria.hpp:20-113)
            subset.for_each_cell(
                [&](const Coord<D>& c)
                {
                    const int fine_level = level;
                    std::array<std::size_t, 1 << D> fo;
                    for (int ch = 0; ch < (1 << D); ++ch)
                    {
                        Coord<D> f;
                        for (int d = 0; d < static_cast<int>(D); ++d)
                        {
                            f[d] = 2 * c[d] + ((ch >> d) & 1);
                        }
                        fo[ch] = static_cast<std::size_t>(m.idx(fine_level, f));
                    }
                    if (fine_level > minl)
                    {
                        bool cond = above(static_cast<std::size_t>(m.idx(level - 1, c)), coarse_eps);
                        if (!cond)
                        {
                            bool ok = true;
                            for (auto o : fo)
                            {
                                if (above(o, eps_l))
                                {
                                    ok = false;
                                    break;
                                }
                            }
                            if (ok)
                            {
                                for (auto o : fo)
                                {
                                    tag[o] = FLAG_COARSEN;
                                }
                            }
                        }
                    }
                    if (fine_level < maxl)
                    {
                        for (auto o : fo)
                        {
                            tag[o] |= static_cast<std::uint8_t>(above(o, fine_eps) * FLAG_REFINE);
                        }
                    }
                });
        }

        // keep_boundary_refined (mr/adapt.hpp:245-274, called at :342-345 when --refine-boundary is given): in
        // each Cartesian direction, the cells of max_level outside the domain translated by -max_stencil_radius
        // times the direction (domain_boundary_layer, boundary.hpp:6-21) are tagged keep, overwriting their tag
        if (mr.refine_boundary)
        {
            const int n = 1 << maxl, w = m.cfg.max_stencil_radius;
            m.cells[maxl].for_each_cell(
                [&](const Coord<D>& c)
                {
                    bool near = false;
                    for (int d = 0; d < static_cast<int>(D); ++d)
                    {
                        near = near || c[d] < w || c[d] >= n - w;
                    }
                    if (near)
                    {
                        tag[static_cast<std::size_t>(m.idx(maxl, c))] = FLAG_KEEP;
                    }
                });
        }

        // tag finalization: update_tag_periodic, then maximum_op (mr/adapt.hpp:348-357, mr/operators.hpp:22-96)
        for (int level = maxl; level > 0; --level)
        {
            update_tag_periodic<D>(m, tag, level);
            auto ks = on(inter(m.cells[level], m.ref[level - 1]), level - 1);
            ks.for_each_cell(
                [&](const Coord<D>& c)
                {
                    std::array<std::size_t, 1 << D> fo;
                    for (int ch = 0; ch < (1 << D); ++ch)
                    {
                        Coord<D> f;
                        for (int d = 0; d < static_cast<int>(D); ++d)
                        {
                            f[d] = 2 * c[d] + ((ch >> d) & 1);
                        }
                        fo[ch] = static_cast<std::size_t>(m.idx(level, f));
                    }
                    auto co = static_cast<std::size_t>(m.idx(level - 1, c));
                    // children in offset order: rows (y,z) outer, x inner
                    std::uint8_t any_keep = 0;
                    for (auto o : fo)
                    {
                        any_keep |= static_cast<std::uint8_t>(tag[o] & FLAG_KEEP);
                    }
                    if (any_keep)
                    {
                        for (auto o : fo)
                        {
                            tag[o] |= FLAG_KEEP;
                        }
                        tag[co] |= FLAG_KEEP;
                        return;
                    }
                    std::uint8_t all_coarsen = FLAG_COARSEN;
                    for (auto o : fo)
                    {
                        all_coarsen &= static_cast<std::uint8_t>(tag[o] & FLAG_COARSEN);
                    }
                    if (all_coarsen)
                    {
                        tag[co] |= FLAG_KEEP;
                    }
                    else
                    {
                        for (auto o : fo)
                        {
                            tag[o] &= static_cast<std::uint8_t>(~FLAG_COARSEN);
                        }
                    }
                });
        }
        if (det_out)
        {
            *det_out = dets[0];
        }
        if (tag_out)
        {
            *tag_out = tag;
        }

        // update_cell_array_from_tag (algorithm/graduation.hpp:743-842)
        std::vector<LSet<D>> add_m, rem_m, add_p, rem_p, nca;
        init_levels(add_m);
        init_levels(rem_m);
        init_levels(add_p);
        init_levels(rem_p);
        init_levels(nca);
        for (int level = 0; level < MAXL; ++level)
        {
            m.cells[level].for_each_cell(
                [&](const Coord<D>& c)
                {
                    bool yz_even = true;
                    for (int d = 1; d < static_cast<int>(D); ++d)
                    {
                        yz_even = yz_even && (c[d] % 2 == 0);
                    }
                    std::uint8_t t    = tag[static_cast<std::size_t>(m.idx(level, c))];
                    bool refine_f     = t & FLAG_REFINE;
                    bool coarsen_nk   = (t & FLAG_COARSEN) && !(t & FLAG_KEEP);
                    if (refine_f && level < maxl)
                    {
                        rem_p[level].add(key_of<D>(c), {c[0], c[0] + 1});
                        for_each_offset<D>(0, 2,
                                           [&](const Key<D>& o)
                                           {
                                               Key<D> kk;
                                               for (int d = 0; d < static_cast<int>(D) - 1; ++d)
                                               {
                                                   kk[d] = 2 * c[d + 1] + o[d];
                                               }
                                               add_p[level + 1].add(kk, {2 * c[0], 2 * c[0] + 2});
                                           });
                    }
                    else if (coarsen_nk && level > minl)
                    {
                        if (c[0] % 2 == 0 && yz_even)
                        {
                            Coord<D> p;
                            for (int d = 0; d < static_cast<int>(D); ++d)
                            {
                                p[d] = c[d] >> 1;
                            }
                            add_m[level - 1].add(key_of<D>(p), {p[0], p[0] + 1});
                        }
                        rem_m[level].add(key_of<D>(c), {c[0], c[0] + 1});
                    }
                });
        }
        for (int level = minl; level <= maxl; ++level)
        {
            nca[level] = diff(uni(uni(m.cells[level], add_m[level]), add_p[level]), uni(rem_m[level], rem_p[level]));
            nca[level].level = level;
        }
        int gi = make_graduation<D>(nca, m.cfg.graduation_width, m.cfg.max_stencil_radius, &m.cfg);
        if (grad_iters)
        {
            *grad_iters = gi;
        }
        bool same = true;
        for (int l = 0; l < MAXL; ++l)
        {
            if (!(nca[l] == m.cells[l]))
            {
                same = false;
            }
        }
        if (same)
        {
            return true;
        }
        Mesh<D> nm = make_mesh_from_cells<D>(m.cfg, nca);
        for (std::size_t k = 0; k < others.size(); ++k)
        {
            update_ghost_mr<D>(m, *others[k], *other_bcs[k]);
        }
        std::vector<Field> nus;
        for (auto* f : fs)
        {
            nus.push_back(update_fields<D>(m, nm, *f));
        }
        for (auto* f : others)
        {
            nus.push_back(update_fields<D>(m, nm, *f));
        }
        m = std::move(nm);
        for (std::size_t k = 0; k < fs.size(); ++k)
        {
            *fs[k] = std::move(nus[k]);
        }
        for (std::size_t k = 0; k < others.size(); ++k)
        {
            *others[k] = std::move(nus[fs.size() + k]);
        }
        return false;
    }

    // Adapt<Field>::harten for one field
    template <std::size_t D>
    bool harten(Mesh<D>& m, Field& u, int ite, const MRConfig& mr, const BcConfig& bc, Field* det_out = nullptr,
                std::vector<std::uint8_t>* tag_out = nullptr, int* grad_iters = nullptr)
    {
        return harten_fields<D>(m, {&u}, {&bc}, ite, mr, {}, {}, det_out, tag_out, grad_iters);
    }

    // Adapt::operator() (mr/adapt.hpp:147-195)
    template <std::size_t D>
    int adapt(Mesh<D>& m, Field& u, const MRConfig& mr, const BcConfig& bc)
    {
        const int minl = m.cfg.min_level, maxl = m.cfg.max_level;
        if (minl == maxl)
        {
            return 0;
        }
        int it = 0;
        for (int i = 0; i < maxl - minl; ++i)
        {
            ++it;
            if (harten<D>(m, u, i, mr, bc))
            {
                break;
            }
        }
        return it;
    }

    // --------------------------------------------------------------- upwind
    enum class Scheme
    {
        UpwindOp   = 0, // unp1 = u - dt * upwind(a, u)   (stencil_field.hpp:38-44, 91-97)
        Readme     = 1, // README lambda, a = (1,1)        (README.md:144-153)
        Convection = 2  // unp1 = u - dt * conv(u), conv = make_convection_upwind<Field>(a)
    };

    // make_convection_upwind(velocity) (schemes/fv/operators/convection_lin.hpp:16-89) applied explicitly:
    // the output field is filled with 0 (explicit_FV_scheme.hpp:51-56), then direction by direction
    // (explicit_FV_scheme.hpp:78-101) every interface adds its contributions in the order of
    // flux_based_scheme__lin_hom.hpp:74-238 with the sequential-context loops of
    // explicit_flux_based_scheme__lin_hom.hpp:39-110 and the boundary loop of :276-318: same-level
    // interfaces level by level, then level jumps (direction, then opposite direction) level by level,
    // then boundary interfaces.  Interfaces come from interface.hpp:36-330 and 440-510.  The upwind flux
    // in direction d is a_d * u_left when a_d >= 0, a_d * u_right otherwise.
    template <std::size_t D>
    Field convection_apply(const Mesh<D>& m, const Field& u, const std::array<double, D>& a)
    {
        Field out(m.nb_ref, 0.0);
        int cmin = MAXL, cmax = -1;
        for (int l = 0; l < MAXL; ++l)
        {
            if (!m.cells[l].empty())
            {
                cmin = std::min(cmin, l);
                cmax = std::max(cmax, l);
            }
        }
        if (cmax < 0)
        {
            return out;
        }
        const int minl = std::max(m.cfg.min_level, cmin - 1);
        const int maxl = std::min(m.cfg.max_level, cmax + 1);
        auto hf        = [](double hface, double hcell) { return std::pow(hface, static_cast<int>(D) - 1) / std::pow(hcell, static_cast<int>(D)); };
        auto length    = [](int level) { return 1.0 / static_cast<double>(1LL << level); };
        auto coord     = [](const Key<D>& k, int x)
        {
            Coord<D> c;
            c[0] = x;
            for (int d = 0; d < static_cast<int>(D) - 1; ++d)
            {
                c[d + 1] = k[d];
            }
            return c;
        };
        auto parent = [](Coord<D> c)
        {
            for (auto& v : c)
            {
                v >>= 1;
            }
            return c;
        };
        auto U = [&](int level, const Coord<D>& c) { return u[static_cast<std::size_t>(m.idx(level, c))]; };
        auto O = [&](int level, const Coord<D>& c) -> double& { return out[static_cast<std::size_t>(m.idx(level, c))]; };

        for (int d = 0; d < static_cast<int>(D); ++d)
        {
            Dir<D> e{};
            e[d]            = 1;
            const Dir<D> me = scale<D>(e, -1);
            // FluxStencilCoeffs (left, right) of the upwind flux (convection_lin.hpp:38-76)
            const double fl = a[d] >= 0 ? a[d] : 0.;
            const double fr = a[d] >= 0 ? 0. : a[d];
            const double flux[2] = {fl, fr};

            // same level (flux_based_scheme__lin_hom.hpp:90-111)
            for (int level = minl; level <= maxl; ++level)
            {
                const double h      = length(level);
                const double factor = hf(h, h);
                const double lc[2]  = {factor * flux[0], factor * flux[1]};
                const double rc[2]  = {-lc[0], -lc[1]};
                const auto I        = inter(m.cells[level], translate(m.cells[level], me));
                for (const auto& [k, r] : I.rows)
                {
                    for (const auto& iv : r)
                    {
                        for (int c = 0; c < 2; ++c)
                        {
                            for (int x = iv.s; x < iv.e; ++x)
                            {
                                const Coord<D> L = coord(k, x);
                                O(level, L) += lc[c] * U(level, add<D>(L, e, c));
                            }
                            for (int x = iv.s; x < iv.e; ++x)
                            {
                                const Coord<D> L = coord(k, x);
                                O(level, add<D>(L, e)) += rc[c] * U(level, add<D>(L, e, c));
                            }
                        }
                    }
                }
            }

            // level jumps (flux_based_scheme__lin_hom.hpp:113-169)
            for (int level = minl; level < maxl; ++level)
            {
                const double hl = length(level), hl1 = length(level + 1);
                {
                    // coarse left, fine right (interface.hpp:125-219)
                    const double lf = hf(hl1, hl), rf = hf(hl1, hl1);
                    const double lc[2] = {lf * flux[0], lf * flux[1]};
                    const double rc[2] = {-rf * flux[0], -rf * flux[1]};
                    const auto P       = on(inter(m.cells[level], translate(m.cells[level + 1], me)), level + 1);
                    for (const auto& [k, r] : P.rows)
                    {
                        for (const auto& iv : r)
                        {
                            const int n = iv.e - iv.s;
                            for (int c = 0; c < 2; ++c)
                            {
                                if (n == 1)
                                {
                                    const Coord<D> p = coord(k, iv.s);
                                    O(level, parent(p)) += lc[c] * U(level + 1, add<D>(p, e, c));
                                    O(level + 1, add<D>(p, e)) += rc[c] * U(level + 1, add<D>(p, e, c));
                                }
                                else
                                {
                                    for (int ii = 0; ii < n / 2; ++ii)
                                    {
                                        const Coord<D> p0 = coord(k, iv.s + 2 * ii), p1 = coord(k, iv.s + 2 * ii + 1);
                                        O(level, parent(p0)) += lc[c] * U(level + 1, add<D>(p0, e, c)) + lc[c] * U(level + 1, add<D>(p1, e, c));
                                    }
                                    for (int x = iv.s; x < iv.e; ++x)
                                    {
                                        const Coord<D> p = coord(k, x);
                                        O(level + 1, add<D>(p, e)) += rc[c] * U(level + 1, add<D>(p, e, c));
                                    }
                                }
                            }
                        }
                    }
                }
                {
                    // fine left, coarse right (interface.hpp:221-328): stencil {Q - e, Q}
                    const double lf = hf(hl1, hl1), rf = hf(hl1, hl);
                    const double lc[2] = {lf * flux[0], lf * flux[1]};
                    const double rc[2] = {-rf * flux[0], -rf * flux[1]};
                    const auto Q       = on(inter(m.cells[level], translate(m.cells[level + 1], e)), level + 1);
                    for (const auto& [k, r] : Q.rows)
                    {
                        for (const auto& iv : r)
                        {
                            const int n = iv.e - iv.s;
                            for (int c = 0; c < 2; ++c)
                            {
                                if (n == 1)
                                {
                                    const Coord<D> q  = coord(k, iv.s);
                                    const Coord<D> fl_ = add<D>(q, me);
                                    O(level + 1, fl_) += lc[c] * U(level + 1, add<D>(fl_, e, c));
                                    O(level, parent(q)) += rc[c] * U(level + 1, add<D>(fl_, e, c));
                                }
                                else
                                {
                                    for (int x = iv.s; x < iv.e; ++x)
                                    {
                                        const Coord<D> fl_ = add<D>(coord(k, x), me);
                                        O(level + 1, fl_) += lc[c] * U(level + 1, add<D>(fl_, e, c));
                                    }
                                    for (int ii = 0; ii < n / 2; ++ii)
                                    {
                                        const Coord<D> q0 = coord(k, iv.s + 2 * ii), q1 = coord(k, iv.s + 2 * ii + 1);
                                        O(level, parent(q0)) += rc[c] * U(level + 1, add<D>(add<D>(q0, me), e, c))
                                                              + rc[c] * U(level + 1, add<D>(add<D>(q1, me), e, c));
                                    }
                                }
                            }
                        }
                    }
                }
            }

            // boundary interfaces (flux_based_scheme__lin_hom.hpp:184-226)
            for (int level = 0; level < MAXL; ++level)
            {
                if (m.cells[level].empty())
                {
                    continue;
                }
                const double h = length(level);
                double co[2]   = {hf(h, h) * flux[0], hf(h, h) * flux[1]};
                for (int side = 0; side < 2; ++side)
                {
                    const Dir<D> dir = side == 0 ? e : me;
                    const auto B     = domain_boundary(m, level, dir);
                    for (const auto& [k, r] : B.rows)
                    {
                        for (const auto& iv : r)
                        {
                            for (int c = 0; c < 2; ++c)
                            {
                                for (int x = iv.s; x < iv.e; ++x)
                                {
                                    const Coord<D> X = coord(k, x);
                                    // stencil {0, e} in the direction, {-e, 0} in the opposite one
                                    const Coord<D> s = side == 0 ? add<D>(X, e, c) : add<D>(add<D>(X, me), e, c);
                                    O(level, X) += co[c] * U(level, s);
                                }
                            }
                        }
                    }
                    co[0] *= -1;
                    co[1] *= -1;
                }
            }
        }
        return out;
    }

    // Returns unp1 on the reference storage; ghost entries are NaN, which
    // is where the reference's resized unp1 holds indeterminate values.
    template <std::size_t D>
    Field upwind_step(const Mesh<D>& m, const Field& u, const std::array<double, D>& a, double dt, Scheme scheme)
    {
        Field unp1(m.nb_ref, std::numeric_limits<double>::quiet_NaN());
        if (scheme == Scheme::Convection)
        {
            // unp1 = u - dt * conv(u) on the cells (field expression, field/field_base.hpp:232-242)
            const Field out = convection_apply<D>(m, u, a);
            for (int level = 0; level < MAXL; ++level)
            {
                m.cells[level].for_each_cell(
                    [&](const Coord<D>& c)
                    {
                        const auto i = static_cast<std::size_t>(m.idx(level, c));
                        unp1[i]      = u[i] - dt * out[i];
                    });
            }
            return unp1;
        }
        for (int level = 0; level < MAXL; ++level)
        {
            const double dx = 1.0 / (1 << level); // cell_length with a unit scaling factor (cell.hpp:17-20)
            m.cells[level].for_each_cell(
                [&](const Coord<D>& c)
                {
                    auto at = [&](int d, int k)
                    {
                        Coord<D> cc = c;
                        cc[d] += k;
                        return u[static_cast<std::size_t>(m.idx(level, cc))];
                    };
                    const double uc = u[static_cast<std::size_t>(m.idx(level, c))];
                    double out;
                    if (scheme == Scheme::Readme)
                    {
                        if constexpr (D == 2)
                        {
                            out = uc - dt / dx * (uc - at(0, -1) + uc - at(1, -1));
                        }
                        else
                        {
                            out = uc - dt / dx * (uc - at(0, -1) + uc - at(1, -1) + uc - at(2, -1));
                        }
                    }
                    else
                    {
                        auto flux = [](double av, double ul, double ur) { return .5 * av * (ul + ur) + .5 * std::abs(av) * (ul - ur); };
                        double lf = flux(a[0], at(0, -1), uc);
                        double rf = flux(a[0], uc, at(0, 1));
                        double df = flux(a[1], at(1, -1), uc);
                        double uf = flux(a[1], uc, at(1, 1));
                        double s  = -lf + rf + -df + uf;
                        if constexpr (D == 3)
                        {
                            double ff = flux(a[2], at(2, -1), uc);
                            double bf = flux(a[2], uc, at(2, 1));
                            s         = s + -ff + bf;
                        }
                        double up = s / dx;
                        out       = uc - dt * up;
                    }
                    unp1[static_cast<std::size_t>(m.idx(level, c))] = out;
                });
        }
        return unp1;
    }

} // namespace oracle
