// Core device-side layout of the GB300 MR mesh.
//
// Every mesh id of samurai's MRMesh (cells, cells_and_ghosts, proj_cells,
// union_cells, reference; mr/mesh.hpp:25-33) is held as a pyramid of
// per-level bitmaps.  Level l covers the padded box
//     x in [-PX, 32*W_l - PX),  y (and z) in [-PY, 2^l + PY)
// with one bit per cell, rows ordered z-outer / y-inner and 32-bit words along
// x.  Words of all levels are concatenated in level order, so a global word
// index w identifies (level, row, x-word).
//
// FP64 fields use the same index space densely: the value of the cell at
// (word w, bit b) lives at element 32*w + b.  A warp that owns one word
// therefore reads/writes 32 consecutive doubles (256 B).
//
// samurai's storage numbering of the reference mesh (level-major, then rows,
// then x: level_cell_array.hpp:775-784, mesh.hpp:894-911) is the exclusive
// prefix popcount of the reference bitmap; rank[w] holds it per word.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sg
{
    constexpr int MAXLEV = 24; // levels 0..23 can be stored
    constexpr int PX     = 32; // x padding in cells, one word on each side
    constexpr int PY     = 8;  // y/z padding in rows on each side

    struct LevelGeom
    {
        int n;       // 2^l cells per axis inside the unit box
        int W;       // 32-bit words per row
        int R;       // rows per axis: n + 2*PY
        int sW;      // division by W: shift
        unsigned mW; // division by W: multiplier
        unsigned mR; // division by R: multiplier
        int sR;      // division by R: shift
        int pad_;
        long long nrows;  // R^(dim-1)
        long long woff;   // first word of the level
        long long nwords; // nrows * W
    };

    // Unsigned 32-bit division by a run-time constant d >= 2 as a multiply-high
    // and shifts (the round-up method of Granlund and Montgomery, "Division by
    // invariant integers using multiplication", 1994): with s = ceil(log2 d)
    // and m = floor(2^32 (2^s - d) / d) + 1, n / d = (t + ((n - t) >> 1)) >> (s - 1)
    // where t = (m n) >> 32, exact for every 32-bit n.
    inline void fastdiv_init(unsigned d, unsigned* m, int* s)
    {
        int l = 0;
        while ((1ull << l) < d)
        {
            ++l;
        }
        *s = l;
        *m = static_cast<unsigned>(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    }

    __host__ __device__ __forceinline__ unsigned fastdiv(unsigned n, unsigned m, int s)
    {
#ifdef __CUDA_ARCH__
        const unsigned t = __umulhi(m, n);
#else
        const unsigned t = static_cast<unsigned>((static_cast<unsigned long long>(m) * n) >> 32);
#endif
        return (t + ((n - t) >> 1)) >> (s - 1);
    }

    // row -> (y row, z row) of a level (3D rows are z-major)
    __host__ __device__ __forceinline__ void split_row(const LevelGeom& L, long long row, int* ry, int* rz)
    {
        const unsigned r = static_cast<unsigned>(row);
        const unsigned z = fastdiv(r, L.mR, L.sR);
        *rz              = static_cast<int>(z);
        *ry              = static_cast<int>(r - z * static_cast<unsigned>(L.R));
    }

    struct Geom
    {
        int dim;
        int nlev; // stored levels: 0..nlev-1 (= max_level + 1)
        int min_level;
        int max_level;
        long long total_words;
        int* err;      // device word of the mesh: set by kernels that met a position outside the stored box
        int periodic;  // bit d set: axis d is periodic (mesh_config::periodic)
        int ghost_width; // max(max_stencil_radius, prediction_radius)
        LevelGeom lv[MAXLEV];
    };

    inline Geom make_geom(int dim, int min_level, int max_level)
    {
        Geom g{};
        g.dim       = dim;
        g.min_level = min_level;
        g.max_level = max_level;
        g.nlev      = max_level + 1;
        long long off = 0;
        for (int l = 0; l < g.nlev; ++l)
        {
            LevelGeom& L = g.lv[l];
            L.n          = 1 << l;
            L.W          = (L.n + 31) / 32 + 2;
            L.R          = L.n + 2 * PY;
            L.nrows      = (dim == 2) ? L.R : static_cast<long long>(L.R) * L.R;
            L.woff       = off;
            L.nwords     = L.nrows * L.W;
            fastdiv_init(static_cast<unsigned>(L.W), &L.mW, &L.sW);
            fastdiv_init(static_cast<unsigned>(L.R), &L.mR, &L.sR);
            off += L.nwords;
        }
        g.total_words = off;
        return g;
    }

    // --------------------------------------------------------- positions
    struct Pos
    {
        long long w; // global word, -1 when outside the stored box
        int b;       // bit
    };

    __host__ __device__ __forceinline__ Pos pos_of(const Geom& g, int l, int x, int y, int z)
    {
        const LevelGeom& L = g.lv[l];
        const int xb       = x + PX;
        const int ry       = y + PY;
        const int rz       = z + PY;
        if (xb < 0 || xb >= 32 * L.W || ry < 0 || ry >= L.R || (g.dim == 3 && (rz < 0 || rz >= L.R)))
        {
            return {-1, 0};
        }
        const long long row = (g.dim == 2) ? ry : static_cast<long long>(rz) * L.R + ry;
        return {L.woff + row * L.W + (xb >> 5), xb & 31};
    }

    __device__ __forceinline__ bool test(const uint32_t* bm, const Pos& p)
    {
        return p.w >= 0 && ((__ldg(bm + p.w) >> p.b) & 1u);
    }

    __device__ __forceinline__ bool test(const uint32_t* bm, const Geom& g, int l, int x, int y, int z)
    {
        return test(bm, pos_of(g, l, x, y, z));
    }

    __host__ __device__ __forceinline__ long long elem(const Pos& p)
    {
        return 32 * p.w + p.b;
    }

    // coordinates of (word, bit) at level l
    struct Cell
    {
        int x, y, z;
    };

    __host__ __device__ __forceinline__ Cell cell_of(const Geom& g, int l, long long w, int b)
    {
        const LevelGeom& L = g.lv[l];
        const unsigned loc = static_cast<unsigned>(w - L.woff);
        const unsigned row = fastdiv(loc, L.mW, L.sW);
        const int wi       = static_cast<int>(loc - row * static_cast<unsigned>(L.W));
        Cell c;
        c.x = wi * 32 + b - PX;
        if (g.dim == 2)
        {
            c.y = static_cast<int>(row) - PY;
            c.z = 0;
        }
        else
        {
            int ry, rz;
            split_row(L, row, &ry, &rz);
            c.y = ry - PY;
            c.z = rz - PY;
        }
        return c;
    }

    // level of a global word (levels are few: linear scan)
    __host__ __device__ __forceinline__ int level_of(const Geom& g, long long w)
    {
        int l = 0;
        while (l + 1 < g.nlev && w >= g.lv[l + 1].woff)
        {
            ++l;
        }
        return l;
    }

    // storage index in samurai's reference numbering
    __device__ __forceinline__ long long ref_index(const uint32_t* ref, const int* rank, const Pos& p)
    {
        return static_cast<long long>(__ldg(rank + p.w)) + __popc(__ldg(ref + p.w) & ((1u << p.b) - 1u));
    }

    // ------------------------------------------------------- bit kernels
    // OR of bit pairs: 64 fine bits -> 32 coarse bits (bit j = b[2j] | b[2j+1])
    __host__ __device__ __forceinline__ uint32_t compress_pairs(uint32_t lo, uint32_t hi)
    {
        uint64_t v = static_cast<uint64_t>(lo) | (static_cast<uint64_t>(hi) << 32);
        v          = (v | (v >> 1)) & 0x5555555555555555ull;
        v          = (v | (v >> 1)) & 0x3333333333333333ull;
        v          = (v | (v >> 2)) & 0x0F0F0F0F0F0F0F0Full;
        v          = (v | (v >> 4)) & 0x00FF00FF00FF00FFull;
        v          = (v | (v >> 8)) & 0x0000FFFF0000FFFFull;
        v          = (v | (v >> 16)) & 0x00000000FFFFFFFFull;
        return static_cast<uint32_t>(v);
    }

    // even bits only: 64 fine bits -> 32 coarse bits (bit j = b[2j])
    __host__ __device__ __forceinline__ uint32_t compress_even(uint32_t lo, uint32_t hi)
    {
        uint64_t v = (static_cast<uint64_t>(lo) | (static_cast<uint64_t>(hi) << 32)) & 0x5555555555555555ull;
        v          = (v | (v >> 1)) & 0x3333333333333333ull;
        v          = (v | (v >> 2)) & 0x0F0F0F0F0F0F0F0Full;
        v          = (v | (v >> 4)) & 0x00FF00FF00FF00FFull;
        v          = (v | (v >> 8)) & 0x0000FFFF0000FFFFull;
        v          = (v | (v >> 16)) & 0x00000000FFFFFFFFull;
        return static_cast<uint32_t>(v);
    }

    // 16 coarse bits -> 32 fine bits (bit j -> bits 2j, 2j+1)
    __host__ __device__ __forceinline__ uint32_t spread16(uint32_t h)
    {
        uint32_t x = h & 0xFFFFu;
        x          = (x | (x << 8)) & 0x00FF00FFu;
        x          = (x | (x << 4)) & 0x0F0F0F0Fu;
        x          = (x | (x << 2)) & 0x33333333u;
        x          = (x | (x << 1)) & 0x55555555u;
        return x | (x << 1);
    }

    // Word of the coarsened set (parent of any member) at level l from the
    // bitmap `fine` at level l+1.  Coarse word wi of row (yc, zc) covers the
    // fine words 2*wi-1 and 2*wi of the fine rows 2*yc+{0,1} (x 2*zc+{0,1}).
    __device__ __forceinline__ uint32_t coarsen_word(const Geom& g, const uint32_t* fine, int l, long long row, int wi)
    {
        const LevelGeom& C = g.lv[l];
        const LevelGeom& F = g.lv[l + 1];
        int yc, zc;
        if (g.dim == 2)
        {
            yc = static_cast<int>(row) - PY;
            zc = 0;
        }
        else
        {
            split_row(C, row, &yc, &zc);
            yc -= PY;
            zc -= PY;
        }
        uint32_t out = 0;
        const int nz = (g.dim == 3) ? 2 : 1;
        for (int sz = 0; sz < nz; ++sz)
        {
            for (int sy = 0; sy < 2; ++sy)
            {
                const int ry = 2 * yc + sy + PY;
                const int rz = 2 * zc + sz + PY;
                if (ry < 0 || ry >= F.R || (g.dim == 3 && (rz < 0 || rz >= F.R)))
                {
                    continue;
                }
                const long long frow = (g.dim == 2) ? ry : static_cast<long long>(rz) * F.R + ry;
                const long long base = F.woff + frow * F.W;
                const int k0         = 2 * wi - 1;
                const uint32_t lo    = (k0 >= 0 && k0 < F.W) ? __ldg(fine + base + k0) : 0u;
                const uint32_t hi    = (k0 + 1 >= 0 && k0 + 1 < F.W) ? __ldg(fine + base + k0 + 1) : 0u;
                out |= compress_pairs(lo, hi);
            }
        }
        return out;
    }

    // Word of the refined set (all children) at level l from `coarse` at
    // level l-1.  Fine word k of row (yf, zf) reads coarse word (k+1)>>1 of
    // row (yf>>1, zf>>1), low half when (k+1) is even, high half otherwise.
    __device__ __forceinline__ uint32_t refine_word(const Geom& g, const uint32_t* coarse, int l, long long row, int k)
    {
        const LevelGeom& F = g.lv[l];
        const LevelGeom& C = g.lv[l - 1];
        int yf, zf;
        if (g.dim == 2)
        {
            yf = static_cast<int>(row) - PY;
            zf = 0;
        }
        else
        {
            split_row(F, row, &yf, &zf);
            yf -= PY;
            zf -= PY;
        }
        const int ry = (yf >> 1) + PY;
        const int rz = (zf >> 1) + PY;
        if (ry < 0 || ry >= C.R || (g.dim == 3 && (rz < 0 || rz >= C.R)))
        {
            return 0u;
        }
        const int wc = (k + 1) >> 1;
        if (wc >= C.W)
        {
            return 0u;
        }
        const long long crow = (g.dim == 2) ? ry : static_cast<long long>(rz) * C.R + ry;
        const uint32_t cw    = __ldg(coarse + C.woff + crow * C.W + wc);
        return spread16(((k + 1) & 1) ? (cw >> 16) : cw);
    }

    // The word one level coarser that holds the parents of the cells of word
    // (row, wi) at level l: bit 0 of the word is x = 32 wi - PX, whose parent
    // x = 16 wi - PX/2 sits at position 16 wi + 16 of the coarse row, so the 16
    // parents of the word's 32 cells occupy bits [shift, shift + 16) of one
    // coarse word.  ok is false when the parents' row leaves the coarse box.
    struct ParentWord
    {
        long long row;
        int wi;
        int shift;
        bool ok;
    };

    __host__ __device__ __forceinline__ ParentWord parent_word(const Geom& g, int l, long long row, int wi)
    {
        const LevelGeom& F = g.lv[l];
        const LevelGeom& C = g.lv[l - 1];
        int y, z;
        if (g.dim == 2)
        {
            y = static_cast<int>(row) - PY;
            z = 0;
        }
        else
        {
            split_row(F, row, &y, &z);
            y -= PY;
            z -= PY;
        }
        const int ry = (y >> 1) + PY, rz = (z >> 1) + PY; // floor halves
        const int base = 16 * wi + 16;
        ParentWord p;
        p.wi    = base >> 5;
        p.shift = base & 31;
        p.ok    = ry >= 0 && ry < C.R && (g.dim == 2 || (rz >= 0 && rz < C.R)) && p.wi < C.W;
        p.row   = (g.dim == 2) ? ry : static_cast<long long>(rz) * C.R + ry;
        return p;
    }

    // Marks in bm the ancestors, at levels l-1 down to lstop, of the cells h
    // of word (row, wi) at level l (bm's coarser levels accumulate by atomic
    // OR).  A walk stops at the first level where its bits were already set:
    // the walk that set them marks everything above.
    __device__ __forceinline__ void mark_ancestors(const Geom& g, uint32_t* bm, int l, long long row, int wi, uint32_t h, int lstop)
    {
        for (int lc = l - 1; lc >= lstop && h; --lc)
        {
            const ParentWord p = parent_word(g, lc + 1, row, wi);
            if (!p.ok)
            {
                return;
            }
            const uint32_t bits = (compress_pairs(h, 0u) & 0xFFFFu) << p.shift;
            const LevelGeom& C  = g.lv[lc];
            const uint32_t old  = atomicOr(bm + C.woff + p.row * C.W + p.wi, bits);
            if ((old & bits) == bits)
            {
                return;
            }
            h   = bits;
            row = p.row;
            wi  = p.wi;
        }
    }

    // Cells of word (row, wi) at level l that lie in bm at level l or whose
    // ancestor (levels l-1 .. lstop) lies in bm: the ancestors of the 32
    // cells at level l - k are 32 >> k cells of one word (one cell from
    // k = 5 on), read independently for every k and spread back.
    __device__ __forceinline__ uint32_t self_or_ancestor(const Geom& g, const uint32_t* bm, int l, long long row, int wi, int lstop)
    {
        const LevelGeom& L = g.lv[l];
        uint32_t acc       = __ldg(bm + L.woff + row * L.W + wi);
        int y, z;
        if (g.dim == 2)
        {
            y = static_cast<int>(row) - PY;
            z = 0;
        }
        else
        {
            split_row(L, row, &y, &z);
            y -= PY;
            z -= PY;
        }
        const int x0 = 32 * wi - PX;
        for (int k = 1; l - k >= lstop; ++k)
        {
            const LevelGeom& A = g.lv[l - k];
            const int ry = (y >> k) + PY, rz = (z >> k) + PY;
            if (ry < 0 || ry >= A.R || (g.dim == 3 && (rz < 0 || rz >= A.R)))
            {
                continue;
            }
            const int pos        = (x0 >> (k < 31 ? k : 31)) + PX;
            const long long arow = (g.dim == 2) ? ry : static_cast<long long>(rz) * A.R + ry;
            const int width      = k >= 5 ? 1 : (32 >> k);
            const uint32_t word  = __ldg(bm + A.woff + arow * A.W + (pos >> 5));
            uint32_t bits        = (word >> (pos & 31)) & (width == 32 ? 0xFFFFFFFFu : ((1u << width) - 1u));
            if (k >= 5)
            {
                acc |= bits ? 0xFFFFFFFFu : 0u;
            }
            else
            {
                for (int s = 0; s < k; ++s)
                {
                    bits = spread16(bits);
                }
                acc |= bits;
            }
        }
        return acc;
    }

    // x-dilation of one word by r (< 32) using its neighbours in the row
    __device__ __forceinline__ uint32_t dilate_x(uint32_t left, uint32_t mid, uint32_t right, int r)
    {
        uint32_t out = mid;
        for (int k = 1; k <= r; ++k)
        {
            out |= (mid << k) | (left >> (32 - k)) | (mid >> k) | (right << (32 - k));
        }
        return out;
    }

    // Box dilation split by axes: dilate_xy_word dilates along x and y within
    // a z plane (the whole box dilation in 2D), dilate_z_word along z; in 3D
    // box = z o xy reads 5 + 15 words instead of 75 for r = 2.
    __device__ __forceinline__ uint32_t dilate_xy_word(const Geom& g, const uint32_t* src, int l, long long row, int wi, int r)
    {
        const LevelGeom& L = g.lv[l];
        int ry, rz;
        if (g.dim == 2)
        {
            ry = static_cast<int>(row);
            rz = 0;
        }
        else
        {
            split_row(L, row, &ry, &rz);
        }
        uint32_t out = 0;
        for (int dy = -r; dy <= r; ++dy)
        {
            const int y2 = ry + dy;
            if (y2 < 0 || y2 >= L.R)
            {
                continue;
            }
            const long long base = L.woff + ((g.dim == 2) ? y2 : static_cast<long long>(rz) * L.R + y2) * L.W;
            const uint32_t mid   = __ldg(src + base + wi);
            const uint32_t left  = wi > 0 ? __ldg(src + base + wi - 1) : 0u;
            const uint32_t right = wi + 1 < L.W ? __ldg(src + base + wi + 1) : 0u;
            out |= dilate_x(left, mid, right, r);
        }
        return out;
    }

    __device__ __forceinline__ uint32_t dilate_z_word(const Geom& g, const uint32_t* src, int l, long long row, int wi, int r)
    {
        const LevelGeom& L = g.lv[l];
        int ry, rz;
        split_row(L, row, &ry, &rz);
        uint32_t out = 0;
        for (int dz = -r; dz <= r; ++dz)
        {
            const int z2 = rz + dz;
            if (z2 < 0 || z2 >= L.R)
            {
                continue;
            }
            out |= __ldg(src + L.woff + (static_cast<long long>(z2) * L.R + ry) * L.W + wi);
        }
        return out;
    }

    // mask of the cells of word (row, wi) at level l inside the box
    // [lo, 2^l + hi) in every direction
    __host__ __device__ __forceinline__ uint32_t box_mask(const Geom& g, int l, long long row, int wi, int lo, int hi)
    {
        const LevelGeom& L = g.lv[l];
        int y, z;
        if (g.dim == 2)
        {
            y = static_cast<int>(row) - PY;
            z = 0;
        }
        else
        {
            split_row(L, row, &y, &z);
            y -= PY;
            z -= PY;
        }
        const int a = -lo, b = L.n + hi; // allowed range [a, b)
        if (y < a || y >= b || (g.dim == 3 && (z < a || z >= b)))
        {
            return 0u;
        }
        const int x0 = wi * 32 - PX; // x of bit 0
        int s        = a - x0;
        int e        = b - x0;
        if (s < 0)
        {
            s = 0;
        }
        if (e > 32)
        {
            e = 32;
        }
        if (e <= s)
        {
            return 0u;
        }
        const uint32_t hiMask = (e == 32) ? 0xFFFFFFFFu : ((1u << e) - 1u);
        const uint32_t loMask = (1u << s) - 1u;
        return hiMask & ~loMask;
    }

    // decompose a global word index within a known level
    struct WordLoc
    {
        long long row;
        int wi;
    };

    __host__ __device__ __forceinline__ WordLoc word_loc(const Geom& g, int l, long long w)
    {
        const LevelGeom& L = g.lv[l];
        const unsigned loc = static_cast<unsigned>(w - L.woff);
        const unsigned row = fastdiv(loc, L.mW, L.sW);
        return {static_cast<long long>(row), static_cast<int>(loc - row * static_cast<unsigned>(L.W))};
    }

    // status word shared with the host
    enum Status : int
    {
        SG_OK           = 0,
        SG_ERR_ARG      = 1,
        SG_ERR_CUDA     = 2,
        SG_ERR_CAPACITY = 3,
        SG_ERR_STATE    = 4,
        SG_ERR_NOTFOUND = 5
    };
    // ------------------------------------------------------- periodic axes
    // A direction with a non-zero component along a periodic axis has no
    // boundary: its boundary conditions, corners included, are skipped
    // (algorithm/update_outer_ghost.hpp:355-366, 379, 426).
    __host__ __device__ __forceinline__ bool crosses_periodic(const Geom& g, const int* d)
    {
        for (int k = 0; k < g.dim; ++k)
        {
            if (d[k] != 0 && ((g.periodic >> k) & 1))
            {
                return true;
            }
        }
        return false;
    }

    // The 32 bits of bitmap `bm` (level l) at the positions of word (row, wi)
    // moved by -t: bit b answers "is p - t in bm" for the position p of bit b.
    // Zero where p - t leaves the stored box.
    __device__ __forceinline__ uint32_t shifted_word(const Geom& g, const uint32_t* bm, int l, long long row, int wi, int tx, int ty, int tz)
    {
        const LevelGeom& L = g.lv[l];
        long long srow;
        if (g.dim == 2)
        {
            srow = row - ty;
            if (srow < 0 || srow >= L.R)
            {
                return 0u;
            }
        }
        else
        {
            int ry, rz;
            split_row(L, row, &ry, &rz);
            const int sy = ry - ty, sz = rz - tz;
            if (sy < 0 || sy >= L.R || sz < 0 || sz >= L.R)
            {
                return 0u;
            }
            srow = static_cast<long long>(sz) * L.R + sy;
        }
        const uint32_t* rp = bm + L.woff + srow * L.W;
        const long long o  = 32LL * wi - tx; // source bit of bit 0
        const long long lw = o >> 5;         // floor division
        const int sh       = static_cast<int>(o & 31);
        const uint32_t a   = (lw >= 0 && lw < L.W) ? rp[lw] : 0u;
        const uint32_t b   = (lw + 1 >= 0 && lw + 1 < L.W) ? rp[lw + 1] : 0u;
        return sh ? ((a >> sh) | (b << (32 - sh))) : a;
    }

    // The union of the translates of bm by every periodic shift t (each
    // periodic axis moved by -n, 0 or +n cells, n = 2^l, not all zero:
    // detail::get_periodic_directions, mesh.hpp:44-80), on word (row, wi).
    __device__ __forceinline__ uint32_t periodic_translates(const Geom& g, const uint32_t* bm, int l, long long row, int wi)
    {
        const int n  = g.lv[l].n;
        uint32_t acc = 0u;
        for (int code = 0; code < 27; ++code)
        {
            const int c0 = code % 3 - 1, c1 = (code / 3) % 3 - 1, c2 = code / 9 - 1;
            if ((c0 == 0 && c1 == 0 && c2 == 0) || (g.dim == 2 && c2 != 0) || (c0 && !(g.periodic & 1)) || (c1 && !(g.periodic & 2))
                || (c2 && !(g.periodic & 4)))
            {
                continue;
            }
            acc |= shifted_word(g, bm, l, row, wi, c0 * n, c1 * n, c2 * n);
        }
        return acc;
    }

} // namespace sg
