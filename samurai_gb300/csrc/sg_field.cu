// FP64 kernels of the MR advection step on the dense level slabs:
// update_ghost_mr (outer ghosts, projection, prediction), wavelet details,
// keep/coarsen/refine criteria, tag finalisation, update_fields and the
// first-order upwind step.  Built with --fmad=false: every FP64 operation is
// rounded on its own, in the reference's association order, so that the
// detail thresholds take the same decisions as the CPU implementation.
#include <algorithm>
#include <cstring>
#include <functional>
#include <type_traits>

#include "sg_access.cuh"
#include "sg_ctx.cuh"

namespace sg
{
    // the mesh's device error word (Geom::err), read and cleared
    int device_error(Ctx& c)
    {
        int v = 0;
        if (read_device_error(c, &v) != cudaSuccess)
        {
            return check(c, "device_error");
        }
        if (v)
        {
            c.err = "a kernel addressed a cell outside the stored level box (invalid mesh)";
            return SG_ERR_STATE;
        }
        return SG_OK;
    }

    int new_cells_from_tags(Ctx& c, const DeviceMesh& m, uint32_t* nc);
    int graduate(Ctx& c, uint32_t* nc, int* iterations);
    int grad_pass(Ctx& c, uint32_t* nc, int slot, const int* guard);
    int bitmaps_differ(Ctx& c, const uint32_t* a, const uint32_t* b, int slot);

    namespace
    {
        constexpr int BLOCK = 256;

        // One warp per listed word, lane b on bit b.  The list holds the
        // non-empty words of a superset (reference or leaf cells) in
        // ascending order; word_of(w) narrows it to the subset a kernel acts
        // on.  Consecutive cells of a word are consecutive doubles, so every
        // field access of a warp is one 256-byte segment.  A null list means
        // every word of [begin, end): the dense range of small levels, which
        // a launch covers with one warp per word without loading the list
        // or its offsets (two dependent loads fewer at the head of the
        // launch; word_of is zero on the words the list leaves out).
        template <class WordF, class CellF>
        __device__ __forceinline__ void warp_list(const int* list, long long begin, long long end, long long warp0, long long nwarps, WordF word_of,
                                                  CellF cell)
        {
            const int lane = threadIdx.x & 31;
            for (long long i = begin + warp0; i < end; i += nwarps)
            {
                const long long w = list ? __ldg(list + i) : i;
                const uint32_t v  = word_of(w);
                if ((v >> lane) & 1u)
                {
                    cell(w, lane);
                }
            }
        }

        // Compacted traversal for the FP64-heavy kernels.  On the traversal
        // above a warp works on one word and the lanes of its empty bits idle
        // while the others issue FP64 instructions, which the narrow FP64 pipe
        // executes for the whole warp (42 % of the lanes of the leaf-cell
        // words of the 2D max_level-12 workload hold a cell).  Here a warp
        // takes ch consecutive words of the list, ranks their set bits with a
        // warp prefix sum and processes them 32 at a time, one per lane.
        // item(valid, w, b) is called by every lane of the warp (so that it
        // may shuffle); only lanes with valid set hold an item, bit b of word w.
        constexpr unsigned FULL_MASK = 0xffffffffu;

        // words per warp: the largest power of two (<= 32) that still leaves
        // every warp of the launch a chunk; 1 on lists shorter than two words
        // per warp, where the launch is latency-bound and the compaction does
        // not pay
        __device__ __forceinline__ int items_chunk(long long n, long long nwarps)
        {
            const long long per = n / (nwarps > 0 ? nwarps : 1);
            int ch              = 1;
            while (ch < 32 && 2 * ch <= per)
            {
                ch <<= 1;
            }
            return ch;
        }

        template <class WordF, class ItemF>
        __device__ __forceinline__ void warp_items(const int* list, long long begin, long long end, long long warp0, long long nwarps, int ch,
                                                   WordF word_of, ItemF item)
        {
            const int lane = threadIdx.x & 31;
            for (long long c0 = begin + warp0 * ch; c0 < end; c0 += nwarps * ch)
            {
                long long w = 0;
                uint32_t m  = 0u;
                if (lane < ch && c0 + lane < end)
                {
                    w = list ? __ldg(list + c0 + lane) : c0 + lane;
                    m = word_of(w);
                }
                int incl = __popc(m); // inclusive prefix of the item counts over the lanes
                for (int o = 1; o < 32; o <<= 1)
                {
                    const int t = __shfl_up_sync(FULL_MASK, incl, o);
                    if (lane >= o)
                    {
                        incl += t;
                    }
                }
                const int total = __shfl_sync(FULL_MASK, incl, 31);
                for (int base = 0; base < total; base += 32)
                {
                    const int j = base + lane;
                    // the word of item j: the first lane whose inclusive prefix exceeds j
                    int lo_k = 0, hi_k = 31;
                    for (int s = 0; s < 5; ++s)
                    {
                        const int mid = (lo_k + hi_k) >> 1;
                        if (__shfl_sync(FULL_MASK, incl, mid) > j)
                        {
                            hi_k = mid;
                        }
                        else
                        {
                            lo_k = mid + 1;
                        }
                    }
                    const long long wk = __shfl_sync(FULL_MASK, w, lo_k);
                    const uint32_t mk  = __shfl_sync(FULL_MASK, m, lo_k);
                    const int before   = __shfl_sync(FULL_MASK, incl, lo_k) - __popc(mk);
                    const bool valid   = j < total;
                    // position of set bit number r (from 0) of mk
                    int r = valid ? j - before : 0, pos = 0;
                    uint32_t x = mk;
                    for (int sh = 16; sh > 0; sh >>= 1)
                    {
                        const int cnt = __popc(x & ((1u << sh) - 1u));
                        if (r >= cnt)
                        {
                            r -= cnt;
                            x >>= sh;
                            pos += sh;
                        }
                    }
                    item(valid, wk, pos);
                }
            }
        }

        // warp_list with the compacted traversal where the list is long enough:
        // cell(w, b) for every set bit
        template <class WordF, class CellF>
        __device__ __forceinline__ void warp_list_compact(const int* list, long long begin, long long end, long long warp0, long long nwarps,
                                                          WordF word_of, CellF cell)
        {
            const int ch = items_chunk(end - begin, nwarps);
            if (ch == 1)
            {
                warp_list(list, begin, end, warp0, nwarps, word_of, cell);
                return;
            }
            warp_items(list, begin, end, warp0, nwarps, ch, word_of,
                       [&](bool valid, long long w, int b)
                       {
                           if (valid)
                           {
                               cell(w, b);
                           }
                       });
        }

        __device__ __forceinline__ long long warp_id()
        {
            return (blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x) >> 5;
        }

        __device__ __forceinline__ long long warp_count()
        {
            return (static_cast<long long>(gridDim.x) * blockDim.x) >> 5;
        }


        // The prediction coefficients interp_coeffs<3> (numeric/prediction.hpp:32-36)
        // of tap t in {0,1,2} for a child of parity q are 1 at t = 1 and
        // +-1/8 at t = 0, 2 (negative at t = 0 for odd children, at t = 2 for
        // even ones); products over the axes are +-8^-k, k = off-centre taps.

        // Element of a cell that the reference algorithm guarantees to be in
        // the stored box.  A position outside it (a bug or an invalid mesh)
        // is recorded in the device error word and redirected to element 0,
        // so that no access leaves the allocation.
        __device__ __forceinline__ long long elem_at(const Geom& g, int l, int x, int y, int z)
        {
            const Pos p = pos_of(g, l, x, y, z);
            if (p.w < 0)
            {
                atomicOr(g.err, 1);
                return 0;
            }
            return elem(p);
        }

        // x * 2^-s (0 < s < 64), exactly, without the FP64 pipe when it can: for
        // a normal x whose product stays normal the product is x with its
        // exponent lowered by s (what the multiplication rounds to, since it is
        // exact); zeros keep their bits; other values take the multiplication.
        __device__ __forceinline__ double scale_down(double x, int s)
        {
            const long long b = __double_as_longlong(x);
            const int e       = static_cast<int>((b >> 52) & 0x7FF);
            if (e > s && e < 0x7FF)
            {
                return __longlong_as_double(b - (static_cast<long long>(s) << 52));
            }
            if ((static_cast<unsigned long long>(b) << 1) == 0)
            {
                return x;
            }
            return x * __longlong_as_double(static_cast<long long>(1023 - s) << 52);
        }

        // x * 8^-k: the prediction coefficients' magnitudes
        __device__ __forceinline__ double scale8(double x, int k)
        {
            return scale_down(x, 3 * k);
        }

        template <int CAP>
        __device__ __forceinline__ LinForm<CAP> scale_down(const LinForm<CAP>& x, int s)
        {
            return x * (1.0 / static_cast<double>(1LL << s));
        }

        // -x when neg, by the sign bit (exact, no FP64 operation)
        __device__ __forceinline__ double negate_if(bool neg, double x)
        {
            return __longlong_as_double(__double_as_longlong(x) ^ (static_cast<long long>(neg) << 63));
        }

        template <int CAP>
        __device__ __forceinline__ LinForm<CAP> scale8(const LinForm<CAP>& x, int k)
        {
            return x * (k == 1 ? 0.125 : (k == 2 ? 0.015625 : 0.001953125));
        }

        template <int CAP>
        __device__ __forceinline__ LinForm<CAP> negate_if(bool neg, const LinForm<CAP>& x)
        {
            return neg ? -x : x;
        }

        // A box of cells [x0, x0+n) x [y0, y0+n) x [z0, z0+n) at level l as a base
        // element and strides: both corners are checked against the stored
        // box (a violation is recorded and every access goes to element 0)
        struct Box3
        {
            long long base, sy, sz;
        };

        template <int DIM>
        __device__ __forceinline__ Box3 box_at(const Geom& g, int l, int x0, int y0, int z0, int n)
        {
            const Pos lo = pos_of(g, l, x0, y0, DIM == 3 ? z0 : 0);
            const Pos hi = pos_of(g, l, x0 + n - 1, y0 + n - 1, DIM == 3 ? z0 + n - 1 : 0);
            if (lo.w < 0 || hi.w < 0)
            {
                atomicOr(g.err, 1);
                return {0, 0, 0};
            }
            const LevelGeom& L = g.lv[l];
            return {elem(lo), 32LL * L.W, 32LL * L.W * L.R};
        }

        // prediction_op<order,false> for one fine cell (numeric/prediction.hpp:286-361)
        template <int DIM, class A>
        __device__ __forceinline__ typename A::V predict_one(const Geom& g, const A& u, int l, int x, int y, int z, int order)
        {
            const int px = x >> 1, py = y >> 1, pz = z >> 1;
            if (order == 0)
            {
                return u.get(elem_at(g, l - 1, px, py, pz));
            }
            // acc + u * coeff with coeff = ((1 * cx) * cy) * cz = +-8^-k (k = axes
            // with an off-centre tap): u * coeff is +-(u * 8^-k) bit for bit
            // (power-of-two scaling is exact) and acc + (-m) is acc - m
            typename A::V acc = A::konst(0.);
            const int qx = x & 1, qy = y & 1, qz = z & 1;
            const Box3 bx     = box_at<DIM>(g, l - 1, px - 1, py - 1, pz - 1, 3);
#pragma unroll
            for (int sz = 0; sz < (DIM == 3 ? 3 : 1); ++sz)
            {
#pragma unroll
                for (int sy = 0; sy < 3; ++sy)
                {
                    const long long base = bx.base + sy * bx.sy + sz * bx.sz;
#pragma unroll
                    for (int sx = 0; sx < 3; ++sx)
                    {
                        const int k      = (sx != 1) + (sy != 1) + (DIM == 3 && sz != 1);
                        const bool neg   = ((sx == 0 && qx) || (sx == 2 && !qx)) ^ ((sy == 0 && qy) || (sy == 2 && !qy))
                                         ^ (DIM == 3 && ((sz == 0 && qz) || (sz == 2 && !qz)));
                        const typename A::V v = u.get(base + sx);
                        // acc + u * coeff == acc + (+-m): one FP64 addition per tap
                        const typename A::V m = k == 0 ? v : scale8(v, k);
                        acc                   = acc + negate_if(neg, m);
                    }
                }
            }
            return acc;
        }

        // projection_op_ (numeric/projection.hpp:15-65)
        template <int DIM, class A>
        __device__ __forceinline__ typename A::V project_one(const Geom& g, const A& u, int lf, int x, int y, int z)
        {
            typename A::V sum = A::konst(0.);
            const Box3 bx     = box_at<DIM>(g, lf, 2 * x, 2 * y, 2 * z, 2);
#pragma unroll
            for (int sz = 0; sz < (DIM == 3 ? 2 : 1); ++sz)
            {
#pragma unroll
                for (int sy = 0; sy < 2; ++sy)
                {
                    const long long e = bx.base + sy * bx.sy + sz * bx.sz;
                    sum               = sum + (u.get(e) + u.get(e + 1));
                }
            }
            // sum * (1 / 2^dim)
            return scale_down(sum, DIM);
        }

        // ----------------------------------------------------------- tags
        __global__ void k_tag_init(const __grid_constant__ Geom gp, const int* wl, const long long* lo, const uint32_t* ref, const uint32_t* cells,
                                   uint8_t* tag, double* det)
        {
            warp_list(wl, lo[LO_REF], lo[LO_REF + gp.nlev], warp_id(), warp_count(), [&](long long w) { return ref[w]; },
                      [&](long long w, int b)
                      {
                          const long long e = 32 * w + b;
                          tag[e]            = static_cast<uint8_t>((cells[w] >> b) & 1u);
                          det[e]            = 0.;
                      });
        }

        // ----------------------------------------------------- outer ghosts
        // k-th diagonal direction in for_each_diagonal_direction order
        // (stencil.hpp:338-349): first coordinate fastest, at least two
        // non-zero components
        __device__ __forceinline__ void diagonal_dir(int dim, int k, int* d)
        {
            int found = 0;
            const int nz = (dim == 3) ? 3 : 1;
            for (int t = 0; t < 9 * nz; ++t)
            {
                const int x = t % 3 - 1, y = (t / 3) % 3 - 1, z = (dim == 3) ? t / 9 - 1 : 0;
                if ((x != 0) + (y != 0) + (z != 0) > 1)
                {
                    if (found == k)
                    {
                        d[0] = x;
                        d[1] = y;
                        d[2] = z;
                        return;
                    }
                    ++found;
                }
            }
            d[0] = d[1] = d[2] = 0;
        }

        // PolynomialExtrapolation of the second ghost layer (bc/polynomial_extrapolation.hpp:22-92, stencil of 4
        // cells along d from c - d): u(c + 2d) = u(c - d) - 3 u(c) + 3 u(c + d), in the reference's operation order
        template <class A>
        __device__ __forceinline__ void extrapolate_layer2(const Geom& g, int l, const int* c, const int* d, const A& u)
        {
            const int z = g.dim == 3;
            const long long em = elem_at(g, l, c[0] - d[0], c[1] - d[1], z ? c[2] - d[2] : 0);
            const long long e0 = elem_at(g, l, c[0], c[1], z ? c[2] : 0);
            const long long e1 = elem_at(g, l, c[0] + d[0], c[1] + d[1], z ? c[2] + d[2] : 0);
            const long long e2 = elem_at(g, l, c[0] + 2 * d[0], c[1] + 2 * d[1], z ? c[2] + 2 * d[2] : 0);
            u.put(e2, (u.get(em) - u.get(e0) * 3.0) + u.get(e1) * 3.0);
        }

        // update_outer_corners_by_polynomial_extrapolation (bc/apply_field_bc.hpp:371-505) followed by
        // project_corner_below (algorithm/update_outer_ghost.hpp:268-337), one block per diagonal direction d:
        // layer 1 copies the corner leaf, layer 2 (ghost width 2) extrapolates along d, then the other ghosts
        // of the corner block copy the diagonal ones (the off-diagonal copies).  parts: 1 the corners, 2 their
        // projection below, 3 both (the projection reads the corners, after a block barrier).
        template <class A>
        __device__ void corner_role(const Geom& g, const int* d, int l, const uint32_t* cells, const uint32_t* ref, const A& u, int parts = 3)
        {
            if (crosses_periodic(g, d))
            {
                return; // no corner across a periodic axis (the test is uniform over the block)
            }
            const int n = g.lv[l].n;
            int nfree   = 0;
            for (int k = 0; k < g.dim; ++k)
            {
                nfree += (d[k] == 0);
            }
            const long long npos = (nfree == 0) ? 1 : n; // 3D edges have one free axis
            for (long long t = threadIdx.x; (parts & 1) && t < npos; t += blockDim.x)
            {
                int c[3];
                for (int k = 0; k < 3; ++k)
                {
                    c[k] = (k < g.dim) ? (d[k] > 0 ? n - 1 : (d[k] < 0 ? 0 : static_cast<int>(t))) : 0;
                }
                const Pos pc = pos_of(g, l, c[0], c[1], c[2]);
                if (test(cells, pc))
                {
                    const long long eg = elem_at(g, l, c[0] + d[0], c[1] + d[1], g.dim == 3 ? c[2] + d[2] : 0);
                    u.put(eg, u.get(elem(pc)));
                    if (g.ghost_width >= 2)
                    {
                        if (test(ref, g, l, c[0] + 2 * d[0], c[1] + 2 * d[1], g.dim == 3 ? c[2] + 2 * d[2] : 0))
                        {
                            extrapolate_layer2(g, l, c, d, u);
                        }
                        // off-diagonal copies: from c + k d (k = 1, 2) to c + k d + delta, delta moving the
                        // non-zero components after the first by g - (k - 1), g in [0, 2), not all zero
                        int nz[3], nnz = 0;
                        for (int k = 0; k < g.dim; ++k)
                        {
                            if (d[k] != 0)
                            {
                                nz[nnz++] = k;
                            }
                        }
                        const int combos = nnz == 3 ? 4 : 2;
                        for (int k = 1; k <= 2; ++k)
                        {
                            const int sx = c[0] + k * d[0], sy = c[1] + k * d[1], sz = g.dim == 3 ? c[2] + k * d[2] : 0;
                            const long long es = elem_at(g, l, sx, sy, sz);
                            for (int combo = 0; combo < combos; ++combo)
                            {
                                int delta[3] = {0, 0, 0};
                                bool source  = true;
                                int tmp      = combo;
                                for (int p = 1; p < nnz; ++p)
                                {
                                    const int dp = (tmp % 2) - (k - 1);
                                    tmp /= 2;
                                    delta[nz[p]] += dp * d[nz[p]];
                                    source = source && dp == 0;
                                }
                                if (!source)
                                {
                                    u.put(elem_at(g, l, sx + delta[0], sy + delta[1], sz + delta[2]), u.get(es));
                                }
                            }
                        }
                    }
                }
            }
            if (parts != 3)
            {
                if (!(parts & 2))
                {
                    return;
                }
            }
            else
            {
                __syncthreads();
            }
            for (int dl = 1; dl <= 2; ++dl)
            {
                const int pl = l - dl;
                if (pl < 0)
                {
                    break;
                }
                const int npl          = g.lv[pl].n;
                const long long npos_c = (nfree == 0) ? 1 : npl;
                for (long long t = threadIdx.x; t < npos_c; t += blockDim.x)
                {
                    int gc[3], ch[3];
                    for (int k = 0; k < 3; ++k)
                    {
                        if (k >= g.dim)
                        {
                            gc[k] = ch[k] = 0;
                            continue;
                        }
                        gc[k] = d[k] > 0 ? npl : (d[k] < 0 ? -1 : static_cast<int>(t));
                        ch[k] = (gc[k] << dl) + (d[k] == -1 ? ((1 << dl) - 1) : 0);
                    }
                    const Pos pg = pos_of(g, pl, gc[0], gc[1], gc[2]);
                    const Pos pf = pos_of(g, l, ch[0], ch[1], ch[2]);
                    if (test(ref, pg) && test(ref, pf))
                    {
                        u.put(elem(pg), u.get(elem(pf)));
                    }
                }
            }
        }

        // face position helper: direction index k in 0..2*dim-1 is
        // (+e0,-e0,+e1,-e1,...) (stencil.hpp:301-317)
        __device__ __forceinline__ void face_cell(const Geom& g, int l, int k, long long t, int* in, int* dir)
        {
            const int axis = k >> 1;
            const int sgn  = (k & 1) ? -1 : 1;
            const int n    = g.lv[l].n;
            const int f0 = static_cast<int>(t % n), f1 = static_cast<int>(t / n);
            // the free coordinates fill the non-normal axes in order
            dir[0] = dir[1] = dir[2] = 0;
            in[2]                    = 0;
            if (axis == 0)
            {
                in[0] = sgn > 0 ? n - 1 : 0;
                in[1] = f0;
                in[2] = (g.dim == 3) ? f1 : 0;
            }
            else if (axis == 1)
            {
                in[0] = f0;
                in[1] = sgn > 0 ? n - 1 : 0;
                in[2] = (g.dim == 3) ? f1 : 0;
            }
            else
            {
                in[0] = f0;
                in[1] = f1;
                in[2] = sgn > 0 ? n - 1 : 0;
            }
            dir[axis] = sgn;
        }

        struct GhostLevelArgs
        {
            int l;
            int do_corners;
            int do_project;   // project_bc: level < max_level
            int do_dirichlet; // apply_field_bc: level >= min_level and a BC is attached
            int do_predict;   // predict_bc: min_level <= level < max_level
            double value;
            int nb_corner;    // blocks of the corner role
            int nb_face;      // blocks of the face role
            long long nfaces; // face positions (2*dim directions)
            int do_proj;      // project the reference of level l onto proj_cells[l-1]
            int corner_parts; // corner_role parts run by the corner blocks
            int do_dirichlet_layer2; // the second ghost layer next to non-leaf boundary cells (level >= min_level, a BC)
        };

        // One launch per level of the top-down pass of update_ghost_mr
        // (algorithm/update_ghost_mr.hpp:206-222).  Within a level the
        // reference's operations touch disjoint cells and read only cells
        // finalised earlier, so they run concurrently as block roles:
        //  - corners: outer corners and their projection two levels down;
        //  - faces: per Cartesian direction, the Dirichlet ghost 2v - u
        //    (bc/dirichlet.hpp:22-29) then predict_bc to level l+1
        //    (update_outer_ghost.hpp:195-266) by the same thread, or project_bc
        //    (update_outer_ghost.hpp:20-155) next to union cells;
        //  - projection of the reference cells of level l onto proj_cells[l-1]
        //    (numeric/projection.hpp:15-65).
        template <int DIM, class A>
        __device__ __forceinline__ void face_work(const Geom& g, const GhostLevelArgs& a, long long t, const uint32_t* cells, const uint32_t* uni,
                                                  const uint32_t* ref, const A& u)
        {
            const int l        = a.l;
            const int n        = g.lv[l].n;
            const long long nf = (DIM == 2) ? n : static_cast<long long>(n) * n;
            const int k        = static_cast<int>(t / nf);
            int in[3], dir[3];
            face_cell(g, l, k, t - k * nf, in, dir);
            if (crosses_periodic(g, dir))
            {
                return; // a periodic axis has no boundary
            }
            const Pos pi = pos_of(g, l, in[0], in[1], in[2]);
            const int gx = in[0] + dir[0], gy = in[1] + dir[1], gz = in[2] + dir[2];
            if ((a.do_dirichlet || a.do_predict) && test(cells, pi))
            {
                const long long eg = elem_at(g, l, gx, gy, gz);
                typename A::V v;
                if (a.do_dirichlet)
                {
                    v = A::konst(2 * a.value) - u.get(elem(pi));
                    u.put(eg, v);
                    // update_further_ghosts_by_polynomial_extrapolation (bc/apply_field_bc.hpp:531-593), ghost
                    // width 2: the second layer beyond a boundary leaf, where it is a reference cell
                    if (g.ghost_width >= 2 && test(ref, g, l, gx + dir[0], gy + dir[1], gz + dir[2]))
                    {
                        extrapolate_layer2(g, l, in, dir, u);
                    }
                }
                else
                {
                    v = u.get(eg);
                }
                if (a.do_predict)
                {
                    for (int sz = 0; sz < (DIM == 3 ? 2 : 1); ++sz)
                    {
                        for (int sy = 0; sy < 2; ++sy)
                        {
                            for (int sx = 0; sx < 2; ++sx)
                            {
                                const Pos pf = pos_of(g, l + 1, 2 * gx + sx, 2 * gy + sy, DIM == 3 ? 2 * gz + sz : 0);
                                if (test(ref, pf))
                                {
                                    u.put(elem(pf), v);
                                }
                            }
                        }
                    }
                }
            }
            else if (a.do_project && test(uni, pi))
            {
                const Pos pg = pos_of(g, l, gx, gy, gz);
                if (!test(ref, pg))
                {
                    return;
                }
                typename A::V sum = A::konst(0.);
                int nch           = 0;
                for (int dl = 1; dl <= 2 && nch == 0 && l + dl < g.nlev; ++dl)
                {
                    const int lc = l + dl;
                    const int m  = 1 << dl;
                    for (int sz = 0; sz < (DIM == 3 ? m : 1); ++sz)
                    {
                        for (int sy = 0; sy < m; ++sy)
                        {
                            for (int sx = 0; sx < m; ++sx)
                            {
                                const Pos pc = pos_of(g, lc, gx * m + sx, gy * m + sy, DIM == 3 ? gz * m + sz : 0);
                                if (test(ref, pc))
                                {
                                    sum = sum + u.get(elem(pc));
                                    ++nch;
                                }
                            }
                        }
                    }
                }
                u.put(elem(pg), nch > 0 ? sum / static_cast<double>(nch) : A::konst(0.));
                // the second ghost layer beyond a boundary cell that is not a leaf but has finer leaves
                // (apply_extrapolation_bc_ghosts, bc/apply_field_bc.hpp:196-214), ghost width 2
                if (g.ghost_width >= 2 && a.do_dirichlet_layer2 && test(ref, g, l, gx + dir[0], gy + dir[1], gz + dir[2]))
                {
                    extrapolate_layer2(g, l, in, dir, u);
                }
            }
        }

        template <class A>
        struct IsRev
        {
            static constexpr bool value = false;
        };
        template <int CAP>
        struct IsRev<RevAcc<CAP>>
        {
            static constexpr bool value = true;
        };

        // The transposes of one projection and one prediction, written out instead of through linear forms: the
        // weights are those the forms would carry (2^-dim for each child; +-8^-k for each tap of the order-1
        // stencil, the signs and k as in predict_one), so the adjoint is the same operator, without building a form
        // in local memory per item.  lam[e] (e the written element) is read, scattered and, in place, cleared.
        template <int DIM, int CAP>
        __device__ __forceinline__ void project_transpose(const Geom& g, const RevAcc<CAP>& u, long long e, int lf, int x, int y, int z)
        {
            const double ld = u.lam_in[e];
            if (u.in_place)
            {
                u.lam_in[e] = 0.;
            }
            if (ld == 0.)
            {
                return;
            }
            const double wch = ld * (1.0 / static_cast<double>(1 << DIM));
            const Box3 bx    = box_at<DIM>(g, lf, 2 * x, 2 * y, 2 * z, 2);
            for (int sz = 0; sz < (DIM == 3 ? 2 : 1); ++sz)
            {
                for (int sy = 0; sy < 2; ++sy)
                {
                    const long long b = bx.base + sy * bx.sy + sz * bx.sz;
                    atomicAdd(u.lam_out + b, wch);
                    atomicAdd(u.lam_out + b + 1, wch);
                }
            }
        }

        template <int DIM, int CAP>
        __device__ __forceinline__ void predict_transpose(const Geom& g, const RevAcc<CAP>& u, long long e, int l, int x, int y, int z, int order)
        {
            const double ld = u.lam_in[e];
            if (u.in_place)
            {
                u.lam_in[e] = 0.;
            }
            if (ld == 0.)
            {
                return;
            }
            const int px = x >> 1, py = y >> 1, pz = z >> 1;
            if (order == 0)
            {
                atomicAdd(u.lam_out + elem_at(g, l - 1, px, py, pz), ld);
                return;
            }
            const int qx = x & 1, qy = y & 1, qz = z & 1;
            const Box3 bx = box_at<DIM>(g, l - 1, px - 1, py - 1, pz - 1, 3);
            for (int sz = 0; sz < (DIM == 3 ? 3 : 1); ++sz)
            {
                for (int sy = 0; sy < 3; ++sy)
                {
                    const long long base = bx.base + sy * bx.sy + sz * bx.sz;
                    for (int sx = 0; sx < 3; ++sx)
                    {
                        const int k    = (sx != 1) + (sy != 1) + (DIM == 3 && sz != 1);
                        const bool neg = ((sx == 0 && qx) || (sx == 2 && !qx)) ^ ((sy == 0 && qy) || (sy == 2 && !qy))
                                         ^ (DIM == 3 && ((sz == 0 && qz) || (sz == 2 && !qz)));
                        const double w = (k == 0 ? 1.0 : (k == 1 ? 0.125 : (k == 2 ? 0.015625 : 0.001953125))) * (neg ? -1.0 : 1.0);
                        atomicAdd(u.lam_out + base + sx, w * ld);
                    }
                }
            }
        }

        // projection of the reference cells of level l onto proj_cells[l-1]
        // (numeric/projection.hpp:15-65), warps warp0, warp0+nwarps, ...
        template <int DIM, class A>
        __device__ __forceinline__ void project_level(const Geom& g, int l, const int* wl_ref, const long long* lo, const uint32_t* proj, const uint32_t* ref,
                                                      const A& u, long long warp0, long long nwarps)
        {
            const int lc = l - 1;
            const LevelGeom& C = g.lv[lc];
            warp_list_compact(lo ? wl_ref : nullptr, lo ? lo[LO_REF + lc] : C.woff, lo ? lo[LO_REF + lc + 1] : C.woff + C.nwords, warp0, nwarps,
                      [&](long long w)
                      {
                          const WordLoc loc = word_loc(g, lc, w);
                          return proj[w] & coarsen_word(g, ref, lc, loc.row, loc.wi);
                      },
                      [&](long long w, int b)
                      {
                          const Cell c = cell_of(g, lc, w, b);
                          if constexpr (IsRev<A>::value)
                          {
                              project_transpose<DIM>(g, u, 32 * w + b, l, c.x, c.y, c.z);
                          }
                          else
                          {
                              u.put(32 * w + b, project_one<DIM>(g, u, l, c.x, c.y, c.z));
                          }
                      });
        }

        // prediction of the ghosts of level l from level l-1
        // (algorithm/update_ghost_mr.hpp:224-233)
        template <int DIM, class A>
        __device__ __forceinline__ void predict_level(const Geom& g, int l, int order, const int* wl_ref, const long long* lo, const uint32_t* cells,
                                                      const uint32_t* proj, const uint32_t* ref, const A& u, long long warp0, long long nwarps)
        {
            const LevelGeom& L = g.lv[l];
            warp_list_compact(lo ? wl_ref : nullptr, lo ? lo[LO_REF + l] : L.woff, lo ? lo[LO_REF + l + 1] : L.woff + L.nwords, warp0, nwarps,
                      [&](long long w)
                      {
                          const WordLoc loc = word_loc(g, l, w);
                          return ref[w] & ~(cells[w] | proj[w]) & box_mask(g, l, loc.row, loc.wi, 0, 0) & refine_word(g, ref, l, loc.row, loc.wi);
                      },
                      [&](long long w, int b)
                      {
                          const Cell c = cell_of(g, l, w, b);
                          if constexpr (IsRev<A>::value)
                          {
                              predict_transpose<DIM>(g, u, 32 * w + b, l, c.x, c.y, c.z, order);
                          }
                          else
                          {
                              u.put(32 * w + b, predict_one<DIM>(g, u, l, c.x, c.y, c.z, order));
                          }
                      });
        }

        // One launch per level of the top-down pass of update_ghost_mr
        // (algorithm/update_ghost_mr.hpp:206-222).  Within a level the
        // reference's operations touch disjoint cells and read only cells
        // finalised earlier, so they run concurrently as block roles:
        //  - corners: outer corners and their projection two levels down;
        //  - faces: per Cartesian direction, the Dirichlet ghost 2v - u
        //    (bc/dirichlet.hpp:22-29) then predict_bc to level l+1
        //    (update_outer_ghost.hpp:195-266) by the same thread, or project_bc
        //    (update_outer_ghost.hpp:20-155) next to union cells;
        //  - projection of the reference cells of level l onto proj_cells[l-1].
        template <int DIM, class A>
        __global__ void k_ghost_level(const __grid_constant__ Geom gp, GhostLevelArgs a, const int* wl_ref, const long long* lo, const uint32_t* cells,
                                      const uint32_t* uni, const uint32_t* proj, const uint32_t* ref, A u)
        {
            const Geom& g = gp;
            const int l   = a.l;
            if (static_cast<int>(blockIdx.x) < a.nb_corner)
            {
                int d[3];
                diagonal_dir(DIM, static_cast<int>(blockIdx.x), d);
                corner_role(g, d, l, cells, ref, u, a.corner_parts);
                return;
            }
            if (static_cast<int>(blockIdx.x) < a.nb_corner + a.nb_face)
            {
                const long long t = static_cast<long long>(blockIdx.x - a.nb_corner) * blockDim.x + threadIdx.x;
                if (t < a.nfaces)
                {
                    face_work<DIM>(g, a, t, cells, uni, ref, u);
                }
                return;
            }
            if (!a.do_proj)
            {
                return;
            }
            const long long rb     = static_cast<long long>(blockIdx.x - a.nb_corner - a.nb_face);
            const long long warp0  = (rb * blockDim.x + threadIdx.x) >> 5;
            const long long nwarps = (static_cast<long long>(gridDim.x - a.nb_corner - a.nb_face) * blockDim.x) >> 5;
            project_level<DIM>(g, l, wl_ref, lo, proj, ref, u, warp0, nwarps);
        }

        // iterate_over_periodic_ghosts (algorithm/update_periodic.hpp:27-140) on
        // axis d, one side: side 0 pairs the ghosts of [n, n + gw) with [0, gw),
        // side 1 those of [-gw, 0) with [n - gw, n); the other axes span
        // [-gw, n + gw).  Only pairs of two reference cells count.  Work item t
        // of the side: gw * (n + 2 gw)^(dim-1) of them.
        __device__ __forceinline__ bool periodic_pair(const Geom& g, int l, int d, int side, long long t, const uint32_t* ref, long long* eg,
                                                      long long* ei)
        {
            const int n = g.lv[l].n, gw = g.ghost_width, span = n + 2 * gw;
            int c[3]    = {0, 0, 0};
            c[d]        = (side == 0 ? n : -gw) + static_cast<int>(t % gw);
            long long r = t / gw;
            for (int k = 0; k < g.dim; ++k)
            {
                if (k != d)
                {
                    c[k] = -gw + static_cast<int>(r % span);
                    r /= span;
                }
            }
            int q[3] = {c[0], c[1], c[2]};
            q[d] += side == 0 ? -n : n;
            const Pos pg = pos_of(g, l, c[0], c[1], c[2]);
            const Pos pi = pos_of(g, l, q[0], q[1], q[2]);
            if (!test(ref, pg) || !test(ref, pi))
            {
                return false;
            }
            *eg = elem(pg);
            *ei = elem(pi);
            return true;
        }

        inline long long periodic_side_items(const Geom& g, int l)
        {
            const long long span = g.lv[l].n + 2 * g.ghost_width;
            return g.ghost_width * (g.dim == 2 ? span : span * span);
        }

        // update_ghost_periodic(level, field) (algorithm/update_periodic.hpp:19-25)
        // on one axis: both sides at once (they read inner cells and write
        // outer ghosts, so no item reads what another writes)
        __global__ void k_periodic_copy(const __grid_constant__ Geom gp, int l, int d, long long per_side, const uint32_t* ref, double* u)
        {
            const Geom& g     = gp;
            const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (t >= 2 * per_side)
            {
                return;
            }
            const int side = t >= per_side ? 1 : 0;
            long long eg, ei;
            if (periodic_pair(g, l, d, side, t - side * per_side, ref, &eg, &ei))
            {
                u[eg] = u[ei];
            }
        }

        // update_tag_periodic(level, tag) (algorithm/update_periodic.hpp:178-300)
        // on one axis and side: both cells of a pair take the union of their tags
        __global__ void k_periodic_tag(const __grid_constant__ Geom gp, int l, int d, int side, long long per_side, const uint32_t* ref, uint8_t* tag)
        {
            const Geom& g     = gp;
            const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (t >= per_side)
            {
                return;
            }
            long long eg, ei;
            if (periodic_pair(g, l, d, side, t, ref, &eg, &ei))
            {
                tag[eg] |= tag[ei];
                tag[ei] |= tag[eg];
            }
        }

        // the periodic ghost copies of one level, axis after axis (a later axis
        // reads the ghosts an earlier one wrote: the corners)
        void periodic_copies(Ctx& c, const DeviceMesh& m, int l, double* u)
        {
            const Geom& g = c.g;
            if (!g.periodic || l < 0 || l >= g.nlev)
            {
                return;
            }
            const long long per = periodic_side_items(g, l);
            for (int d = 0; d < g.dim; ++d)
            {
                if ((g.periodic >> d) & 1)
                {
                    k_periodic_copy<<<static_cast<int>((2 * per + BLOCK - 1) / BLOCK), BLOCK, 0, c.stream>>>(c.g, l, d, per, m.ref, u);
                    launched(c, "periodic_copy");
                }
            }
        }

        void periodic_tags(Ctx& c, const DeviceMesh& m, int l)
        {
            const Geom& g = c.g;
            if (!g.periodic || l < 0 || l >= g.nlev)
            {
                return;
            }
            const long long per = periodic_side_items(g, l);
            for (int d = 0; d < g.dim; ++d)
            {
                if ((g.periodic >> d) & 1)
                {
                    for (int side = 0; side < 2; ++side)
                    {
                        k_periodic_tag<<<static_cast<int>((per + BLOCK - 1) / BLOCK), BLOCK, 0, c.stream>>>(c.g, l, d, side, per, m.ref, c.tag);
                        launched(c, "periodic_tag");
                    }
                }
            }
        }

        struct GhostChainArgs
        {
            int l_hi, l_lo; // levels of the chain, walked from l_hi down to l_lo
            int lmin;       // lowest level holding reference cells
            int has_bc;
            double value;
        };

        // The small levels of the top-down pass in one block: the roles of
        // k_ghost_level one level after the other.
        template <int DIM>
        __global__ void __launch_bounds__(1024, 1) k_ghost_levels_small(const __grid_constant__ Geom gp, GhostChainArgs ca, const int* wl_ref, const long long* lo, const uint32_t* cells,
                                             const uint32_t* uni, const uint32_t* proj, const uint32_t* ref, ValAcc u)
        {
            const Geom& g         = gp;
            const int minl        = g.min_level, maxl = g.max_level;
            const int ndiag       = (DIM == 2) ? 4 : 20;
            const long long warp0 = threadIdx.x >> 5;
            const long long nw    = blockDim.x >> 5;
            for (int l = ca.l_hi; l >= ca.l_lo; --l)
            {
                GhostLevelArgs a{};
                a.l            = l;
                a.do_project   = l < maxl;
                a.do_dirichlet = (l >= minl) && ca.has_bc;
                a.do_dirichlet_layer2 = a.do_dirichlet;
                a.do_predict   = (l >= minl && l < maxl);
                a.value        = ca.value;
                if (l >= minl && l <= maxl)
                {
                    for (int k = 0; k < ndiag; ++k)
                    {
                        int d[3];
                        diagonal_dir(DIM, k, d);
                        corner_role(g, d, l, cells, ref, u);
                    }
                }
                if (a.do_project || a.do_dirichlet || a.do_predict)
                {
                    const int n              = g.lv[l].n;
                    const long long nfaces   = static_cast<long long>(2 * DIM) * ((DIM == 2) ? n : static_cast<long long>(n) * n);
                    for (long long t = threadIdx.x; t < nfaces; t += blockDim.x)
                    {
                        face_work<DIM>(g, a, t, cells, uni, ref, u);
                    }
                }
                if (l > ca.lmin)
                {
                    project_level<DIM>(g, l, wl_ref, lo, proj, ref, u, warp0, nw);
                }
                __syncthreads();
            }
        }

        template <int DIM, class A>
        __global__ void k_predict(const __grid_constant__ Geom gp, int l, int order, const int* wl_ref, const long long* lo, const uint32_t* cells,
                                  const uint32_t* proj, const uint32_t* ref, A u)
        {
            predict_level<DIM>(gp, l, order, wl_ref, lo, cells, proj, ref, u, warp_id(), warp_count());
        }

        // the small levels of the bottom-up pass in one block
        template <int DIM>
        __global__ void __launch_bounds__(1024, 1) k_predict_small(const __grid_constant__ Geom gp, int l_lo, int l_hi, int order, const int* wl_ref, const long long* lo,
                                        const uint32_t* cells, const uint32_t* proj, const uint32_t* ref, ValAcc u)
        {
            const long long warp0 = threadIdx.x >> 5;
            const long long nw    = blockDim.x >> 5;
            for (int l = l_lo; l <= l_hi; ++l)
            {
                predict_level<DIM>(gp, l, order, wl_ref, lo, cells, proj, ref, u, warp0, nw);
                __syncthreads();
            }
        }

        // -------------------------------------------------------- details
        // compute_detail_op (mr/operators.hpp:139-540) on
        // intersection(all_cells[l], union(cells[l+1], cells[l+2])).on(l)
        template <int DIM>
        __global__ void k_detail(const __grid_constant__ Geom gp, int order, const int* wl, const long long* lo, int l0, int l1, const int* d_ite,
                                 const uint32_t* ref, const uint32_t* hc, const uint32_t* hc2, const double* u, double* det)
        {
            const Geom& g = gp;
            // levels l0 .. min(l1, max_level - ite - 1) (mr/adapt.hpp:310-317)
            const int le = min(l1, g.max_level - *d_ite - 1);
            if (le < l0)
            {
                return;
            }
            warp_list_compact(wl, lo[LO_REF + l0], lo[LO_REF + le + 1], warp_id(), warp_count(), [&](long long w) { return ref[w] & (hc[w] | hc2[w]); },
                      [&](long long w, int b)
                      {
                          const int l    = level_of(g, w);
                          const Cell c   = cell_of(g, l, w, b);
                          long long ce[8];
                          const Box3 cb = box_at<DIM>(g, l + 1, 2 * c.x, 2 * c.y, 2 * c.z, 2);
                          for (int ch = 0; ch < (1 << DIM); ++ch)
                          {
                              ce[ch] = cb.base + (ch & 1) + ((ch >> 1) & 1) * cb.sy + ((ch >> 2) & 1) * cb.sz;
                          }
                          if (order == 0)
                          {
                              const double uc = u[32 * w + b];
                              for (int ch = 0; ch < (1 << DIM); ++ch)
                              {
                                  det[ce[ch]] = u[ce[ch]] - uc;
                              }
                              return;
                          }
                          double d[8];
                          for (int ch = 0; ch < (1 << DIM); ++ch)
                          {
                              d[ch] = u[ce[ch]];
                          }
                          // d -= cf * src with cf = prod interp1 = +-8^-k (k = axes with
                          // an off-centre tap): cf * src is +-(src * 8^-k) bit for bit
                          // (power-of-two scaling is exact), and d - (-m) is d + m, so
                          // one product per source serves all children
                          const int nz  = (DIM == 3) ? 3 : 1;
                          const Box3 sb = box_at<DIM>(g, l, c.x - 1, c.y - 1, c.z - 1, 3);
#pragma unroll
                          for (int sz = 0; sz < nz; ++sz)
                          {
#pragma unroll
                              for (int sy = 0; sy < 3; ++sy)
                              {
                                  const long long base = sb.base + sy * sb.sy + sz * sb.sz;
                                  for (int sx = 0; sx < 3; ++sx)
                                  {
                                      const double src = u[base + sx];
                                      const int k      = (sx != 1) + (sy != 1) + (DIM == 3 && sz != 1);
                                      const double m   = k == 0 ? src : scale8(src, k);
                                      for (int ch = 0; ch < (1 << DIM); ++ch)
                                      {
                                          // interp1(parity, t) < 0: t == 0 on odd children, t == 2 on even ones
                                          const int px = ch & 1, py = (ch >> 1) & 1, pz = (ch >> 2) & 1;
                                          const bool neg = ((sx == 0 && px) || (sx == 2 && !px)) ^ ((sy == 0 && py) || (sy == 2 && !py))
                                                           ^ (DIM == 3 && ((sz == 0 && pz) || (sz == 2 && !pz)));
                                          d[ch]          = neg ? d[ch] + m : d[ch] - m;
                                      }
                                  }
                              }
                          }
                          for (int ch = 0; ch < (1 << DIM); ++ch)
                          {
                              det[ce[ch]] = d[ch];
                          }
                      });
        }

        // mr_criteria_op (mr/criteria.hpp:20-113) on
        // intersection(cells[l], all_cells[l-1]).on(l-1), fine levels l0..l1
        template <int DIM>
        __global__ void k_criteria(const __grid_constant__ Geom gp, const double* __restrict__ eps, const int* wl, const long long* lo, int l0, int l1,
                                   const int* d_ite, const uint32_t* ref, const uint32_t* hc, const double* det, uint8_t* tag, int ncomp,
                                   long long cstride)
        {
            // |detail| above a threshold in one of the components (one per
            // adapted field, mr/criteria.hpp:45-107)
            auto above = [&](long long e, double thr)
            {
                for (int k = 0; k < ncomp; ++k)
                {
                    if (fabs(det[k * cstride + e]) > thr)
                    {
                        return true;
                    }
                }
                return false;
            };
            const Geom& g = gp;
            // fine levels l0 .. min(l1, max_level - ite) (mr/adapt.hpp:325-339); the
            // operator runs on their parents
            const int le = min(l1, g.max_level - *d_ite);
            if (le < l0)
            {
                return;
            }
            warp_list(wl, lo[LO_REF + l0 - 1], lo[LO_REF + le], warp_id(), warp_count(), [&](long long w) { return ref[w] & hc[w]; },
                      [&](long long w, int b)
                      {
                          const int lc  = level_of(g, w);
                          const int lf  = lc + 1;
                          const Cell c  = cell_of(g, lc, w, b);
                          long long fo[8];
                          const Box3 fb = box_at<DIM>(g, lf, 2 * c.x, 2 * c.y, 2 * c.z, 2);
                          for (int ch = 0; ch < (1 << DIM); ++ch)
                          {
                              fo[ch] = fb.base + (ch & 1) + ((ch >> 1) & 1) * fb.sy + ((ch >> 2) & 1) * fb.sz;
                          }
                          if (lf > g.min_level)
                          {
                              const bool cond = above(32 * w + b, eps[2 * MAXLEV + lf]);
                              if (!cond)
                              {
                                  bool ok = true;
                                  for (int ch = 0; ch < (1 << DIM); ++ch)
                                  {
                                      if (above(fo[ch], eps[lf]))
                                      {
                                          ok = false;
                                          break;
                                      }
                                  }
                                  if (ok)
                                  {
                                      for (int ch = 0; ch < (1 << DIM); ++ch)
                                      {
                                          tag[fo[ch]] = 2;
                                      }
                                  }
                              }
                          }
                          if (lf < g.max_level)
                          {
                              for (int ch = 0; ch < (1 << DIM); ++ch)
                              {
                                  if (above(fo[ch], eps[MAXLEV + lf]))
                                  {
                                      tag[fo[ch]] |= 4;
                                  }
                              }
                          }
                      });
        }

        // compute_relative_detail (mr/rel_detail.hpp:75-111), for a scalar
        // field: max |u| over the leaf cells (the bits of non-negative doubles
        // order like the doubles, so an integer atomic max is exact and
        // independent of the order), then every reference detail times
        // 1 / max (1 when max is below the machine epsilon)
        __global__ void k_absmax_init(unsigned long long* m)
        {
            *m = static_cast<unsigned long long>(__double_as_longlong(2.2250738585072014e-308)); // numeric_limits<double>::min()
        }

        __global__ void k_absmax(const int* wl, const long long* lo, int nlev, const uint32_t* cells, const double* u, unsigned long long* m)
        {
            const int lane    = threadIdx.x & 31;
            unsigned long long best = 0;
            for (long long i = lo[LO_CELLS] + warp_id(); i < lo[LO_CELLS + nlev]; i += warp_count())
            {
                const long long w = __ldg(wl + i);
                if ((__ldg(cells + w) >> lane) & 1u)
                {
                    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(fabs(u[32 * w + lane])));
                    best                       = b > best ? b : best;
                }
            }
            for (int o = 16; o > 0; o >>= 1)
            {
                const unsigned long long x = __shfl_xor_sync(0xffffffffu, best, o);
                best                       = x > best ? x : best;
            }
            if (lane == 0 && best)
            {
                atomicMax(m, best);
            }
        }

        __global__ void k_rel_scale(const int* wl, const long long* lo, int nlev, const uint32_t* ref, const unsigned long long* m, double* det)
        {
            double mx = __longlong_as_double(static_cast<long long>(*m));
            if (mx < 2.220446049250313e-16) // numeric_limits<double>::epsilon()
            {
                mx = 1.0;
            }
            const double inv = 1. / mx;
            warp_list(wl, lo[LO_REF], lo[LO_REF + nlev], warp_id(), warp_count(), [&](long long w) { return ref[w]; },
                      [&](long long w, int b) { det[32 * w + b] *= inv; });
        }

        // keep_boundary_refined (mr/adapt.hpp:245-274): in each Cartesian
        // direction, the cells of max_level outside the domain translated by
        // -max_stencil_radius times the direction (domain_boundary_layer,
        // boundary.hpp:6-21), i.e. the leaves of max_level within r cells of
        // the boundary, are tagged keep (the tag is overwritten)
        __global__ void k_keep_boundary(const __grid_constant__ Geom gp, const int* wl, const long long* lo, const uint32_t* cells, int r, uint8_t* tag)
        {
            const Geom& g = gp;
            const int l   = g.max_level;
            warp_list(wl, lo[LO_CELLS + l], lo[LO_CELLS + l + 1], warp_id(), warp_count(),
                      [&](long long w)
                      {
                          const WordLoc loc = word_loc(g, l, w);
                          return cells[w] & ~box_mask(g, l, loc.row, loc.wi, -r, -r);
                      },
                      [&](long long w, int b) { tag[32 * w + b] = 1; });
        }

        // maximum_op (mr/operators.hpp:22-96), children at level l
        template <int DIM>
        __device__ __forceinline__ void maximum_level(const Geom& g, int l, const int* wl, const long long* lo, const uint32_t* ref, const uint32_t* hc,
                                                      uint8_t* tag, long long warp0, long long nwarps)
        {
            const int lc = l - 1;
            const LevelGeom& C = g.lv[lc];
            warp_list(lo ? wl : nullptr, lo ? lo[LO_REF + lc] : C.woff, lo ? lo[LO_REF + l] : C.woff + C.nwords, warp0, nwarps,
                      [&](long long w) { return ref[w] & hc[w]; },
                      [&](long long w, int b)
                      {
                          const Cell c  = cell_of(g, lc, w, b);
                          long long fo[8];
                          uint8_t keep = 0, coarsen = 2;
                          const Box3 fb = box_at<DIM>(g, l, 2 * c.x, 2 * c.y, 2 * c.z, 2);
                          for (int ch = 0; ch < (1 << DIM); ++ch)
                          {
                              fo[ch] = fb.base + (ch & 1) + ((ch >> 1) & 1) * fb.sy + ((ch >> 2) & 1) * fb.sz;
                              const uint8_t t = tag[fo[ch]];
                              keep |= t & 1;
                              coarsen &= t & 2;
                          }
                          const long long co = 32 * w + b;
                          if (keep)
                          {
                              for (int ch = 0; ch < (1 << DIM); ++ch)
                              {
                                  tag[fo[ch]] |= 1;
                              }
                              tag[co] |= 1;
                          }
                          else if (coarsen)
                          {
                              tag[co] |= 1;
                          }
                          else
                          {
                              for (int ch = 0; ch < (1 << DIM); ++ch)
                              {
                                  tag[fo[ch]] &= static_cast<uint8_t>(~2);
                              }
                          }
                      });
        }

        // byte-wise atomic OR / AND on the tag array (through its 32-bit word)
        __device__ __forceinline__ void tag_or_atomic(uint8_t* t, unsigned v)
        {
            const unsigned long long a = reinterpret_cast<unsigned long long>(t);
            atomicOr(reinterpret_cast<unsigned*>(a & ~3ull), v << (8 * (a & 3)));
        }

        __device__ __forceinline__ void tag_and_atomic(uint8_t* t, unsigned v)
        {
            const unsigned long long a = reinterpret_cast<unsigned long long>(t);
            atomicAnd(reinterpret_cast<unsigned*>(a & ~3ull), ~((~v & 0xFFu) << (8 * (a & 3))));
        }

        // Two consecutive levels of maximum_op in one launch: the operator with children at level l (parents at
        // l-1) and the one with children at level l-1 (parents at l-2), which in sequence runs after it.  A parent
        // at l-2 needs the keep bits its children at l-1 carry after the first operator; it derives them itself
        // from their children at l: keep(p) = keep bit of p, or p is a parent of leaves (reference and hc) whose
        // children hold a keep bit or are all tagged coarsen.  Those inputs are the same before and after the
        // first operator's writes (it sets keep bits on all children only when one already holds one, and clears
        // coarsen bits only when not all hold one), so the two operators' threads run concurrently.  The bytes of
        // level l-1, written by both, take atomic updates.
        template <int DIM>
        __global__ void k_maximum2(const __grid_constant__ Geom gp, int l, const int* wl, const long long* lo, const uint32_t* ref,
                                   const uint32_t* hc, uint8_t* tag)
        {
            const Geom& g      = gp;
            const long long w1 = g.lv[l - 1].woff; // first word of level l-1
            const LevelGeom& C = g.lv[l - 1];
            warp_list(lo ? wl : nullptr, lo ? lo[LO_REF + l - 2] : g.lv[l - 2].woff, lo ? lo[LO_REF + l] : C.woff + C.nwords, warp_id(), warp_count(),
                      [&](long long w) { return ref[w] & hc[w]; },
                      [&](long long w, int b)
                      {
                          const long long co = 32 * w + b;
                          if (w >= w1)
                          {
                              // parent at l-1, children at l (maximum_op, mr/operators.hpp:22-96)
                              const Cell c  = cell_of(g, l - 1, w, b);
                              const Box3 fb = box_at<DIM>(g, l, 2 * c.x, 2 * c.y, 2 * c.z, 2);
                              long long fo[8];
                              uint8_t keep = 0, coarsen = 2;
                              for (int ch = 0; ch < (1 << DIM); ++ch)
                              {
                                  fo[ch]          = fb.base + (ch & 1) + ((ch >> 1) & 1) * fb.sy + ((ch >> 2) & 1) * fb.sz;
                                  const uint8_t t = tag[fo[ch]];
                                  keep |= t & 1;
                                  coarsen &= t & 2;
                              }
                              if (keep)
                              {
                                  for (int ch = 0; ch < (1 << DIM); ++ch)
                                  {
                                      tag[fo[ch]] |= 1;
                                  }
                                  tag_or_atomic(tag + co, 1u);
                              }
                              else if (coarsen)
                              {
                                  tag_or_atomic(tag + co, 1u);
                              }
                              else
                              {
                                  for (int ch = 0; ch < (1 << DIM); ++ch)
                                  {
                                      tag[fo[ch]] &= static_cast<uint8_t>(~2);
                                  }
                              }
                              return;
                          }
                          // parent at l-2, children p at l-1
                          const Cell c  = cell_of(g, l - 2, w, b);
                          const Box3 pb = box_at<DIM>(g, l - 1, 2 * c.x, 2 * c.y, 2 * c.z, 2);
                          long long po[8];
                          uint8_t keep = 0, coarsen = 2;
                          for (int ch = 0; ch < (1 << DIM); ++ch)
                          {
                              const int px = 2 * c.x + (ch & 1), py = 2 * c.y + ((ch >> 1) & 1), pz = 2 * c.z + ((ch >> 2) & 1);
                              po[ch]          = pb.base + (ch & 1) + ((ch >> 1) & 1) * pb.sy + ((ch >> 2) & 1) * pb.sz;
                              const uint8_t t = tag[po[ch]];
                              uint8_t k       = t & 1;
                              const Pos pp    = pos_of(g, l - 1, px, py, DIM == 3 ? pz : 0);
                              if (!k && test(ref, pp) && test(hc, pp))
                              {
                                  // p's own operator: a child's keep bit, or all children tagged coarsen
                                  const Box3 fb = box_at<DIM>(g, l, 2 * px, 2 * py, 2 * pz, 2);
                                  uint8_t ck = 0, cc = 2;
                                  for (int gc = 0; gc < (1 << DIM); ++gc)
                                  {
                                      const uint8_t tt = tag[fb.base + (gc & 1) + ((gc >> 1) & 1) * fb.sy + ((gc >> 2) & 1) * fb.sz];
                                      ck |= tt & 1;
                                      cc &= tt & 2;
                                  }
                                  k = (ck | cc) ? 1 : 0;
                              }
                              keep |= k;
                              coarsen &= t & 2;
                          }
                          if (keep)
                          {
                              for (int ch = 0; ch < (1 << DIM); ++ch)
                              {
                                  tag_or_atomic(tag + po[ch], 1u);
                              }
                              tag[co] |= 1;
                          }
                          else if (coarsen)
                          {
                              tag[co] |= 1;
                          }
                          else
                          {
                              for (int ch = 0; ch < (1 << DIM); ++ch)
                              {
                                  tag_and_atomic(tag + po[ch], static_cast<unsigned>(static_cast<uint8_t>(~2)));
                              }
                          }
                      });
        }

        template <int DIM>
        __global__ void k_maximum(const __grid_constant__ Geom gp, int l, const int* wl, const long long* lo, const uint32_t* ref, const uint32_t* hc,
                                  uint8_t* tag)
        {
            maximum_level<DIM>(gp, l, wl, lo, ref, hc, tag, warp_id(), warp_count());
        }

        // the small levels of the tag finalisation in one block, l_hi down to l_lo
        template <int DIM>
        __global__ void __launch_bounds__(1024, 1) k_maximum_small(const __grid_constant__ Geom gp, int l_hi, int l_lo, const int* wl, const long long* lo,
                                                                   const uint32_t* ref, const uint32_t* hc, uint8_t* tag)
        {
            const long long warp0 = threadIdx.x >> 5;
            const long long nw    = blockDim.x >> 5;
            for (int l = l_hi; l >= l_lo; --l)
            {
                maximum_level<DIM>(gp, l, wl, lo, ref, hc, tag, warp0, nw);
                __syncthreads();
            }
        }

        // update_fields (algorithm/update_fields.hpp:27-127): copy on
        // reference ∩ new cells, projection on coarsened cells, prediction on
        // refined cells; every other reference entry of the new field is 0.
        template <int DIM, class A>
        __global__ void k_update_fields(const __grid_constant__ Geom gp, int order, const int* wl, const long long* lo, const uint32_t* nref,
                                        const uint32_t* ncells, const uint32_t* oref, const uint32_t* ocells, const uint32_t* ohc, A uo, A un)
        {
            const Geom& g = gp;
            warp_list_compact(wl, lo[LO_REF], lo[LO_REF + g.nlev], warp_id(), warp_count(), [&](long long w) { return nref[w]; },
                      [&](long long w, int b)
                      {
                          const long long e = 32 * w + b;
                          typename A::V v   = A::konst(0.);
                          if ((ncells[w] >> b) & 1u)
                          {
                              const int l  = level_of(g, w);
                              const Cell c = cell_of(g, l, w, b);
                              if ((ohc[w] >> b) & 1u)
                              {
                                  v = project_one<DIM>(g, uo, l + 1, c.x, c.y, c.z);
                              }
                              else if (l >= 1 && test(ocells, g, l - 1, c.x >> 1, c.y >> 1, c.z >> 1))
                              {
                                  v = predict_one<DIM>(g, uo, l, c.x, c.y, c.z, order);
                              }
                              else if ((oref[w] >> b) & 1u)
                              {
                                  v = uo.get(e);
                              }
                          }
                          un.put(e, v);
                      });
        }

        // -------------------------------------------------------- upwind
        // unp1 = u - dt * upwind(a, u) (stencil_field.hpp:38-44, 91-97;
        // demos/FiniteVolume/advection_2d.cpp:144) or the README lambda
        // (README.md:144-153).  Neighbours at the same level are reference
        // cells, at fixed offsets in the dense slabs.
        // 2^l as a double from its exponent bits (no FP64 instruction)
        __device__ __forceinline__ double pow2(int l)
        {
            return __longlong_as_double(static_cast<long long>(1023 + l) << 52);
        }

        // x * 2^l (l >= 0), exactly, by raising the exponent when x and the
        // product are normal numbers; zeros keep their bits; otherwise the
        // multiplication
        __device__ __forceinline__ double scale2(double x, int l)
        {
            const long long b = __double_as_longlong(x);
            const int e       = static_cast<int>((b >> 52) & 0x7FF);
            if (e > 0 && e + l < 0x7FF)
            {
                return __longlong_as_double(b + (static_cast<long long>(l) << 52));
            }
            if ((static_cast<unsigned long long>(b) << 1) == 0)
            {
                return x;
            }
            return x * pow2(l);
        }

        struct UpwindArgs
        {
            double ha[3]; // .5 * a_d, as the reference's flux forms it
            double hb[3]; // .5 * |a_d|
            double dt;
            int scheme;
        };

        // unp1 = u - dt * upwind(a, u) (stencil_field.hpp:38-44, 91-97;
        // demos/FiniteVolume/advection_2d.cpp:144) or the README lambda
        // (README.md:144-153).  Same-level neighbours are reference cells at
        // fixed offsets in the dense slabs.  On GB300 the FP64 pipe, not HBM,
        // bounds this kernel, so FP64 work is cut without changing a rounding:
        //  - the x-face flux between two leaf cells of a word is computed once
        //    (lane b's right flux is lane b+1's left flux: same operands, same
        //    operations, same bits) and passed by a shuffle;
        //  - /dx and dt/dx use dx = 2^-l exactly: x / 2^-l == x * 2^l.
        template <int DIM>
        __global__ void k_upwind(const __grid_constant__ Geom gp, const int* wl, const long long* lo, const uint32_t* cells, const double* __restrict__ u,
                                 double* __restrict__ unp1, UpwindArgs p)
        {
            const Geom& g  = gp;
            const int lane = threadIdx.x & 31;
            // the leaf cells compacted over the lanes (warp_items); a cell's left
            // flux is its left neighbour's right flux when that neighbour is the
            // previous lane's cell (the same face, the same expression)
            const long long nb = lo[LO_CELLS], ne = lo[LO_CELLS + g.nlev];
            warp_items(wl, nb, ne, warp_id(), warp_count(), items_chunk(ne - nb, warp_count()), [&](long long w) { return __ldg(cells + w); },
                           [&](bool valid, long long w, int b)
                           {
                               int l = 0;
                               long long e = 0, sy = 0, sz = 0;
                               double uc = 0., rf = 0.;
                               if (valid)
                               {
                                   l                  = level_of(g, w);
                                   const LevelGeom& L = g.lv[l];
                                   e                  = 32 * w + b;
                                   sy                 = 32LL * L.W;
                                   sz                 = sy * L.R;
                                   uc                 = u[e];
                               }
                               if (p.scheme == 1)
                               {
                                   if (valid)
                                   {
                                       double s = uc - u[e - 1];
                                       s        = s + uc;
                                       s        = s - u[e - sy];
                                       if (DIM == 3)
                                       {
                                           s = s + uc;
                                           s = s - u[e - sz];
                                       }
                                       unp1[e] = uc - (p.dt * pow2(l)) * s;
                                   }
                                   return;
                               }
                               if (valid)
                               {
                                   const double ur = u[e + 1];
                                   rf              = p.ha[0] * (uc + ur) + p.hb[0] * (uc - ur);
                               }
                               const double rf_left = __shfl_up_sync(FULL_MASK, rf, 1);
                               const long long wl_  = __shfl_up_sync(FULL_MASK, w, 1);
                               const int bl         = __shfl_up_sync(FULL_MASK, valid ? b : -2, 1);
                               if (!valid)
                               {
                                   return;
                               }
                               double lf;
                               if (lane > 0 && wl_ == w && bl == b - 1)
                               {
                                   lf = rf_left;
                               }
                               else
                               {
                                   const double ul = u[e - 1];
                                   lf              = p.ha[0] * (ul + uc) + p.hb[0] * (ul - uc);
                               }
                               const double ud = u[e - sy], uu = u[e + sy];
                               const double df = p.ha[1] * (ud + uc) + p.hb[1] * (ud - uc);
                               const double uf = p.ha[1] * (uc + uu) + p.hb[1] * (uc - uu);
                               double s        = -lf + rf;
                               s               = s + -df;
                               s               = s + uf;
                               if (DIM == 3)
                               {
                                   const double uf2 = u[e - sz], ub2 = u[e + sz];
                                   const double ff  = p.ha[2] * (uf2 + uc) + p.hb[2] * (uf2 - uc);
                                   const double bf  = p.ha[2] * (uc + ub2) + p.hb[2] * (uc - ub2);
                                   s                = s + -ff;
                                   s                = s + bf;
                               }
                               const double up = scale2(s, l); // s / dx with dx = 2^-l
                               unp1[e]         = uc - p.dt * up;
                           });
        }


        // ---------------------------------------------- flux-form convection
        // unp1 = u - dt * conv(u) with conv = make_convection_upwind<Field>(a)
        // (schemes/fv/operators/convection_lin.hpp:16-89), explicit application
        // (explicit_flux_based_scheme__lin_hom.hpp:39-319).  The reference
        // visits interfaces (same level by level, then level jumps, then the
        // boundary, direction by direction) and adds each face's contributions
        // to both cells; one thread per leaf cell here gathers the same terms
        // in the order they reach that cell:
        //  same level   d = 0: [+lc0 u_X], [+rc0 u_X-e], [+lc1 u_X+e], [+rc1 u_X]
        //               (X left / right of a same-level face, one x-interval);
        //               d > 0: the face below (previous row) first: [+rc0 u_X-e,
        //               +rc1 u_X] then [+lc0 u_X, +lc1 u_X+e];
        //  jumps, X fine (iteration level-1): coarse on the left, then coarse on
        //               the right, neighbour values from the ghosts at X's level;
        //  jumps, X coarse (iteration level): fine on the right, then on the
        //               left, row by row; a face along x adds one term per
        //               fine row, other faces add the pair sum of the two fine
        //               cells of a row (the i.size()==1 / pair branches);
        //  boundary:    +(2^l f) terms with the outer ghost.
        // Coefficients: face length^(dim-1) / cell volume times the upwind flux
        // coefficients (a, 0) for a >= 0, (0, a) otherwise; every factor is a
        // power of two.
        template <int DIM>
        __global__ void k_convection(const __grid_constant__ Geom gp, const int* wl, const long long* lo, const uint32_t* cells, const double* __restrict__ u,
                                     double* __restrict__ unp1, UpwindArgs p, const double* __restrict__ av)
        {
            const Geom& g     = gp;
            const long long n = lo[LO_CELLS + g.nlev];
            warp_list_compact(wl, lo[LO_CELLS], n, warp_id(), warp_count(), [&](long long w) { return __ldg(cells + w); },
                              [&](long long w, int b)
                              {
                                  const int m        = level_of(g, w);
                                  const Cell cc      = cell_of(g, m, w, b);
                                  const int c[3]     = {cc.x, cc.y, cc.z};
                                  const long long eX = 32 * w + b;
                                  const double uX    = u[eX];
                                  const int nm       = 1 << m;
                                  auto leaf = [&](int l, const int* q) { return l >= 0 && l <= g.max_level && test(cells, g, l, q[0], q[1], DIM == 3 ? q[2] : 0); };
                                  auto val  = [&](int l, const int* q) { return u[elem_at(g, l, q[0], q[1], DIM == 3 ? q[2] : 0)]; };
                                  double acc = 0.;
                                  for (int d = 0; d < DIM; ++d)
                                  {
                                      const double a  = av[d];
                                      const double fl = a >= 0 ? a : 0.;
                                      const double fr = a >= 0 ? 0. : a;
                                      int xp[3] = {c[0], c[1], c[2]}, xm[3] = {c[0], c[1], c[2]};
                                      ++xp[d];
                                      --xm[d];
                                      const double s2   = pow2(m);
                                      const double lc0 = s2 * fl, lc1 = s2 * fr;
                                      const double rc0 = -lc0, rc1 = -lc1;
                                      const bool rs = leaf(m, xp), ls = leaf(m, xm);
                                      // same level
                                      if (d == 0)
                                      {
                                          if (rs) acc = acc + lc0 * uX;
                                          if (ls) acc = acc + rc0 * val(m, xm);
                                          if (rs) acc = acc + lc1 * val(m, xp);
                                          if (ls) acc = acc + rc1 * uX;
                                      }
                                      else
                                      {
                                          if (ls)
                                          {
                                              acc = acc + rc0 * val(m, xm);
                                              acc = acc + rc1 * uX;
                                          }
                                          if (rs)
                                          {
                                              acc = acc + lc0 * uX;
                                              acc = acc + lc1 * val(m, xp);
                                          }
                                      }
                                      const bool out_r = xp[d] >= nm, out_l = xm[d] < 0;
                                      // level jumps with X the fine cell
                                      int pp[3] = {xp[0] >> 1, xp[1] >> 1, xp[2] >> 1}, pm[3] = {xm[0] >> 1, xm[1] >> 1, xm[2] >> 1};
                                      const bool lcoarse = !ls && !out_l && m >= 1 && leaf(m - 1, pm);
                                      const bool rcoarse = !rs && !out_r && m >= 1 && leaf(m - 1, pp);
                                      if (lcoarse)
                                      {
                                          acc = acc + rc0 * val(m, xm);
                                          acc = acc + rc1 * uX;
                                      }
                                      if (rcoarse)
                                      {
                                          acc = acc + lc0 * uX;
                                          acc = acc + lc1 * val(m, xp);
                                      }
                                      // level jumps with X the coarse cell: its face children at m+1
                                      const double sf = pow2(m - DIM + 1);
                                      int ch[3]       = {2 * c[0], 2 * c[1], 2 * c[2]};
                                      ch[d]           = 2 * c[d] + 2;
                                      const bool rfine = !rs && !rcoarse && !out_r && leaf(m + 1, ch);
                                      ch[d]            = 2 * c[d] - 1;
                                      const bool lfine = !ls && !lcoarse && !out_l && leaf(m + 1, ch);
                                      // fine rows of the face in row order (z outer, y inner); a face
                                      // normal to y or z has the pair of fine cells within each row
                                      const int nrow = (d == 0) ? (DIM == 3 ? 4 : 2) : (DIM == 3 ? 2 : 1);
                                      if (rfine)
                                      {
                                          const double j0 = sf * fl, j1 = sf * fr;
                                          for (int r = 0; r < nrow; ++r)
                                          {
                                              int q[3] = {2 * c[0], 2 * c[1], 2 * c[2]};
                                              q[d]     = 2 * c[d] + 1;
                                              if (d == 0)
                                              {
                                                  q[1] += r & 1;
                                                  if (DIM == 3)
                                                  {
                                                      q[2] += r >> 1;
                                                  }
                                                  int qe[3] = {q[0] + 1, q[1], q[2]};
                                                  acc       = acc + j0 * val(m + 1, q);
                                                  acc       = acc + j1 * val(m + 1, qe);
                                              }
                                              else
                                              {
                                                  if (DIM == 3)
                                                  {
                                                      q[d == 1 ? 2 : 1] += r;
                                                  }
                                                  int qb[3] = {q[0] + 1, q[1], q[2]};
                                                  int qe[3] = {q[0], q[1], q[2]}, qbe[3] = {qb[0], qb[1], qb[2]};
                                                  ++qe[d];
                                                  ++qbe[d];
                                                  acc = acc + (j0 * val(m + 1, q) + j0 * val(m + 1, qb));
                                                  acc = acc + (j1 * val(m + 1, qe) + j1 * val(m + 1, qbe));
                                              }
                                          }
                                      }
                                      if (lfine)
                                      {
                                          const double j0 = -sf * fl, j1 = -sf * fr;
                                          for (int r = 0; r < nrow; ++r)
                                          {
                                              int q[3] = {2 * c[0], 2 * c[1], 2 * c[2]}; // Q, inside X on its left face
                                              if (d == 0)
                                              {
                                                  q[1] += r & 1;
                                                  if (DIM == 3)
                                                  {
                                                      q[2] += r >> 1;
                                                  }
                                                  int qm[3] = {q[0] - 1, q[1], q[2]};
                                                  acc       = acc + j0 * val(m + 1, qm);
                                                  acc       = acc + j1 * val(m + 1, q);
                                              }
                                              else
                                              {
                                                  if (DIM == 3)
                                                  {
                                                      q[d == 1 ? 2 : 1] += r;
                                                  }
                                                  int qb[3] = {q[0] + 1, q[1], q[2]};
                                                  int qm[3] = {q[0], q[1], q[2]}, qbm[3] = {qb[0], qb[1], qb[2]};
                                                  --qm[d];
                                                  --qbm[d];
                                                  acc = acc + (j0 * val(m + 1, qm) + j0 * val(m + 1, qbm));
                                                  acc = acc + (j1 * val(m + 1, q) + j1 * val(m + 1, qb));
                                              }
                                          }
                                      }
                                      // boundary interfaces
                                      if (out_r)
                                      {
                                          acc = acc + lc0 * uX;
                                          acc = acc + lc1 * val(m, xp);
                                      }
                                      if (out_l)
                                      {
                                          acc = acc + (-lc0) * val(m, xm);
                                          acc = acc + (-lc1) * uX;
                                      }
                                  }
                                  unp1[eX] = uX - p.dt * acc;
            });
        }

        // --------------------------------------------------- layout moves
        __global__ void k_gather(const int* wl, const long long* lo, int nlev, const uint32_t* ref, const int* rank, const double* dense, double* compact)
        {
            warp_list(wl, lo[LO_REF], lo[LO_REF + nlev], warp_id(), warp_count(), [&](long long w) { return ref[w]; },
                      [&](long long w, int b) { compact[ref_index(ref, rank, Pos{w, b})] = dense[32 * w + b]; });
        }

        __global__ void k_scatter(const int* wl, const long long* lo, int nlev, const uint32_t* ref, const int* rank, const double* compact, double* dense)
        {
            warp_list(wl, lo[LO_REF], lo[LO_REF + nlev], warp_id(), warp_count(), [&](long long w) { return ref[w]; },
                      [&](long long w, int b) { dense[32 * w + b] = compact[ref_index(ref, rank, Pos{w, b})]; });
        }

        __global__ void k_fill(const int* wl, const long long* lo, int nlev, const uint32_t* ref, double* dense, double v)
        {
            warp_list(wl, lo[LO_REF], lo[LO_REF + nlev], warp_id(), warp_count(), [&](long long w) { return ref[w]; }, [&](long long w, int b) { dense[32 * w + b] = v; });
        }
    } // namespace

    namespace
    {
        // one warp per word of levels l0..l1, at most the mesh's block limit
        // blocks of c.block threads: one warp per word of levels l0..l1, at most
        // max_blocks blocks of 8 warps' worth of warps
        int blocks_words(const Ctx& c, int l0, int l1)
        {
            if (l1 < l0)
            {
                return 1;
            }
            const Geom& g          = c.g;
            const long long wpb    = c.block / 32;
            const long long nb     = (g.lv[l1].woff + g.lv[l1].nwords - g.lv[l0].woff + wpb - 1) / wpb;
            const long long cap    = std::max(1LL, c.max_blocks * 8 / wpb);
            return static_cast<int>(nb < 1 ? 1 : (nb > cap ? cap : nb));
        }
    } // namespace

    namespace
    {
        // the offsets argument of a level-chain launch over levels l0..l1: null (the dense word range, no list)
        // when the launch's grid gives every word of those levels a warp of its own, else the mesh's offsets
        const long long* level_offsets(const Ctx& c, const DeviceMesh& m, int l0, int l1)
        {
            const Geom& g       = c.g;
            const long long wpb = c.block / 32;
            const long long cap = std::max(1LL, c.max_blocks * 8 / wpb) * wpb;
            const long long n   = g.lv[l1].woff + g.lv[l1].nwords - g.lv[l0].woff;
            return n <= cap ? nullptr : m.d_lo;
        }
    } // namespace

    cudaError_t launch_gather(Ctx& c, const DeviceMesh& m, const double* dense, double* compact)
    {
        k_gather<<<blocks_words(c, 0, c.g.nlev - 1), c.block, 0, c.stream>>>(m.wl_ref, m.d_lo, c.g.nlev, m.ref, m.rank, dense, compact);
        launched(c, "gather");
        return cudaGetLastError();
    }

    int gather_compact(Ctx& c, const DeviceMesh& m, const double* dense, double* compact)
    {
        if (launch_gather(c, m, dense, compact) != cudaSuccess)
        {
            c.err = "gather: kernel launch failed";
            return SG_ERR_CUDA;
        }
        return SG_OK;
    }

    cudaError_t read_device_error(Ctx& c, int* v)
    {
        *v            = 0;
        cudaError_t e = cudaMemcpyAsync(v, c.g.err, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
        if (e == cudaSuccess)
        {
            e = cudaStreamSynchronize(c.stream);
        }
        if (e == cudaSuccess && *v)
        {
            e = cudaMemsetAsync(c.g.err, 0, sizeof(int), c.stream);
        }
        return e;
    }

    int scatter_compact(Ctx& c, const DeviceMesh& m, const double* compact, double* dense)
    {
        k_scatter<<<blocks_words(c, 0, c.g.nlev - 1), c.block, 0, c.stream>>>(m.wl_ref, m.d_lo, c.g.nlev, m.ref, m.rank, compact, dense);
        launched(c, "scatter");
        return check(c, "scatter");
    }

    int fill_ref(Ctx& c, const DeviceMesh& m, double* dense, double value)
    {
        k_fill<<<blocks_words(c, 0, c.g.nlev - 1), c.block, 0, c.stream>>>(m.wl_ref, m.d_lo, c.g.nlev, m.ref, dense, value);
        launched(c, "fill");
        return check(c, "fill");
    }

    // --------------------------------------------------------------- graphs
    // The launch sequences below depend only on the level geometry and on
    // the buffers they touch: list sizes and level ranges are read on the
    // device.  Each is captured once per buffer combination into a CUDA graph
    // and replayed.
    template <class F>
    int run_cached(Ctx& c, unsigned long long k0, unsigned long long k1, unsigned long long k2, unsigned long long k3, F seq)
    {
        if (!c.use_graphs || c.timers.enabled)
        {
            if (c.trace.enabled)
            {
                trace_mark(c, nullptr);
            }
            return seq();
        }
        // a traced sequence carries its trace events as graph nodes (a head event first): a graph of its own
        if (c.trace.enabled)
        {
            k0 |= 1ull << 63;
        }
        for (auto& e : c.graphs)
        {
            if (e.key[0] == k0 && e.key[1] == k1 && e.key[2] == k2 && e.key[3] == k3)
            {
                if (cudaGraphLaunch(e.exec, c.stream) != cudaSuccess)
                {
                    return check(c, "cudaGraphLaunch");
                }
                c.n_launches += e.kernels;
                if (c.trace.enabled)
                {
                    for (const auto& mk : e.marks)
                    {
                        for (const auto& seen : c.trace.marks)
                        {
                            c.trace.reused = c.trace.reused || seen.second == mk.second;
                        }
                        c.trace.marks.push_back(mk);
                    }
                }
                return SG_OK;
            }
        }
        if (cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        {
            return check(c, "cudaStreamBeginCapture");
        }
        const int before      = c.n_launches;
        const size_t marks0   = c.trace.marks.size();
        if (c.trace.enabled)
        {
            trace_mark(c, nullptr);
        }
        int st                = seq();
        cudaGraph_t graph     = nullptr;
        cudaError_t e         = cudaStreamEndCapture(c.stream, &graph);
        // the trace events recorded during the capture belong to the graph
        std::vector<std::pair<const char*, cudaEvent_t>> marks(c.trace.marks.begin() + static_cast<long>(std::min(marks0, c.trace.marks.size())),
                                                               c.trace.marks.end());
        c.trace.marks.resize(std::min(marks0, c.trace.marks.size()));
        if (st || e != cudaSuccess)
        {
            if (graph)
            {
                cudaGraphDestroy(graph);
            }
            for (const auto& mk : marks)
            {
                give_event(c, mk.second);
            }
            if (!st)
            {
                c.err = std::string("graph capture: ") + cudaGetErrorString(e);
                st    = SG_ERR_CUDA;
            }
            cudaGetLastError();
            return st;
        }
        cudaGraphExec_t exec = nullptr;
        e                    = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess)
        {
            for (const auto& mk : marks)
            {
                give_event(c, mk.second);
            }
            return check(c, "cudaGraphInstantiate");
        }
        if (c.graphs.size() >= 64)
        {
            cudaGraphExecDestroy(c.graphs.front().exec);
            for (const auto& mk : c.graphs.front().marks)
            {
                give_event(c, mk.second);
            }
            c.graphs.erase(c.graphs.begin());
        }
        const int kernels = c.n_launches - before;
        c.graphs.push_back({{k0, k1, k2, k3}, exec, kernels, marks});
        c.trace.marks.insert(c.trace.marks.end(), marks.begin(), marks.end());
        if (cudaGraphLaunch(exec, c.stream) != cudaSuccess)
        {
            return check(c, "cudaGraphLaunch");
        }
        return SG_OK;
    }

    namespace
    {
        // A captured chain of kernel launches (one stream, no other node types) rebuilt with its kernels in the
        // opposite order.  The kernel parameters are copied from the captured nodes.
        cudaError_t reverse_chain(cudaGraph_t in, cudaGraph_t* out)
        {
            *out     = nullptr;
            size_t n = 0, nr = 0;
            cudaError_t e = cudaGraphGetNodes(in, nullptr, &n);
            if (e == cudaSuccess)
            {
                e = cudaGraphGetRootNodes(in, nullptr, &nr);
            }
            if (e != cudaSuccess)
            {
                return e;
            }
            std::vector<cudaGraphNode_t> order;
            if (n > 0)
            {
                if (nr != 1)
                {
                    return cudaErrorInvalidValue;
                }
                cudaGraphNode_t cur = nullptr;
                if ((e = cudaGraphGetRootNodes(in, &cur, &nr)) != cudaSuccess)
                {
                    return e;
                }
                while (order.size() <= n)
                {
                    order.push_back(cur);
                    size_t nd = 0;
                    if ((e = cudaGraphNodeGetDependentNodes(cur, nullptr, nullptr, &nd)) != cudaSuccess)
                    {
                        return e;
                    }
                    if (nd == 0)
                    {
                        break;
                    }
                    if (nd != 1 || (e = cudaGraphNodeGetDependentNodes(cur, &cur, nullptr, &nd)) != cudaSuccess)
                    {
                        return nd != 1 ? cudaErrorInvalidValue : e;
                    }
                }
                if (order.size() != n)
                {
                    return cudaErrorInvalidValue;
                }
            }
            if ((e = cudaGraphCreate(out, 0)) != cudaSuccess)
            {
                return e;
            }
            cudaGraphNode_t prev = nullptr;
            for (auto it = order.rbegin(); it != order.rend(); ++it)
            {
                cudaGraphNodeType t;
                cudaKernelNodeParams kp{};
                cudaGraphNode_t node = nullptr;
                if ((e = cudaGraphNodeGetType(*it, &t)) != cudaSuccess || t != cudaGraphNodeTypeKernel
                    || (e = cudaGraphKernelNodeGetParams(*it, &kp)) != cudaSuccess
                    || (e = cudaGraphAddKernelNode(&node, *out, prev ? &prev : nullptr, prev ? 1 : 0, &kp)) != cudaSuccess)
                {
                    cudaGraphDestroy(*out);
                    *out = nullptr;
                    return e != cudaSuccess ? e : cudaErrorInvalidValue;
                }
                prev = node;
            }
            return cudaSuccess;
        }
    } // namespace

    // run_cached for a launch sequence whose launches must run in the opposite order (the transpose of a chain of
    // linear operators): captured once per key, reversed, cached and replayed.  Always a graph (the reversal needs
    // the captured chain), and with no trace events inside.
    template <class F>
    int run_reversed(Ctx& c, unsigned long long k0, unsigned long long k1, unsigned long long k2, unsigned long long k3, F seq)
    {
        k0 |= 1ull << 62;
        for (auto& e : c.graphs)
        {
            if (e.key[0] == k0 && e.key[1] == k1 && e.key[2] == k2 && e.key[3] == k3)
            {
                c.n_launches += e.kernels;
                return cudaGraphLaunch(e.exec, c.stream) != cudaSuccess ? check(c, "cudaGraphLaunch") : SG_OK;
            }
        }
        const bool traced = c.trace.enabled;
        c.trace.enabled   = false;
        if (cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        {
            c.trace.enabled = traced;
            return check(c, "cudaStreamBeginCapture");
        }
        const int before  = c.n_launches;
        int st            = seq();
        cudaGraph_t graph = nullptr;
        cudaError_t e     = cudaStreamEndCapture(c.stream, &graph);
        c.trace.enabled   = traced;
        cudaGraph_t rev   = nullptr;
        if (!st && e == cudaSuccess)
        {
            e = reverse_chain(graph, &rev);
        }
        if (graph)
        {
            cudaGraphDestroy(graph);
        }
        if (st || e != cudaSuccess)
        {
            if (!st)
            {
                c.err = std::string("reversed graph: ") + cudaGetErrorString(e);
                st    = SG_ERR_CUDA;
            }
            cudaGetLastError();
            return st;
        }
        cudaGraphExec_t exec = nullptr;
        e                    = cudaGraphInstantiate(&exec, rev, 0);
        cudaGraphDestroy(rev);
        if (e != cudaSuccess)
        {
            return check(c, "cudaGraphInstantiate");
        }
        if (c.graphs.size() >= 64)
        {
            cudaGraphExecDestroy(c.graphs.front().exec);
            for (const auto& mk : c.graphs.front().marks)
            {
                give_event(c, mk.second);
            }
            c.graphs.erase(c.graphs.begin());
        }
        c.graphs.push_back({{k0, k1, k2, k3}, exec, c.n_launches - before, {}});
        return cudaGraphLaunch(exec, c.stream) != cudaSuccess ? check(c, "cudaGraphLaunch") : SG_OK;
    }

    namespace
    {
        // the Harten pass index and the criteria thresholds of one pass, baked
        // into a captured graph (the host computes them exactly as for the
        // staged copies of the per-pass path)
        struct PassSetup
        {
            double eps[3 * MAXLEV];
            int ite;
        };

        __global__ void k_pass_setup(PassSetup p, double* d_eps, int* d_ite)
        {
            for (int i = threadIdx.x; i < 3 * MAXLEV; i += blockDim.x)
            {
                d_eps[i] = p.eps[i];
            }
            if (threadIdx.x == 0)
            {
                *d_ite = p.ite;
            }
        }

        // the condition of a conditional graph node from a device word
        __global__ void k_cond_set(cudaGraphConditionalHandle h, const int* flag, int invert)
        {
            cudaGraphSetConditional(h, ((*flag != 0) ? 1u : 0u) ^ static_cast<unsigned>(invert));
        }

        // end of a loop body: repeat while *flag is set, at most limit times
        // (the count at *iter, reset before the loop); past the limit the
        // mesh's error word records it and the loop stops
        __global__ void k_loop_next(cudaGraphConditionalHandle h, const int* flag, int* iter, int limit, int* err)
        {
            const int n = ++*iter;
            bool go     = *flag != 0;
            if (go && n >= limit)
            {
                atomicOr(err, 4);
                go = false;
            }
            cudaGraphSetConditional(h, go ? 1u : 0u);
        }

        // after the passes: which final buffers (parity of the transitions) and whether the ghosts need updating
        __global__ void k_step_flags(int* a)
        {
            const int trans = a[A_TRANS];
            a[A_PAR0]       = (trans & 1) == 0;
            a[A_PAR1]       = (trans & 1) == 1;
            a[A_NEEDG]      = a[A_PASSES] == trans;
        }

        // the leaf bitmap of a transition into recording slot a[A_TRANS] (before the count moves on)
        __global__ void k_record_bits(const uint32_t* cells, uint32_t* slots, const int* a, long long words)
        {
            uint32_t* dst = slots + static_cast<long long>(a[A_TRANS]) * words;
            for (long long w = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; w < words; w += static_cast<long long>(gridDim.x) * blockDim.x)
            {
                dst[w] = cells[w];
            }
        }

        __global__ void k_adapt_words(int* a, int slot, const int* src, int value, int add)
        {
            // a[slot] = src ? *src : value, or += when add
            const int v = src ? *src : value;
            a[slot]     = add ? a[slot] + v : v;
        }

        // Appends to the graph captured on c.stream a conditional node (IF:
        // its body runs once when the condition holds; WHILE: while it holds)
        // whose condition is set by set_cond(handle) just before the node and
        // whose body is captured from body(handle) on a capture stream of its
        // own.  Conditional bodies hold kernels, memsets and copies only.
        template <class SetCond, class Body>
        int capture_conditional(Ctx& c, cudaGraphConditionalNodeType type, SetCond set_cond, Body body)
        {
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            cudaGraph_t graph          = nullptr;
            if (cudaStreamGetCaptureInfo(c.stream, &cs, nullptr, &graph) != cudaSuccess || cs != cudaStreamCaptureStatusActive)
            {
                c.err = "conditional node outside a capture";
                return SG_ERR_STATE;
            }
            if (c.cap_depth >= Ctx::CAPTURE_DEPTH || !c.cap_streams[c.cap_depth])
            {
                c.err = "conditional nodes nested too deep";
                return SG_ERR_STATE;
            }
            cudaGraphConditionalHandle h{};
            if (cudaGraphConditionalHandleCreate(&h, graph, 0, cudaGraphCondAssignDefault) != cudaSuccess)
            {
                return check(c, "cudaGraphConditionalHandleCreate");
            }
            set_cond(h);
            const cudaGraphNode_t* deps = nullptr;
            size_t nd                   = 0;
            if (cudaStreamGetCaptureInfo(c.stream, &cs, nullptr, &graph, &deps, nullptr, &nd) != cudaSuccess)
            {
                return check(c, "cudaStreamGetCaptureInfo");
            }
            cudaGraphNodeParams np{};
            np.type                 = cudaGraphNodeTypeConditional;
            np.conditional.handle   = h;
            np.conditional.type     = type;
            np.conditional.size     = 1;
            cudaGraphNode_t node    = nullptr;
            if (cudaGraphAddNode(&node, graph, deps, nullptr, nd, &np) != cudaSuccess)
            {
                return check(c, "cudaGraphAddNode (conditional)");
            }
            cudaGraph_t bodyg = np.conditional.phGraph_out[0];
            if (cudaStreamUpdateCaptureDependencies(c.stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
            {
                return check(c, "cudaStreamUpdateCaptureDependencies");
            }
            cudaStream_t s2 = c.cap_streams[c.cap_depth];
            if (cudaStreamBeginCaptureToGraph(s2, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            {
                return check(c, "cudaStreamBeginCaptureToGraph");
            }
            ++c.cap_depth;
            std::swap(c.stream, s2);
            int st = body(h);
            std::swap(c.stream, s2);
            --c.cap_depth;
            cudaGraph_t out = nullptr;
            const cudaError_t e = cudaStreamEndCapture(s2, &out);
            if (!st && e != cudaSuccess)
            {
                c.err = std::string("conditional body capture: ") + cudaGetErrorString(e);
                st    = SG_ERR_CUDA;
            }
            return st;
        }

        template <class Body>
        int capture_if(Ctx& c, const int* flag, Body body)
        {
            return capture_conditional(
                c, cudaGraphCondTypeIf,
                [&](cudaGraphConditionalHandle h)
                {
                    k_cond_set<<<1, 1, 0, c.stream>>>(h, flag, 0);
                    launched(c, "cond_set");
                },
                [&](cudaGraphConditionalHandle) { return body(); });
        }

        unsigned long long bits_of(double v)
        {
            unsigned long long b;
            std::memcpy(&b, &v, sizeof(b));
            return b;
        }

        unsigned long long ptr_key(const void* p)
        {
            return static_cast<unsigned long long>(reinterpret_cast<uintptr_t>(p));
        }

        // update_ghost_mr / update_ghost_mr_aggregated (algorithm/update_ghost_mr.hpp:195-270)
        // as a sequence of launches on accessor u.  ft: levels 0..ft run as
        // one-block chains (value accessor only; -2 for none).  split: the
        // corner projection of each level gets a launch of its own, so that
        // no launch reads what it writes (needed to record the operator).
        // after() runs after every launch.
        template <class A, class After>
        int ghost_launches(Ctx& c, DeviceMesh& m, const A& u, bool has_bc, double bcv, int ft, bool split, After after)
        {
            const Geom& g   = c.g;
            if (g.periodic)
            {
                // the periodic copies sit between the levels of both passes: no
                // level is fused into a one-block chain
                ft = -2 * MAXLEV;
            }
            // update_ghost_periodic after the boundary conditions of a level and
            // after its prediction (update_ghost_mr.hpp:205-234).  The copy the
            // reference also makes before the boundary conditions is overwritten
            // by this one before anything reads it: the boundary conditions of a
            // serial run read and write no ghost across a periodic axis.
            auto periodic = [&](int lev)
            {
                if constexpr (std::is_same<A, ValAcc>::value)
                {
                    if (g.periodic)
                    {
                        periodic_copies(c, m, lev, u.u);
                        after();
                    }
                }
            };
            const int minl  = c.cfg.min_level;
            const int maxl  = c.cfg.max_level;
            const int lmin  = minl >= 2 ? minl - 2 : 0; // no reference cell below min_level-2
            const int ndiag = (g.dim == 2) ? 4 : 20;
            int l           = maxl;
            for (; l >= lmin && l - 1 > ft; --l)
            {
                GhostLevelArgs a{};
                a.l            = l;
                a.do_corners   = (l >= minl && l <= maxl) ? 1 : 0;
                a.do_project   = l < maxl;
                a.do_dirichlet = (l >= minl) && has_bc;
                a.do_dirichlet_layer2 = a.do_dirichlet;
                a.do_predict   = (l >= minl && l < maxl);
                a.value        = bcv;
                a.nb_corner    = a.do_corners ? ndiag : 0;
                a.corner_parts = split ? 1 : 3;
                const int n    = g.lv[l].n;
                a.nfaces       = (a.do_project || a.do_dirichlet || a.do_predict)
                                     ? static_cast<long long>(2 * g.dim) * ((g.dim == 2) ? n : static_cast<long long>(n) * n)
                                     : 0;
                a.nb_face         = static_cast<int>((a.nfaces + c.block - 1) / c.block);
                a.do_proj         = l > lmin;
                const int nb_proj = a.do_proj ? blocks_words(c, l - 1, l - 1) : 0;
                const long long* proj_lo = a.do_proj ? level_offsets(c, m, l - 1, l - 1) : m.d_lo;
                const int grid    = a.nb_corner + a.nb_face + nb_proj;
                if (grid > 0)
                {
                    if (g.dim == 2)
                    {
                        k_ghost_level<2><<<grid, c.block, 0, c.stream>>>(c.g, a, m.wl_ref, proj_lo, m.cells, m.uni, m.proj, m.ref, u);
                    }
                    else
                    {
                        k_ghost_level<3><<<grid, c.block, 0, c.stream>>>(c.g, a, m.wl_ref, proj_lo, m.cells, m.uni, m.proj, m.ref, u);
                    }
                    launched(c, "ghost_level");
                    after();
                }
                if (split && a.nb_corner > 0)
                {
                    GhostLevelArgs b = a;
                    b.corner_parts   = 2;
                    b.nb_face        = 0;
                    b.nfaces         = 0;
                    b.do_proj        = 0;
                    if (g.dim == 2)
                    {
                        k_ghost_level<2><<<b.nb_corner, c.block, 0, c.stream>>>(c.g, b, m.wl_ref, m.d_lo, m.cells, m.uni, m.proj, m.ref, u);
                    }
                    else
                    {
                        k_ghost_level<3><<<b.nb_corner, c.block, 0, c.stream>>>(c.g, b, m.wl_ref, m.d_lo, m.cells, m.uni, m.proj, m.ref, u);
                    }
                    launched(c, "ghost_corner_projection");
                    after();
                }
                periodic(l);
            }
            const int lp0 = lmin > 1 ? lmin : 1;
            int lp        = lp0;
            if constexpr (std::is_same<A, ValAcc>::value)
            {
                if (l >= lmin)
                {
                    GhostChainArgs ca{l, lmin, lmin, has_bc ? 1 : 0, bcv};
                    if (g.dim == 2)
                    {
                        k_ghost_levels_small<2><<<1, 1024, 0, c.stream>>>(c.g, ca, m.wl_ref, m.d_lo, m.cells, m.uni, m.proj, m.ref, u);
                    }
                    else
                    {
                        k_ghost_levels_small<3><<<1, 1024, 0, c.stream>>>(c.g, ca, m.wl_ref, m.d_lo, m.cells, m.uni, m.proj, m.ref, u);
                    }
                    launched(c, "ghost_levels_small");
                    after();
                }
                if (lp <= maxl && lp <= ft)
                {
                    const int e = maxl < ft ? maxl : ft;
                    if (g.dim == 2)
                    {
                        k_predict_small<2><<<1, 1024, 0, c.stream>>>(c.g, lp, e, c.cfg.prediction_radius, m.wl_ref, m.d_lo, m.cells, m.proj, m.ref, u);
                    }
                    else
                    {
                        k_predict_small<3><<<1, 1024, 0, c.stream>>>(c.g, lp, e, c.cfg.prediction_radius, m.wl_ref, m.d_lo, m.cells, m.proj, m.ref, u);
                    }
                    launched(c, "predict_small");
                    after();
                    lp = e + 1;
                }
            }
            for (; lp <= maxl; ++lp)
            {
                if (g.dim == 2)
                {
                    k_predict<2><<<blocks_words(c, lp, lp), c.block, 0, c.stream>>>(c.g, lp, c.cfg.prediction_radius, m.wl_ref, level_offsets(c, m, lp, lp), m.cells, m.proj,
                                                                                   m.ref, u);
                }
                else
                {
                    k_predict<3><<<blocks_words(c, lp, lp), c.block, 0, c.stream>>>(c.g, lp, c.cfg.prediction_radius, m.wl_ref, level_offsets(c, m, lp, lp), m.cells, m.proj,
                                                                                   m.ref, u);
                }
                launched(c, "predict");
                after();
                periodic(lp);
            }
            return check(c, "update_ghost_mr");
        }

        int seq_ghost(Ctx& c, DeviceMesh& m, double* u, bool has_bc, double bcv)
        {
            ScopedTimer timer(c, T_GHOST);
            return ghost_launches(c, m, ValAcc{u}, has_bc, bcv, c.fuse_top_field, false, [] {});
        }

        // update_fields (algorithm/update_fields.hpp:27-127) from mesh m to nm
        template <class A>
        void update_fields_launch(Ctx& c, DeviceMesh& m, DeviceMesh& nm, const A& uo, const A& un)
        {
            const Geom& g = c.g;
            if (g.dim == 2)
            {
                k_update_fields<2><<<blocks_words(c, 0, g.nlev - 1), c.block, 0, c.stream>>>(c.g, c.cfg.prediction_radius, nm.wl_ref, nm.d_lo, nm.ref,
                                                                                            nm.cells, m.ref, m.cells, m.hc, uo, un);
            }
            else
            {
                k_update_fields<3><<<blocks_words(c, 0, g.nlev - 1), c.block, 0, c.stream>>>(c.g, c.cfg.prediction_radius, nm.wl_ref, nm.d_lo, nm.ref,
                                                                                            nm.cells, m.ref, m.cells, m.hc, uo, un);
            }
            launched(c, "update_fields");
        }

        // Adapt::harten up to the fixed-point test (mr/adapt.hpp:276-375):
        // tags, ghost update, details, criteria, tag finalisation, new cells,
        // two graduation passes and the comparison with the current cells.
        // Reads the pass index and thresholds staged in pinned memory; leaves
        // the flags in pinned memory.  No host synchronisation.
        // The fields fs drive the criteria, one detail component each, the
        // components stored one dense slab after the other.
        int seq_front(Ctx& c, DeviceMesh& m, DeviceMesh& nm, const std::vector<DeviceField*>& fs, const PassSetup* graphed = nullptr)
        {
            const Geom& g  = c.g;
            const int minl = c.cfg.min_level;
            const int maxl = c.cfg.max_level;
            const int nf   = static_cast<int>(fs.size());
            int st;
            if (graphed)
            {
                k_pass_setup<<<1, 128, 0, c.stream>>>(*graphed, c.d_eps, c.d_ite);
                launched(c, "pass_setup");
            }
            else
            {
                cudaMemcpyAsync(c.d_ite, c.h_ite, sizeof(int), cudaMemcpyHostToDevice, c.stream);
                cudaMemcpyAsync(c.d_eps, c.h_eps, 3 * MAXLEV * sizeof(double), cudaMemcpyHostToDevice, c.stream);
            }
            cudaMemsetAsync(c.d_flags, 0, F_COUNT * sizeof(int), c.stream);
            k_tag_init<<<blocks_words(c, 0, g.nlev - 1), c.block, 0, c.stream>>>(c.g, m.wl_ref, m.d_lo, m.ref, m.cells, c.tag, c.detail);
            launched(c, "tag_init");
            for (int k = 1; k < nf; ++k)
            {
                k_fill<<<blocks_words(c, 0, g.nlev - 1), c.block, 0, c.stream>>>(m.wl_ref, m.d_lo, g.nlev, m.ref, c.detail + k * c.capacity, 0.);
                launched(c, "fill");
            }
            if ((st = check(c, "tag_init")))
            {
                return st;
            }
            for (DeviceField* f : fs)
            {
                if ((st = seq_ghost(c, m, f->data, f->has_bc, f->bc_value)))
                {
                    return st;
                }
            }

            timer_start(c, T_DETAIL);
            const int dl0 = minl > 0 ? minl - 1 : 0;
            const int dl1 = maxl - 1;
            for (int k = 0; k < nf && dl1 >= dl0; ++k)
            {
                const double* u = fs[k]->data;
                double* det     = c.detail + k * c.capacity;
                if (g.dim == 2)
                {
                    k_detail<2><<<blocks_words(c, dl0, dl1), c.block, 0, c.stream>>>(c.g, c.cfg.prediction_radius, m.wl_ref, m.d_lo, dl0, dl1, c.d_ite,
                                                                                    m.ref, m.hc, m.hc2, u, det);
                }
                else
                {
                    k_detail<3><<<blocks_words(c, dl0, dl1), c.block, 0, c.stream>>>(c.g, c.cfg.prediction_radius, m.wl_ref, m.d_lo, dl0, dl1, c.d_ite,
                                                                                    m.ref, m.hc, m.hc2, u, det);
                }
                launched(c, "detail");
            }
            for (int k = 0; k < nf && c.rel_detail; ++k)
            {
                k_absmax_init<<<1, 1, 0, c.stream>>>(c.d_absmax);
                k_absmax<<<blocks_words(c, 0, g.nlev - 1), c.block, 0, c.stream>>>(m.wl_cells, m.d_lo, g.nlev, m.cells, fs[k]->data, c.d_absmax);
                k_rel_scale<<<blocks_words(c, 0, g.nlev - 1), c.block, 0, c.stream>>>(m.wl_ref, m.d_lo, g.nlev, m.ref, c.d_absmax, c.detail + k * c.capacity);
                launched(c, "absmax", 3);
            }
            timer_stop(c, T_DETAIL);

            timer_start(c, T_TAG);
            if (minl >= 1 && maxl >= minl)
            {
                if (g.dim == 2)
                {
                    k_criteria<2><<<blocks_words(c, minl - 1, maxl - 1), c.block, 0, c.stream>>>(c.g, c.d_eps, m.wl_ref, m.d_lo, minl, maxl, c.d_ite,
                                                                                                m.ref, m.hc, c.detail, c.tag, nf, c.capacity);
                }
                else
                {
                    k_criteria<3><<<blocks_words(c, minl - 1, maxl - 1), c.block, 0, c.stream>>>(c.g, c.d_eps, m.wl_ref, m.d_lo, minl, maxl, c.d_ite,
                                                                                                m.ref, m.hc, c.detail, c.tag, nf, c.capacity);
                }
                launched(c, "criteria");
            }
            if (c.refine_boundary)
            {
                // "refine boundary" (mr/adapt.hpp:341-346), between tag cells and tag finalization
                k_keep_boundary<<<blocks_words(c, maxl, maxl), c.block, 0, c.stream>>>(c.g, m.wl_cells, m.d_lo, m.cells, c.cfg.max_stencil_radius,
                                                                                   c.tag);
                launched(c, "keep_boundary");
            }
            timer_stop(c, T_TAG);

            timer_start(c, T_FINALIZE);
            {
                // children at levels maxl .. min_level: below min_level no parent
                // has a leaf child, so the operator has nothing to do there
                const int lstop = std::max(1, c.cfg.min_level);
                int l           = maxl;
                // periodic axes: update_tag_periodic before each level's operator
                // (mr/adapt.hpp:348-357), so no level is fused into a one-block chain
                const int top   = g.periodic ? -2 * MAXLEV : c.fuse_top_max;
                while (l >= lstop && l - 1 > top)
                {
                    periodic_tags(c, m, l);
                    if (c.level_pairs && !g.periodic && l - 1 >= lstop && l - 2 > top)
                    {
                        // children at levels l and l-1 in one launch
                        if (g.dim == 2)
                        {
                            k_maximum2<2><<<blocks_words(c, l - 2, l - 1), c.block, 0, c.stream>>>(c.g, l, m.wl_ref, level_offsets(c, m, l - 2, l - 1), m.ref, m.hc,
                                                                                         c.tag);
                        }
                        else
                        {
                            k_maximum2<3><<<blocks_words(c, l - 2, l - 1), c.block, 0, c.stream>>>(c.g, l, m.wl_ref, level_offsets(c, m, l - 2, l - 1), m.ref, m.hc,
                                                                                         c.tag);
                        }
                        launched(c, "maximum"); // the trace groups the one- and two-level launches
                        l -= 2;
                        continue;
                    }
                    if (g.dim == 2)
                    {
                        k_maximum<2><<<blocks_words(c, l - 1, l - 1), c.block, 0, c.stream>>>(c.g, l, m.wl_ref, level_offsets(c, m, l - 1, l - 1), m.ref, m.hc, c.tag);
                    }
                    else
                    {
                        k_maximum<3><<<blocks_words(c, l - 1, l - 1), c.block, 0, c.stream>>>(c.g, l, m.wl_ref, level_offsets(c, m, l - 1, l - 1), m.ref, m.hc, c.tag);
                    }
                    launched(c, "maximum");
                    --l;
                }
                if (l >= lstop)
                {
                    if (g.dim == 2)
                    {
                        k_maximum_small<2><<<1, 1024, 0, c.stream>>>(c.g, l, lstop, m.wl_ref, m.d_lo, m.ref, m.hc, c.tag);
                    }
                    else
                    {
                        k_maximum_small<3><<<1, 1024, 0, c.stream>>>(c.g, l, lstop, m.wl_ref, m.d_lo, m.ref, m.hc, c.tag);
                    }
                    launched(c, "maximum_small");
                }
                // the levels below hold no operator but still exchange their tags
                for (int lt = lstop - 1; g.periodic && lt >= 1; --lt)
                {
                    periodic_tags(c, m, lt);
                }
            }
            timer_stop(c, T_FINALIZE);
            if ((st = check(c, "criteria")))
            {
                return st;
            }

            timer_start(c, T_MESH_UPDATE);
            // the second pass runs on the device only if the first one refined
            if ((st = new_cells_from_tags(c, m, nm.cells)) || (st = grad_pass(c, nm.cells, F_GRAD0, nullptr))
                || (!graphed && (st = grad_pass(c, nm.cells, F_GRAD1, c.d_flags + F_GRAD0))))
            {
                return st;
            }
            if (graphed)
            {
                // make_graduation to its fixed point on the device: further passes while the last one refined
                // (at most 64, as on the host path)
                k_adapt_words<<<1, 1, 0, c.stream>>>(c.d_adapt, A_LOOP, c.d_flags + F_GRAD0, 0, 0);
                k_adapt_words<<<1, 1, 0, c.stream>>>(c.d_adapt, A_ITER, nullptr, 0, 0);
                launched(c, "adapt_words", 2);
                st = capture_conditional(
                    c, cudaGraphCondTypeWhile,
                    [&](cudaGraphConditionalHandle h)
                    {
                        k_cond_set<<<1, 1, 0, c.stream>>>(h, c.d_adapt + A_LOOP, 0);
                        launched(c, "cond_set");
                    },
                    [&](cudaGraphConditionalHandle h)
                    {
                        cudaMemsetAsync(c.d_flags + F_GRADX, 0, sizeof(int), c.stream);
                        int s2 = grad_pass(c, nm.cells, F_GRADX, nullptr);
                        if (!s2)
                        {
                            k_adapt_words<<<1, 1, 0, c.stream>>>(c.d_adapt, A_LOOP, c.d_flags + F_GRADX, 0, 0);
                            k_loop_next<<<1, 1, 0, c.stream>>>(h, c.d_adapt + A_LOOP, c.d_adapt + A_ITER, 64, c.g.err);
                            launched(c, "loop_next", 2);
                        }
                        return s2;
                    });
                if (st)
                {
                    return st;
                }
            }
            if ((st = bitmaps_differ(c, nm.cells, m.cells, F_DIFFER)))
            {
                return st;
            }
            timer_stop(c, T_MESH_UPDATE);
            if (!graphed)
            {
                cudaMemcpyAsync(c.h_flags, c.d_flags, F_COUNT * sizeof(int), cudaMemcpyDeviceToHost, c.stream);
            }
            return check(c, "harten front");
        }

        // new mesh from the new cells and update_fields (mr/adapt.hpp:380-386)
        // for the adapted fields fs and the fields os carried along (their
        // ghosts are updated first, mr/adapt.hpp:383)
        int seq_back(Ctx& c, DeviceMesh& m, DeviceMesh& nm, const std::vector<DeviceField*>& fs, const std::vector<DeviceField*>& os)
        {
            int st;
            for (DeviceField* f : os)
            {
                if ((st = seq_ghost(c, m, f->data, f->has_bc, f->bc_value)))
                {
                    return st;
                }
            }
            if ((st = build_mesh(c, nm)))
            {
                return st;
            }
            ScopedTimer tf(c, T_FIELDS_UPDATE);
            for (const auto* list : {&fs, &os})
            {
                for (DeviceField* f : *list)
                {
                    update_fields_launch(c, m, nm, ValAcc{f->data}, ValAcc{f->spare});
                }
            }
            return check(c, "update_fields");
        }

        // graph-cache key of a list of fields: their buffers and boundary values
        unsigned long long fields_key(const std::vector<DeviceField*>& fs, bool spares)
        {
            unsigned long long h = 1469598103934665603ull;
            auto mix             = [&](unsigned long long v)
            {
                h ^= v;
                h *= 1099511628211ull;
            };
            for (const DeviceField* f : fs)
            {
                mix(ptr_key(spares ? f->spare : f->data));
                mix(f->has_bc ? bits_of(f->bc_value) : 1ull);
            }
            return h;
        }
    } // namespace

    int update_ghost_mr(Ctx& c, DeviceField& f)
    {
        if (c.cfg.ghost_width > 2)
        {
            c.err = "update_ghost_mr: ghost widths 1 and 2 are implemented";
            return SG_ERR_ARG;
        }
        if (f.ghosts_valid && f.ghost_version == c.mesh_version)
        {
            return SG_OK;
        }
        DeviceMesh& m = c.m();
        double* u     = f.data;
        int st        = run_cached(c, 1, static_cast<unsigned long long>(c.cur), ptr_key(u), f.has_bc ? bits_of(f.bc_value) : 1ull,
                                   [&]() { return seq_ghost(c, m, u, f.has_bc, f.bc_value); });
        if (!st)
        {
            f.ghosts_valid  = true;
            f.ghost_version = c.mesh_version;
        }
        return st;
    }

    // Adapt::harten (mr/adapt.hpp:276-389) for one field, in two halves:
    // harten_begin launches everything up to the fixed-point test without
    // waiting; harten_end waits for it, finishes the graduation if needed and
    // launches the new mesh and update_fields.  Between the two halves the
    // host may launch other meshes' work (batched mode).
    int harten_begin(Ctx& c, DeviceField& f, int ite, double eps, double regularity, bool relative_detail)
    {
        return harten_begin_fields(c, {&f}, ite, eps, regularity, relative_detail);
    }

    namespace
    {
        // the criteria thresholds of Harten pass ite (mr/adapt.hpp:325-339,
        // mr/criteria.hpp:20-113): per level eps_l, 2^(reg+dim) eps_l and that
        // over 2^dim, zero on the levels the pass does not examine
        void pass_thresholds(const Ctx& c, int ite, double eps, double regularity, double* out)
        {
            const int minl = c.cfg.min_level, maxl = c.cfg.max_level, dim = c.g.dim;
            for (int l = 0; l < 3 * MAXLEV; ++l)
            {
                out[l] = 0.;
            }
            for (int l = minl; l <= maxl - ite; ++l)
            {
                const int exponent     = dim * (maxl - l);
                out[l]                 = eps / (1 << exponent);
                out[MAXLEV + l]        = std::pow(2.0, regularity + dim) * out[l];
                out[2 * MAXLEV + l]    = out[MAXLEV + l] / (1 << dim);
            }
        }
    } // namespace

    int harten_begin_fields(Ctx& c, const std::vector<DeviceField*>& fs, int ite, double eps, double regularity, bool relative_detail)
    {
        if (c.cfg.ghost_width > 2)
        {
            c.err = "harten: ghost widths 1 and 2 are implemented";
            return SG_ERR_ARG;
        }
        const int minl = c.cfg.min_level;
        const int maxl = c.cfg.max_level;
        const int dim  = c.g.dim;
        DeviceMesh& m  = c.m();
        DeviceMesh& nm = c.spare();
        // the pinned inputs staged here were consumed by the previous pass,
        // which ended with harten_end's synchronisation
        *c.h_ite = ite;
        pass_thresholds(c, ite, eps, regularity, c.h_eps);
        // the captured front differs with relative details and with the
        // number of fields: keys of their own
        c.rel_detail = relative_detail;
        // the keep_boundary launch is part of the captured front only with --refine-boundary
        const unsigned long long rb = c.refine_boundary ? 256ull : 0ull;
        if (fs.size() == 1)
        {
            DeviceField& f = *fs[0];
            return run_cached(c, (relative_detail ? 4 : 2) | rb, static_cast<unsigned long long>(c.cur), ptr_key(f.data),
                              f.has_bc ? bits_of(f.bc_value) : 1ull, [&]() { return seq_front(c, m, nm, fs); });
        }
        return run_cached(c, (relative_detail ? 6 : 5) | rb, static_cast<unsigned long long>(c.cur), fields_key(fs, false), fs.size(),
                          [&]() { return seq_front(c, m, nm, fs); });
    }

    int harten_end(Ctx& c, DeviceField& f, bool* converged)
    {
        return harten_end_fields(c, {&f}, {}, converged);
    }

    int harten_end_fields(Ctx& c, const std::vector<DeviceField*>& fs, const std::vector<DeviceField*>& os, bool* converged)
    {
        DeviceMesh& m  = c.m();
        DeviceMesh& nm = c.spare();
        int st;
        if (cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            return check(c, "harten front sync");
        }
        for (DeviceField* f : fs)
        {
            f->ghosts_valid  = true; // the front's ghost update ran on the current mesh
            f->ghost_version = c.mesh_version;
        }
        if (c.h_flags[F_GRAD1])
        {
            // graduation still refining after two passes: finish the fixed
            // point with host-tested passes, then compare again
            if ((st = graduate(c, nm.cells, nullptr)))
            {
                return st;
            }
            cudaMemsetAsync(c.d_flags + F_DIFFER, 0, sizeof(int), c.stream);
            if ((st = bitmaps_differ(c, nm.cells, m.cells, F_DIFFER)))
            {
                return st;
            }
            cudaMemcpyAsync(c.h_flags + F_DIFFER, c.d_flags + F_DIFFER, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
            if (cudaStreamSynchronize(c.stream) != cudaSuccess)
            {
                return check(c, "harten compare sync");
            }
        }
        if (!c.h_flags[F_DIFFER])
        {
            *converged = true;
            return SG_OK;
        }
        *converged = false;
        if (fs.size() == 1 && os.empty())
        {
            DeviceField& f = *fs[0];
            st             = run_cached(c, 3, static_cast<unsigned long long>(c.cur), ptr_key(f.data), ptr_key(f.spare),
                                        [&]() { return seq_back(c, m, nm, fs, os); });
        }
        else
        {
            std::vector<DeviceField*> all(fs);
            all.insert(all.end(), os.begin(), os.end());
            st = run_cached(c, 7 + 16 * fs.size(), static_cast<unsigned long long>(c.cur), fields_key(all, false), fields_key(all, true),
                            [&]() { return seq_back(c, m, nm, fs, os); });
        }
        if (st)
        {
            return st;
        }
        nm.host_valid = false; // a replayed graph refreshed the counters without host code
        for (const auto* list : {&fs, &os})
        {
            for (DeviceField* f : *list)
            {
                std::swap(f->data, f->spare);
                f->ghosts_valid = false;
            }
        }
        c.cur = 1 - c.cur;
        ++c.mesh_version;
        return SG_OK;
    }

    // No synchronisation before the pass: the pinned thresholds it rewrites
    // were consumed before the previous pass's harten_end returned, and its
    // launches queue behind whatever the stream still runs.
    int harten(Ctx& c, DeviceField& f, int ite, double eps, double regularity, bool* converged, bool relative_detail)
    {
        int st = harten_begin(c, f, ite, eps, regularity, relative_detail);
        if (st)
        {
            return st;
        }
        return harten_end(c, f, converged);
    }

    // ---------------------------------------------------------------
    // Operators of one step on a given (frozen) mesh, for the replay and the
    // adjoint: the ghost update and update_fields applied (value) or
    // transposed (reverse: the RevAcc accessor, launches in reverse order).
    int ghost_value(Ctx& c, DeviceMesh& m, double* u, bool has_bc, double bcv)
    {
        return ghost_launches(c, m, ValAcc{u}, has_bc, bcv, c.fuse_top_field, false, [] {});
    }

    // lam := G^T lam for the ghost update G of mesh m, in place.  The launch sequence is the one that separates
    // every read from every write (corner projections in launches of their own, no one-block chains), captured
    // once per mesh buffer and adjoint array and replayed backwards.
    int ghost_reverse(Ctx& c, DeviceMesh& m, double* lam, int* overflow, bool has_bc)
    {
        const unsigned long long kind = 40ull | (has_bc ? 256ull : 0ull);
        return run_reversed(c, kind, ptr_key(m.ref), ptr_key(lam), ptr_key(overflow),
                            [&]()
                            {
                                if (c.g.dim == 2)
                                {
                                    return ghost_launches(c, m, RevAcc<FormCap<2>::value>{lam, lam, overflow, 1}, has_bc, 0., -2, true, [] {});
                                }
                                return ghost_launches(c, m, RevAcc<FormCap<3>::value>{lam, lam, overflow, 1}, has_bc, 0., -2, true, [] {});
                            });
    }

    int update_fields_value(Ctx& c, DeviceMesh& m, DeviceMesh& nm, const double* uo, double* un)
    {
        update_fields_launch(c, m, nm, ValAcc{const_cast<double*>(uo)}, ValAcc{un});
        return check(c, "update_fields");
    }

    // lam_old += T^T lam_new for update_fields T from mesh m to mesh nm (lam_old is not cleared here)
    int update_fields_reverse(Ctx& c, DeviceMesh& m, DeviceMesh& nm, double* lam_new, double* lam_old, int* overflow)
    {
        if (c.g.dim == 2)
        {
            const RevAcc<FormCap<2>::value> r{lam_new, lam_old, overflow, 0};
            update_fields_launch(c, m, nm, r, r);
        }
        else
        {
            const RevAcc<FormCap<3>::value> r{lam_new, lam_old, overflow, 0};
            update_fields_launch(c, m, nm, r, r);
        }
        return check(c, "update_fields (transpose)");
    }

    namespace
    {
        // The whole adaptation (Adapt::operator(), mr/adapt.hpp:147-195) as one
        // captured graph: Harten pass i (at most max_level - min_level of them)
        // runs under a conditional node that holds while the previous pass
        // changed the mesh, and its second half (new mesh, update_fields) under
        // one that holds when this pass changed it; graduation iterates in a
        // conditional loop.  Pass i works on mesh buffer (cur + i) mod 2 and on
        // the field buffers that many swaps away, all known when capturing.
        struct StepTail
        {
            DeviceField* u;    // the adapted field (fs[0])
            DeviceField* unp1; // the upwind's output
            double a[3];
            double dt;
            int scheme;
        };

        int seq_adapt(Ctx& c, const std::vector<DeviceField*>& fs, const std::vector<DeviceField*>& os, double eps, double regularity,
                      const StepTail* tail = nullptr)
        {
            const int passes = c.cfg.max_level - c.cfg.min_level;
            std::vector<DeviceField> fa, oa; // the fields as they stand at each pass (buffers swapped per transition)
            for (DeviceField* f : fs)
            {
                fa.push_back(*f);
            }
            for (DeviceField* f : os)
            {
                oa.push_back(*f);
            }
            cudaMemsetAsync(c.d_adapt, 0, A_COUNT * sizeof(int), c.stream);
            k_adapt_words<<<1, 1, 0, c.stream>>>(c.d_adapt, A_GO, nullptr, 1, 0);
            launched(c, "adapt_words");
            int st = SG_OK;
            for (int i = 0; i < passes && !st; ++i)
            {
                const int cur = (c.cur + i) & 1;
                DeviceMesh& m  = c.mesh[cur];
                DeviceMesh& nm = c.mesh[1 - cur];
                std::vector<DeviceField*> fp, op;
                for (auto& f : fa)
                {
                    fp.push_back(&f);
                }
                for (auto& f : oa)
                {
                    op.push_back(&f);
                }
                PassSetup ps{};
                pass_thresholds(c, i, eps, regularity, ps.eps);
                ps.ite    = i;
                auto pass = [&]()
                {
                    int s1 = seq_front(c, m, nm, fp, &ps);
                    if (s1)
                    {
                        return s1;
                    }
                    k_adapt_words<<<1, 1, 0, c.stream>>>(c.d_adapt, A_PASSES, nullptr, i + 1, 0);
                    k_adapt_words<<<1, 1, 0, c.stream>>>(c.d_adapt, A_GO, c.d_flags + F_DIFFER, 0, 0);
                    launched(c, "adapt_words", 2);
                    return capture_if(c, c.d_flags + F_DIFFER,
                                      [&]()
                                      {
                                          int s2 = seq_back(c, m, nm, fp, op);
                                          if (c.rec_slots)
                                          {
                                              k_record_bits<<<grid_for(c.g.total_words), 256, 0, c.stream>>>(nm.cells, c.rec_slots, c.d_adapt,
                                                                                                              c.g.total_words);
                                              launched(c, "record_bits");
                                          }
                                          k_adapt_words<<<1, 1, 0, c.stream>>>(c.d_adapt, A_TRANS, nullptr, 1, 1);
                                          launched(c, "adapt_words");
                                          return s2;
                                      });
                };
                st = i == 0 ? pass() : capture_if(c, c.d_adapt + A_GO, pass);
                for (auto* list : {&fa, &oa})
                {
                    for (auto& f : *list)
                    {
                        std::swap(f.data, f.spare);
                    }
                }
            }
            if (!st && tail)
            {
                // the rest of the time step on the final mesh: the mesh buffer and the field's buffer depend on the
                // parity of the number of transitions, the ghost update on whether the last pass changed the mesh
                // (when it kept it, its own ghost update left the ghosts valid)
                k_step_flags<<<1, 1, 0, c.stream>>>(c.d_adapt);
                launched(c, "adapt_words");
                for (int par = 0; par < 2 && !st; ++par)
                {
                    const int cur    = (c.cur + par) & 1;
                    DeviceMesh& mf   = c.mesh[cur];
                    double* ud       = par ? tail->u->spare : tail->u->data;
                    const bool bc    = tail->u->has_bc;
                    const double bcv = tail->u->bc_value;
                    st               = capture_if(c, c.d_adapt + (par ? A_PAR1 : A_PAR0),
                                                  [&]()
                                                  {
                                                      int s1 = capture_if(c, c.d_adapt + A_NEEDG,
                                                                          [&]() { return ghost_launches(c, mf, ValAcc{ud}, bc, bcv, c.fuse_top_field, false, [] {}); });
                                                      return s1 ? s1 : upwind_on(c, mf, ud, tail->unp1->data, tail->a, tail->dt, tail->scheme, true);
                                                  });
                }
            }
            if (!st)
            {
                cudaMemcpyAsync(c.h_adapt, c.d_adapt, A_COUNT * sizeof(int), cudaMemcpyDeviceToHost, c.stream);
            }
            return st ? st : check(c, "adaptation graph");
        }

        bool graph_applies(const Ctx& c)
        {
            return c.graphed_adapt && c.use_graphs && !c.timers.enabled && !c.trace.enabled && c.cfg.max_level != c.cfg.min_level;
        }

        // launches seq_adapt's graph (captured on first use) without waiting
        int adapt_graph_launch(Ctx& c, const std::vector<DeviceField*>& fs, const std::vector<DeviceField*>& os, double eps, double regularity,
                               bool relative_detail, const StepTail* tail)
        {
            if (c.cfg.ghost_width > 2)
            {
                c.err = "harten: ghost widths 1 and 2 are implemented";
                return SG_ERR_ARG;
            }
            c.rel_detail = relative_detail;
            std::vector<DeviceField*> all(fs);
            all.insert(all.end(), os.begin(), os.end());
            unsigned long long kind = 9ull | (relative_detail ? 16ull : 0ull) | (c.refine_boundary ? 256ull : 0ull)
                                      | (static_cast<unsigned long long>(fs.size()) << 20);
            unsigned long long thr  = bits_of(eps) * 0x9E3779B97F4A7C15ull ^ bits_of(regularity);
            unsigned long long bufs = fields_key(all, false) ^ (fields_key(all, true) << 1) ^ (ptr_key(c.rec_slots) * 0x9E3779B97F4A7C15ull);
            if (tail)
            {
                kind |= (static_cast<unsigned long long>(tail->scheme) + 1) << 10;
                bufs ^= ptr_key(tail->unp1->data) * 0xC2B2AE3D27D4EB4Full;
                for (double v : {tail->a[0], tail->a[1], tail->a[2], tail->dt})
                {
                    thr = (thr ^ bits_of(v)) * 0x100000001B3ull;
                }
            }
            return run_cached(c, kind, static_cast<unsigned long long>(c.cur), bufs, thr, [&]() { return seq_adapt(c, fs, os, eps, regularity, tail); });
        }

        // waits for a launched adaptation graph and applies its outcome on the host: the buffer swaps of the
        // transitions, the current mesh, ghost validity and the step's own swap
        int adapt_graph_finish(Ctx& c, const std::vector<DeviceField*>& fs, const std::vector<DeviceField*>& os, const StepTail* tail,
                               int* n_harten)
        {
            if (cudaStreamSynchronize(c.stream) != cudaSuccess)
            {
                return check(c, "adaptation sync");
            }
            std::vector<DeviceField*> all(fs);
            all.insert(all.end(), os.begin(), os.end());
            const int passes = c.h_adapt[A_PASSES], trans = c.h_adapt[A_TRANS];
            for (int t = 0; t < trans; ++t)
            {
                for (DeviceField* f : all)
                {
                    std::swap(f->data, f->spare);
                }
                c.cur = 1 - c.cur;
                ++c.mesh_version;
            }
            if (trans > 0)
            {
                c.mesh[0].host_valid = c.mesh[1].host_valid = false;
            }
            // the last pass's ghost update ran on the final mesh when that pass kept it
            for (DeviceField* f : all)
            {
                f->ghosts_valid = false;
            }
            if (passes > trans || tail)
            {
                // the last pass kept the mesh, or the step's tail updated the ghosts
                for (DeviceField* f : fs)
                {
                    f->ghosts_valid  = true;
                    f->ghost_version = c.mesh_version;
                }
            }
            if (tail)
            {
                // unp1 = u - dt * upwind(a, u) then std::swap(u.array(), unp1.array())
                std::swap(tail->u->data, tail->unp1->data);
                tail->u->ghosts_valid    = false;
                tail->unp1->ghosts_valid = false;
            }
            if (n_harten)
            {
                *n_harten = passes;
            }
            return device_error(c);
        }

        // the adaptation (and the rest of the step when tail is given) through
        // the graph; false when that path does not apply (graphs off, timers or
        // the kernel trace on)
        bool adapt_graphed(Ctx& c, const std::vector<DeviceField*>& fs, const std::vector<DeviceField*>& os, double eps, double regularity,
                           bool relative_detail, int* n_harten, int* status, const StepTail* tail = nullptr)
        {
            if (!graph_applies(c))
            {
                return false;
            }
            *status = adapt_graph_launch(c, fs, os, eps, regularity, relative_detail, tail);
            if (!*status)
            {
                *status = adapt_graph_finish(c, fs, os, tail, n_harten);
            }
            return true;
        }

        StepTail make_tail(const Ctx& c, DeviceField& u, DeviceField& unp1, const double* a, double dt, int scheme)
        {
            StepTail t{};
            t.u    = &u;
            t.unp1 = &unp1;
            for (int d = 0; d < c.g.dim; ++d)
            {
                t.a[d] = a[d];
            }
            t.dt     = dt;
            t.scheme = scheme;
            return t;
        }
    } // namespace

    bool step_graph_applies(const Ctx& c)
    {
        return graph_applies(c);
    }

    // the time step's graph in two halves (batched mode: launch every instance's, then wait for each);
    // step_launch returns SG_ERR_NOTFOUND when the graph path does not apply to this mesh
    int step_launch(Ctx& c, DeviceField& u, DeviceField& unp1, double eps, double regularity, const double* a, double dt, int scheme)
    {
        if (!graph_applies(c))
        {
            return SG_ERR_NOTFOUND;
        }
        const StepTail t = make_tail(c, u, unp1, a, dt, scheme);
        return adapt_graph_launch(c, {&u}, {}, eps, regularity, false, &t);
    }

    int step_finish(Ctx& c, DeviceField& u, DeviceField& unp1, int* n_harten)
    {
        const double zero[3] = {0., 0., 0.};
        const StepTail t     = make_tail(c, u, unp1, zero, 0., 0);
        return adapt_graph_finish(c, {&u}, {}, &t, n_harten);
    }

    // One iteration of the demo's time loop (demos/FiniteVolume/advection_2d.cpp:140-147): MRadaptation(eps,
    // regularity), update_ghost_mr(u), unp1 = u - dt * upwind(a, u) (or the flux form / README scheme),
    // std::swap(u.array(), unp1.array()) — one captured graph and one synchronisation when graphs apply,
    // otherwise the separate calls.
    int step(Ctx& c, DeviceField& u, DeviceField& unp1, double eps, double regularity, const double* a, double dt, int scheme, int* n_harten)
    {
        const StepTail t = make_tail(c, u, unp1, a, dt, scheme);
        int st           = SG_OK;
        {
            ScopedTimer timer(c, T_ADAPT);
            if (adapt_graphed(c, {&u}, {}, eps, regularity, false, n_harten, &st, &t))
            {
                return st;
            }
        }
        if ((st = adapt(c, u, eps, regularity, n_harten, false)) || (st = update_ghost_mr(c, u)) || (st = upwind(c, u, unp1, a, dt, scheme)))
        {
            return st;
        }
        std::swap(u.data, unp1.data);
        u.ghosts_valid    = false;
        unp1.ghosts_valid = false;
        return SG_OK;
    }

    // Adapt<Fields...>::operator()(mra_config, other_fields...) (mr/adapt.hpp:147-195)
    int adapt_fields(Ctx& c, const std::vector<DeviceField*>& fs, const std::vector<DeviceField*>& os, double eps, double regularity,
                     bool relative_detail, int* n_harten)
    {
        ScopedTimer timer(c, T_ADAPT);
        int gst = SG_OK;
        if (adapt_graphed(c, fs, os, eps, regularity, relative_detail, n_harten, &gst))
        {
            return gst;
        }
        const int minl = c.cfg.min_level, maxl = c.cfg.max_level;
        int it         = 0;
        for (int i = 0; minl != maxl && i < maxl - minl; ++i)
        {
            ++it;
            bool conv = false;
            int st    = harten_begin_fields(c, fs, i, eps, regularity, relative_detail);
            if (!st)
            {
                st = harten_end_fields(c, fs, os, &conv);
            }
            if (st)
            {
                return st;
            }
            if (conv)
            {
                break;
            }
        }
        if (n_harten)
        {
            *n_harten = it;
        }
        return device_error(c);
    }

    // Adapt::operator() (mr/adapt.hpp:147-195)
    int adapt(Ctx& c, DeviceField& f, double eps, double regularity, int* n_harten, bool relative_detail)
    {
        ScopedTimer timer(c, T_ADAPT);
        int gst = SG_OK;
        if (adapt_graphed(c, {&f}, {}, eps, regularity, relative_detail, n_harten, &gst))
        {
            return gst;
        }
        const int minl = c.cfg.min_level, maxl = c.cfg.max_level;
        int it         = 0;
        if (minl != maxl)
        {
            for (int i = 0; i < maxl - minl; ++i)
            {
                ++it;
                bool conv = false;
                int st    = harten(c, f, i, eps, regularity, &conv, relative_detail);
                if (st)
                {
                    return st;
                }
                if (conv)
                {
                    break;
                }
            }
        }
        if (n_harten)
        {
            *n_harten = it;
        }
        return device_error(c);
    }

    namespace
    {
        __global__ void k_set_velocity(double* av, double a0, double a1, double a2)
        {
            av[0] = a0;
            av[1] = a1;
            av[2] = a2;
        }
    } // namespace

    // the upwind step on mesh m from the values at ud into unp1d; baked: the
    // velocity of the flux form is written by a kernel (inside a captured
    // graph) instead of copied from the host array
    int upwind_on(Ctx& c, const DeviceMesh& m, const double* ud, double* unp1d, const double* a, double dt, int scheme, bool baked)
    {
        const Geom& g = c.g;
        UpwindArgs p{};
        for (int d = 0; d < g.dim; ++d)
        {
            p.ha[d] = .5 * a[d];
            p.hb[d] = .5 * std::fabs(a[d]);
        }
        p.dt     = dt;
        p.scheme = scheme;
        const int nb = blocks_words(c, 0, g.nlev - 1);
        if (scheme == 2)
        {
            double* av = c.d_eps + EPS_VELOCITY;
            if (baked)
            {
                k_set_velocity<<<1, 1, 0, c.stream>>>(av, a[0], a[1], g.dim == 3 ? a[2] : 0.);
                launched(c, "set_velocity");
            }
            else
            {
                cudaMemcpyAsync(av, a, g.dim * sizeof(double), cudaMemcpyHostToDevice, c.stream);
            }
            if (g.dim == 2)
            {
                k_convection<2><<<nb, c.block, 0, c.stream>>>(c.g, m.wl_cells, m.d_lo, m.cells, ud, unp1d, p, av);
            }
            else
            {
                k_convection<3><<<nb, c.block, 0, c.stream>>>(c.g, m.wl_cells, m.d_lo, m.cells, ud, unp1d, p, av);
            }
        }
        else if (g.dim == 2)
        {
            k_upwind<2><<<nb, c.block, 0, c.stream>>>(c.g, m.wl_cells, m.d_lo, m.cells, ud, unp1d, p);
        }
        else
        {
            k_upwind<3><<<nb, c.block, 0, c.stream>>>(c.g, m.wl_cells, m.d_lo, m.cells, ud, unp1d, p);
        }
        launched(c, scheme == 2 ? "convection" : "upwind");
        return check(c, "upwind");
    }

    int upwind(Ctx& c, DeviceField& u, DeviceField& unp1, const double* a, double dt, int scheme)
    {
        ScopedTimer timer(c, T_UPWIND);
        return upwind_on(c, c.m(), u.data, unp1.data, a, dt, scheme, false);
    }
} // namespace sg
