#include <algorithm>
// Mesh construction on the device: the MRMesh ids from a leaf-cell bitmap,
// and the integer kernels of the adaptation (tags -> new cells, graduation).
//
// Set algebra follows samurai's subset semantics: operators act on cells of
// one level, coarser operands are refined, .on(l) coarsens to the parent of
// any member (subset/projection.hpp:68-177).  On bitmaps these are word-wise
// AND/OR/ANDNOT, bit-pair compression (coarsen) and bit spreading (refine).
#include <nvtx3/nvToolsExt.h>

#include "sg_ctx.cuh"

namespace sg
{
    cudaEvent_t take_event(Ctx& c)
    {
        if (!c.timers.pool.empty())
        {
            cudaEvent_t e = c.timers.pool.back();
            c.timers.pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }

    void give_event(Ctx& c, cudaEvent_t e)
    {
        if (e)
        {
            c.timers.pool.push_back(e);
        }
    }

    void clear_graphs(Ctx& c)
    {
        for (auto& ge : c.graphs)
        {
            cudaGraphExecDestroy(ge.exec);
            for (const auto& mk : ge.marks)
            {
                bool in_window = false;
                for (const auto& tm : c.trace.marks)
                {
                    in_window = in_window || tm.second == mk.second;
                }
                if (!in_window)
                {
                    give_event(c, mk.second);
                }
            }
        }
        c.graphs.clear();
    }

    void launched(Ctx& c, const char* name, int count)
    {
        c.n_launches += count;
        if (c.trace.enabled)
        {
            trace_mark(c, name);
        }
    }

    // a trace event after the work queued so far; name null for the head of a launch sequence (the time before
    // it, a host round trip included, is charged to no kernel)
    void trace_mark(Ctx& c, const char* name)
    {
        // inside a stream capture an external record becomes an event-record node of the graph (a plain
        // record would only order the capture); outside a capture it is a plain record
        cudaEvent_t e              = take_event(c);
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(c.stream, &cs);
        if (cs == cudaStreamCaptureStatusActive)
        {
            cudaEventRecordWithFlags(e, c.stream, cudaEventRecordExternal);
        }
        else
        {
            cudaEventRecord(e, c.stream);
        }
        c.trace.marks.push_back({name, e});
    }

    namespace
    {
        // samurai's timer names (timers.hpp:111-1036) as NVTX ranges, so that a
        // profiler's timeline shows the phases under the reference's names
        const char* const TIMER_NAMES[T_COUNT] = {"mesh adaptation",  "ghost update",    "detail computation", "tag cells",     "tag finalization",
                                                  "mesh update",      "make_graduation", "mesh construction",  "fields update", "field expressions"};
    } // namespace

    void timer_start(Ctx& c, int id)
    {
        nvtxRangePushA(TIMER_NAMES[id]);
        if (!c.timers.enabled)
        {
            return;
        }
        cudaEvent_t e = take_event(c);
        cudaEventRecord(e, c.stream);
        c.timers.pending[id] = e;
    }

    void timer_stop(Ctx& c, int id)
    {
        nvtxRangePop();
        if (!c.timers.enabled || !c.timers.pending[id])
        {
            return;
        }
        cudaEvent_t e = take_event(c);
        cudaEventRecord(e, c.stream);
        c.timers.open[id].push_back({c.timers.pending[id], e});
        c.timers.pending[id] = nullptr;
        ++c.timers.calls[id];
    }

    void timers_flush(Ctx& c)
    {
        cudaStreamSynchronize(c.stream);
        for (int id = 0; id < T_COUNT; ++id)
        {
            for (auto& pr : c.timers.open[id])
            {
                float ms = 0.f;
                if (cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess)
                {
                    c.timers.ms[id] += ms;
                }
                c.timers.pool.push_back(pr.first);
                c.timers.pool.push_back(pr.second);
            }
            c.timers.open[id].clear();
        }
        cudaGetLastError();
    }

    namespace
    {
        // ------------------------------------------------------------- words
        // guard: when not null, the launch does nothing unless *guard != 0
        template <class F>
        __global__ void k_words(const __grid_constant__ Geom gp, int l0, int l1, F f, const int* guard)
        {
            if (guard && *guard == 0)
            {
                return;
            }
            const Geom& g         = gp;
            const long long begin = g.lv[l0].woff;
            const long long end   = g.lv[l1].woff + g.lv[l1].nwords;
            for (long long w = begin + blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; w < end;
                 w += static_cast<long long>(gridDim.x) * blockDim.x)
            {
                int l = l0;
                while (l < l1 && w >= g.lv[l + 1].woff)
                {
                    ++l;
                }
                const WordLoc loc = word_loc(g, l, w);
                f(g, l, w, loc.row, loc.wi);
            }
        }

        // one block walks the levels l_first -> l_last (either direction)
        template <class F>
        __global__ void __launch_bounds__(1024, 1) k_words_chain(const __grid_constant__ Geom gp, int l_first, int l_last, F f, const int* guard)
        {
            if (guard && *guard == 0)
            {
                return;
            }
            const Geom& g  = gp;
            const int step = l_last >= l_first ? 1 : -1;
            for (int l = l_first;; l += step)
            {
                const LevelGeom& L = g.lv[l];
                for (long long k = threadIdx.x; k < L.nwords; k += blockDim.x)
                {
                    const long long w   = L.woff + k;
                    const unsigned row = fastdiv(static_cast<unsigned>(k), L.mW, L.sW);
                    f(g, l, w, static_cast<long long>(row), static_cast<int>(static_cast<unsigned>(k) - row * static_cast<unsigned>(L.W)));
                }
                __syncthreads();
                if (l == l_last)
                {
                    break;
                }
            }
        }

        template <class F>
        int launch_words(Ctx& c, int l0, int l1, F f, const char* what);

        // the levels l_first -> l_last one after the other: the large ones by
        // separate launches, the small ones (<= fuse_top) by one block
        template <class F>
        int launch_chain(Ctx& c, int l_first, int l_last, F f, const char* what)
        {
            const int ft = c.fuse_top;
            int st       = SG_OK;
            if (l_first >= l_last)
            {
                int l = l_first;
                for (; l >= l_last && l > ft; --l)
                {
                    if ((st = launch_words(c, l, l, f, what)))
                    {
                        return st;
                    }
                }
                if (l >= l_last)
                {
                    k_words_chain<<<1, 1024, 0, c.stream>>>(c.g, l, l_last, f, c.guard);
                    launched(c, what);
                    st = check(c, what);
                }
            }
            else
            {
                int l = l_first;
                if (l <= ft)
                {
                    const int e = l_last < ft ? l_last : ft;
                    k_words_chain<<<1, 1024, 0, c.stream>>>(c.g, l, e, f, c.guard);
                    launched(c, what);
                    if ((st = check(c, what)))
                    {
                        return st;
                    }
                    l = e + 1;
                }
                for (; l <= l_last; ++l)
                {
                    if ((st = launch_words(c, l, l, f, what)))
                    {
                        return st;
                    }
                }
            }
            return st;
        }

        template <class F>
        int launch_words(Ctx& c, int l0, int l1, F f, const char* what)
        {
            if (l0 > l1)
            {
                return SG_OK;
            }
            const long long n = c.g.lv[l1].woff + c.g.lv[l1].nwords - c.g.lv[l0].woff;
            k_words<<<grid_for(n, 256, 4LL * c.max_blocks), 256, 0, c.stream>>>(c.g, l0, l1, f, c.guard);
            launched(c, what);
            return check(c, what);
        }

        // --------------------------------------------------------------- scan
        constexpr int SCAN_T   = 256;
        constexpr int SCAN_PER = 16;
        constexpr int SCAN_CHUNK = SCAN_T * SCAN_PER;

        __device__ __forceinline__ long long block_exclusive_scan(long long v, long long* total)
        {
            __shared__ long long warp_tot[32];
            const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
            long long x    = v;
            for (int o = 1; o < 32; o <<= 1)
            {
                long long y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o)
                {
                    x += y;
                }
            }
            if (lane == 31)
            {
                warp_tot[wid] = x;
            }
            __syncthreads();
            const int nw = blockDim.x >> 5;
            if (wid == 0)
            {
                long long t = lane < nw ? warp_tot[lane] : 0;
                for (int o = 1; o < 32; o <<= 1)
                {
                    long long y = __shfl_up_sync(0xffffffffu, t, o);
                    if (lane >= o)
                    {
                        t += y;
                    }
                }
                if (lane < nw)
                {
                    warp_tot[lane] = t;
                }
            }
            __syncthreads();
            const long long before = wid > 0 ? warp_tot[wid - 1] : 0;
            if (total)
            {
                *total = warp_tot[nw - 1];
            }
            const long long r = before + x - v;
            __syncthreads();
            return r;
        }

        // Four scans in one pass over the words: popcount of the reference
        // (rank), non-empty reference words, popcount of the cells and
        // non-empty cell words (the word lists the field kernels iterate).
        struct Quad
        {
            long long v[4];
        };

        __device__ __forceinline__ Quad thread_quad(const uint32_t* ref, const uint32_t* cells, long long base, long long n)
        {
            Quad q{};
            for (int k = 0; k < SCAN_PER; ++k)
            {
                if (base + k < n)
                {
                    const uint32_t r = ref[base + k], c = cells[base + k];
                    q.v[0] += __popc(r);
                    q.v[1] += (r != 0u);
                    q.v[2] += __popc(c);
                    q.v[3] += (c != 0u);
                }
            }
            return q;
        }

        __global__ void k_scan_sums(const uint32_t* ref, const uint32_t* cells, long long n, long long nb, long long* sums)
        {
            const long long base = static_cast<long long>(blockIdx.x) * SCAN_CHUNK + threadIdx.x * SCAN_PER;
            const Quad q         = thread_quad(ref, cells, base, n);
            for (int k = 0; k < 4; ++k)
            {
                long long tot;
                block_exclusive_scan(q.v[k], &tot);
                if (threadIdx.x == 0)
                {
                    sums[k * nb + blockIdx.x] = tot;
                }
            }
        }

        __global__ void k_scan_top(long long* sums, long long nb, long long* counts, int nlev)
        {
            const long long per = (nb + blockDim.x - 1) / blockDim.x;
            const long long b0  = threadIdx.x * per;
            for (int k = 0; k < 4; ++k)
            {
                long long* a = sums + k * nb;
                long long s  = 0;
                for (long long j = 0; j < per; ++j)
                {
                    if (b0 + j < nb)
                    {
                        s += a[b0 + j];
                    }
                }
                long long tot;
                long long off = block_exclusive_scan(s, &tot);
                for (long long j = 0; j < per; ++j)
                {
                    if (b0 + j < nb)
                    {
                        const long long v = a[b0 + j];
                        a[b0 + j]         = off;
                        off += v;
                    }
                }
                if (threadIdx.x == 0)
                {
                    counts[k] = tot;
                    if (k == 1)
                    {
                        counts[LO_REF + nlev] = tot;
                    }
                    if (k == 3)
                    {
                        counts[LO_CELLS + nlev] = tot;
                    }
                }
            }
        }

        __global__ void k_scan_write(const __grid_constant__ Geom gp, const uint32_t* ref, const uint32_t* cells, long long n, long long nb, const long long* sums, int* rank,
                                     int* wl_ref, int* wl_cells, long long* counts)
        {
            const Geom& g = gp;
            const long long base = static_cast<long long>(blockIdx.x) * SCAN_CHUNK + threadIdx.x * SCAN_PER;
            const Quad q         = thread_quad(ref, cells, base, n);
            long long off[4];
            for (int k = 0; k < 4; ++k)
            {
                off[k] = block_exclusive_scan(q.v[k], nullptr) + sums[k * nb + blockIdx.x];
            }
            for (int k = 0; k < SCAN_PER; ++k)
            {
                const long long w = base + k;
                if (w >= n)
                {
                    break;
                }
                for (int l = 0; l < g.nlev; ++l)
                {
                    if (g.lv[l].woff == w)
                    {
                        counts[LO_REF + l]   = off[1];
                        counts[LO_CELLS + l] = off[3];
                    }
                }
                const uint32_t r = ref[w], c = cells[w];
                rank[w]          = static_cast<int>(off[0]);
                off[0] += __popc(r);
                if (r)
                {
                    wl_ref[off[1]++] = static_cast<int>(w);
                }
                off[2] += __popc(c);
                if (c)
                {
                    wl_cells[off[3]++] = static_cast<int>(w);
                }
            }
        }
    } // namespace

    int scan_rank(Ctx& c, DeviceMesh& m)
    {
        const long long n  = c.g.total_words;
        const long long nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
        k_scan_sums<<<static_cast<unsigned>(nb), SCAN_T, 0, c.stream>>>(m.ref, m.cells, n, nb, c.block_sums);
        launched(c, "scan_sums");
        k_scan_top<<<1, 1024, 0, c.stream>>>(c.block_sums, nb, m.d_lo, c.g.nlev);
        launched(c, "scan_top");
        k_scan_write<<<static_cast<unsigned>(nb), SCAN_T, 0, c.stream>>>(c.g, m.ref, m.cells, n, nb, c.block_sums, m.rank, m.wl_ref, m.wl_cells,
                                                                          m.d_lo);
        launched(c, "scan_write");
        cudaMemcpyAsync(m.h_lo, m.d_lo, COUNTS * sizeof(long long), cudaMemcpyDeviceToHost, c.stream);
        m.host_valid = false;
        return check(c, "scan_rank");
    }

    int host_counts(Ctx& c, DeviceMesh& m)
    {
        if (m.host_valid)
        {
            return SG_OK;
        }
        if (cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            return check(c, "host_counts");
        }
        m.nb_ref     = m.h_lo[0];
        m.nb_cells   = m.h_lo[2];
        m.host_valid = true;
        if (m.nb_ref >= (1LL << 31))
        {
            c.err = "reference mesh exceeds 2^31 cells";
            return SG_ERR_CAPACITY;
        }
        return SG_OK;
    }

    // Mesh_base::finalize_mesh for the serial unit-box case:
    // construct_union (mesh.hpp:1231-1262), MRMesh::update_sub_mesh_impl
    // (mr/mesh.hpp:222-455) and renumbering (mesh.hpp:894-911).
    int build_mesh(Ctx& c, DeviceMesh& m)
    {
        ScopedTimer timer(c, T_CONSTRUCTION);
        const Geom g       = c.g;
        const int maxl     = c.cfg.max_level;
        const int r        = c.cfg.max_stencil_radius;
        const int p        = c.cfg.prediction_radius;
        const bool multi   = c.cfg.max_level != c.cfg.min_level;
        uint32_t* cells    = m.cells;
        uint32_t* hc       = m.hc;
        uint32_t* hc2      = m.hc2;
        uint32_t* uni      = m.uni;
        uint32_t* cag      = m.cag;
        uint32_t* ref      = m.ref;
        uint32_t* proj     = m.proj;
        uint32_t* t1       = c.t1;
        const size_t bytes = static_cast<size_t>(g.total_words) * 4;
        int st;

        // Leaf cells lie in levels min_level .. max_level, so each set below
        // can be non-empty only on a known range of levels; it is computed on
        // that range, and its other levels keep the zeros they were created
        // with (no pass ever writes them).
        const int minl = c.cfg.min_level;
        const int lmin = minl >= 2 ? minl - 2 : 0; // lowest level of the reference

        // Passes that read the same inputs share a launch:
        //  1. hc = cells[l+1].on(l) (levels min-1 .. max-1: cells with a leaf
        //     child) and the expansion of the cells by the stencil radius
        //     (cells_and_ghosts, levels min .. max; in 3D its xy part);
        //  2. hc2 = hc.on(l) (cells with a leaf grandchild, min-2 .. max-2) with,
        //     in 2D, cells_and_ghosts.on(l) (t1, min-1 .. max-1) and, in 3D, the
        //     z part of cells_and_ghosts;
        //  3. (3D) t1 = cells_and_ghosts.on(l).
        const int hlo  = std::max(minl - 1, 0), hhi = maxl - 1;
        const int h2lo = std::max(minl - 2, 0), h2hi = maxl - 2;
        const int t1lo = std::max(minl - 1, 0), t1hi = maxl - 1; // t1 is read on these levels only
        uint32_t* t0   = c.t0;
        uint32_t* cxy  = (g.dim == 2) ? cag : t0;
        // union cells (construct_union, mesh.hpp:1231-1262): union[l] =
        // (cells[l+1] | union[l+1]).on(l) for levels max-1 .. 0, i.e. every
        // cell with a leaf among its descendants: the same launch marks the
        // ancestors of each word of hc = cells[l+1].on(l) into the zeroed union
        // bitmap (union[max] stays zero)
        cudaMemsetAsync(uni, 0, bytes, c.stream);
        st = launch_words(c, std::min(hlo, minl), maxl,
                          [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                          {
                              if (l >= hlo && l <= hhi)
                              {
                                  const uint32_t h = coarsen_word(g, cells, l, row, wi);
                                  hc[w]            = h;
                                  if (h && (atomicOr(uni + w, h) & h) != h)
                                  {
                                      mark_ancestors(g, uni, l, row, wi, h, 0);
                                  }
                              }
                              if (l >= minl)
                              {
                                  cxy[w] = dilate_xy_word(g, cells, l, row, wi, r);
                              }
                          },
                          "hc_cag");
        if (st)
        {
            return st;
        }
        if (g.dim == 2)
        {
            const bool with_t1 = multi;
            const int lo2      = with_t1 ? std::min(h2lo, t1lo) : h2lo;
            const int hi2      = with_t1 ? std::max(h2hi, t1hi) : h2hi;
            st                 = launch_words(c, lo2, hi2,
                                              [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                              {
                                                  if (l >= h2lo && l <= h2hi)
                                                  {
                                                      hc2[w] = coarsen_word(g, hc, l, row, wi);
                                                  }
                                                  if (with_t1 && l >= t1lo && l <= t1hi)
                                                  {
                                                      t1[w] = coarsen_word(g, cag, l, row, wi);
                                                  }
                                              },
                                              "hc2_cag_on");
        }
        else
        {
            st = launch_words(c, std::min(h2lo, minl), maxl,
                              [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                              {
                                  if (l >= h2lo && l <= h2hi)
                                  {
                                      hc2[w] = coarsen_word(g, hc, l, row, wi);
                                  }
                                  if (l >= minl)
                                  {
                                      cag[w] = dilate_z_word(g, t0, l, row, wi, r);
                                  }
                              },
                              "hc2_cag_z");
            if (!st && multi)
            {
                st = launch_words(c, t1lo, t1hi,
                                  [=] __device__(const Geom& g, int l, long long w, long long row, int wi) { t1[w] = coarsen_word(g, cag, l, row, wi); },
                                  "cag_on");
            }
        }
        if (st)
        {
            return st;
        }


        if (!multi)
        {
            cudaMemcpyAsync(ref, cag, bytes, cudaMemcpyDeviceToDevice, c.stream);
            cudaMemsetAsync(proj, 0, bytes, c.stream);
            if (g.periodic)
            {
                // the translated cells expanded by the stencil radius, within the
                // expanded domain (mr/mesh.hpp:294-317)
                st = launch_words(c, minl, maxl,
                                  [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                  { ref[w] |= periodic_translates(g, cag, l, row, wi) & box_mask(g, l, row, wi, r, r); },
                                  "ref_periodic");
                if (st)
                {
                    return st;
                }
            }
            return scan_rank(c, m);
        }

        // prediction ghosts: cag[l+1].on(l) (= t1, above) expanded by p within the
        // expanded domain, and cells[l+2].on(l) expanded by p
        // the reference starts at level min-2: cag (min .. max), t1 (min-1 ..
        // max-1) and hc2 (min-2 .. max-2)
        // the reference before the children of the projection cells (ref0) goes
        // to a scratch bitmap (the refine flags of the adaptation, free here)
        // in the non-periodic case: the pass below reads it while it writes ref
        uint32_t* ref0 = g.periodic ? ref : c.rf;
        if (g.dim == 2)
        {
            st = launch_words(c, lmin, maxl,
                              [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                              {
                                  uint32_t v = cag[w];
                                  if (l >= t1lo && l <= t1hi)
                                  {
                                      v |= dilate_xy_word(g, t1, l, row, wi, p) & box_mask(g, l, row, wi, p, p);
                                  }
                                  if (l >= h2lo && l <= h2hi) // hc2 is empty elsewhere
                                  {
                                      v |= dilate_xy_word(g, hc2, l, row, wi, p);
                                  }
                                  ref0[w] = v;
                              },
                              "ref0");
        }
        else
        {
            uint32_t* t2 = c.t2;
            uint32_t* t3 = c.t3;
            st           = launch_words(c, lmin, maxl,
                                        [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                        {
                                            t2[w] = (l >= t1lo && l <= t1hi) ? dilate_xy_word(g, t1, l, row, wi, p) : 0u;
                                            t3[w] = (l >= h2lo && l <= h2hi) ? dilate_xy_word(g, hc2, l, row, wi, p) : 0u;
                                        },
                                        "ref0_xy");
            if (!st)
            {
                st = launch_words(c, lmin, maxl,
                                  [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                  {
                                      uint32_t v = cag[w];
                                      // t2 and t3 are empty outside the levels of t1 and hc2
                                      if (l >= t1lo && l <= t1hi)
                                      {
                                          v |= dilate_z_word(g, t2, l, row, wi, p) & box_mask(g, l, row, wi, p, p);
                                      }
                                      if (l >= h2lo && l <= h2hi)
                                      {
                                          v |= dilate_z_word(g, t3, l, row, wi, p);
                                      }
                                      ref0[w] = v;
                                  },
                                  "ref0_z");
            }
        }
        if (st)
        {
            return st;
        }

        if (g.periodic)
        {
            // periodic parts of the reference (mr/mesh.hpp:294-317, 356-368): the
            // translates of cells_and_ghosts within the domain expanded by the
            // stencil radius, and those of the two prediction-ghost sets (the
            // dilations above, written in full into scratch bitmaps) within the
            // domain.  translate commutes with on() and the dilations.
            uint32_t* pa = c.t0;
            uint32_t* pb = c.t1; // cells_and_ghosts.on(l) is no longer needed
            if (g.dim == 2)
            {
                uint32_t* t2 = c.t2;
                st           = launch_words(c, lmin, maxl,
                                            [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                            {
                                                pa[w] = (l >= t1lo && l <= t1hi) ? dilate_xy_word(g, t1, l, row, wi, p) : 0u;
                                                t2[w] = dilate_xy_word(g, hc2, l, row, wi, p);
                                            },
                                            "ref_periodic_sources");
                pb = t2;
            }
            else
            {
                uint32_t* t2 = c.t2;
                uint32_t* t3 = c.t3;
                st           = launch_words(c, lmin, maxl,
                                            [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                            {
                                                pa[w] = dilate_z_word(g, t2, l, row, wi, p);
                                                pb[w] = dilate_z_word(g, t3, l, row, wi, p);
                                            },
                                            "ref_periodic_sources");
            }
            if (!st)
            {
                st = launch_words(c, lmin, maxl,
                                  [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                  {
                                      uint32_t v = ref[w];
                                      if (l >= minl)
                                      {
                                          v |= periodic_translates(g, cag, l, row, wi) & box_mask(g, l, row, wi, r, r);
                                      }
                                      v |= (periodic_translates(g, pa, l, row, wi) | periodic_translates(g, pb, l, row, wi)) & box_mask(g, l, row, wi, 0, 0);
                                      ref[w] = v;
                                  },
                                  "ref_periodic");
            }
            if (st)
            {
                return st;
            }
        }

        // children of the projection cells, bottom-up:
        // reference[l+1] |= (reference[l] & union[l]) refined; the reference
        // starts at min_level - 2, so the first level with a source is above it
        const int ref_lo = std::max(1, std::max(c.cfg.min_level - 2, 0) + 1);
        if (!g.periodic && maxl >= ref_lo)
        {
            // In one pass instead of level by level: the parent of a union cell
            // is a union cell, so a cell whose parent p is in the union joins the
            // reference exactly when p or one of p's ancestors (down to the
            // reference's first level) is in ref0; and proj = reference & union.
            // Each word reads its parent word's ancestors in ref0 directly.
            const uint32_t* r0 = ref0;
            const int rlo      = ref_lo;
            st                 = launch_words(c, ref_lo - 1, maxl,
                                              [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                              {
                                                  uint32_t v = r0[w];
                                                  if (l >= rlo)
                                                  {
                                                      const ParentWord pw = parent_word(g, l, row, wi);
                                                      if (pw.ok)
                                                      {
                                                          const LevelGeom& C = g.lv[l - 1];
                                                          const uint32_t pc  = self_or_ancestor(g, r0, l - 1, pw.row, pw.wi, rlo - 1)
                                                                              & uni[C.woff + pw.row * C.W + pw.wi];
                                                          v |= spread16(pc >> pw.shift);
                                                      }
                                                  }
                                                  ref[w] = v;
                                                  if (l < g.max_level)
                                                  {
                                                      proj[w] = v & uni[w];
                                                  }
                                              },
                                              "ref_children");
            if (st)
            {
                return st;
            }
            return scan_rank(c, m);
        }
        if (maxl >= ref_lo)
        {
            st = launch_chain(c, ref_lo, maxl,
                              [=] __device__(const Geom& g, int lf, long long w, long long row, int k)
                              {
                                  const LevelGeom& F = g.lv[lf];
                                  const LevelGeom& C = g.lv[lf - 1];
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
                                  const int ry = (yf >> 1) + PY, rz = (zf >> 1) + PY;
                                  const int wc = (k + 1) >> 1;
                                  if (ry < 0 || ry >= C.R || (g.dim == 3 && (rz < 0 || rz >= C.R)) || wc >= C.W)
                                  {
                                      return;
                                  }
                                  const long long cw = C.woff + ((g.dim == 2) ? ry : static_cast<long long>(rz) * C.R + ry) * C.W + wc;
                                  const uint32_t pc  = ref[cw] & uni[cw];
                                  // proj_cells of the coarse level, final once the chain has passed it;
                                  // the fine words of one coarse word all write this same value
                                  proj[cw]           = pc;
                                  const uint32_t add = spread16(((k + 1) & 1) ? (pc >> 16) : pc);
                                  if (add)
                                  {
                                      ref[w] |= add;
                                  }
                              },
                              "ref_children");
            if (st)
            {
                return st;
            }
        }
        if (maxl < ref_lo)
        {
            // no chain ran: proj_cells = reference & union directly
            st = launch_words(c, lmin, maxl, [=] __device__(const Geom&, int, long long w, long long, int) { proj[w] = ref[w] & uni[w]; }, "proj");
            if (st)
            {
                return st;
            }
        }
        return scan_rank(c, m);
    }

    // ------------------------------------------------------------------
    // adaptation: integer part
    // ------------------------------------------------------------------
    namespace
    {
        // refine / coarsen_even flags of leaf cells from the tags
        // (update_cell_array_from_tag, algorithm/graduation.hpp:743-842)
        __global__ void k_tag_flags(const __grid_constant__ Geom gp, const uint32_t* cells, const uint8_t* tag, uint32_t* rf, uint32_t* cf, int minl, int maxl)
        {
            const Geom& g = gp;
            for (long long w = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; w < g.total_words;
                 w += static_cast<long long>(gridDim.x) * blockDim.x)
            {
                const uint32_t cw = cells[w];
                uint32_t r = 0, k = 0;
                if (cw)
                {
                    const int l = level_of(g, w);
                    const uint8_t* t = tag + 32 * w;
                    for (int b = 0; b < 32; ++b)
                    {
                        if ((cw >> b) & 1u)
                        {
                            const uint8_t tv = t[b];
                            const bool refine = (tv & 4) && l < maxl;
                            const bool coarsen = (tv & 2) && !(tv & 1) && l > minl;
                            if (refine)
                            {
                                r |= 1u << b;
                            }
                            else if (coarsen)
                            {
                                k |= 1u << b;
                            }
                        }
                    }
                }
                rf[w] = r;
                cf[w] = k;
            }
        }
    } // namespace

    int new_cells_from_tags(Ctx& c, const DeviceMesh& m, uint32_t* nc)
    {
        const Geom g = c.g;
        k_tag_flags<<<grid_for(g.total_words, 256, 4LL * c.max_blocks), 256, 0, c.stream>>>(c.g, m.cells, c.tag, c.rf, c.cf, c.cfg.min_level, c.cfg.max_level);
        launched(c, "tag_flags");
        int st = check(c, "tag_flags");
        if (st)
        {
            return st;
        }
        const uint32_t* cells = m.cells;
        const uint32_t* rf    = c.rf;
        const uint32_t* cf    = c.cf;
        const int minl = c.cfg.min_level, maxl = c.cfg.max_level;
        return launch_words(c, 0, g.nlev - 1,
                            [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                            {
                                uint32_t v = 0;
                                if (l >= minl && l <= maxl)
                                {
                                    v = cells[w] & ~rf[w] & ~cf[w];
                                    if (l >= 1)
                                    {
                                        v |= refine_word(g, rf, l, row, wi);
                                    }
                                    if (l + 1 < g.nlev)
                                    {
                                        // parent of the coarsened (even) child
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
                                        const int ry = 2 * yc + PY, rz = 2 * zc + PY;
                                        if (ry >= 0 && ry < F.R && (g.dim == 2 || (rz >= 0 && rz < F.R)))
                                        {
                                            const long long base = F.woff + ((g.dim == 2) ? ry : static_cast<long long>(rz) * F.R + ry) * F.W;
                                            const int k0         = 2 * wi - 1;
                                            const uint32_t lo    = (k0 >= 0 && k0 < F.W) ? cf[base + k0] : 0u;
                                            const uint32_t hi    = (k0 + 1 < F.W) ? cf[base + k0 + 1] : 0u;
                                            v |= compress_even(lo, hi);
                                        }
                                    }
                                }
                                nc[w] = v;
                            },
                            "new_cells");
    }

    // One pass of make_graduation (algorithm/graduation.hpp:573-726,
    // 245-330): the cells of level l that lie under the
    // (2*grad_width)-expansion of a leaf cell two or more levels finer are
    // refined.  flag[slot] is set when the pass refined something.  A pass
    // that finds nothing leaves the cells unchanged, so extra passes after the
    // fixed point are no-ops.  The contiguous-boundary pass
    // (graduation.hpp:121-249) is a no-op for a max_stencil_radius of 1.
    namespace
    {
        // list_interval_to_refine_for_contiguous_boundary_cells for a max_stencil_radius of 2
        // (algorithm/graduation.hpp:370-497): in each non-periodic Cartesian direction t, a leaf P of level lc is
        // refined when a leaf b of level lc + 1 on the boundary the direction points to has b - 2 t among P's
        // children, i.e. P sits at coordinate n - 2 (t = +e) or 1 (t = -e) along the axis and one of its children's
        // neighbours across the boundary layer is a leaf.  The bits of word (row, wi) of level lc to refine.
        __device__ __forceinline__ uint32_t contiguous_boundary_word(const Geom& g, const uint32_t* nc, int lc, long long w, long long row, int wi)
        {
            const uint32_t v = nc[w];
            if (!v)
            {
                return 0u;
            }
            const LevelGeom& C = g.lv[lc];
            const LevelGeom& F = g.lv[lc + 1];
            int y, z;
            if (g.dim == 2)
            {
                y = static_cast<int>(row) - PY;
                z = 0;
            }
            else
            {
                split_row(C, row, &y, &z);
                y -= PY;
                z -= PY;
            }
            const int x0   = 32 * wi - PX;
            const int nz   = g.dim == 3 ? 2 : 1;
            uint32_t out   = 0u;
            auto fine_word = [&](int fy, int fz, int k) -> uint32_t
            {
                const int ry = fy + PY, rz = fz + PY;
                if (ry < 0 || ry >= F.R || (g.dim == 3 && (rz < 0 || rz >= F.R)) || k < 0 || k >= F.W)
                {
                    return 0u;
                }
                const long long frow = (g.dim == 2) ? ry : static_cast<long long>(rz) * F.R + ry;
                return nc[F.woff + frow * F.W + k];
            };
            for (int d = 0; d < g.dim; ++d)
            {
                if ((g.periodic >> d) & 1)
                {
                    continue;
                }
                for (int sgn = 1; sgn >= -1; sgn -= 2)
                {
                    const int p  = sgn > 0 ? C.n - 2 : 1;  // coordinate of P along d
                    const int bf = sgn > 0 ? F.n - 1 : 0;  // coordinate of b along d
                    if (d == 0)
                    {
                        const int bit = p - x0;
                        if (bit < 0 || bit >= 32 || !((v >> bit) & 1u))
                        {
                            continue;
                        }
                        const int xb = bf + PX;
                        bool hit     = false;
                        for (int sz = 0; sz < nz && !hit; ++sz)
                        {
                            for (int sy = 0; sy < 2 && !hit; ++sy)
                            {
                                hit = (fine_word(2 * y + sy, 2 * z + sz, xb >> 5) >> (xb & 31)) & 1u;
                            }
                        }
                        out |= hit ? (1u << bit) : 0u;
                    }
                    else
                    {
                        if ((d == 1 ? y : z) != p)
                        {
                            continue;
                        }
                        // the fine boundary row (or plane) under the word's cells: any of a cell's two x children
                        for (int s2 = 0; s2 < 2 && (d == 1 ? s2 < nz : true); ++s2)
                        {
                            const int fy = d == 1 ? bf : 2 * y + s2;
                            const int fz = d == 1 ? 2 * z + s2 : bf;
                            if (g.dim == 2 && s2 > 0)
                            {
                                break;
                            }
                            out |= compress_pairs(fine_word(fy, fz, 2 * wi - 1), fine_word(fy, fz, 2 * wi));
                        }
                    }
                }
            }
            return out & v;
        }

        // refine the cells flagged in rr (levels dlo .. dtop): levels dlo .. dtop + 1 change
        int grad_apply(Ctx& c, uint32_t* nc, const uint32_t* rr, int dlo, int dtop)
        {
            return launch_words(c, dlo, dtop + 1,
                                [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                {
                                    const uint32_t r = l <= dtop ? rr[w] : 0u;
                                    uint32_t v       = nc[w] & ~r;
                                    if (l - 1 >= dlo)
                                    {
                                        v |= refine_word(g, rr, l, row, wi);
                                    }
                                    if (v != nc[w])
                                    {
                                        nc[w] = v;
                                    }
                                },
                                "grad_apply");
        }
    } // namespace

    int grad_pass(Ctx& c, uint32_t* nc, int slot, const int* guard)
    {
        // every launch of the pass is skipped on the device when *guard == 0
        struct GuardScope
        {
            Ctx& c;
            const int* saved;
            GuardScope(Ctx& cc, const int* gd)
                : c(cc)
                , saved(cc.guard)
            {
                c.guard = gd;
            }
            ~GuardScope()
            {
                c.guard = saved;
            }
        } scope(c, guard);
        const Geom g   = c.g;
        const int maxl = c.cfg.max_level;
        const int gw   = c.cfg.graduation_width;
        uint32_t* hcn  = c.t0;
        uint32_t* ec1  = c.t1;
        uint32_t* d    = c.t2;
        uint32_t* rr   = c.t3;
        int* flag      = c.d_flags + slot;
        // A cell of level l must be refined when a cell of level l+2 or finer
        // lies within 2 gw cells of it at that finer level: d[l] collects, on
        // level l, the finer cells dilated by 2 gw (graduation.hpp:628-723).
        // Levels min_level .. max_level-2 can hold such cells.
        const int dtop = maxl - 2;
        const int dlo  = c.cfg.min_level;
        // radius 2: the contiguous-boundary cells refine leaves of levels min_level .. max_level-1 too
        const bool contiguous = c.cfg.max_stencil_radius == 2;
        const int rtop        = contiguous ? maxl - 1 : dtop; // rr covers levels dlo .. rtop
        if (dtop < dlo && contiguous && maxl > dlo)
        {
            // no graduation between two levels, the contiguous-boundary pass alone
            int st = launch_words(c, dlo, rtop,
                                  [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                  {
                                      const uint32_t rv = contiguous_boundary_word(g, nc, l, w, row, wi);
                                      rr[w]             = rv;
                                      if (rv)
                                      {
                                          atomicOr(flag, 1);
                                      }
                                  },
                                  "grad_boundary");
            return st ? st : grad_apply(c, nc, rr, dlo, rtop);
        }
        if (dtop < dlo)
        {
            return SG_OK;
        }
        // ec1[l] = dilate_2gw(cells[l+1]).on(l), computed as
        // dilate_gw(cells[l+1].on(l)): per axis the parents of [a - 2gw, b + 2gw]
        // are [a/2 - gw, b/2 + gw], so both give the same set, and the
        // dilation then runs on the coarser level
        const int elo = dlo + 1, ehi = dtop + 1;
        int st        = launch_words(c, elo, ehi,
                                     [=] __device__(const Geom& g, int l, long long w, long long row, int wi) { hcn[w] = coarsen_word(g, nc, l, row, wi); },
                                     "grad_coarsen");
        if (st)
        {
            return st;
        }
        if (!g.periodic)
        {
            // d[l] = (ec1[l+1] | d[l+1]).on(l) on levels max-2 .. min_level is
            // the set of the cells with a cell of ec1 among their descendants:
            // the expansion marks the ancestors of each ec1 word into the zeroed
            // d (levels min_level .. max-2), and rr = nc & d follows in one pass
            const size_t off   = static_cast<size_t>(g.lv[dlo].woff);
            const size_t words = static_cast<size_t>(g.lv[dtop].woff + g.lv[dtop].nwords) - off;
            cudaMemsetAsync(d + off, 0, words * 4, c.stream);
            auto mark = [=] __device__(const Geom& g, int l, long long w, long long row, int wi, uint32_t e)
            {
                ec1[w] = e;
                if (e)
                {
                    const ParentWord pw = parent_word(g, l, row, wi);
                    if (pw.ok)
                    {
                        const LevelGeom& C  = g.lv[l - 1];
                        const uint32_t bits = (compress_pairs(e, 0u) & 0xFFFFu) << pw.shift;
                        if (bits && (atomicOr(d + C.woff + pw.row * C.W + pw.wi, bits) & bits) != bits)
                        {
                            mark_ancestors(g, d, l - 1, pw.row, pw.wi, bits, dlo);
                        }
                    }
                }
            };
            if (g.dim == 2)
            {
                st = launch_words(c, elo, ehi,
                                  [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                  { mark(g, l, w, row, wi, dilate_xy_word(g, hcn, l, row, wi, gw)); },
                                  "grad_expand");
            }
            else
            {
                // xy part into rr (written again below), then z with the marking
                st = launch_words(c, elo, ehi,
                                  [=] __device__(const Geom& g, int l, long long w, long long row, int wi) { rr[w] = dilate_xy_word(g, hcn, l, row, wi, gw); },
                                  "grad_expand_xy");
                if (!st)
                {
                    st = launch_words(c, elo, ehi,
                                      [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                      { mark(g, l, w, row, wi, dilate_z_word(g, rr, l, row, wi, gw)); },
                                      "grad_expand_z");
                }
            }
            if (!st)
            {
                const int dt = dtop;
                st           = launch_words(c, dlo, rtop,
                                  [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                  {
                                      uint32_t rv = l <= dt ? (nc[w] & d[w]) : 0u;
                                      if (contiguous)
                                      {
                                          rv |= contiguous_boundary_word(g, nc, l, w, row, wi);
                                      }
                                      rr[w] = rv;
                                      if (rv)
                                      {
                                          atomicOr(flag, 1);
                                      }
                                  },
                                  "grad_refine");
            }
            if (st)
            {
                return st;
            }
            return grad_apply(c, nc, rr, dlo, rtop);
        }
        if (g.dim == 2)
        {
            st = launch_words(c, elo, ehi,
                              [=] __device__(const Geom& g, int l, long long w, long long row, int wi) { ec1[w] = dilate_xy_word(g, hcn, l, row, wi, gw); },
                              "grad_expand");
        }
        else
        {
            // xy into d (written by the chain only after this), then z
            st = launch_words(c, elo, ehi,
                              [=] __device__(const Geom& g, int l, long long w, long long row, int wi) { d[w] = dilate_xy_word(g, hcn, l, row, wi, gw); },
                              "grad_expand_xy");
            if (!st)
            {
                st = launch_words(c, elo, ehi,
                                  [=] __device__(const Geom& g, int l, long long w, long long row, int wi) { ec1[w] = dilate_z_word(g, d, l, row, wi, gw); },
                                  "grad_expand_z");
            }
        }
        if (st)
        {
            return st;
        }
        if (g.periodic)
        {
            // with periodic axes the finer cells also act through their
            // translates (graduation.hpp:309-318): ec1 gains its translates
            // within the domain (translation commutes with the dilation and
            // with on(), so the chain below carries them down); the coarsened
            // cells in hcn are no longer needed and take the result
            const uint32_t* src = ec1;
            st                  = launch_words(c, elo, ehi,
                                               [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                                               { hcn[w] = src[w] | (periodic_translates(g, src, l, row, wi) & box_mask(g, l, row, wi, 0, 0)); },
                                               "grad_periodic");
            if (st)
            {
                return st;
            }
            ec1 = hcn;
        }
        // d[l] = (ec1[l+1] | d[l+1]).on(l), levels max-2 .. min_level; d and rr
        // are written on every word of those levels and read as 0 outside them
        st = launch_chain(c, dtop, dlo,
                          [=] __device__(const Geom& g, int ll, long long w, long long row, int wi)
                          {
                              const uint32_t dv = coarsen_word(g, ec1, ll, row, wi) | (ll + 1 <= dtop ? coarsen_word(g, d, ll, row, wi) : 0u);
                              d[w]              = dv;
                              const uint32_t rv = nc[w] & dv;
                              rr[w]             = rv;
                              if (rv)
                              {
                                  atomicOr(flag, 1);
                              }
                          },
                          "grad_down");
        if (st)
        {
            return st;
        }
        if (contiguous)
        {
            // the contiguous-boundary cells join the chain's graduation flags (levels above dtop had none)
            const int dt = dtop;
            st           = launch_words(c, dlo, rtop,
                              [=] __device__(const Geom& g, int l, long long w, long long row, int wi)
                              {
                                  const uint32_t add = contiguous_boundary_word(g, nc, l, w, row, wi);
                                  const uint32_t rv  = (l <= dt ? rr[w] : 0u) | add;
                                  rr[w]              = rv;
                                  if (add)
                                  {
                                      atomicOr(flag, 1);
                                  }
                              },
                              "grad_boundary");
            if (st)
            {
                return st;
            }
        }
        return grad_apply(c, nc, rr, dlo, rtop);
    }

    // make_graduation to the fixed point, with a host test after each pass
    int graduate(Ctx& c, uint32_t* nc, int* iterations)
    {
        ScopedTimer timer(c, T_GRADUATION);
        int nit = 0;
        for (;;)
        {
            ++nit;
            cudaMemsetAsync(c.d_flags + F_GRADX, 0, sizeof(int), c.stream);
            int st = grad_pass(c, nc, F_GRADX, nullptr);
            if (st)
            {
                return st;
            }
            cudaMemcpyAsync(c.h_flags + F_GRADX, c.d_flags + F_GRADX, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
            if (cudaStreamSynchronize(c.stream) != cudaSuccess)
            {
                return check(c, "graduate sync");
            }
            if (!c.h_flags[F_GRADX])
            {
                break;
            }
            if (nit > 64)
            {
                c.err = "graduation did not converge";
                return SG_ERR_STATE;
            }
        }
        if (iterations)
        {
            *iterations = nit - 1;
        }
        return SG_OK;
    }

    // flag[slot] = (a != b), without synchronisation
    int bitmaps_differ(Ctx& c, const uint32_t* a, const uint32_t* b, int slot)
    {
        int* flag = c.d_flags + slot;
        return launch_words(c, 0, c.g.nlev - 1,
                            [=] __device__(const Geom&, int, long long w, long long, int)
                            {
                                if (a[w] != b[w])
                                {
                                    atomicOr(flag, 1);
                                }
                            },
                            "compare");
    }

} // namespace sg
