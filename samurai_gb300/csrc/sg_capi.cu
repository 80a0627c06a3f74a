// C ABI of libsamurai_gpu.so (declared in include/samurai_gpu.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/samurai_gpu.h"
#include "sg_ctx.cuh"

#include "sg_handles.cuh"

namespace
{
    // per-thread message of the last failure; a fixed buffer, so that
    // reporting an error never allocates
    thread_local char g_err[512] = "";

    int fail(int code, const char* msg, const char* detail = nullptr)
    {
        std::snprintf(g_err, sizeof(g_err), "%s%s", msg ? msg : "", detail ? detail : "");
        return code;
    }

} // namespace


namespace
{
    // launch-shape tuning: a positive integer in the environment overrides a
    // default threshold (read when a mesh is created)
    long long tuned(const char* name, long long dflt)
    {
        const char* v = std::getenv(name);
        if (!v || !*v)
        {
            return dflt;
        }
        char* end          = nullptr;
        const long long x  = std::strtoll(v, &end, 10);
        return (end && *end == '\0' && x >= 0) ? x : dflt;
    }

    int from_ctx(sg::Ctx& c, int st)
    {
        if (st != sg::SG_OK)
        {
            fail(st, c.err.empty() ? "error" : c.err.c_str());
        }
        return st;
    }

    template <class T>
    int dalloc(sg::Ctx& c, T** p, size_t n)
    {
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), n * sizeof(T) + 256);
        if (e != cudaSuccess)
        {
            c.err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
            *p    = nullptr;
            return sg::SG_ERR_CUDA;
        }
        return sg::SG_OK;
    }

    template <class T>
    void dfree(T*& p)
    {
        if (p)
        {
            cudaFree(p);
            p = nullptr;
        }
    }

    int alloc_mesh(sg::Ctx& c, sg::DeviceMesh& m)
    {
        const size_t n = static_cast<size_t>(c.g.total_words);
        int st         = 0;
        st |= dalloc(c, &m.cells, n);
        st |= dalloc(c, &m.cag, n);
        st |= dalloc(c, &m.proj, n);
        st |= dalloc(c, &m.uni, n);
        st |= dalloc(c, &m.ref, n);
        st |= dalloc(c, &m.hc, n);
        st |= dalloc(c, &m.hc2, n);
        st |= dalloc(c, &m.rank, n);
        st |= dalloc(c, &m.wl_ref, n);
        st |= dalloc(c, &m.wl_cells, n);
        st |= dalloc(c, &m.d_lo, static_cast<size_t>(sg::COUNTS));
        if (!st && cudaMallocHost(reinterpret_cast<void**>(&m.h_lo), sg::COUNTS * sizeof(long long)) != cudaSuccess)
        {
            m.h_lo = nullptr;
            st     = sg::SG_ERR_CUDA;
        }
        return st ? sg::SG_ERR_CUDA : sg::SG_OK;
    }

    void free_mesh(sg::DeviceMesh& m)
    {
        dfree(m.cells);
        dfree(m.cag);
        dfree(m.proj);
        dfree(m.uni);
        dfree(m.ref);
        dfree(m.hc);
        dfree(m.hc2);
        dfree(m.rank);
        dfree(m.wl_ref);
        dfree(m.wl_cells);
        dfree(m.d_lo);
        if (m.h_lo)
        {
            cudaFreeHost(m.h_lo);
            m.h_lo = nullptr;
        }
    }

    void destroy_ctx(sg_mesh_s* h)
    {
        sg::Ctx& c = h->ctx;
        if (c.stream)
        {
            cudaStreamSynchronize(c.stream);
        }
        sg::timers_flush(c);
        sg::clear_graphs(c);
        for (const auto& mk : c.trace.marks)
        {
            sg::give_event(c, mk.second);
        }
        c.trace.marks.clear();
        sg::give_event(c, c.trace.start);
        c.trace.start = nullptr;
        std::sort(c.timers.pool.begin(), c.timers.pool.end());
        c.timers.pool.erase(std::unique(c.timers.pool.begin(), c.timers.pool.end()), c.timers.pool.end());
        for (cudaEvent_t e : c.timers.pool)
        {
            cudaEventDestroy(e);
        }
        dfree(c.d_ite);
        if (c.h_ite)
        {
            cudaFreeHost(c.h_ite);
        }
        free_mesh(c.mesh[0]);
        free_mesh(c.mesh[1]);
        dfree(c.t0);
        dfree(c.t1);
        dfree(c.t2);
        dfree(c.t3);
        dfree(c.rf);
        dfree(c.cf);
        dfree(c.detail);
        dfree(c.tag);
        dfree(c.block_sums);
        dfree(c.d_counts);
        dfree(c.d_flags);
        dfree(c.d_eps);
        dfree(c.d_absmax);
        dfree(c.g.err);
        if (c.h_eps)
        {
            cudaFreeHost(c.h_eps);
        }
        dfree(h->staging);
        if (c.h_counts)
        {
            cudaFreeHost(c.h_counts);
        }
        if (c.h_flags)
        {
            cudaFreeHost(c.h_flags);
        }
        dfree(c.d_adapt);
        if (c.h_adapt)
        {
            cudaFreeHost(c.h_adapt);
        }
        for (cudaStream_t cs : c.cap_streams)
        {
            if (cs)
            {
                cudaStreamDestroy(cs);
            }
        }
        if (c.stream)
        {
            cudaStreamDestroy(c.stream);
        }
        delete h;
    }

    __global__ void k_box_cells(const __grid_constant__ sg::Geom gp, int l, uint32_t* cells)
    {
        const sg::Geom& g      = gp;
        const sg::LevelGeom& L = g.lv[l];
        for (long long w = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; w < L.nwords; w += static_cast<long long>(gridDim.x) * blockDim.x)
        {
            const unsigned row = sg::fastdiv(static_cast<unsigned>(w), L.mW, L.sW);
            const int wi       = static_cast<int>(static_cast<unsigned>(w) - row * static_cast<unsigned>(L.W));
            cells[L.woff + w]   = sg::box_mask(g, l, row, wi, 0, 0);
        }
    }

    // FP64 throughput probe: independent multiply/add chains (built with
    // --fmad=false, so each step is one DMUL and one DADD)
    __global__ void k_fp64_probe(double* out, int iters, double a, double b)
    {
        double x0 = threadIdx.x * 1e-3, x1 = x0 + 1., x2 = x0 + 2., x3 = x0 + 3., x4 = x0 + 4., x5 = x0 + 5., x6 = x0 + 6., x7 = x0 + 7.;
        for (int k = 0; k < iters; ++k)
        {
            x0 = x0 * a + b;
            x1 = x1 * a + b;
            x2 = x2 * a + b;
            x3 = x3 * a + b;
            x4 = x4 * a + b;
            x5 = x5 * a + b;
            x6 = x6 * a + b;
            x7 = x7 * a + b;
        }
        const double r = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
        if (r == 12345.678)
        {
            out[0] = r; // keeps the chains alive
        }
    }

    int stage(sg_mesh_s* h, long long n)
    {
        if (n <= h->staging_n)
        {
            return sg::SG_OK;
        }
        dfree(h->staging);
        h->staging_n = 0;
        if (dalloc(h->ctx, &h->staging, static_cast<size_t>(n)))
        {
            return sg::SG_ERR_CUDA;
        }
        h->staging_n = n;
        return sg::SG_OK;
    }

    struct HostMesh
    {
        std::vector<uint32_t> bm;
        std::vector<uint32_t> ref;
        std::vector<int> rank;
    };

    int pull(sg::Ctx& c, const uint32_t* dbm, HostMesh& hm, bool with_ref)
    {
        const size_t n = static_cast<size_t>(c.g.total_words);
        hm.bm.resize(n);
        cudaMemcpyAsync(hm.bm.data(), dbm, n * 4, cudaMemcpyDeviceToHost, c.stream);
        if (with_ref)
        {
            hm.ref.resize(n);
            hm.rank.resize(n);
            cudaMemcpyAsync(hm.ref.data(), c.m().ref, n * 4, cudaMemcpyDeviceToHost, c.stream);
            cudaMemcpyAsync(hm.rank.data(), c.m().rank, n * 4, cudaMemcpyDeviceToHost, c.stream);
        }
        if (cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            return sg::check(c, "pull");
        }
        return sg::SG_OK;
    }

    long long host_ref_index(const HostMesh& hm, long long w, int b)
    {
        return static_cast<long long>(hm.rank[w]) + __builtin_popcount(hm.ref[w] & ((1u << b) - 1u));
    }

    const uint32_t* mesh_bitmap(sg::Ctx& c, int id)
    {
        sg::DeviceMesh& m = c.m();
        switch (id)
        {
            case SG_CELLS: return m.cells;
            case SG_CELLS_AND_GHOSTS: return m.cag;
            case SG_PROJ_CELLS: return m.proj;
            case SG_UNION_CELLS: return m.uni;
            case SG_REFERENCE: return m.ref;
            default: return nullptr;
        }
    }
} // namespace

namespace sg
{
    // the C ABI's error text, for entry points defined in other files
    void set_last_error(const char* msg, const char* detail)
    {
        fail(0, msg, detail);
    }

    // one-block chain limits of a mesh; the captured launch sequences are
    // dropped, since they were recorded with the previous limits
    void set_fusion_tops(Ctx& c, int mesh_top, int field_top, int max_top)
    {
        cudaStreamSynchronize(c.stream);
        c.fuse_top       = mesh_top;
        c.fuse_top_field = field_top;
        c.fuse_top_max   = max_top;
        sg::clear_graphs(c);
    }

    void set_fusion(Ctx& c, long long mesh_words, long long field_words, long long max_words)
    {
        c.fuse_words_mesh  = mesh_words;
        c.fuse_words_field = field_words;
        c.fuse_words_max   = max_words;
        set_fusion_tops(c, fuse_top_of(c.g, mesh_words), fuse_top_of(c.g, field_words), fuse_top_of(c.g, max_words));
    }

    // the spare buffer adaptation swaps into, allocated on first use
    int ensure_spare(Ctx& c, DeviceField& f)
    {
        if (!f.spare && dalloc(c, &f.spare, static_cast<size_t>(c.capacity)))
        {
            return SG_ERR_CUDA;
        }
        return SG_OK;
    }
} // namespace sg

extern "C"
{
    const char* sg_last_error(void)
    {
        return g_err;
    }

    int sg_version(int* major, int* minor)
    try
    {
        if (major)
        {
            *major = 0;
        }
        if (minor)
        {
            *minor = 1;
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_version)

    int sg_mesh_create(int dim, int min_level, int max_level, int max_stencil_radius, int prediction_radius, int graduation_width, sg_mesh_t* out)
    try
    {
        return sg_mesh_create_periodic(dim, min_level, max_level, max_stencil_radius, prediction_radius, graduation_width, nullptr, out);
    }
    SG_API_CATCH(sg_mesh_create)

    int sg_mesh_create_periodic(int dim, int min_level, int max_level, int max_stencil_radius, int prediction_radius, int graduation_width,
                                const int* periodic, sg_mesh_t* out)
    try
    {
        if (!out)
        {
            return fail(SG_ERR_ARG, "sg_mesh_create: null output");
        }
        *out = nullptr;
        if (dim != 2 && dim != 3)
        {
            return fail(SG_ERR_ARG, "sg_mesh_create: dim must be 2 or 3");
        }
        if (min_level < 1 || max_level < min_level || max_level + 1 > sg::MAXLEV)
        {
            return fail(SG_ERR_ARG, "sg_mesh_create: need 1 <= min_level <= max_level <= 23");
        }
        if (max_stencil_radius < 1 || prediction_radius < 0 || prediction_radius > 1 || graduation_width < 1 || graduation_width > 4)
        {
            return fail(SG_ERR_ARG, "sg_mesh_create: unsupported stencil radius / prediction radius / graduation width");
        }
        if (max_stencil_radius > 2)
        {
            return fail(SG_ERR_ARG, "sg_mesh_create: max_stencil_radius 1 and 2 are implemented (samurai's demos and its default)");
        }
        {
            // the dense slabs of all levels (the bitmap words of sg::make_geom, 32 cells each), counted in
            // floating point so that levels whose sizes overflow 64-bit integers (3D beyond about 20) are refused
            double words = 0.0;
            for (int l = 0; l <= max_level; ++l)
            {
                const double n = std::ldexp(1.0, l), W = std::ceil(n / 32.0) + 2.0, R = n + 2.0 * sg::PY;
                words += (dim == 2 ? R : R * R) * W;
            }
            if (words * 32.0 * sizeof(double) > std::ldexp(1.0, 47))
            {
                return fail(SG_ERR_CAPACITY, "sg_mesh_create: max_level too fine: one field's dense slabs would exceed 128 TiB");
            }
        }
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        {
            cudaGetLastError();
            return fail(SG_ERR_CUDA, "sg_mesh_create: no CUDA device");
        }
        {
            // device memory of the mesh (two meshes of 10 word arrays, 6 scratch bitmaps, the dense detail and tag
            // slabs) and of one field with its update_fields buffer, against the free memory of the device: a
            // configuration that cannot fit is refused here rather than by a failing allocation midway
            const sg::Geom gg    = sg::make_geom(dim, min_level, max_level);
            const double words   = static_cast<double>(gg.total_words);
            const double cap     = 32.0 * words;
            const double mesh_b  = (2.0 * 10.0 + 6.0) * 4.0 * words + 9.0 * cap;
            const double field_b = 16.0 * cap;
            size_t free_b = 0, total_b = 0;
            if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess)
            {
                cudaGetLastError();
                return fail(SG_ERR_CUDA, "sg_mesh_create: cudaMemGetInfo failed");
            }
            if (mesh_b + field_b > static_cast<double>(free_b))
            {
                char msg[256];
                std::snprintf(msg, sizeof msg,
                              "sg_mesh_create: the mesh needs %.1f GB of device memory and each field %.1f GB (dense level slabs), "
                              "%.1f GB are free",
                              mesh_b / 1e9, field_b / 1e9, static_cast<double>(free_b) / 1e9);
                return fail(SG_ERR_CAPACITY, msg);
            }
        }
        sg_mesh_s* h = new (std::nothrow) sg_mesh_s();
        if (!h)
        {
            return fail(SG_ERR_CAPACITY, "sg_mesh_create: out of host memory");
        }
        sg::Ctx& c                 = h->ctx;
        c.cfg.dim                  = dim;
        c.cfg.min_level            = min_level;
        c.cfg.max_level            = max_level;
        c.cfg.max_stencil_radius   = max_stencil_radius;
        c.cfg.prediction_radius    = prediction_radius;
        c.cfg.graduation_width     = graduation_width;
        c.cfg.ghost_width          = max_stencil_radius > prediction_radius ? max_stencil_radius : prediction_radius;
        c.g                        = sg::make_geom(dim, min_level, max_level);
        c.g.ghost_width            = c.cfg.ghost_width;
        c.g.periodic               = 0;
        for (int d = 0; periodic && d < dim; ++d)
        {
            c.g.periodic |= periodic[d] ? (1 << d) : 0;
        }
        c.capacity                 = 32 * c.g.total_words;
        c.fuse_words_mesh          = tuned("SG_FUSE_WORDS", sg::FUSE_WORDS);
        c.fuse_words_field         = tuned("SG_FUSE_WORDS_FIELD", sg::FUSE_WORDS_FIELD);
        c.fuse_words_max           = tuned("SG_FUSE_WORDS_MAX", sg::FUSE_WORDS_MAX);
        c.max_blocks               = std::max(1LL, tuned("SG_MAX_BLOCKS", c.max_blocks));
        c.block                    = static_cast<int>(std::min(1024LL, std::max(32LL, tuned("SG_BLOCK", c.block))) / 32 * 32);
        // the pass-by-pass path by default: on GB300 with driver 580 a conditional graph node costs about 9 us
        // (measured), more than the host round trip per Harten pass it replaces
        c.graphed_adapt = tuned("SG_GRAPHED_ADAPT", 0) != 0;
        c.level_pairs   = tuned("SG_LEVEL_PAIRS", 1) != 0;
        if (cudaGetDevice(&c.device) != cudaSuccess)
        {
            cudaGetLastError();
            delete h;
            return fail(SG_ERR_CUDA, "sg_mesh_create: no CUDA device");
        }
        sg::apply_tuned_launch(c); // the autotuner's choice for this device and level range, unless overridden above
        c.fuse_top                 = sg::fuse_top_of(c.g, c.fuse_words_mesh);
        c.fuse_top_field           = sg::fuse_top_of(c.g, c.fuse_words_field);
        c.fuse_top_max             = sg::fuse_top_of(c.g, c.fuse_words_max);
        if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess)
        {
            cudaGetLastError();
            delete h;
            return fail(SG_ERR_CUDA, "sg_mesh_create: cudaStreamCreate failed");
        }
        for (auto& cs : c.cap_streams)
        {
            if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess)
            {
                cudaGetLastError();
                cs = nullptr;
            }
        }

        const size_t nw = static_cast<size_t>(c.g.total_words);
        int st          = alloc_mesh(c, c.mesh[0]);
        st |= alloc_mesh(c, c.mesh[1]);
        st |= dalloc(c, &c.t0, nw);
        st |= dalloc(c, &c.t1, nw);
        st |= dalloc(c, &c.t2, nw);
        st |= dalloc(c, &c.t3, nw);
        st |= dalloc(c, &c.rf, nw);
        st |= dalloc(c, &c.cf, nw);
        st |= dalloc(c, &c.detail, static_cast<size_t>(c.capacity));
        st |= dalloc(c, &c.tag, static_cast<size_t>(c.capacity));
        c.n_scan_blocks = (c.g.total_words + 4095) / 4096;
        st |= dalloc(c, &c.block_sums, 4 * static_cast<size_t>(c.n_scan_blocks) + 4);
        st |= dalloc(c, &c.d_counts, static_cast<size_t>(sg::COUNTS));
        st |= dalloc(c, &c.d_flags, 8);
        st |= dalloc(c, &c.d_adapt, static_cast<size_t>(sg::A_COUNT));
        st |= dalloc(c, &c.d_ite, 1);
        st |= dalloc(c, &c.d_eps, sg::EPS_VELOCITY + 3);
        st |= dalloc(c, &c.d_absmax, 1);
        st |= dalloc(c, &c.g.err, 1);
        if (!st)
        {
            if (cudaMallocHost(reinterpret_cast<void**>(&c.h_ite), sizeof(int)) != cudaSuccess
                || cudaMallocHost(reinterpret_cast<void**>(&c.h_eps), 3 * sg::MAXLEV * sizeof(double)) != cudaSuccess
                || cudaMallocHost(reinterpret_cast<void**>(&c.h_counts), sg::COUNTS * sizeof(long long)) != cudaSuccess
                || cudaMallocHost(reinterpret_cast<void**>(&c.h_flags), 8 * sizeof(int)) != cudaSuccess
                || cudaMallocHost(reinterpret_cast<void**>(&c.h_adapt), sg::A_COUNT * sizeof(int)) != cudaSuccess)
            {
                st = SG_ERR_CUDA;
                c.err = "cudaMallocHost failed";
            }
        }
        if (st)
        {
            std::string msg = c.err;
            destroy_ctx(h);
            return fail(SG_ERR_CUDA, "sg_mesh_create: ", msg.c_str());
        }
        cudaMemsetAsync(c.g.err, 0, sizeof(int), c.stream);
        // every bitmap starts empty: the mesh construction writes only the
        // levels where a set can be non-empty and relies on zeros elsewhere
        for (int k = 0; k < 2; ++k)
        {
            sg::DeviceMesh& mk = c.mesh[k];
            for (uint32_t* bm : {mk.cells, mk.cag, mk.proj, mk.uni, mk.ref, mk.hc, mk.hc2})
            {
                cudaMemsetAsync(bm, 0, nw * 4, c.stream);
            }
        }
        cudaMemsetAsync(c.detail, 0, static_cast<size_t>(c.capacity) * sizeof(double), c.stream);
        cudaMemsetAsync(c.tag, 0, static_cast<size_t>(c.capacity), c.stream);
        k_box_cells<<<sg::grid_for(c.g.lv[max_level].nwords), 256, 0, c.stream>>>(c.g, max_level, c.m().cells);
        st = sg::check(c, "initial cells");
        if (!st)
        {
            st = sg::build_mesh(c, c.m());
        }
        if (!st)
        {
            st = sg::host_counts(c, c.m());
        }
        if (st)
        {
            std::string msg = c.err;
            destroy_ctx(h);
            return fail(st, "sg_mesh_create: ", msg.c_str());
        }
        *out = h;
        return SG_OK;
    }
    SG_API_CATCH(sg_mesh_create_periodic)

    int sg_mesh_destroy(sg_mesh_t mesh)
    try
    {
        if (mesh && !mesh->destroyed)
        {
            mesh->destroyed = true;
            if (mesh->attached == 0)
            {
                destroy_ctx(mesh);
            }
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_mesh_destroy)

    int sg_mesh_counts(sg_mesh_t mesh, long long* nb_cells, long long* nb_reference)
    try
    {
        if (!mesh)
        {
            return fail(SG_ERR_ARG, "sg_mesh_counts: null mesh");
        }
        if (int st = sg::host_counts(mesh->ctx, mesh->ctx.m()))
        {
            return from_ctx(mesh->ctx, st);
        }
        if (nb_cells)
        {
            *nb_cells = mesh->ctx.m().nb_cells;
        }
        if (nb_reference)
        {
            *nb_reference = mesh->ctx.m().nb_ref;
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_mesh_counts)

    int sg_mesh_get_cells(sg_mesh_t mesh, int* level, int* coords, long long* index, long long capacity)
    try
    {
        if (!mesh)
        {
            return fail(SG_ERR_ARG, "sg_mesh_get_cells: null mesh");
        }
        sg::Ctx& c = mesh->ctx;
        if (int st = sg::host_counts(c, c.m()))
        {
            return from_ctx(c, st);
        }
        if (capacity < c.m().nb_cells)
        {
            return fail(SG_ERR_CAPACITY, "sg_mesh_get_cells: output too small");
        }
        HostMesh hm;
        if (int st = pull(c, c.m().cells, hm, true))
        {
            return from_ctx(c, st);
        }
        const int D  = c.g.dim;
        long long k  = 0;
        for (long long w = 0; w < c.g.total_words; ++w)
        {
            uint32_t v = hm.bm[w];
            if (!v)
            {
                continue;
            }
            const int l = sg::level_of(c.g, w);
            while (v)
            {
                const int b = __builtin_ctz(v);
                v &= v - 1;
                const sg::Cell cc = sg::cell_of(c.g, l, w, b);
                if (level)
                {
                    level[k] = l;
                }
                if (coords)
                {
                    coords[D * k]     = cc.x;
                    coords[D * k + 1] = cc.y;
                    if (D == 3)
                    {
                        coords[D * k + 2] = cc.z;
                    }
                }
                if (index)
                {
                    index[k] = host_ref_index(hm, w, b);
                }
                ++k;
            }
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_mesh_get_cells)

    int sg_mesh_count_intervals(sg_mesh_t mesh, int mesh_id, int level, long long* n)
    try
    {
        if (!mesh || !n)
        {
            return fail(SG_ERR_ARG, "sg_mesh_count_intervals: null argument");
        }
        sg::Ctx& c = mesh->ctx;
        const uint32_t* dbm = mesh_bitmap(c, mesh_id);
        if (!dbm || level < 0 || level >= c.g.nlev)
        {
            return fail(SG_ERR_ARG, "sg_mesh_count_intervals: bad mesh id or level");
        }
        HostMesh hm;
        if (int st = pull(c, dbm, hm, false))
        {
            return from_ctx(c, st);
        }
        const sg::LevelGeom& L = c.g.lv[level];
        long long cnt          = 0;
        for (long long r = 0; r < L.nrows; ++r)
        {
            bool prev = false;
            for (int x = 0; x < 32 * L.W; ++x)
            {
                const long long w = L.woff + r * L.W + (x >> 5);
                const bool on     = (hm.bm[w] >> (x & 31)) & 1u;
                if (on && !prev)
                {
                    ++cnt;
                }
                prev = on;
            }
        }
        *n = cnt;
        return SG_OK;
    }
    SG_API_CATCH(sg_mesh_count_intervals)

    int sg_mesh_get_intervals(sg_mesh_t mesh, int mesh_id, int level, long long* out, long long capacity)
    try
    {
        if (!mesh || !out)
        {
            return fail(SG_ERR_ARG, "sg_mesh_get_intervals: null argument");
        }
        sg::Ctx& c = mesh->ctx;
        const uint32_t* dbm = mesh_bitmap(c, mesh_id);
        if (!dbm || level < 0 || level >= c.g.nlev)
        {
            return fail(SG_ERR_ARG, "sg_mesh_get_intervals: bad mesh id or level");
        }
        HostMesh hm;
        if (int st = pull(c, dbm, hm, true))
        {
            return from_ctx(c, st);
        }
        const int D            = c.g.dim;
        const int rec          = D + 2;
        const sg::LevelGeom& L = c.g.lv[level];
        long long k            = 0;
        for (long long r = 0; r < L.nrows; ++r)
        {
            int start = 0;
            bool prev = false;
            for (int xb = 0; xb <= 32 * L.W; ++xb)
            {
                bool on = false;
                if (xb < 32 * L.W)
                {
                    const long long w = L.woff + r * L.W + (xb >> 5);
                    on                = (hm.bm[w] >> (xb & 31)) & 1u;
                }
                if (on && !prev)
                {
                    start = xb;
                }
                if (!on && prev)
                {
                    if (k >= capacity)
                    {
                        return fail(SG_ERR_CAPACITY, "sg_mesh_get_intervals: output too small");
                    }
                    const long long w0 = L.woff + r * L.W + (start >> 5);
                    const int x0       = start - sg::PX;
                    const sg::Cell cc  = sg::cell_of(c.g, level, w0, start & 31);
                    long long idx      = -1;
                    if ((hm.ref[w0] >> (start & 31)) & 1u)
                    {
                        idx = host_ref_index(hm, w0, start & 31) - x0;
                    }
                    out[rec * k]     = x0;
                    out[rec * k + 1] = xb - sg::PX;
                    out[rec * k + 2] = cc.y;
                    if (D == 3)
                    {
                        out[rec * k + 3] = cc.z;
                    }
                    out[rec * k + D + 1] = idx;
                    ++k;
                }
                prev = on;
            }
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_mesh_get_intervals)

    int sg_mesh_set_cells(sg_mesh_t mesh, long long n, const int* level, const int* coords)
    try
    {
        if (!mesh || n < 0 || (n > 0 && (!level || !coords)))
        {
            return fail(SG_ERR_ARG, "sg_mesh_set_cells: null argument or negative count");
        }
        sg::Ctx& c = mesh->ctx;
        const int D = c.g.dim;
        std::vector<uint32_t> bm(static_cast<size_t>(c.g.total_words), 0u);
        for (long long i = 0; i < n; ++i)
        {
            const int l = level[i];
            if (l < c.cfg.min_level || l > c.cfg.max_level)
            {
                return fail(SG_ERR_ARG, "sg_mesh_set_cells: level out of [min_level, max_level]");
            }
            const int x = coords[D * i], y = coords[D * i + 1], z = D == 3 ? coords[D * i + 2] : 0;
            const int nl = 1 << l;
            if (x < 0 || x >= nl || y < 0 || y >= nl || z < 0 || (D == 3 && z >= nl))
            {
                return fail(SG_ERR_ARG, "sg_mesh_set_cells: cell outside the unit box");
            }
            const sg::Pos p = sg::pos_of(c.g, l, x, y, z);
            bm[static_cast<size_t>(p.w)] |= 1u << p.b;
        }
        cudaMemcpyAsync(c.m().cells, bm.data(), bm.size() * 4, cudaMemcpyHostToDevice, c.stream);
        ++c.mesh_version;
        int st = sg::build_mesh(c, c.m());
        if (!st)
        {
            st = sg::host_counts(c, c.m());
        }
        return from_ctx(c, st);
    }
    SG_API_CATCH(sg_mesh_set_cells)

    int sg_mesh_stream(sg_mesh_t mesh, void** stream)
    try
    {
        if (!mesh || !stream)
        {
            return fail(SG_ERR_ARG, "sg_mesh_stream: null argument");
        }
        *stream = mesh->ctx.stream;
        return SG_OK;
    }
    SG_API_CATCH(sg_mesh_stream)

    int sg_mesh_synchronize(sg_mesh_t mesh)
    try
    {
        if (!mesh)
        {
            return fail(SG_ERR_ARG, "sg_mesh_synchronize: null mesh");
        }
        cudaError_t e = cudaStreamSynchronize(mesh->ctx.stream);
        if (e != cudaSuccess)
        {
            return fail(SG_ERR_CUDA, "sg_mesh_synchronize: ", cudaGetErrorString(e));
        }
        return from_ctx(mesh->ctx, sg::device_error(mesh->ctx));
    }
    SG_API_CATCH(sg_mesh_synchronize)

    int sg_mesh_version(sg_mesh_t mesh, unsigned long long* version)
    try
    {
        if (!mesh || !version)
        {
            return fail(SG_ERR_ARG, "sg_mesh_version: null argument");
        }
        *version = mesh->ctx.mesh_version;
        return SG_OK;
    }
    SG_API_CATCH(sg_mesh_version)

    int sg_mesh_launch_count(sg_mesh_t mesh, int reset, long long* count)
    try
    {
        if (!mesh)
        {
            return fail(SG_ERR_ARG, "sg_mesh_launch_count: null mesh");
        }
        if (count)
        {
            *count = mesh->ctx.n_launches;
        }
        if (reset)
        {
            mesh->ctx.n_launches = 0;
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_mesh_launch_count)

    int sg_device_fp64_rate(double* gflops)
    try
    {
        if (!gflops)
        {
            return fail(SG_ERR_ARG, "sg_device_fp64_rate: null output");
        }
        int dev = 0, nsm = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        {
            cudaGetLastError();
            return fail(SG_ERR_CUDA, "sg_device_fp64_rate: no CUDA device");
        }
        double* d = nullptr;
        cudaMalloc(&d, 64);
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        const int blocks = nsm * 8, threads = 256, iters = 4096;
        k_fp64_probe<<<blocks, threads>>>(d, 64, 1.0000001, 1e-9); // warm up
        cudaEventRecord(e0);
        k_fp64_probe<<<blocks, threads>>>(d, iters, 1.0000001, 1e-9);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(d);
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess)
        {
            return fail(SG_ERR_CUDA, "sg_device_fp64_rate: ", cudaGetErrorString(err));
        }
        const double ops = 2.0 * 8.0 * iters * static_cast<double>(blocks) * threads;
        *gflops          = ops / (ms * 1e-3) / 1e9;
        return SG_OK;
    }
    SG_API_CATCH(sg_device_fp64_rate)

    int sg_mesh_set_adapt_graph(sg_mesh_t mesh, int enable)
    try
    {
        if (!mesh)
        {
            return fail(SG_ERR_ARG, "sg_mesh_set_adapt_graph: null mesh");
        }
        mesh->ctx.graphed_adapt = enable != 0;
        return SG_OK;
    }
    SG_API_CATCH(sg_mesh_set_adapt_graph)

    int sg_mesh_set_refine_boundary(sg_mesh_t mesh, int enable)
    try
    {
        if (!mesh)
        {
            return fail(SG_ERR_ARG, "sg_mesh_set_refine_boundary: null mesh");
        }
        mesh->ctx.refine_boundary = enable != 0;
        return SG_OK;
    }
    SG_API_CATCH(sg_mesh_set_refine_boundary)

    int sg_kernel_trace(sg_mesh_t mesh, int enable)
    try
    {
        if (!mesh)
        {
            return fail(SG_ERR_ARG, "sg_kernel_trace: null mesh");
        }
        sg::Ctx& c = mesh->ctx;
        if (enable)
        {
            if (cudaStreamSynchronize(c.stream) != cudaSuccess)
            {
                return fail(SG_ERR_CUDA, "sg_kernel_trace: CUDA error");
            }
            // the events of the previous window that no captured sequence holds go back to the pool
            for (const auto& mk : c.trace.marks)
            {
                bool held = false;
                for (const auto& ge : c.graphs)
                {
                    for (const auto& gm : ge.marks)
                    {
                        held = held || gm.second == mk.second;
                    }
                }
                if (!held)
                {
                    sg::give_event(c, mk.second);
                }
            }
            c.trace.marks.clear();
            c.trace.reused = false;
            c.trace.results.clear();
            if (!c.trace.start)
            {
                c.trace.start = sg::take_event(c);
            }
            cudaEventRecord(c.trace.start, c.stream);
            c.trace.enabled = true;
            return SG_OK;
        }
        if (!c.trace.enabled)
        {
            return SG_OK;
        }
        c.trace.enabled = false;
        if (cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            return fail(SG_ERR_CUDA, "sg_kernel_trace: CUDA error");
        }
        cudaEvent_t prev = c.trace.start;
        for (const auto& mk : c.trace.marks)
        {
            if (!mk.first)
            {
                prev = mk.second; // the head of a launch sequence: the gap before it belongs to no kernel
                continue;
            }
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, prev, mk.second) != cudaSuccess)
            {
                cudaGetLastError();
                c.trace.reused = true;
                ms             = 0.f;
            }
            prev   = mk.second;
            bool found = false;
            for (auto& r : c.trace.results)
            {
                if (r.name == mk.first)
                {
                    r.launches += 1;
                    r.ms += ms;
                    found = true;
                    break;
                }
            }
            if (!found)
            {
                c.trace.results.push_back({mk.first, 1, static_cast<double>(ms)});
            }
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_kernel_trace)

    int sg_kernel_trace_read(sg_mesh_t mesh, int i, const char** name, long long* launches, double* ms, int* valid)
    try
    {
        if (!mesh || i < 0)
        {
            return fail(SG_ERR_ARG, "sg_kernel_trace_read: null mesh or negative index");
        }
        const auto& res = mesh->ctx.trace.results;
        if (static_cast<size_t>(i) >= res.size())
        {
            return SG_ERR_NOTFOUND;
        }
        if (name)
        {
            *name = res[static_cast<size_t>(i)].name;
        }
        if (launches)
        {
            *launches = res[static_cast<size_t>(i)].launches;
        }
        if (ms)
        {
            *ms = res[static_cast<size_t>(i)].ms;
        }
        if (valid)
        {
            *valid = mesh->ctx.trace.reused ? 0 : 1;
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_kernel_trace_read)

    int sg_timers_enable(sg_mesh_t mesh, int enable)
    try
    {
        if (!mesh)
        {
            return fail(SG_ERR_ARG, "sg_timers_enable: null mesh");
        }
        mesh->ctx.timers.enabled = enable != 0;
        return SG_OK;
    }
    SG_API_CATCH(sg_timers_enable)

    int sg_timers_get(sg_mesh_t mesh, int timer_id, double* total_ms, long long* calls)
    try
    {
        if (!mesh || timer_id < 0 || timer_id >= sg::T_COUNT)
        {
            return fail(SG_ERR_ARG, "sg_timers_get: bad mesh or timer id");
        }
        sg::timers_flush(mesh->ctx);
        if (total_ms)
        {
            *total_ms = mesh->ctx.timers.ms[timer_id];
        }
        if (calls)
        {
            *calls = mesh->ctx.timers.calls[timer_id];
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_timers_get)

    int sg_timers_reset(sg_mesh_t mesh)
    try
    {
        if (!mesh)
        {
            return fail(SG_ERR_ARG, "sg_timers_reset: null mesh");
        }
        sg::timers_flush(mesh->ctx);
        for (int i = 0; i < sg::T_COUNT; ++i)
        {
            mesh->ctx.timers.ms[i]    = 0.;
            mesh->ctx.timers.calls[i] = 0;
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_timers_reset)

    int sg_field_create(sg_mesh_t mesh, const char* name, sg_field_t* out)
    try
    {
        if (!mesh || !out)
        {
            return fail(SG_ERR_ARG, "sg_field_create: null argument");
        }
        sg_field_s* f = new (std::nothrow) sg_field_s();
        if (!f)
        {
            return fail(SG_ERR_CAPACITY, "sg_field_create: out of host memory");
        }
        f->mesh  = mesh;
        f->f.ctx = &mesh->ctx;
        f->f.name = name ? name : "";
        {
            // the field's slab and the buffer update_fields gives it on the first adaptation
            size_t free_b = 0, total_b = 0;
            const double need = 16.0 * static_cast<double>(mesh->ctx.capacity);
            if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && need > static_cast<double>(free_b))
            {
                delete f;
                char msg[200];
                std::snprintf(msg, sizeof msg, "sg_field_create: the field needs %.1f GB of device memory, %.1f GB are free", need / 1e9,
                              static_cast<double>(free_b) / 1e9);
                return fail(SG_ERR_CAPACITY, msg);
            }
            cudaGetLastError();
        }
        if (dalloc(mesh->ctx, &f->f.data, static_cast<size_t>(mesh->ctx.capacity)))
        {
            delete f;
            return fail(SG_ERR_CUDA, "sg_field_create: ", mesh->ctx.err.c_str());
        }
        cudaMemsetAsync(f->f.data, 0, static_cast<size_t>(mesh->ctx.capacity) * sizeof(double), mesh->ctx.stream);
        ++mesh->attached;
        *out = f;
        return SG_OK;
    }
    SG_API_CATCH(sg_field_create)

    int sg_field_destroy(sg_field_t field)
    try
    {
        if (field)
        {
            sg_mesh_s* mesh = field->mesh;
            cudaStreamSynchronize(mesh->ctx.stream);
            dfree(field->f.data);
            dfree(field->f.spare);
            delete field;
            if (--mesh->attached == 0 && mesh->destroyed)
            {
                destroy_ctx(mesh);
            }
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_field_destroy)

    int sg_field_set_dirichlet(sg_field_t field, double value)
    try
    {
        if (!field)
        {
            return fail(SG_ERR_ARG, "sg_field_set_dirichlet: null field");
        }
        field->f.has_bc   = true;
        field->f.bc_value = value;
        return SG_OK;
    }
    SG_API_CATCH(sg_field_set_dirichlet)

    int sg_field_upload_device(sg_field_t field, const double* dvalues, long long n)
    try
    {
        if (!field || !dvalues)
        {
            return fail(SG_ERR_ARG, "sg_field_upload_device: null argument");
        }
        sg::Ctx& c = field->mesh->ctx;
        if (int st = sg::host_counts(c, c.m()))
        {
            return from_ctx(c, st);
        }
        if (n != c.m().nb_ref)
        {
            return fail(SG_ERR_ARG, "sg_field_upload_device: size differs from the reference mesh");
        }
        field->f.ghosts_valid = false;
        return from_ctx(c, sg::scatter_compact(c, c.m(), dvalues, field->f.data));
    }
    SG_API_CATCH(sg_field_upload_device)

    int sg_field_download_device(sg_field_t field, double* dvalues, long long n)
    try
    {
        if (!field || !dvalues)
        {
            return fail(SG_ERR_ARG, "sg_field_download_device: null argument");
        }
        sg::Ctx& c = field->mesh->ctx;
        if (int st = sg::host_counts(c, c.m()))
        {
            return from_ctx(c, st);
        }
        if (n != c.m().nb_ref)
        {
            return fail(SG_ERR_ARG, "sg_field_download_device: size differs from the reference mesh");
        }
        return from_ctx(c, sg::gather_compact(c, c.m(), field->f.data, dvalues));
    }
    SG_API_CATCH(sg_field_download_device)

    int sg_field_upload(sg_field_t field, const double* values, long long n)
    try
    {
        if (!field || !values)
        {
            return fail(SG_ERR_ARG, "sg_field_upload: null argument");
        }
        sg_mesh_s* h = field->mesh;
        sg::Ctx& c   = h->ctx;
        if (int st = sg::host_counts(c, c.m()))
        {
            return from_ctx(c, st);
        }
        if (n != c.m().nb_ref)
        {
            return fail(SG_ERR_ARG, "sg_field_upload: size differs from the reference mesh");
        }
        if (stage(h, n))
        {
            return from_ctx(c, SG_ERR_CUDA);
        }
        cudaMemcpyAsync(h->staging, values, static_cast<size_t>(n) * sizeof(double), cudaMemcpyHostToDevice, c.stream);
        field->f.ghosts_valid = false;
        int st = sg::scatter_compact(c, c.m(), h->staging, field->f.data);
        if (!st && cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            st = sg::check(c, "upload");
        }
        return from_ctx(c, st);
    }
    SG_API_CATCH(sg_field_upload)

    int sg_field_download(sg_field_t field, double* values, long long n)
    try
    {
        if (!field || !values)
        {
            return fail(SG_ERR_ARG, "sg_field_download: null argument");
        }
        sg_mesh_s* h = field->mesh;
        sg::Ctx& c   = h->ctx;
        if (int st = sg::host_counts(c, c.m()))
        {
            return from_ctx(c, st);
        }
        if (n != c.m().nb_ref)
        {
            return fail(SG_ERR_ARG, "sg_field_download: size differs from the reference mesh");
        }
        if (stage(h, n))
        {
            return from_ctx(c, SG_ERR_CUDA);
        }
        int st = sg::gather_compact(c, c.m(), field->f.data, h->staging);
        if (st)
        {
            return from_ctx(c, st);
        }
        cudaMemcpyAsync(values, h->staging, static_cast<size_t>(n) * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
        if (cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            return from_ctx(c, sg::check(c, "download"));
        }
        return from_ctx(c, sg::device_error(c));
    }
    SG_API_CATCH(sg_field_download)

    int sg_field_set_cells(sg_field_t field, const double* values, long long n)
    try
    {
        if (!field || !values)
        {
            return fail(SG_ERR_ARG, "sg_field_set_cells: null argument");
        }
        sg::Ctx& c = field->mesh->ctx;
        if (int st = sg::host_counts(c, c.m()))
        {
            return from_ctx(c, st);
        }
        if (n != c.m().nb_cells)
        {
            return fail(SG_ERR_ARG, "sg_field_set_cells: size differs from the number of cells");
        }
        std::vector<long long> idx(static_cast<size_t>(n));
        if (int st = sg_mesh_get_cells(field->mesh, nullptr, nullptr, idx.data(), n))
        {
            return st;
        }
        std::vector<double> full(static_cast<size_t>(c.m().nb_ref), 0.);
        for (long long i = 0; i < n; ++i)
        {
            full[static_cast<size_t>(idx[i])] = values[i];
        }
        return sg_field_upload(field, full.data(), c.m().nb_ref);
    }
    SG_API_CATCH(sg_field_set_cells)

    int sg_field_get_cells(sg_field_t field, double* values, long long n)
    try
    {
        if (!field || !values)
        {
            return fail(SG_ERR_ARG, "sg_field_get_cells: null argument");
        }
        sg::Ctx& c = field->mesh->ctx;
        if (int st = sg::host_counts(c, c.m()))
        {
            return from_ctx(c, st);
        }
        if (n != c.m().nb_cells)
        {
            return fail(SG_ERR_ARG, "sg_field_get_cells: size differs from the number of cells");
        }
        std::vector<long long> idx(static_cast<size_t>(n));
        if (int st = sg_mesh_get_cells(field->mesh, nullptr, nullptr, idx.data(), n))
        {
            return st;
        }
        std::vector<double> full(static_cast<size_t>(c.m().nb_ref));
        if (int st = sg_field_download(field, full.data(), c.m().nb_ref))
        {
            return st;
        }
        for (long long i = 0; i < n; ++i)
        {
            values[i] = full[static_cast<size_t>(idx[i])];
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_field_get_cells)

    int sg_field_fill(sg_field_t field, double value)
    try
    {
        if (!field)
        {
            return fail(SG_ERR_ARG, "sg_field_fill: null field");
        }
        sg::Ctx& c = field->mesh->ctx;
        if (int st = sg::host_counts(c, c.m()))
        {
            return from_ctx(c, st);
        }
        field->f.ghosts_valid = false;
        return from_ctx(c, sg::fill_ref(c, c.m(), field->f.data, value));
    }
    SG_API_CATCH(sg_field_fill)

    int sg_field_swap(sg_field_t a, sg_field_t b)
    try
    {
        if (!a || !b || a->mesh != b->mesh)
        {
            return fail(SG_ERR_ARG, "sg_field_swap: fields must live on the same mesh");
        }
        std::swap(a->f.data, b->f.data);
        a->f.ghosts_valid = false;
        b->f.ghosts_valid = false;
        return SG_OK;
    }
    SG_API_CATCH(sg_field_swap)

    int sg_adapt(sg_field_t u, double eps, double regularity, int* n_harten)
    try
    {
        return sg_adapt_ex(u, eps, regularity, 0, n_harten);
    }
    SG_API_CATCH(sg_adapt)

    int sg_adapt_ex(sg_field_t u, double eps, double regularity, int relative_detail, int* n_harten)
    try
    {
        if (!u)
        {
            return fail(SG_ERR_ARG, "sg_adapt: null field");
        }
        sg::Ctx& c = u->mesh->ctx;
        if (!u->f.spare && dalloc(c, &u->f.spare, static_cast<size_t>(c.capacity)))
        {
            return from_ctx(c, SG_ERR_CUDA);
        }
        return from_ctx(c, sg::adapt(c, u->f, eps, regularity, n_harten, relative_detail != 0));
    }
    SG_API_CATCH(sg_adapt_ex)

    int sg_harten(sg_field_t u, int ite, double eps, double regularity, int* converged)
    try
    {
        return sg_harten_ex(u, ite, eps, regularity, 0, converged);
    }
    SG_API_CATCH(sg_harten)

    int sg_adapt_fields(int n, const sg_field_t* fields, int n_other, const sg_field_t* others, double eps, double regularity,
                        int relative_detail, int* n_harten)
    try
    {
        if (n < 1 || !fields || n_other < 0 || (n_other > 0 && !others) || !fields[0])
        {
            return fail(SG_ERR_ARG, "sg_adapt_fields: need n >= 1 fields (and n_other >= 0 others)");
        }
        sg_mesh_s* mesh = fields[0]->mesh;
        sg::Ctx& c      = mesh->ctx;
        std::vector<sg::DeviceField*> fs, os;
        for (int k = 0; k < n + n_other; ++k)
        {
            sg_field_t f = k < n ? fields[k] : others[k - n];
            if (!f || f->mesh != mesh)
            {
                return fail(SG_ERR_ARG, "sg_adapt_fields: every field must live on the first field's mesh");
            }
            for (auto* g : fs)
            {
                if (g == &f->f)
                {
                    return fail(SG_ERR_ARG, "sg_adapt_fields: a field is listed twice");
                }
            }
            for (auto* g : os)
            {
                if (g == &f->f)
                {
                    return fail(SG_ERR_ARG, "sg_adapt_fields: a field is listed twice");
                }
            }
            if (!f->f.spare && dalloc(c, &f->f.spare, static_cast<size_t>(c.capacity)))
            {
                return from_ctx(c, SG_ERR_CUDA);
            }
            (k < n ? fs : os).push_back(&f->f);
        }
        if (n > c.detail_comps)
        {
            // one dense detail slab per adapted field; the contents are rebuilt by every pass
            cudaStreamSynchronize(c.stream);
            dfree(c.detail);
            if (dalloc(c, &c.detail, static_cast<size_t>(c.capacity) * static_cast<size_t>(n)))
            {
                c.detail_comps = 0;
                return from_ctx(c, SG_ERR_CUDA);
            }
            cudaMemsetAsync(c.detail, 0, static_cast<size_t>(c.capacity) * n * sizeof(double), c.stream);
            c.detail_comps = n;
            sg::clear_graphs(c); // they hold the old detail buffer
        }
        return from_ctx(c, sg::adapt_fields(c, fs, os, eps, regularity, relative_detail != 0, n_harten));
    }
    SG_API_CATCH(sg_adapt_fields)

    int sg_update_ghost_mr_fields(int n, const sg_field_t* fields)
    try
    {
        if (n < 0 || (n > 0 && !fields))
        {
            return fail(SG_ERR_ARG, "sg_update_ghost_mr_fields: null field list");
        }
        for (int k = 0; k < n; ++k)
        {
            if (int st = sg_update_ghost_mr(fields[k]))
            {
                return st;
            }
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_update_ghost_mr_fields)

    int sg_harten_ex(sg_field_t u, int ite, double eps, double regularity, int relative_detail, int* converged)
    try
    {
        if (!u)
        {
            return fail(SG_ERR_ARG, "sg_harten: null field");
        }
        sg::Ctx& c = u->mesh->ctx;
        if (!u->f.spare && dalloc(c, &u->f.spare, static_cast<size_t>(c.capacity)))
        {
            return from_ctx(c, SG_ERR_CUDA);
        }
        bool conv = false;
        int st    = sg::harten(c, u->f, ite, eps, regularity, &conv, relative_detail != 0);
        if (converged)
        {
            *converged = conv ? 1 : 0;
        }
        return from_ctx(c, st);
    }
    SG_API_CATCH(sg_harten_ex)

    int sg_update_ghost_mr(sg_field_t u)
    try
    {
        if (!u)
        {
            return fail(SG_ERR_ARG, "sg_update_ghost_mr: null field");
        }
        return from_ctx(u->mesh->ctx, sg::update_ghost_mr(u->mesh->ctx, u->f));
    }
    SG_API_CATCH(sg_update_ghost_mr)

    int sg_upwind(sg_field_t u, sg_field_t unp1, const double* a, double dt, int scheme)
    try
    {
        if (!u || !unp1 || !a || u->mesh != unp1->mesh || u == unp1)
        {
            return fail(SG_ERR_ARG, "sg_upwind: need two distinct fields on the same mesh");
        }
        if (scheme != SG_UPWIND_OP && scheme != SG_README && scheme != SG_CONVECTION)
        {
            return fail(SG_ERR_ARG, "sg_upwind: unknown scheme");
        }
        sg::Ctx& c = u->mesh->ctx;
        if (scheme == SG_README && c.g.dim != 2)
        {
            return fail(SG_ERR_ARG, "sg_upwind: the README scheme is two-dimensional");
        }
        if (scheme == SG_CONVECTION && c.g.periodic)
        {
            return fail(SG_ERR_ARG, "sg_upwind: the flux form is not available on a mesh with a periodic axis");
        }
        unp1->f.ghosts_valid = false;
        return from_ctx(c, sg::upwind(c, u->f, unp1->f, a, dt, scheme));
    }
    SG_API_CATCH(sg_upwind)

    int sg_step(sg_field_t u, sg_field_t unp1, double eps, double regularity, const double* a, double dt, int scheme, int* n_harten)
    try
    {
        if (!u || !unp1 || !a || u->mesh != unp1->mesh || u == unp1)
        {
            return fail(SG_ERR_ARG, "sg_step: need two distinct fields on the same mesh");
        }
        if (scheme != SG_UPWIND_OP && scheme != SG_README && scheme != SG_CONVECTION)
        {
            return fail(SG_ERR_ARG, "sg_step: unknown scheme");
        }
        sg::Ctx& c = u->mesh->ctx;
        if (scheme == SG_README && c.g.dim != 2)
        {
            return fail(SG_ERR_ARG, "sg_step: the README scheme is two-dimensional");
        }
        if (scheme == SG_CONVECTION && c.g.periodic)
        {
            return fail(SG_ERR_ARG, "sg_step: the flux form is not available on a mesh with a periodic axis");
        }
        if (!u->f.spare && dalloc(c, &u->f.spare, static_cast<size_t>(c.capacity)))
        {
            return from_ctx(c, SG_ERR_CUDA);
        }
        unp1->f.ghosts_valid = false;
        return from_ctx(c, sg::step(c, u->f, unp1->f, eps, regularity, a, dt, scheme, n_harten));
    }
    SG_API_CATCH(sg_step)

    int sg_detail_download(sg_field_t u, double* values, long long n)
    try
    {
        if (!u || !values)
        {
            return fail(SG_ERR_ARG, "sg_detail_download: null argument");
        }
        sg_mesh_s* h = u->mesh;
        sg::Ctx& c   = h->ctx;
        if (int st = sg::host_counts(c, c.m()))
        {
            return from_ctx(c, st);
        }
        if (n != c.m().nb_ref)
        {
            return fail(SG_ERR_ARG, "sg_detail_download: size differs from the reference mesh");
        }
        if (stage(h, n))
        {
            return from_ctx(c, SG_ERR_CUDA);
        }
        int st = sg::gather_compact(c, c.m(), c.detail, h->staging);
        if (st)
        {
            return from_ctx(c, st);
        }
        cudaMemcpyAsync(values, h->staging, static_cast<size_t>(n) * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
        if (cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            return from_ctx(c, sg::check(c, "detail download"));
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_detail_download)

    int sg_tag_download(sg_field_t u, unsigned char* values, long long n)
    try
    {
        if (!u || !values)
        {
            return fail(SG_ERR_ARG, "sg_tag_download: null argument");
        }
        sg::Ctx& c = u->mesh->ctx;
        if (int st = sg::host_counts(c, c.m()))
        {
            return from_ctx(c, st);
        }
        if (n != c.m().nb_ref)
        {
            return fail(SG_ERR_ARG, "sg_tag_download: size differs from the reference mesh");
        }
        HostMesh hm;
        if (int st = pull(c, c.m().ref, hm, true))
        {
            return from_ctx(c, st);
        }
        std::vector<uint8_t> dense(static_cast<size_t>(c.capacity));
        cudaMemcpyAsync(dense.data(), c.tag, dense.size(), cudaMemcpyDeviceToHost, c.stream);
        if (cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            return from_ctx(c, sg::check(c, "tag download"));
        }
        for (long long w = 0; w < c.g.total_words; ++w)
        {
            uint32_t v = hm.ref[w];
            while (v)
            {
                const int b = __builtin_ctz(v);
                v &= v - 1;
                values[host_ref_index(hm, w, b)] = dense[static_cast<size_t>(32 * w + b)];
            }
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_tag_download)
}
