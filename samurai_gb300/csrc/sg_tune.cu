// Launch-shape autotuner (no samurai counterpart).
//
// The level-serial chains of the step are latency-bound and the FP64 list
// kernels compete for the narrow FP64 pipe, so the best launch shapes depend
// on the device and on the size of the mesh: the threads per block of the
// FP64 list kernels, the grid limit of the one-warp-per-word launches, the
// level sizes up to which a chain (ghost update, tag finalisation, mesh
// construction) runs its levels in one block, whether the adaptation runs
// as one graph with conditional nodes or pass by pass, and whether the
// tag-finalisation chain takes two levels per launch.  sg_autotune times the time
// step of a given problem under candidate shapes (coordinate descent, each
// candidate from the same saved state, its graphs captured afresh), keeps the
// fastest on the mesh and caches it per device and level range; later meshes
// of the same device and levels start from the cached choice.  Environment
// variables (SG_BLOCK, SG_MAX_BLOCKS, SG_FUSE_WORDS, SG_FUSE_WORDS_FIELD,
// SG_FUSE_WORDS_MAX, SG_GRAPHED_ADAPT, SG_LEVEL_PAIRS) override
// both the defaults and the cache.  With
// SG_TUNE_FILE set, the cache is also read from and appended to that file.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "sg_handles.cuh"

namespace sg
{
    void set_fusion(Ctx& c, long long mesh_words, long long field_words, long long max_words);
    void clear_graphs(Ctx& c);

    namespace
    {
        struct LaunchShape
        {
            int block;
            long long max_blocks, fuse_mesh, fuse_field, fuse_max;
            int graphed;     // the adaptation as one graph with conditional nodes (1) or pass by pass (0)
            int level_pairs; // tag finalisation two levels per launch (1) or one (0)
        };

        using TuneKey = std::tuple<std::string, int, int, int>; // device name, dim, min_level, max_level

        std::mutex g_tune_mutex;
        std::map<TuneKey, LaunchShape> g_tune_cache;
        bool g_tune_file_read = false;

        std::string device_name(int dev)
        {
            cudaDeviceProp p{};
            if (cudaGetDeviceProperties(&p, dev) != cudaSuccess)
            {
                cudaGetLastError();
                return "device" + std::to_string(dev);
            }
            std::string n = p.name;
            std::replace(n.begin(), n.end(), ' ', '_');
            return n;
        }

        // SG_TUNE_FILE: lines "device dim min max block max_blocks fuse_mesh fuse_field fuse_max graphed level_pairs" (the last line of a
        // key wins); read once, under the cache mutex
        void read_tune_file()
        {
            if (g_tune_file_read)
            {
                return;
            }
            g_tune_file_read = true;
            const char* path = std::getenv("SG_TUNE_FILE");
            if (!path || !*path)
            {
                return;
            }
            FILE* f = std::fopen(path, "r");
            if (!f)
            {
                return;
            }
            char name[256];
            int dim, lo, hi, block, gr, lp;
            long long mb, fm, ff, fx;
            while (std::fscanf(f, "%255s %d %d %d %d %lld %lld %lld %lld %d %d", name, &dim, &lo, &hi, &block, &mb, &fm, &ff, &fx, &gr, &lp) == 11)
            {
                if (block >= 32 && block <= 1024 && block % 32 == 0 && mb > 0 && fm >= 0 && ff >= 0 && fx >= 0 && (gr == 0 || gr == 1)
                    && (lp == 0 || lp == 1))
                {
                    g_tune_cache[TuneKey{name, dim, lo, hi}] = LaunchShape{block, mb, fm, ff, fx, gr, lp};
                }
            }
            std::fclose(f);
        }

        void append_tune_file(const TuneKey& k, const LaunchShape& s)
        {
            const char* path = std::getenv("SG_TUNE_FILE");
            if (!path || !*path)
            {
                return;
            }
            if (FILE* f = std::fopen(path, "a"))
            {
                std::fprintf(f, "%s %d %d %d %d %lld %lld %lld %lld %d %d\n", std::get<0>(k).c_str(), std::get<1>(k), std::get<2>(k), std::get<3>(k),
                             s.block, s.max_blocks, s.fuse_mesh, s.fuse_field, s.fuse_max, s.graphed, s.level_pairs);
                std::fclose(f);
            }
        }

        TuneKey key_of(const Ctx& c)
        {
            return TuneKey{device_name(c.device), c.g.dim, c.cfg.min_level, c.cfg.max_level};
        }

        bool env_set(const char* name)
        {
            const char* v = std::getenv(name);
            return v && *v;
        }

        LaunchShape shape_of(const Ctx& c)
        {
            return LaunchShape{c.block, c.max_blocks, c.fuse_words_mesh, c.fuse_words_field, c.fuse_words_max, c.graphed_adapt ? 1 : 0, c.level_pairs ? 1 : 0};
        }

        // applies a shape to a mesh (its captured graphs were recorded with the old one and are dropped)
        void apply_shape(Ctx& c, const LaunchShape& s)
        {
            c.block         = s.block;
            c.max_blocks    = s.max_blocks;
            c.graphed_adapt = s.graphed != 0;
            c.level_pairs   = s.level_pairs != 0;
            set_fusion(c, s.fuse_mesh, s.fuse_field, s.fuse_max); // drops the captured graphs
        }
    } // namespace

    // the cached shape for this device and level range, where no environment variable sets the value
    void apply_tuned_launch(Ctx& c)
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        read_tune_file();
        const auto it = g_tune_cache.find(key_of(c));
        if (it == g_tune_cache.end())
        {
            return;
        }
        const LaunchShape& s = it->second;
        if (!env_set("SG_BLOCK"))
        {
            c.block = s.block;
        }
        if (!env_set("SG_MAX_BLOCKS"))
        {
            c.max_blocks = s.max_blocks;
        }
        if (!env_set("SG_FUSE_WORDS"))
        {
            c.fuse_words_mesh = s.fuse_mesh;
        }
        if (!env_set("SG_FUSE_WORDS_FIELD"))
        {
            c.fuse_words_field = s.fuse_field;
        }
        if (!env_set("SG_FUSE_WORDS_MAX"))
        {
            c.fuse_words_max = s.fuse_max;
        }
        if (!env_set("SG_GRAPHED_ADAPT"))
        {
            c.graphed_adapt = s.graphed != 0;
        }
        if (!env_set("SG_LEVEL_PAIRS"))
        {
            c.level_pairs = s.level_pairs != 0;
        }
    }
} // namespace sg

namespace
{
    int tfail(int code, const std::string& msg)
    {
        sg::set_last_error(msg.c_str(), nullptr);
        return code;
    }
}

extern "C"
{
    int sg_autotune(sg_field_t u, sg_field_t unp1, double eps, double regularity, const double* a, double dt, int scheme, int steps,
                    double* default_ms, double* tuned_ms)
    try
    {
        if (!u || !unp1 || !a || u->mesh != unp1->mesh || u == unp1 || steps < 1 || steps > 1000)
        {
            return tfail(SG_ERR_ARG, "sg_autotune: need two distinct fields on one mesh and 1 <= steps <= 1000");
        }
        sg_mesh_s* mesh = u->mesh;
        sg::Ctx& c      = mesh->ctx;
        // the state every candidate starts from: leaf cells and leaf values
        long long nc = 0, nr = 0;
        if (int st = sg_mesh_counts(mesh, &nc, &nr))
        {
            return st;
        }
        std::vector<int> lv(static_cast<size_t>(nc)), co(static_cast<size_t>(nc) * c.g.dim);
        std::vector<long long> idx(static_cast<size_t>(nc));
        std::vector<double> vals(static_cast<size_t>(nc));
        if (int st = sg_mesh_get_cells(mesh, lv.data(), co.data(), idx.data(), nc))
        {
            return st;
        }
        if (int st = sg_field_get_cells(u, vals.data(), nc))
        {
            return st;
        }
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        {
            cudaGetLastError();
            return tfail(SG_ERR_CUDA, "sg_autotune: cudaEventCreate failed");
        }
        auto restore = [&]() -> int
        {
            if (int st = sg_mesh_set_cells(mesh, nc, lv.data(), co.data()))
            {
                return st;
            }
            return sg_field_set_cells(u, vals.data(), nc);
        };
        // every timed step starts with a cold L2 (a 256 MiB write before it, not timed), as a step does that follows
        // other work
        const size_t flush_bytes = 256u << 20;
        void* flush              = nullptr;
        if (cudaMalloc(&flush, flush_bytes) != cudaSuccess)
        {
            cudaGetLastError();
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return tfail(SG_ERR_CUDA, "sg_autotune: no device memory for the L2 flush");
        }
        // ms per step of `steps` steps from the saved state (the best of two runs), after an untimed run that
        // captures the shape's graphs
        auto measure = [&](double* ms) -> int
        {
            float best = 1e30f;
            for (int rep = 0; rep < 3; ++rep)
            {
                if (int st = restore())
                {
                    return st;
                }
                const int n = rep == 0 ? std::max(steps, 8) : steps; // rep 0 captures the graphs of every buffer combination
                float total = 0.f;
                for (int k = 0; k < n; ++k)
                {
                    cudaMemsetAsync(flush, k & 0xFF, flush_bytes, c.stream);
                    cudaEventRecord(e0, c.stream);
                    int passes = 0;
                    if (int st = sg_step(u, unp1, eps, regularity, a, dt, scheme, &passes))
                    {
                        return st;
                    }
                    cudaEventRecord(e1, c.stream);
                    if (cudaEventSynchronize(e1) != cudaSuccess)
                    {
                        return tfail(SG_ERR_CUDA, "sg_autotune: CUDA error while timing");
                    }
                    float t = 0.f;
                    cudaEventElapsedTime(&t, e0, e1);
                    total += t;
                }
                if (rep > 0)
                {
                    best = std::min(best, total / static_cast<float>(n));
                }
            }
            *ms = best;
            return SG_OK;
        };
        const sg::LaunchShape start = sg::shape_of(c);
        double base = 0.;
        int st      = measure(&base);
        sg::LaunchShape best = start;
        double best_ms       = base;
        // coordinate descent over the launch parameters, each from the best shape so far
        const std::vector<long long> blocks = {128, 256, 512};
        const std::vector<long long> grids  = {152LL * 4, 152LL * 8, 152LL * 16};
        const std::vector<long long> fuses  = {0, 32, 128, 512};
        const std::vector<long long> flags  = {0, 1};
        for (int param = 0; param < 6 && !st; ++param)
        {
            const std::vector<long long>& cands = param <= 1 ? flags : (param == 2 ? blocks : (param == 3 ? grids : fuses));
            const sg::LaunchShape from          = best;
            for (long long v : cands)
            {
                sg::LaunchShape s = from;
                switch (param)
                {
                case 0: s.graphed = static_cast<int>(v); break;
                case 1: s.level_pairs = static_cast<int>(v); break;
                case 2: s.block = static_cast<int>(v); break;
                case 3: s.max_blocks = v; break;
                case 4: s.fuse_field = v; break;
                default: s.fuse_max = v; break;
                }
                if (s.graphed == from.graphed && s.level_pairs == from.level_pairs && s.block == from.block
                    && s.max_blocks == from.max_blocks && s.fuse_field == from.fuse_field && s.fuse_max == from.fuse_max)
                {
                    continue;
                }
                sg::apply_shape(c, s);
                double ms = 0.;
                if ((st = measure(&ms)))
                {
                    break;
                }
                if (ms < best_ms * 0.99) // a change must win by more than the timing noise
                {
                    best_ms = ms;
                    best    = s;
                }
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(flush);
        sg::apply_shape(c, st ? start : best);
        const int rs = restore();
        if (st)
        {
            return st;
        }
        if (rs)
        {
            return rs;
        }
        {
            std::lock_guard<std::mutex> lock(sg::g_tune_mutex);
            const sg::TuneKey k       = sg::key_of(c);
            sg::g_tune_cache[k]       = best;
            sg::append_tune_file(k, best);
        }
        if (default_ms)
        {
            *default_ms = base;
        }
        if (tuned_ms)
        {
            *tuned_ms = best_ms;
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_autotune)

    int sg_launch_shape(sg_mesh_t mesh, int* block, long long* max_blocks, long long* fuse_mesh_words, long long* fuse_field_words,
                        long long* fuse_max_words, int* graphed_adapt, int* level_pairs)
    try
    {
        if (!mesh)
        {
            return tfail(SG_ERR_ARG, "sg_launch_shape: null mesh");
        }
        const sg::Ctx& c = mesh->ctx;
        if (block)
        {
            *block = c.block;
        }
        if (max_blocks)
        {
            *max_blocks = c.max_blocks;
        }
        if (fuse_mesh_words)
        {
            *fuse_mesh_words = c.fuse_words_mesh;
        }
        if (fuse_field_words)
        {
            *fuse_field_words = c.fuse_words_field;
        }
        if (fuse_max_words)
        {
            *fuse_max_words = c.fuse_words_max;
        }
        if (graphed_adapt)
        {
            *graphed_adapt = c.graphed_adapt ? 1 : 0;
        }
        if (level_pairs)
        {
            *level_pairs = c.level_pairs ? 1 : 0;
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_launch_shape)
}
