// Host-side state of one GB300 MR mesh and its fields (one stream, one GPU).
#pragma once

#include <cstdio>
#include <functional>
#include <string>
#include <vector>

#include "sg_core.cuh"

namespace sg
{
    struct MeshCfg
    {
        int dim                = 2;
        int min_level          = 0;
        int max_level          = 0;
        int max_stencil_radius = 1; // mesh_config::max_stencil_radius (mesh_config.hpp:42-80)
        int prediction_radius  = 1; // config_t::prediction_stencil_radius
        int graduation_width   = 1;
        int ghost_width        = 1; // max(max_stencil_radius, prediction_radius)
    };

    // One mesh: the bitmaps of the MRMesh ids plus helper sets and the rank.
    struct DeviceMesh
    {
        uint32_t* cells = nullptr; // MRMeshId::cells
        uint32_t* cag   = nullptr; // MRMeshId::cells_and_ghosts
        uint32_t* proj  = nullptr; // MRMeshId::proj_cells
        uint32_t* uni   = nullptr; // MRMeshId::union_cells
        uint32_t* ref   = nullptr; // MRMeshId::reference (all_cells)
        uint32_t* hc    = nullptr; // cells[l+1].on(l): cells with a leaf child
        uint32_t* hc2   = nullptr; // cells[l+2].on(l)
        int* rank       = nullptr; // exclusive popcount prefix of ref
        int* wl_ref     = nullptr; // indices of the non-empty reference words, ascending
        int* wl_cells   = nullptr; // indices of the non-empty leaf-cell words, ascending
        // Counters written by scan_rank on the device (layout below) and
        // mirrored asynchronously into pinned host memory; kernels read the
        // device copy, so no launch waits for the host.
        long long* d_lo = nullptr;
        long long* h_lo = nullptr;
        bool host_valid = false; // h_lo reflects d_lo (after a synchronisation)
        long long nb_ref   = 0;  // host copies, valid when host_valid
        long long nb_cells = 0;
    };

    // counters of a mesh: [0] reference size, [1] non-empty reference words,
    // [2] leaf cells, [3] non-empty leaf words, then the word-list offsets:
    // the reference words of level l are wl_ref[lo[LO_REF+l] .. lo[LO_REF+l+1]),
    // the leaf words wl_cells[lo[LO_CELLS+l] .. lo[LO_CELLS+l+1]).
    constexpr int LO_REF   = 4;
    constexpr int LO_CELLS = LO_REF + MAXLEV + 1;
    constexpr int COUNTS   = LO_CELLS + MAXLEV + 1;

    // state of an adaptation run as one graph (device words, mirrored to pinned host at its end)
    enum AdaptSlot : int
    {
        A_GO     = 0,  // the next Harten pass runs (the previous one changed the mesh)
        A_PASSES = 1,  // Harten passes run
        A_TRANS  = 2,  // passes that changed the mesh
        A_LOOP   = 3,  // condition of the graduation loop
        A_ITER   = 4,  // iterations of the graduation loop
        A_PAR0   = 5,  // a time step's tail: an even number of transitions (the starting buffers are final)
        A_PAR1   = 6,  //   an odd number
        A_NEEDG  = 7,  //   the last pass changed the mesh: the ghosts need an update
        A_COUNT  = 8
    };

    // flags written by the adaptation kernels (device, mirrored to pinned host)
    enum FlagSlot : int
    {
        F_GRAD0 = 0,  // graduation pass 1 found cells to refine
        F_GRAD1 = 1,  // graduation pass 2 found cells to refine (more passes needed)
        F_DIFFER = 2, // new leaf cells differ from the current ones
        F_GRADX = 3,  // scratch for extra graduation passes
        F_COUNT = 8
    };

    // Named phase timers with samurai's scope names (timers.hpp:111-1036;
    // mr/adapt.hpp:151-387, update_ghost_mr.hpp:263, field/field_base.hpp:234).
    // Disabled by default; when enabled, CUDA events on the mesh stream
    // bracket each phase and the host sums the intervals on request.
    enum TimerId : int
    {
        T_ADAPT = 0,      // "mesh adaptation"
        T_GHOST,          // "ghost update"
        T_DETAIL,         // "detail computation"
        T_TAG,            // "tag cells"
        T_FINALIZE,       // "tag finalization"
        T_MESH_UPDATE,    // "mesh update" (tags -> cells, graduation, fixed-point test)
        T_GRADUATION,     // "make_graduation"
        T_CONSTRUCTION,   // "mesh construction"
        T_FIELDS_UPDATE,  // "fields update"
        T_UPWIND,         // "field expressions" (the upwind step)
        T_COUNT
    };

    // Kernel trace: while enabled, every launch records an event on the mesh
    // stream right after the kernel (inside captured graphs the events become
    // event-record nodes, replayed with the graph), so that the time between
    // consecutive events is one launch's share of the timeline: its run time
    // plus the gap before it.  Times are read once the stream is idle.
    struct KernelTrace
    {
        bool enabled = false;
        cudaEvent_t start = nullptr;
        std::vector<std::pair<const char*, cudaEvent_t>> marks; // launch order
        bool reused = false; // an event was recorded twice in the window (a graph replayed twice)
        struct Result
        {
            const char* name;
            long long launches;
            double ms;
        };
        std::vector<Result> results; // per kernel name, filled when the trace stops
    };

    struct Timers
    {
        bool enabled = false;
        std::vector<cudaEvent_t> pool;
        std::vector<std::pair<cudaEvent_t, cudaEvent_t>> open[T_COUNT];
        double ms[T_COUNT]    = {};
        long long calls[T_COUNT] = {};
        cudaEvent_t pending[T_COUNT] = {};
    };

    struct Ctx
    {
        Timers timers;
        KernelTrace trace;
        MeshCfg cfg;
        Geom g{};                // geometry: kernels take it by value as a __grid_constant__ parameter
        double* d_eps = nullptr; // per-level thresholds of the criteria (3 x MAXLEV)
        unsigned long long* d_absmax = nullptr; // bits of max |u| over the leaf cells (relative details)
        int detail_comps             = 1;       // dense detail slabs allocated (one per adapted field)
        bool rel_detail = false;                // the Harten pass in flight divides the details by max |u|
        bool refine_boundary = false;           // args::refine_boundary: keep the boundary cells of max_level
        double* h_eps = nullptr; // pinned staging of d_eps
        cudaStream_t stream = nullptr;
        int device          = -1; // the device current at creation: every buffer of the mesh lives there
        // streams that capture the bodies of conditional graph nodes (one per nesting depth)
        static constexpr int CAPTURE_DEPTH = 4;
        cudaStream_t cap_streams[CAPTURE_DEPTH] = {};
        int cap_depth = 0;
        bool level_pairs = true; // tag finalisation two levels per launch (k_maximum2)
        int* d_adapt  = nullptr; // device state of a graphed adaptation (AdaptSlot)
        int* h_adapt  = nullptr; // pinned mirror of d_adapt
        bool graphed_adapt = true; // the whole adaptation as one graph with conditional nodes
        uint32_t* rec_slots = nullptr; // when set, the adaptation graph copies the leaf bitmap of transition t into slot t (adjoint recording)
        DeviceMesh mesh[2];
        int cur = 0;
        // scratch bitmaps
        uint32_t* t0 = nullptr;
        uint32_t* t1 = nullptr;
        uint32_t* t2 = nullptr;
        uint32_t* t3 = nullptr;
        uint32_t* rf = nullptr; // refine flags of leaf cells
        uint32_t* cf = nullptr; // coarsen (and not keep) flags of leaf cells
        // adaptation fields (dense layout)
        double* detail = nullptr;
        uint8_t* tag   = nullptr;
        // scan scratch
        long long* block_sums = nullptr;
        long long n_scan_blocks = 0;
        // device/host flags and counters
        long long* d_counts = nullptr; // [0] = popcount total, [1..] misc
        long long* h_counts = nullptr; // pinned mirror
        int* d_flags        = nullptr;
        int* h_flags        = nullptr; // pinned mirror
        long long capacity  = 0;       // dense elements per field (32 * total_words)
        int* d_ite          = nullptr; // Harten pass index seen by the detail/criteria kernels
        int* h_ite          = nullptr; // pinned staging
        bool use_graphs     = true;    // replay captured launch sequences
        unsigned long long mesh_version = 1; // bumped at every change of the current mesh
        int fuse_top        = -1;      // levels 0..fuse_top are small enough for one-block mesh chains
        int fuse_top_field  = -1;      // the same for the FP64 field chains
        int fuse_top_max    = -1;      // the same for the tag-finalisation chain
        const int* guard    = nullptr; // device flag: word launches do nothing while it is 0
        long long max_blocks = 152LL * 8; // grid limit of the one-warp-per-word launches, in blocks of 8 warps (x4 for one thread per word)
        int block            = 256;       // threads per block of the FP64 list kernels
        long long fuse_words_mesh  = 0; // one-block chain limits (words per level) behind fuse_top, fuse_top_field, fuse_top_max
        long long fuse_words_field = 0;
        long long fuse_words_max   = 0;
        struct GraphEntry
        {
            unsigned long long key[4];
            cudaGraphExec_t exec;
            int kernels;
            std::vector<std::pair<const char*, cudaEvent_t>> marks; // trace events captured into the graph
        };
        std::vector<GraphEntry> graphs;
        int n_launches      = 0;       // kernel launches since the last reset (instrumentation)
        std::string err;

        DeviceMesh& m()
        {
            return mesh[cur];
        }

        DeviceMesh& spare()
        {
            return mesh[1 - cur];
        }
    };

    struct DeviceField
    {
        Ctx* ctx       = nullptr;
        double* data   = nullptr;
        double* spare  = nullptr; // second buffer for update_fields
        bool has_bc    = false;
        double bc_value = 0.;
        std::string name;
        // update_ghost_mr is idempotent: when neither the leaf values nor the
        // mesh changed since the last one, a new call would rewrite the same
        // ghost values, and is skipped
        bool ghosts_valid          = false;
        unsigned long long ghost_version = 0;
    };

    // kernels and drivers (sg_mesh.cu / sg_field.cu)
    int build_mesh(Ctx& c, DeviceMesh& m);           // from m.cells; asynchronous
    int scan_rank(Ctx& c, DeviceMesh& m);            // rank, word lists, counters; asynchronous
    int host_counts(Ctx& c, DeviceMesh& m);          // synchronises and refreshes nb_ref / nb_cells
    int update_ghost_mr(Ctx& c, DeviceField& f);     // update_ghost_mr(u)
    int adapt(Ctx& c, DeviceField& f, double eps, double regularity, int* n_harten, bool relative_detail = false);
    int upwind(Ctx& c, DeviceField& u, DeviceField& unp1, const double* a, double dt, int scheme);
    int upwind_on(Ctx& c, const DeviceMesh& m, const double* ud, double* unp1d, const double* a, double dt, int scheme, bool baked);
    int step(Ctx& c, DeviceField& u, DeviceField& unp1, double eps, double regularity, const double* a, double dt, int scheme, int* n_harten);
    int gather_compact(Ctx& c, const DeviceMesh& m, const double* dense, double* compact);
    cudaError_t launch_gather(Ctx& c, const DeviceMesh& m, const double* dense, double* compact); // no error text
    cudaError_t read_device_error(Ctx& c, int* v);                                                  // reads and clears
    int scatter_compact(Ctx& c, const DeviceMesh& m, const double* compact, double* dense);
    int fill_ref(Ctx& c, const DeviceMesh& m, double* dense, double value);
    int harten(Ctx& c, DeviceField& f, int ite, double eps, double regularity, bool* converged, bool relative_detail = false);
    int harten_begin(Ctx& c, DeviceField& f, int ite, double eps, double regularity, bool relative_detail = false); // no synchronisation
    // one step's linear operators on a frozen mesh (replay and adjoint)
    int ghost_value(Ctx& c, DeviceMesh& m, double* u, bool has_bc, double bcv);
    int ghost_reverse(Ctx& c, DeviceMesh& m, double* lam, int* overflow, bool has_bc); // lam := G^T lam
    int update_fields_value(Ctx& c, DeviceMesh& m, DeviceMesh& nm, const double* uo, double* un);
    int update_fields_reverse(Ctx& c, DeviceMesh& m, DeviceMesh& nm, double* lam_new, double* lam_old, int* overflow); // lam_old += T^T lam_new
    int harten_end(Ctx& c, DeviceField& f, bool* converged);
    // the same for the fields fs driving the criteria and the fields os carried along
    int harten_begin_fields(Ctx& c, const std::vector<DeviceField*>& fs, int ite, double eps, double regularity, bool relative_detail);
    int harten_end_fields(Ctx& c, const std::vector<DeviceField*>& fs, const std::vector<DeviceField*>& os, bool* converged);
    int adapt_fields(Ctx& c, const std::vector<DeviceField*>& fs, const std::vector<DeviceField*>& os, double eps, double regularity,
                     bool relative_detail, int* n_harten);
    int device_error(Ctx& c); // reads and clears the device error word (synchronises)

    void timer_start(Ctx& c, int id);
    void timer_stop(Ctx& c, int id);
    void timers_flush(Ctx& c); // synchronises and accumulates

    // bookkeeping after every kernel launch: the launch counter and, while the
    // kernel trace is on, the trace event of the launch
    void launched(Ctx& c, const char* name, int count = 1);
    void trace_mark(Ctx& c, const char* name); // a trace event (name null: the head of a launch sequence)
    void clear_graphs(Ctx& c); // drops the captured launch sequences (their trace events go back to the pool)
    void apply_tuned_launch(Ctx& c); // the autotuner's cached launch shape for the mesh's device and levels (sg_tune.cu)
    cudaEvent_t take_event(Ctx& c);
    void give_event(Ctx& c, cudaEvent_t e);

    struct ScopedTimer
    {
        Ctx& c;
        int id;

        ScopedTimer(Ctx& cc, int i)
            : c(cc)
            , id(i)
        {
            timer_start(c, id);
        }

        ~ScopedTimer()
        {
            timer_stop(c, id);
        }
    };

    // A level-serial chain (union, reference children, graduation, tag
    // finalisation, ghost passes) runs its levels of at most FUSE_WORDS words
    // in a single block that steps through them with __syncthreads(), instead
    // of one launch per level.
    // The integer word chains of the mesh construction stay in one block up
    // to 1K words per level (on the 2D max_level-12 step: 1.14 ms/step at 1K,
    // 1.16 at 4K, 1.25 at 16K, 1.20 without fusion).  The FP64 field chains
    // and the tag finalisation are not fused: their cells wait on memory, and
    // one block serialises that latency (measured slower than one launch per
    // level even at 1K-2K words), so their limit is 0.
    // device thresholds buffer: [eps | fine | coarse] x MAXLEV, then a velocity
    constexpr int EPS_VELOCITY = 3 * MAXLEV;

    constexpr long long FUSE_WORDS       = 1024;
    constexpr long long FUSE_WORDS_FIELD = 0;
    constexpr long long FUSE_WORDS_MAX   = 0;
    // In batched mode many meshes share the GPU and the launch rate, not one
    // mesh's latency, sets the pace: every chain runs its levels of at most
    // 10K words in one block (measured on 256 meshes of max_level 7..11:
    // 23.7 ms per batched step against 28.9 ms with the single-mesh limits
    // and 25.0 ms with every level in one block).
    constexpr long long BATCH_FUSE_WORDS = 10000;

    inline int fuse_top_of(const Geom& g, long long limit)
    {
        int t = -1;
        for (int l = 0; l < g.nlev; ++l)
        {
            if (g.lv[l].nwords <= limit)
            {
                t = l;
            }
        }
        return t;
    }

    // blocks of 256 threads (8 warps) for a warp-per-item loop over at most
    // max_items list entries: one wave of resident warps at most
    inline int blocks_for_items(long long max_items)
    {
        long long b = (max_items + 7) / 8;
        if (b < 1)
        {
            b = 1;
        }
        const long long cap = 152LL * 8;
        return static_cast<int>(b > cap ? cap : b);
    }

    // launch helpers
    inline int grid_for(long long n, int block = 256, long long cap = 152LL * 32)
    {
        long long b = (n + block - 1) / block;
        if (b < 1)
        {
            b = 1;
        }
        if (b > cap)
        {
            b = cap;
        }
        return static_cast<int>(b);
    }

    inline int check(Ctx& c, const char* where)
    {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
        {
            c.err = std::string(where) + ": " + cudaGetErrorString(e);
            return SG_ERR_CUDA;
        }
        return SG_OK;
    }
} // namespace sg
