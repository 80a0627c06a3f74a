// Discrete adjoint of the MR advection time loop (sg_adjoint_*).
//
// samurai has no adjoint; this extends its time loop
// (demos/FiniteVolume/advection_2d.cpp:124-156: MRadaptation, update_ghost_mr,
// upwind, swap) with reverse-mode derivatives.  The adaptation decisions
// (thresholds on details, graduation) are piecewise constant in the field,
// so the derivative is that of the loop on its recorded mesh sequence:
//
//   record    the forward with adaptation; keeps every mesh the loop visits
//             (leaf bitmaps) and the dense field every K steps (checkpoints);
//   replay    the same steps on the recorded meshes from any u0 and velocity:
//             the frozen-mesh map whose derivative the adjoint computes;
//   backward  segment by segment from the last: recompute the segment from its
//             checkpoint on the recorded meshes, keeping the ghosted field of
//             every step; then walk the segment backwards applying transposes:
//             the upwind step (and its velocity derivative) by dedicated
//             kernels, the ghost update and update_fields by their own kernels
//             on the transposing accessor (sg_access.cuh), launched in reverse
//             order (a captured ghost update replayed backwards), rebuilding
//             the recorded meshes on the way back.
//
// Every operator of a step is linear in the field on a frozen mesh; the
// Dirichlet value only adds a constant.  The upwind step is bilinear in (a, u);
// d|a|/da = sign(a), 0 at a = 0.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/samurai_gpu.h"
#include "sg_access.cuh"
#include "sg_ctx.cuh"
#include "sg_handles.cuh"

namespace sg
{
    int ensure_spare(Ctx& c, DeviceField& f);
    bool step_graph_applies(const Ctx& c);

    namespace
    {
        constexpr int ABLOCK = 256;

        __device__ __forceinline__ long long gtid()
        {
            return blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
        }
        __device__ __forceinline__ long long gstride()
        {
            return static_cast<long long>(gridDim.x) * blockDim.x;
        }

        __device__ __forceinline__ double pow2d(int l)
        {
            return __longlong_as_double(static_cast<long long>(1023 + l) << 52);
        }

        struct UpwindAdj
        {
            double ha[3], hb[3]; // .5 a_d and .5 |a_d|
            double sgn[3];       // sign(a_d)
            double dt;
            int scheme;
        };

        // the leaf cell of level l at (x, y, z), if any
        template <int DIM>
        __device__ __forceinline__ bool leaf_at(const Geom& g, const uint32_t* cells, int l, int x, int y, int z, long long* e)
        {
            const Pos p = pos_of(g, l, x, y, z);
            if (p.w < 0 || !((cells[p.w] >> p.b) & 1u))
            {
                return false;
            }
            *e = elem(p);
            return true;
        }

        // mu = U^T lam for unp1 = u - dt * upwind(a, u) on the leaf cells of
        // one mesh (the forward is k_upwind); gather form, one thread per
        // dense element, deterministic.
        // Only the reference cells of the mesh are visited (the words of its reference list, a thread per bit):
        // every value the upwind step reads is a reference cell (a leaf or a same-level neighbour of one), so mu
        // is complete there; the transposes that follow read no other element.
        template <int DIM>
        __global__ void k_upwind_adjoint(const __grid_constant__ Geom gp, const int* __restrict__ wl_ref, const long long* __restrict__ lo,
                                         const uint32_t* __restrict__ ref, const uint32_t* __restrict__ cells, const double* __restrict__ lam,
                                         double* __restrict__ mu, UpwindAdj p)
        {
            const Geom& g       = gp;
            const long long b0  = lo[LO_REF];
            const long long tot = 32 * (lo[LO_REF + g.nlev] - b0);
            for (long long t = gtid(); t < tot; t += gstride())
            {
                const long long w = wl_ref[b0 + (t >> 5)];
                const int b       = static_cast<int>(t & 31);
                if (!((ref[w] >> b) & 1u))
                {
                    continue;
                }
                const long long k = 32 * w + b;
                const int l       = level_of(g, w);
                const Cell c      = cell_of(g, l, w, b);
                const double s    = p.dt * pow2d(l);
                double acc        = 0.;
                long long e;
                if ((cells[w] >> b) & 1u)
                {
                    double self = 0.;
                    for (int d = 0; d < DIM; ++d)
                    {
                        self += p.scheme == 1 ? 1. : 2. * p.hb[d];
                    }
                    acc += lam[k] * (1. - s * self);
                }
                for (int d = 0; d < DIM; ++d)
                {
                    const int dx = d == 0, dy = d == 1, dz = d == 2;
                    // cell c - e_d sees k as its right neighbour
                    if (p.scheme == 0 && leaf_at<DIM>(g, cells, l, c.x - dx, c.y - dy, c.z - dz, &e))
                    {
                        acc += lam[e] * (-s * (p.ha[d] - p.hb[d]));
                    }
                    // cell c + e_d sees k as its left neighbour
                    if (leaf_at<DIM>(g, cells, l, c.x + dx, c.y + dy, c.z + dz, &e))
                    {
                        acc += lam[e] * (p.scheme == 1 ? s : s * (p.ha[d] + p.hb[d]));
                    }
                }
                mu[k] = acc;
            }
        }

        // per-block partial sums of lam . dU/da_d u for the leaf cells (the words of the leaf list, a thread per bit)
        template <int DIM>
        __global__ void k_upwind_da(const __grid_constant__ Geom gp, const int* __restrict__ wl_cells, const long long* __restrict__ lo,
                                    const uint32_t* __restrict__ cells, const double* __restrict__ lam, const double* __restrict__ u, UpwindAdj p,
                                    double* partial)
        {
            const Geom& g       = gp;
            const long long b0  = lo[LO_CELLS];
            const long long tot = 32 * (lo[LO_CELLS + g.nlev] - b0);
            double acc[3]       = {0., 0., 0.};
            for (long long t = gtid(); t < tot; t += gstride())
            {
                const long long w = wl_cells[b0 + (t >> 5)];
                const int b       = static_cast<int>(t & 31);
                const long long k = 32 * w + b;
                if (!((cells[w] >> b) & 1u) || lam[k] == 0.)
                {
                    continue;
                }
                const int l        = level_of(g, w);
                const LevelGeom& L = g.lv[l];
                const double s     = p.dt * pow2d(l);
                const long long st[3] = {1, 32LL * L.W, 32LL * L.W * L.R};
                const double uc       = u[k];
                for (int d = 0; d < DIM; ++d)
                {
                    const double ur = u[k + st[d]], ul = u[k - st[d]];
                    // dF(uL,uR)/da = .5 (uL + uR) + .5 sign(a) (uL - uR)
                    const double dr = .5 * (uc + ur) + .5 * p.sgn[d] * (uc - ur);
                    const double dl = .5 * (ul + uc) + .5 * p.sgn[d] * (ul - uc);
                    acc[d] += lam[k] * (-s * (dr - dl));
                }
            }
            __shared__ double red[3][ABLOCK];
            for (int d = 0; d < 3; ++d)
            {
                red[d][threadIdx.x] = acc[d];
            }
            __syncthreads();
            for (int h = ABLOCK / 2; h > 0; h >>= 1)
            {
                if (static_cast<int>(threadIdx.x) < h)
                {
                    for (int d = 0; d < 3; ++d)
                    {
                        red[d][threadIdx.x] += red[d][threadIdx.x + h];
                    }
                }
                __syncthreads();
            }
            if (threadIdx.x == 0)
            {
                for (int d = 0; d < 3; ++d)
                {
                    partial[3 * blockIdx.x + d] = red[d][0];
                }
            }
        }

        // ga[d] += sum of the partials: thread t of one ABLOCK-thread block sums partials t, t + ABLOCK, ... in that
        // order, then a fixed tree adds the threads' sums (deterministic: the order depends on nb only)
        __global__ void k_sum_partials(const double* partial, int nb, double* ga)
        {
            __shared__ double red[3][ABLOCK];
            double acc[3] = {0., 0., 0.};
            for (int k = static_cast<int>(threadIdx.x); k < nb; k += ABLOCK)
            {
                for (int d = 0; d < 3; ++d)
                {
                    acc[d] += partial[3 * k + d];
                }
            }
            for (int d = 0; d < 3; ++d)
            {
                red[d][threadIdx.x] = acc[d];
            }
            __syncthreads();
            for (int h = ABLOCK / 2; h > 0; h >>= 1)
            {
                if (static_cast<int>(threadIdx.x) < h)
                {
                    for (int d = 0; d < 3; ++d)
                    {
                        red[d][threadIdx.x] += red[d][threadIdx.x + h];
                    }
                }
                __syncthreads();
            }
            if (threadIdx.x < 3)
            {
                ga[threadIdx.x] += red[threadIdx.x][0];
            }
        }

        __global__ void k_leaf_scatter(const long long* __restrict__ el, const double* __restrict__ v, long long n, double* dense)
        {
            for (long long i = gtid(); i < n; i += gstride())
            {
                dense[el[i]] = v[i];
            }
        }

        __global__ void k_leaf_gather(const long long* __restrict__ el, const double* __restrict__ dense, long long n, double* v)
        {
            for (long long i = gtid(); i < n; i += gstride())
            {
                v[i] = dense[el[i]];
            }
        }

        int grid_of(long long n)
        {
            long long b = (n + ABLOCK - 1) / ABLOCK;
            b           = std::max(1LL, std::min(b, 152LL * 16));
            return static_cast<int>(b);
        }
    } // namespace
} // namespace sg

struct sg_adjoint_s
{
    sg_mesh_t mesh  = nullptr; // private copy of the initial mesh, then the loop's meshes
    sg_field_t u    = nullptr;
    sg_field_t unp1 = nullptr;
    int K           = 16; // checkpoint interval

    // recorded loop
    struct Step
    {
        int mesh0;   // index in bits of the mesh at the start of the step
        int n_trans; // meshes bits[mesh0+1 .. mesh0+n_trans] visited by the adaptation
    };
    std::vector<uint32_t*> bits;       // leaf bitmaps, device
    std::vector<uint32_t*> spare_bits; // bitmaps of earlier recordings, reused before allocating
    uint32_t* rec_slots = nullptr;     // where the step graph leaves the meshes of a step's transitions
    std::vector<Step> steps;
    double a[3] = {0., 0., 0.};
    double dt = 0., eps = 0., reg = 0.;
    int scheme = 0;
    bool have_forward = false;
    std::vector<double*> ckpt; // dense field at the start of steps 0, K, 2K, ...

    // leaf cells of the initial and the final mesh (for_each_cell order)
    std::vector<int> lev0, co0, levT, coT;
    long long* d_el0 = nullptr;
    long long* d_elT = nullptr;
    long long n0 = 0, nT = 0, cap0 = 0, capT = 0;
    double* d_uT     = nullptr; // final leaf values of the last forward
    long long uT_cap = 0;

    // adjoint buffers
    int* d_overflow = nullptr; // set when a linear form of the transposed operators overflowed
    double* lam[2]  = {nullptr, nullptr};
    std::vector<double*> ug; // ghosted field of each step of a segment
    double* d_partial = nullptr;
    double* d_ga      = nullptr;
    double* d_vals    = nullptr; // leaf-value staging
    long long vals_cap = 0;
    char err[512]      = "";
};

namespace
{
    using sg::Ctx;

    int afail(int code, const char* msg, const char* detail = nullptr)
    {
        sg::set_last_error(msg, detail);
        return code;
    }

    Ctx& ctx_of(sg_adjoint_t adj)
    {
        return adj->mesh->ctx;
    }

    int cuda_ok(Ctx& c, const char* what)
    {
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
        {
            c.err = std::string(what) + ": " + cudaGetErrorString(e);
            return SG_ERR_CUDA;
        }
        return SG_OK;
    }

    template <class T>
    int dmalloc(T** p, size_t n)
    {
        if (cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess)
        {
            cudaGetLastError();
            *p = nullptr;
            return SG_ERR_CUDA;
        }
        return SG_OK;
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

    size_t bitmap_bytes(Ctx& c)
    {
        return static_cast<size_t>(c.g.total_words) * sizeof(uint32_t);
    }
    size_t dense_bytes(Ctx& c)
    {
        return static_cast<size_t>(c.capacity) * sizeof(double);
    }

    // the current mesh becomes the recorded mesh k
    int load_mesh(sg_adjoint_t adj, int k)
    {
        Ctx& c = ctx_of(adj);
        cudaMemcpyAsync(c.m().cells, adj->bits[static_cast<size_t>(k)], bitmap_bytes(c), cudaMemcpyDeviceToDevice, c.stream);
        int st = sg::build_mesh(c, c.m());
        c.m().host_valid = false;
        ++c.mesh_version;
        adj->u->f.ghosts_valid    = false;
        adj->unp1->f.ghosts_valid = false;
        return st;
    }

    // a bitmap for the mesh sequence: one of an earlier recording's, or a new allocation
    int take_bits(sg_adjoint_t adj, uint32_t** out)
    {
        Ctx& c = ctx_of(adj);
        if (!adj->spare_bits.empty())
        {
            *out = adj->spare_bits.back();
            adj->spare_bits.pop_back();
            return SG_OK;
        }
        if (dmalloc(out, static_cast<size_t>(c.g.total_words)))
        {
            c.err = "adjoint: out of device memory for the mesh sequence";
            return SG_ERR_CUDA;
        }
        return SG_OK;
    }

    int push_bits_from(sg_adjoint_t adj, const uint32_t* src)
    {
        Ctx& c      = ctx_of(adj);
        uint32_t* b = nullptr;
        if (int st = take_bits(adj, &b))
        {
            return st;
        }
        cudaMemcpyAsync(b, src, bitmap_bytes(c), cudaMemcpyDeviceToDevice, c.stream);
        adj->bits.push_back(b);
        return SG_OK;
    }

    int push_current_bits(sg_adjoint_t adj)
    {
        return push_bits_from(adj, ctx_of(adj).m().cells);
    }

    // leaf cells of the current mesh: levels, coordinates and dense elements
    int current_leaves(sg_adjoint_t adj, std::vector<int>& lev, std::vector<int>& co, long long** d_el, long long* n, long long* cap)
    {
        Ctx& c = ctx_of(adj);
        if (int st = sg::host_counts(c, c.m()))
        {
            return st;
        }
        const long long nc = c.m().nb_cells;
        const int dim      = c.g.dim;
        lev.assign(static_cast<size_t>(nc), 0);
        co.assign(static_cast<size_t>(nc * dim), 0);
        if (int st = sg_mesh_get_cells(adj->mesh, lev.data(), co.data(), nullptr, nc))
        {
            return st;
        }
        std::vector<long long> el(static_cast<size_t>(nc));
        for (long long i = 0; i < nc; ++i)
        {
            const int* x = &co[static_cast<size_t>(i * dim)];
            const sg::Pos p = sg::pos_of(c.g, lev[static_cast<size_t>(i)], x[0], x[1], dim == 3 ? x[2] : 0);
            el[static_cast<size_t>(i)] = sg::elem(p);
        }
        if (nc > *cap)
        {
            dfree(*d_el);
            if (dmalloc(d_el, static_cast<size_t>(nc)))
            {
                c.err = "adjoint: out of device memory";
                return SG_ERR_CUDA;
            }
            *cap = nc;
        }
        cudaMemcpyAsync(*d_el, el.data(), static_cast<size_t>(nc) * sizeof(long long), cudaMemcpyHostToDevice, c.stream);
        if (cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            return sg::check(c, "adjoint leaves");
        }
        *n = nc;
        return SG_OK;
    }

    int stage_vals(sg_adjoint_t adj, long long n)
    {
        if (n > adj->vals_cap)
        {
            dfree(adj->d_vals);
            if (dmalloc(&adj->d_vals, static_cast<size_t>(n)))
            {
                ctx_of(adj).err = "adjoint: out of device memory";
                return SG_ERR_CUDA;
            }
            adj->vals_cap = n;
        }
        return SG_OK;
    }

    // dense field of the initial mesh from leaf values (host), other entries 0
    int set_initial_field(sg_adjoint_t adj, const double* u0, double* dense)
    {
        Ctx& c = ctx_of(adj);
        if (int st = stage_vals(adj, adj->n0))
        {
            return st;
        }
        cudaMemsetAsync(dense, 0, dense_bytes(c), c.stream);
        // u0: host memory or device memory of the mesh's GPU (unified addressing tells them apart)
        cudaMemcpyAsync(adj->d_vals, u0, static_cast<size_t>(adj->n0) * sizeof(double), cudaMemcpyDefault, c.stream);
        sg::k_leaf_scatter<<<sg::grid_of(adj->n0), sg::ABLOCK, 0, c.stream>>>(adj->d_el0, adj->d_vals, adj->n0, dense);
        return cuda_ok(c, "adjoint initial field");
    }

    int ensure_ckpt(sg_adjoint_t adj, size_t k)
    {
        Ctx& c = ctx_of(adj);
        while (adj->ckpt.size() <= k)
        {
            double* p = nullptr;
            if (dmalloc(&p, static_cast<size_t>(c.capacity)))
            {
                c.err = "adjoint: out of device memory for checkpoints";
                return SG_ERR_CUDA;
            }
            adj->ckpt.push_back(p);
        }
        return SG_OK;
    }

    void free_recording(sg_adjoint_t adj)
    {
        // the bitmaps go back to the pool of the next recording (no allocation or free per transition)
        for (size_t k = 1; k < adj->bits.size(); ++k)
        {
            adj->spare_bits.push_back(adj->bits[k]);
        }
        if (!adj->bits.empty())
        {
            adj->bits.resize(1);
        }
        adj->steps.clear();
        adj->have_forward = false;
    }

    // the recorded steps [s, e) on their meshes, value mode, from the field
    // already in u (on the mesh of step s, loaded by the caller); with keep_ug
    // the ghosted field of step n is kept in ug[n-s] (the velocity derivative
    // of its upwind step reads it)
    int replay_range(sg_adjoint_t adj, int s, int e, bool keep_ug, bool store_ckpt)
    {
        Ctx& c               = ctx_of(adj);
        sg::DeviceField& u   = adj->u->f;
        sg::DeviceField& up1 = adj->unp1->f;
        int st;
        for (int n = s; n < e; ++n)
        {
            const auto& S = adj->steps[static_cast<size_t>(n)];
            if (store_ckpt && n % adj->K == 0)
            {
                if ((st = ensure_ckpt(adj, static_cast<size_t>(n / adj->K))))
                {
                    return st;
                }
                cudaMemcpyAsync(adj->ckpt[static_cast<size_t>(n / adj->K)], u.data, dense_bytes(c), cudaMemcpyDeviceToDevice, c.stream);
            }
            for (int t = 1; t <= S.n_trans; ++t)
            {
                if ((st = sg::ghost_value(c, c.m(), u.data, u.has_bc, u.bc_value)))
                {
                    return st;
                }
                sg::DeviceMesh& nm = c.spare();
                cudaMemcpyAsync(nm.cells, adj->bits[static_cast<size_t>(S.mesh0 + t)], bitmap_bytes(c), cudaMemcpyDeviceToDevice, c.stream);
                if ((st = sg::build_mesh(c, nm)) || (st = sg::update_fields_value(c, c.m(), nm, u.data, u.spare)))
                {
                    return st;
                }
                nm.host_valid = false;
                std::swap(u.data, u.spare);
                c.cur = 1 - c.cur;
                ++c.mesh_version;
            }
            if ((st = sg::ghost_value(c, c.m(), u.data, u.has_bc, u.bc_value)))
            {
                return st;
            }
            if (keep_ug)
            {
                cudaMemcpyAsync(adj->ug[static_cast<size_t>(n - s)], u.data, dense_bytes(c), cudaMemcpyDeviceToDevice, c.stream);
            }
            u.ghosts_valid = false;
            if ((st = sg::upwind(c, u, up1, adj->a, adj->dt, adj->scheme)))
            {
                return st;
            }
            std::swap(u.data, up1.data);
            up1.ghosts_valid = false;
        }
        return cuda_ok(c, "adjoint replay");
    }

    // leaves of the final mesh and their values (kept for sg_adjoint_final)
    int final_leaves(sg_adjoint_t adj)
    {
        Ctx& c = ctx_of(adj);
        if (int st = current_leaves(adj, adj->levT, adj->coT, &adj->d_elT, &adj->nT, &adj->capT))
        {
            return st;
        }
        if (adj->nT > adj->uT_cap)
        {
            dfree(adj->d_uT);
            if (dmalloc(&adj->d_uT, static_cast<size_t>(adj->nT)))
            {
                c.err = "adjoint: out of device memory";
                return SG_ERR_CUDA;
            }
            adj->uT_cap = adj->nT;
        }
        sg::k_leaf_gather<<<sg::grid_of(adj->nT), sg::ABLOCK, 0, c.stream>>>(adj->d_elT, adj->u->f.data, adj->nT, adj->d_uT);
        return cuda_ok(c, "adjoint final field");
    }

    sg::UpwindAdj upwind_adj(sg_adjoint_t adj)
    {
        sg::UpwindAdj p{};
        for (int d = 0; d < 3; ++d)
        {
            p.ha[d]  = .5 * adj->a[d];
            p.hb[d]  = .5 * std::fabs(adj->a[d]);
            p.sgn[d] = adj->a[d] > 0. ? 1. : (adj->a[d] < 0. ? -1. : 0.);
        }
        p.dt     = adj->dt;
        p.scheme = adj->scheme;
        return p;
    }

    // reverse pass over the steps [s, e) of one segment, replayed just before (the current mesh is the one the
    // segment ends on, ug holds the ghosted field of each step); lam[0] holds the adjoint of the field after the
    // segment and ends as the adjoint of the field at its start
    int reverse_segment(sg_adjoint_t adj, int s, int e)
    {
        Ctx& c                 = ctx_of(adj);
        const sg::UpwindAdj p  = upwind_adj(adj);
        const int nb_da        = sg::grid_of(32 * c.g.total_words); // grid-stride loops over the lists: a fixed grid for every mesh
        const sg::DeviceField& u = adj->u->f;
        int st;
        for (int n = e - 1; n >= s; --n)
        {
            const auto& S         = adj->steps[static_cast<size_t>(n)];
            const sg::DeviceMesh& m = c.m(); // the step's last mesh (its leaves are bits[mesh0 + n_trans])
            const uint32_t* cells = m.cells;
            const double* ugn     = adj->ug[static_cast<size_t>(n - s)];
            // the upwind step u <- u - dt upwind(a, u) and its velocity derivative
            if (p.scheme == 0)
            {
                if (c.g.dim == 2)
                {
                    sg::k_upwind_da<2><<<nb_da, sg::ABLOCK, 0, c.stream>>>(c.g, m.wl_cells, m.d_lo, cells, adj->lam[0], ugn, p, adj->d_partial);
                }
                else
                {
                    sg::k_upwind_da<3><<<nb_da, sg::ABLOCK, 0, c.stream>>>(c.g, m.wl_cells, m.d_lo, cells, adj->lam[0], ugn, p, adj->d_partial);
                }
                sg::k_sum_partials<<<1, sg::ABLOCK, 0, c.stream>>>(adj->d_partial, nb_da, adj->d_ga);
            }
            if (c.g.dim == 2)
            {
                sg::k_upwind_adjoint<2><<<nb_da, sg::ABLOCK, 0, c.stream>>>(c.g, m.wl_ref, m.d_lo, m.ref, cells, adj->lam[0], adj->lam[1], p);
            }
            else
            {
                sg::k_upwind_adjoint<3><<<nb_da, sg::ABLOCK, 0, c.stream>>>(c.g, m.wl_ref, m.d_lo, m.ref, cells, adj->lam[0], adj->lam[1], p);
            }
            std::swap(adj->lam[0], adj->lam[1]);
            // the ghost update before it, on the step's last mesh
            if ((st = sg::ghost_reverse(c, c.m(), adj->lam[0], adj->d_overflow, u.has_bc)))
            {
                return st;
            }
            // the adaptation's transitions, last first: update_fields from mesh t-1 to mesh t, then the ghost
            // update that preceded it on mesh t-1
            for (int t = S.n_trans; t >= 1; --t)
            {
                sg::DeviceMesh& om = c.spare();
                cudaMemcpyAsync(om.cells, adj->bits[static_cast<size_t>(S.mesh0 + t - 1)], bitmap_bytes(c), cudaMemcpyDeviceToDevice, c.stream);
                if ((st = sg::build_mesh(c, om)))
                {
                    return st;
                }
                om.host_valid = false;
                cudaMemsetAsync(adj->lam[1], 0, dense_bytes(c), c.stream);
                if ((st = sg::update_fields_reverse(c, om, c.m(), adj->lam[0], adj->lam[1], adj->d_overflow)))
                {
                    return st;
                }
                std::swap(adj->lam[0], adj->lam[1]);
                c.cur = 1 - c.cur;
                ++c.mesh_version;
                if ((st = sg::ghost_reverse(c, c.m(), adj->lam[0], adj->d_overflow, u.has_bc)))
                {
                    return st;
                }
            }
        }
        return cuda_ok(c, "adjoint reverse");
    }
} // namespace

extern "C"
{
    int sg_adjoint_create(sg_field_t u, int checkpoint_every, sg_adjoint_t* out)
    try
    {
        if (!u || !out || checkpoint_every < 1)
        {
            return afail(SG_ERR_ARG, "sg_adjoint_create: need a field, checkpoint_every >= 1 and an output handle");
        }
        *out         = nullptr;
        sg::Ctx& uc  = u->mesh->ctx;
        const auto& cfg = uc.cfg;
        if (uc.g.periodic)
        {
            return afail(SG_ERR_ARG, "sg_adjoint_create: the adjoint is not available on a mesh with a periodic axis");
        }
        if (cfg.ghost_width != 1)
        {
            return afail(SG_ERR_ARG, "sg_adjoint_create: the adjoint covers a ghost width of 1 (max_stencil_radius 1)");
        }
        auto* adj    = new (std::nothrow) sg_adjoint_s();
        if (!adj)
        {
            return afail(SG_ERR_CAPACITY, "sg_adjoint_create: out of host memory");
        }
        adj->K = checkpoint_every;
        int st = sg_mesh_create(cfg.dim, cfg.min_level, cfg.max_level, cfg.max_stencil_radius, cfg.prediction_radius, cfg.graduation_width, &adj->mesh);
        if (st)
        {
            delete adj;
            return st;
        }
        // the initial mesh: u's current leaf cells
        long long nc = 0, nref = 0;
        if ((st = sg_mesh_counts(u->mesh, &nc, &nref)))
        {
            sg_adjoint_destroy(adj);
            return st;
        }
        std::vector<int> lev(static_cast<size_t>(nc)), co(static_cast<size_t>(nc * cfg.dim));
        if ((st = sg_mesh_get_cells(u->mesh, lev.data(), co.data(), nullptr, nc)) || (st = sg_mesh_set_cells(adj->mesh, nc, lev.data(), co.data()))
            || (st = sg_field_create(adj->mesh, "u", &adj->u)) || (st = sg_field_create(adj->mesh, "unp1", &adj->unp1)))
        {
            sg_adjoint_destroy(adj);
            return st;
        }
        if (u->f.has_bc && (st = sg_field_set_dirichlet(adj->u, u->f.bc_value)))
        {
            sg_adjoint_destroy(adj);
            return st;
        }
        Ctx& c = ctx_of(adj);
        if (c.capacity >= (1LL << 31))
        {
            sg_adjoint_destroy(adj);
            return afail(SG_ERR_CAPACITY, "sg_adjoint_create: the transposed operators index elements with 32 bits; this mesh has more");
        }
        if (sg::ensure_spare(c, adj->u->f) || push_current_bits(adj)
            || current_leaves(adj, adj->lev0, adj->co0, &adj->d_el0, &adj->n0, &adj->cap0) != SG_OK)
        {
            const int code = SG_ERR_CUDA;
            sg::set_last_error(c.err.c_str(), nullptr);
            sg_adjoint_destroy(adj);
            return code;
        }
        if (dmalloc(&adj->d_overflow, 1) || dmalloc(&adj->lam[0], static_cast<size_t>(c.capacity))
            || dmalloc(&adj->lam[1], static_cast<size_t>(c.capacity)) || dmalloc(&adj->d_partial, static_cast<size_t>(3 * 152 * 16))
            || dmalloc(&adj->d_ga, 3))
        {
            sg_adjoint_destroy(adj);
            return afail(SG_ERR_CUDA, "sg_adjoint_create: out of device memory");
        }
        *out = adj;
        return SG_OK;
    }
    SG_API_CATCH(sg_adjoint_create)

    int sg_adjoint_destroy(sg_adjoint_t adj)
    try
    {
        if (!adj)
        {
            return SG_OK;
        }
        if (adj->mesh)
        {
            cudaStreamSynchronize(adj->mesh->ctx.stream);
        }
        for (auto*& b : adj->bits)
        {
            dfree(b);
        }
        for (auto*& b : adj->spare_bits)
        {
            dfree(b);
        }
        dfree(adj->rec_slots);
        for (auto*& p : adj->ckpt)
        {
            dfree(p);
        }
        for (auto*& p : adj->ug)
        {
            dfree(p);
        }
        dfree(adj->d_el0);
        dfree(adj->d_elT);
        dfree(adj->d_uT);
        dfree(adj->d_overflow);
        dfree(adj->lam[0]);
        dfree(adj->lam[1]);
        dfree(adj->d_partial);
        dfree(adj->d_ga);
        dfree(adj->d_vals);
        if (adj->u)
        {
            sg_field_destroy(adj->u);
        }
        if (adj->unp1)
        {
            sg_field_destroy(adj->unp1);
        }
        if (adj->mesh)
        {
            sg_mesh_destroy(adj->mesh);
        }
        delete adj;
        return SG_OK;
    }
    SG_API_CATCH(sg_adjoint_destroy)

    int sg_adjoint_counts(sg_adjoint_t adj, long long* n0, long long* nT, int* n_steps)
    try
    {
        if (!adj)
        {
            return afail(SG_ERR_ARG, "sg_adjoint_counts: null handle");
        }
        if (n0)
        {
            *n0 = adj->n0;
        }
        if (nT)
        {
            *nT = adj->have_forward ? adj->nT : 0;
        }
        if (n_steps)
        {
            *n_steps = static_cast<int>(adj->steps.size());
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_adjoint_counts)

    int sg_adjoint_cells(sg_adjoint_t adj, int which, int* level, int* coords, long long n)
    try
    {
        if (!adj || (which != 0 && which != 1))
        {
            return afail(SG_ERR_ARG, "sg_adjoint_cells: which is 0 (initial mesh) or 1 (final mesh)");
        }
        if (which == 1 && !adj->have_forward)
        {
            return afail(SG_ERR_STATE, "sg_adjoint_cells: no forward run yet");
        }
        const auto& lev = which ? adj->levT : adj->lev0;
        const auto& co  = which ? adj->coT : adj->co0;
        if (n != static_cast<long long>(lev.size()))
        {
            return afail(SG_ERR_ARG, "sg_adjoint_cells: size differs from the number of cells");
        }
        if (level)
        {
            std::copy(lev.begin(), lev.end(), level);
        }
        if (coords)
        {
            std::copy(co.begin(), co.end(), coords);
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_adjoint_cells)

    int sg_adjoint_record(sg_adjoint_t adj, const double* u0, int n_steps, double eps, double regularity, const double* a, double dt, int scheme,
                          long long* nT)
    try
    {
        if (!adj || !u0 || !a || n_steps < 0 || (scheme != SG_UPWIND_OP && scheme != SG_README))
        {
            return afail(SG_ERR_ARG, "sg_adjoint_record: invalid argument (the adjoint covers the upwind operator and the README scheme)");
        }
        Ctx& c = ctx_of(adj);
        if (scheme == SG_README && c.g.dim != 2)
        {
            return afail(SG_ERR_ARG, "sg_adjoint_record: the README scheme is two-dimensional");
        }
        free_recording(adj);
        for (int d = 0; d < 3; ++d)
        {
            adj->a[d] = d < c.g.dim ? a[d] : 0.;
        }
        adj->dt     = dt;
        adj->eps    = eps;
        adj->reg    = regularity;
        adj->scheme = scheme;
        sg::DeviceField& u   = adj->u->f;
        sg::DeviceField& up1 = adj->unp1->f;
        int st;
        if ((st = load_mesh(adj, 0)) || (st = set_initial_field(adj, u0, u.data)))
        {
            return afail(st, c.err.c_str());
        }
        const int passes = c.cfg.max_level - c.cfg.min_level;
        if (!adj->rec_slots && passes > 0 && dmalloc(&adj->rec_slots, static_cast<size_t>(passes) * static_cast<size_t>(c.g.total_words)))
        {
            adj->rec_slots = nullptr; // the pass-by-pass recording below needs no slots
            cudaGetLastError();
        }
        for (int n = 0; n < n_steps; ++n)
        {
            if (n % adj->K == 0)
            {
                if ((st = ensure_ckpt(adj, static_cast<size_t>(n / adj->K))))
                {
                    return afail(st, c.err.c_str());
                }
                cudaMemcpyAsync(adj->ckpt[static_cast<size_t>(n / adj->K)], u.data, dense_bytes(c), cudaMemcpyDeviceToDevice, c.stream);
            }
            sg_adjoint_s::Step S{static_cast<int>(adj->bits.size()) - 1, 0};
            if (sg::step_graph_applies(c) && adj->rec_slots)
            {
                // the whole step as one graph (sg_step) that leaves the mesh of each transition in a slot
                int np       = 0;
                c.rec_slots  = adj->rec_slots;
                st           = sg::step(c, u, up1, eps, regularity, adj->a, dt, scheme, &np);
                c.rec_slots  = nullptr;
                if (st)
                {
                    return afail(st, c.err.c_str());
                }
                const int trans = c.h_adapt[sg::A_TRANS];
                for (int t = 0; t < trans; ++t)
                {
                    if ((st = push_bits_from(adj, adj->rec_slots + static_cast<size_t>(t) * static_cast<size_t>(c.g.total_words))))
                    {
                        return afail(st, c.err.c_str());
                    }
                }
                S.n_trans = trans;
                adj->steps.push_back(S);
                continue;
            }
            for (int i = 0; i < passes; ++i)
            {
                bool conv = false;
                if ((st = sg::harten(c, u, i, eps, regularity, &conv)))
                {
                    return afail(st, c.err.c_str());
                }
                if (conv)
                {
                    break;
                }
                if ((st = push_current_bits(adj)))
                {
                    return afail(st, c.err.c_str());
                }
                ++S.n_trans;
            }
            adj->steps.push_back(S);
            if ((st = sg::update_ghost_mr(c, u)) || (st = sg::upwind(c, u, up1, adj->a, dt, scheme)))
            {
                return afail(st, c.err.c_str());
            }
            std::swap(u.data, up1.data);
            u.ghosts_valid   = false;
            up1.ghosts_valid = false;
        }
        if ((st = sg::device_error(c)) || (st = final_leaves(adj)))
        {
            return afail(st, c.err.c_str());
        }
        adj->have_forward = true;
        if (nT)
        {
            *nT = adj->nT;
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_adjoint_record)

    int sg_adjoint_final(sg_adjoint_t adj, double* uT, long long n)
    try
    {
        if (!adj || !uT)
        {
            return afail(SG_ERR_ARG, "sg_adjoint_final: null argument");
        }
        if (!adj->have_forward || n != adj->nT)
        {
            return afail(SG_ERR_STATE, "sg_adjoint_final: no forward run, or n differs from the final number of cells");
        }
        Ctx& c = ctx_of(adj);
        cudaMemcpyAsync(uT, adj->d_uT, static_cast<size_t>(n) * sizeof(double), cudaMemcpyDefault, c.stream); // host or device
        if (cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            return afail(SG_ERR_CUDA, "sg_adjoint_final: CUDA error");
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_adjoint_final)

    int sg_adjoint_replay(sg_adjoint_t adj, const double* u0, const double* a, double* uT)
    try
    {
        if (!adj || !u0 || !a)
        {
            return afail(SG_ERR_ARG, "sg_adjoint_replay: null argument");
        }
        if (!adj->have_forward)
        {
            return afail(SG_ERR_STATE, "sg_adjoint_replay: nothing recorded");
        }
        Ctx& c = ctx_of(adj);
        for (int d = 0; d < 3; ++d)
        {
            adj->a[d] = d < c.g.dim ? a[d] : 0.;
        }
        int st;
        if ((st = load_mesh(adj, 0)) || (st = set_initial_field(adj, u0, adj->u->f.data))
            || (st = replay_range(adj, 0, static_cast<int>(adj->steps.size()), false, true)))
        {
            return afail(st, c.err.c_str());
        }
        if ((st = sg::device_error(c)))
        {
            return afail(st, c.err.c_str());
        }
        // the final mesh is the recorded one: same leaves as after record
        sg::k_leaf_gather<<<sg::grid_of(adj->nT), sg::ABLOCK, 0, c.stream>>>(adj->d_elT, adj->u->f.data, adj->nT, adj->d_uT);
        return uT ? sg_adjoint_final(adj, uT, adj->nT) : SG_OK;
    }
    SG_API_CATCH(sg_adjoint_replay)

    int sg_adjoint_backward(sg_adjoint_t adj, const double* gT, double* g0, double* ga)
    try
    {
        if (!adj || !gT || !g0)
        {
            return afail(SG_ERR_ARG, "sg_adjoint_backward: null argument");
        }
        if (!adj->have_forward)
        {
            return afail(SG_ERR_STATE, "sg_adjoint_backward: nothing recorded");
        }
        Ctx& c         = ctx_of(adj);
        const int T    = static_cast<int>(adj->steps.size());
        const int K    = adj->K;
        int st;
        // lam = dJ/du_T on the final leaves, 0 elsewhere
        if ((st = stage_vals(adj, std::max(adj->nT, adj->n0))))
        {
            return afail(st, c.err.c_str());
        }
        cudaMemsetAsync(adj->lam[0], 0, dense_bytes(c), c.stream);
        cudaMemcpyAsync(adj->d_vals, gT, static_cast<size_t>(adj->nT) * sizeof(double), cudaMemcpyDefault, c.stream); // host or device
        sg::k_leaf_scatter<<<sg::grid_of(adj->nT), sg::ABLOCK, 0, c.stream>>>(adj->d_elT, adj->d_vals, adj->nT, adj->lam[0]);
        cudaMemsetAsync(adj->d_ga, 0, 3 * sizeof(double), c.stream);
        while (static_cast<int>(adj->ug.size()) < std::min(K, std::max(T, 1)))
        {
            double* p = nullptr;
            if (dmalloc(&p, static_cast<size_t>(c.capacity)))
            {
                return afail(SG_ERR_CUDA, "sg_adjoint_backward: out of device memory");
            }
            adj->ug.push_back(p);
        }
        cudaMemsetAsync(adj->d_overflow, 0, sizeof(int), c.stream);
        for (int s = ((T - 1) / K) * K; s >= 0 && T > 0; s -= K)
        {
            const int e = std::min(T, s + K);
            if ((st = load_mesh(adj, adj->steps[static_cast<size_t>(s)].mesh0)))
            {
                return afail(st, c.err.c_str());
            }
            cudaMemcpyAsync(adj->u->f.data, adj->ckpt[static_cast<size_t>(s / K)], dense_bytes(c), cudaMemcpyDeviceToDevice, c.stream);
            if ((st = replay_range(adj, s, e, true, false)) || (st = reverse_segment(adj, s, e)))
            {
                return afail(st, c.err.c_str());
            }
        }
        int overflow = 0;
        cudaMemcpyAsync(&overflow, adj->d_overflow, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
        if (cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            return afail(SG_ERR_CUDA, "sg_adjoint_backward: CUDA error");
        }
        if (overflow)
        {
            return afail(SG_ERR_CAPACITY, "sg_adjoint_backward: an operator has more terms than a linear form holds");
        }
        if ((st = sg::device_error(c)))
        {
            return afail(st, c.err.c_str());
        }
        sg::k_leaf_gather<<<sg::grid_of(adj->n0), sg::ABLOCK, 0, c.stream>>>(adj->d_el0, adj->lam[0], adj->n0, adj->d_vals);
        cudaMemcpyAsync(g0, adj->d_vals, static_cast<size_t>(adj->n0) * sizeof(double), cudaMemcpyDefault, c.stream); // host or device
        double h_ga[3] = {0., 0., 0.};
        cudaMemcpyAsync(h_ga, adj->d_ga, 3 * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
        if (cudaStreamSynchronize(c.stream) != cudaSuccess)
        {
            return afail(SG_ERR_CUDA, "sg_adjoint_backward: CUDA error");
        }
        if (ga)
        {
            for (int d = 0; d < c.g.dim; ++d)
            {
                ga[d] = h_ga[d];
            }
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_adjoint_backward)
}
