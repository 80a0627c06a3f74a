// C ABI over the CPU oracle (samurai_oracle.hpp) so that the Python tests and
// bench.py's CPU-baseline leg can drive it through ctypes.  TEST
// INFRASTRUCTURE ONLY: the product library never links this file.
#include "samurai_oracle.hpp"

#include <cstring>
#include <memory>

namespace
{
    struct Base
    {
        virtual ~Base() = default;
        int dim              = 2;
        bool refine_boundary = false; // --refine-boundary for this problem's adaptations
    };

    template <std::size_t D>
    struct Sim : Base
    {
        oracle::Mesh<D> mesh;
        oracle::Field u;
        oracle::BcConfig bc;
        // more fields on the same mesh (field k >= 1 is extra[k-1])
        std::vector<oracle::Field> extra;
        std::vector<oracle::BcConfig> extra_bc;
        oracle::Field last_detail;
        std::vector<std::uint8_t> last_tag;
    };

    template <std::size_t D>
    Sim<D>* as(void* h)
    {
        return static_cast<Sim<D>*>(static_cast<Base*>(h));
    }

    int dim_of(void* h)
    {
        return static_cast<Base*>(h)->dim;
    }

    template <std::size_t D>
    const std::vector<oracle::LSet<D>>& mesh_id(const oracle::Mesh<D>& m, int id)
    {
        switch (id)
        {
            case 0: return m.cells;
            case 1: return m.cag;
            case 2: return m.proj;
            case 3: return m.uni;
            default: return m.ref;
        }
    }

    // field k of the state: 0 is u, k >= 1 the fields added by oracle_add_field
    template <std::size_t D>
    oracle::Field& field_k(Sim<D>* s, int k)
    {
        return k == 0 ? s->u : s->extra[static_cast<std::size_t>(k - 1)];
    }
    template <std::size_t D>
    oracle::BcConfig& bc_k(Sim<D>* s, int k)
    {
        return k == 0 ? s->bc : s->extra_bc[static_cast<std::size_t>(k - 1)];
    }

#define DISPATCH(h, ...)                 \
    do                                    \
    {                                     \
        if (dim_of(h) == 2)               \
        {                                 \
            auto* s = as<2>(h);           \
            __VA_ARGS__;                  \
        }                                 \
        else                              \
        {                                 \
            auto* s = as<3>(h);           \
            __VA_ARGS__;                  \
        }                                 \
    } while (0)
}

extern "C"
{
    void* oracle_create_periodic(int dim, int min_level, int max_level, int max_stencil_radius, int prediction_radius, int graduation_width,
                                 double dirichlet, int periodic_mask);

    void* oracle_create(int dim, int min_level, int max_level, int max_stencil_radius, int prediction_radius, int graduation_width, double dirichlet)
    {
        return oracle_create_periodic(dim, min_level, max_level, max_stencil_radius, prediction_radius, graduation_width, dirichlet, 0);
    }

    // mesh_config<dim>().periodic({bit 0, bit 1, bit 2 of periodic_mask})
    void* oracle_create_periodic(int dim, int min_level, int max_level, int max_stencil_radius, int prediction_radius, int graduation_width,
                                 double dirichlet, int periodic_mask)
    {
        oracle::MeshConfig cfg;
        for (int d = 0; d < 3; ++d)
        {
            cfg.periodic[static_cast<std::size_t>(d)] = ((periodic_mask >> d) & 1) != 0;
        }
        cfg.min_level          = min_level;
        cfg.max_level          = max_level;
        cfg.max_stencil_radius = max_stencil_radius;
        cfg.prediction_radius  = prediction_radius;
        cfg.graduation_width   = graduation_width;
        cfg.ghost_width        = std::max(max_stencil_radius, prediction_radius);
        try
        {
            if (dim == 2)
            {
                auto* s            = new Sim<2>();
                s->dim             = 2;
                s->mesh            = oracle::make_uniform_mesh<2>(cfg);
                s->bc.dirichlet_value = dirichlet;
                s->u.assign(s->mesh.nb_ref, std::numeric_limits<double>::quiet_NaN());
                return static_cast<Base*>(s);
            }
            if (dim == 3)
            {
                auto* s            = new Sim<3>();
                s->dim             = 3;
                s->mesh            = oracle::make_uniform_mesh<3>(cfg);
                s->bc.dirichlet_value = dirichlet;
                s->u.assign(s->mesh.nb_ref, std::numeric_limits<double>::quiet_NaN());
                return static_cast<Base*>(s);
            }
        }
        catch (...)
        {
        }
        return nullptr;
    }

    void oracle_destroy(void* h)
    {
        delete static_cast<Base*>(h);
    }

    long long oracle_nb_cells(void* h)
    {
        long long n = 0;
        DISPATCH(h, for (auto& l : s->mesh.cells) n += static_cast<long long>(l.count()));
        return n;
    }

    long long oracle_nb_ref(void* h)
    {
        long long n = 0;
        DISPATCH(h, n = static_cast<long long>(s->mesh.nb_ref));
        return n;
    }

    // leaf cells in for_each_cell order: level, coords (n x dim), storage index
    void oracle_get_cells(void* h, int* level, int* coords, long long* index)
    {
        long long k = 0;
        if (dim_of(h) == 2)
        {
            auto* s = as<2>(h);
            for (int l = 0; l < oracle::MAXL; ++l)
            {
                s->mesh.cells[l].for_each_cell(
                    [&](const oracle::Coord<2>& c)
                    {
                        level[k]          = l;
                        coords[2 * k]     = c[0];
                        coords[2 * k + 1] = c[1];
                        index[k]          = s->mesh.idx(l, c);
                        ++k;
                    });
            }
        }
        else
        {
            auto* s = as<3>(h);
            for (int l = 0; l < oracle::MAXL; ++l)
            {
                s->mesh.cells[l].for_each_cell(
                    [&](const oracle::Coord<3>& c)
                    {
                        level[k]          = l;
                        coords[3 * k]     = c[0];
                        coords[3 * k + 1] = c[1];
                        coords[3 * k + 2] = c[2];
                        index[k]          = s->mesh.idx(l, c);
                        ++k;
                    });
            }
        }
    }

    void oracle_get_field(void* h, double* out)
    {
        DISPATCH(h, std::memcpy(out, s->u.data(), s->u.size() * sizeof(double)));
    }

    void oracle_set_field(void* h, const double* in)
    {
        DISPATCH(h, std::memcpy(s->u.data(), in, s->u.size() * sizeof(double)));
    }

    // a new field on the current mesh (values NaN until set), with make_bc<Dirichlet<1>>(f, value)
    int oracle_add_field(void* h, double dirichlet)
    {
        int k = -1;
        DISPATCH(h,
                 {
                     s->extra.emplace_back(s->mesh.nb_ref, std::numeric_limits<double>::quiet_NaN());
                     oracle::BcConfig b;
                     b.dirichlet_value = dirichlet;
                     s->extra_bc.push_back(b);
                     k = static_cast<int>(s->extra.size());
                 });
        return k;
    }

    void oracle_get_field_k(void* h, int k, double* out)
    {
        DISPATCH(h, { auto& f = field_k(s, k); std::memcpy(out, f.data(), f.size() * sizeof(double)); });
    }

    void oracle_set_field_k(void* h, int k, const double* in)
    {
        DISPATCH(h, { auto& f = field_k(s, k); std::memcpy(f.data(), in, f.size() * sizeof(double)); });
    }

    int oracle_update_ghost_k(void* h, int k)
    {
        try
        {
            DISPATCH(h, oracle::update_ghost_mr(s->mesh, field_k(s, k), bc_k(s, k)));
            return 0;
        }
        catch (...)
        {
            return -1;
        }
    }

    // make_MRAdapt(f_0 .. f_{n_crit-1})(mra_config, f_{n_crit} .. f_{n_crit+n_other-1}): the first fields drive the
    // adaptation, the others follow the mesh; returns the number of Harten passes
    int oracle_adapt_fields(void* h, double eps, double regularity, int relative_detail, int n_crit, int n_other)
    {
        try
        {
            int it = 0;
            DISPATCH(h,
                     {
                         std::vector<oracle::Field*> fs, os;
                         std::vector<const oracle::BcConfig*> bs, obs;
                         for (int k = 0; k < n_crit; ++k)
                         {
                             fs.push_back(&field_k(s, k));
                             bs.push_back(&bc_k(s, k));
                         }
                         for (int k = n_crit; k < n_crit + n_other; ++k)
                         {
                             os.push_back(&field_k(s, k));
                             obs.push_back(&bc_k(s, k));
                         }
                         oracle::MRConfig mr{eps, regularity, relative_detail != 0, s->refine_boundary};
                         const int minl = s->mesh.cfg.min_level, maxl = s->mesh.cfg.max_level;
                         for (int i = 0; minl != maxl && i < maxl - minl; ++i)
                         {
                             ++it;
                             if (oracle::harten_fields(s->mesh, fs, bs, i, mr, os, obs, &s->last_detail, &s->last_tag))
                             {
                                 break;
                             }
                         }
                     });
            return it;
        }
        catch (...)
        {
            return -1;
        }
    }

    void oracle_get_detail(void* h, double* out)
    {
        DISPATCH(h, std::memcpy(out, s->last_detail.data(), s->last_detail.size() * sizeof(double)));
    }

    void oracle_get_tag(void* h, unsigned char* out)
    {
        DISPATCH(h, std::memcpy(out, s->last_tag.data(), s->last_tag.size()));
    }

    // MRadaptation(eps, regularity): returns the number of harten passes, -1 on error
    int oracle_adapt_rel(void* h, double eps, double regularity, int relative_detail);

    int oracle_adapt(void* h, double eps, double regularity)
    {
        return oracle_adapt_rel(h, eps, regularity, 0);
    }

    // the same with mra_config().relative_detail(relative_detail)
    int oracle_adapt_rel(void* h, double eps, double regularity, int relative_detail)
    {
        try
        {
            int it = 0;
            DISPATCH(h,
                     {
                         oracle::MRConfig mr{eps, regularity, relative_detail != 0, s->refine_boundary};
                         const int minl = s->mesh.cfg.min_level, maxl = s->mesh.cfg.max_level;
                         if (minl != maxl)
                         {
                             for (int i = 0; i < maxl - minl; ++i)
                             {
                                 ++it;
                                 if (oracle::harten(s->mesh, s->u, i, mr, s->bc, &s->last_detail, &s->last_tag))
                                 {
                                     break;
                                 }
                             }
                         }
                     });
            return it;
        }
        catch (...)
        {
            return -1;
        }
    }

    // a single harten pass (for parity tests of the adaptation internals);
    // returns 1 at the fixed point, 0 if the mesh changed, -1 on error
    int oracle_harten(void* h, int ite, double eps, double regularity)
    {
        try
        {
            int r = 0;
            DISPATCH(h,
                     {
                         oracle::MRConfig mr{eps, regularity, false, s->refine_boundary};
                         r = oracle::harten(s->mesh, s->u, ite, mr, s->bc, &s->last_detail, &s->last_tag) ? 1 : 0;
                     });
            return r;
        }
        catch (...)
        {
            return -1;
        }
    }

    int oracle_update_ghost(void* h)
    {
        try
        {
            DISPATCH(h, oracle::update_ghost_mr(s->mesh, s->u, s->bc));
            return 0;
        }
        catch (...)
        {
            return -1;
        }
    }

    int oracle_upwind_k(void* h, int k, const double* a, double dt, int scheme);

    // u <- u - dt * upwind(a, u) on the cells; ghost storage becomes NaN
    // (scheme 0: upwind operator, 1: README lambda, 2: make_convection_upwind)
    int oracle_upwind(void* h, const double* a, double dt, int scheme)
    {
        return oracle_upwind_k(h, 0, a, dt, scheme);
    }

    // the same on field k (a component of a vector field is upwinded alone, stencil_field.hpp:91-179)
    int oracle_upwind_k(void* h, int k, const double* a, double dt, int scheme)
    {
        try
        {
            if (dim_of(h) == 2)
            {
                auto* s = as<2>(h);
                auto& f = field_k(s, k);
                f       = oracle::upwind_step<2>(s->mesh, f, {a[0], a[1]}, dt, static_cast<oracle::Scheme>(scheme));
            }
            else
            {
                auto* s = as<3>(h);
                auto& f = field_k(s, k);
                f       = oracle::upwind_step<3>(s->mesh, f, {a[0], a[1], a[2]}, dt, static_cast<oracle::Scheme>(scheme));
            }
            return 0;
        }
        catch (...)
        {
            return -1;
        }
    }

    // intervals of a mesh id at a level, canonical (maximal) form, rows in
    // for_each_interval order.  Each record: start, end, y[, z].
    long long oracle_count_intervals(void* h, int id, int level)
    {
        long long n = 0;
        DISPATCH(h, for (auto& [k, r] : mesh_id(s->mesh, id)[level].rows) n += static_cast<long long>(r.size()));
        return n;
    }

    void oracle_get_intervals(void* h, int id, int level, int* out)
    {
        long long k = 0;
        if (dim_of(h) == 2)
        {
            auto* s = as<2>(h);
            for (auto& [key, r] : mesh_id(s->mesh, id)[level].rows)
            {
                for (auto& iv : r)
                {
                    out[3 * k]     = iv.s;
                    out[3 * k + 1] = iv.e;
                    out[3 * k + 2] = key[0];
                    ++k;
                }
            }
        }
        else
        {
            auto* s = as<3>(h);
            for (auto& [key, r] : mesh_id(s->mesh, id)[level].rows)
            {
                for (auto& iv : r)
                {
                    out[4 * k]     = iv.s;
                    out[4 * k + 1] = iv.e;
                    out[4 * k + 2] = key[0];
                    out[4 * k + 3] = key[1];
                    ++k;
                }
            }
        }
    }

    // One recorded mesh transition of a frozen-mesh replay: the mesh becomes
    // the one of the given leaf cells and field 0 follows it through
    // update_fields (algorithm/update_fields.hpp:27-127), as the end of a
    // Harten pass that changed the mesh does (mr/adapt.hpp:380-386).  The
    // caller updates the ghosts before, as that pass did.
    int oracle_transfer_cells(void* h, long long n, const int* level, const int* coords)
    {
        try
        {
            if (dim_of(h) == 2)
            {
                auto* s = as<2>(h);
                std::vector<oracle::LSet<2>> cells;
                oracle::init_levels(cells);
                for (long long i = 0; i < n; ++i)
                {
                    cells[level[i]].add({coords[2 * i + 1]}, {coords[2 * i], coords[2 * i] + 1});
                }
                oracle::Mesh<2> nm = oracle::make_mesh_from_cells<2>(s->mesh.cfg, cells);
                oracle::Field nu   = oracle::update_fields<2>(s->mesh, nm, s->u);
                s->mesh            = std::move(nm);
                s->u               = std::move(nu);
            }
            else
            {
                auto* s = as<3>(h);
                std::vector<oracle::LSet<3>> cells;
                oracle::init_levels(cells);
                for (long long i = 0; i < n; ++i)
                {
                    cells[level[i]].add({coords[3 * i + 1], coords[3 * i + 2]}, {coords[3 * i], coords[3 * i] + 1});
                }
                oracle::Mesh<3> nm = oracle::make_mesh_from_cells<3>(s->mesh.cfg, cells);
                oracle::Field nu   = oracle::update_fields<3>(s->mesh, nm, s->u);
                s->mesh            = std::move(nm);
                s->u               = std::move(nu);
            }
            return 0;
        }
        catch (...)
        {
            return -1;
        }
    }

    // args::refine_boundary (--refine-boundary) for this problem's adaptations
    void oracle_set_refine_boundary(void* h, int enable)
    {
        static_cast<Base*>(h)->refine_boundary = enable != 0;
    }

    // rebuild the mesh from leaf cells given as (level, coords) lists; used by
    // tests that start from a prescribed adapted mesh.  Field reset to NaN.
    int oracle_set_cells(void* h, long long n, const int* level, const int* coords)
    {
        try
        {
            if (dim_of(h) == 2)
            {
                auto* s = as<2>(h);
                std::vector<oracle::LSet<2>> cells;
                oracle::init_levels(cells);
                for (long long i = 0; i < n; ++i)
                {
                    cells[level[i]].add({coords[2 * i + 1]}, {coords[2 * i], coords[2 * i] + 1});
                }
                s->mesh = oracle::make_mesh_from_cells<2>(s->mesh.cfg, cells);
                s->u.assign(s->mesh.nb_ref, std::numeric_limits<double>::quiet_NaN());
            }
            else
            {
                auto* s = as<3>(h);
                std::vector<oracle::LSet<3>> cells;
                oracle::init_levels(cells);
                for (long long i = 0; i < n; ++i)
                {
                    cells[level[i]].add({coords[3 * i + 1], coords[3 * i + 2]}, {coords[3 * i], coords[3 * i] + 1});
                }
                s->mesh = oracle::make_mesh_from_cells<3>(s->mesh.cfg, cells);
                s->u.assign(s->mesh.nb_ref, std::numeric_limits<double>::quiet_NaN());
            }
            return 0;
        }
        catch (...)
        {
            return -1;
        }
    }
}
