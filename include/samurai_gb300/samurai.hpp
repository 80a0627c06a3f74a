// C++ drop-in for samurai's MR advection API, backed by libsamurai_gpu.so.
//
// A samurai program of the form of demos/FiniteVolume/advection_2d.cpp or
// the README example compiles against this header with its calls unchanged:
//
//   auto config = samurai::mesh_config<2>().min_level(4).max_level(10)
//                     .max_stencil_size(2).disable_minimal_ghost_width();   // mesh_config.hpp:16-433
//   auto mesh   = samurai::mra::make_mesh(box, config);                      // mr/mesh.hpp:511-518
//   auto u      = samurai::make_scalar_field<double>("u", mesh);             // field/scalar_field.hpp:173-216
//   samurai::for_each_cell(mesh, [&](auto& cell) { u[cell] = ...; });        // algorithm.hpp:301-363 (host mirror)
//   samurai::for_each_interval(mesh, [&](auto level, auto& i, auto& index) {  // algorithm.hpp:75-123 (host mirror)
//       for (int x = i.start; x < i.end; ++x) u(level, x, index[0]) = ...; });
//   samurai::make_bc<samurai::Dirichlet<1>>(u, 0.);                          // bc/bc.hpp:786-800
//   auto MRadaptation = samurai::make_MRAdapt(u);                            // mr/adapt.hpp:391-397
//   MRadaptation(samurai::mra_config().epsilon(2e-4));                       // mr/adapt.hpp:147-195
//   samurai::update_ghost_mr(u);                                             // algorithm/update_ghost_mr.hpp:261-270
//   unp1 = u - dt * samurai::upwind(a, u);                                   // stencil_field.hpp:175-179
//   std::swap(u.array(), unp1.array());                                      // advection_2d.cpp:146
//
// The mesh and the fields live on the GPU.  for_each_cell / for_each_interval
// with user lambdas run on a host mirror (downloaded on demand); writes made
// through u[cell] are uploaded at the next GPU call.  Errors raise
// std::runtime_error with the library's message.
#pragma once

#include <array>
#include <cstddef>
#include <filesystem>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "../samurai_gpu.h"

namespace samurai
{
    namespace detail
    {
        inline void check(int status, const char* what)
        {
            if (status != SG_OK)
            {
                throw std::runtime_error(std::string(what) + ": " + sg_last_error());
            }
        }
    }

    template <class value_t, std::size_t dim>
    struct Box
    {
        std::array<value_t, dim> min_corner, max_corner;

        Box(const std::array<value_t, dim>& a, const std::array<value_t, dim>& b)
            : min_corner(a)
            , max_corner(b)
        {
            for (std::size_t d = 0; d < dim; ++d)
            {
                if (a[d] != 0 || b[d] != 1)
                {
                    throw std::invalid_argument("samurai_gb300: only the unit box is supported");
                }
            }
        }
    };

    namespace default_config
    {
        static constexpr int prediction_stencil_radius = 1;
    }

    // samurai's command-line switches that act on this path (arguments.hpp:26, 67): refine_boundary
    // (--refine-boundary) keeps the boundary cells of max_level refined in every adaptation
    namespace args
    {
        inline bool refine_boundary = false;
    }

    template <std::size_t dim_, int prediction_stencil_radius_ = default_config::prediction_stencil_radius>
    class mesh_config
    {
      public:

        static constexpr std::size_t dim            = dim_;
        static constexpr int prediction_stencil_radius = prediction_stencil_radius_;

        auto& min_level(std::size_t l)
        {
            m_min = l;
            return *this;
        }

        auto& max_level(std::size_t l)
        {
            m_max = l;
            return *this;
        }

        auto& max_stencil_radius(int r)
        {
            m_r = r;
            return *this;
        }

        auto& max_stencil_size(int s)
        {
            m_r = s / 2 + (s % 2);
            return *this;
        }

        auto& graduation_width(std::size_t w)
        {
            m_grad = w;
            return *this;
        }

        auto& disable_minimal_ghost_width()
        {
            m_no_min_gw = true;
            return *this;
        }

        auto& disable_args_parse()
        {
            return *this;
        }

        std::size_t min_level() const
        {
            return m_min;
        }

        std::size_t max_level() const
        {
            return m_max;
        }

        std::size_t graduation_width() const
        {
            return m_grad;
        }

        // periodicity (mesh_config.hpp:279-331): one flag for every axis, or one per axis
        auto& periodic(bool p)
        {
            m_periodic.fill(p);
            return *this;
        }

        auto& periodic(const std::array<bool, dim>& p)
        {
            m_periodic = p;
            return *this;
        }

        const std::array<bool, dim>& periodic() const
        {
            return m_periodic;
        }

        bool periodic(std::size_t i) const
        {
            return m_periodic[i];
        }

        // mesh_config::parse_args (mesh_config.hpp:358-396), without CLI overrides
        int parsed_stencil_radius() const
        {
            if (m_max < m_min)
            {
                throw std::invalid_argument("Max level must be greater than min level.");
            }
            return m_no_min_gw ? m_r : (m_r > 2 ? m_r : 2);
        }

      private:

        std::size_t m_min = 0, m_max = 6, m_grad = 1;
        int m_r           = 1;
        bool m_no_min_gw  = false;
        std::array<bool, dim> m_periodic{};
    };

    // deprecated MRConfig<dim> used by the README (mr/mesh.hpp:45-72)
    template <std::size_t dim_>
    struct MRConfig
    {
        static constexpr std::size_t dim               = dim_;
        static constexpr int prediction_stencil_radius = 1;
    };

    // coordinates of a point: c[d] and samurai's c(d) (coords_t, cell.hpp)
    template <std::size_t dim>
    struct Coords : std::array<double, dim>
    {
        double operator()(std::size_t d) const
        {
            return (*this)[d];
        }
    };

    template <std::size_t dim>
    struct Cell
    {
        std::size_t level;
        std::array<int, dim> indices;
        long long index;
        double length;

        Coords<dim> center() const
        {
            Coords<dim> c;
            for (std::size_t d = 0; d < dim; ++d)
            {
                c[d] = length * (indices[d] + 0.5); // cell.hpp:130-133 with a zero origin
            }
            return c;
        }

        std::array<double, dim> corner() const
        {
            std::array<double, dim> c;
            for (std::size_t d = 0; d < dim; ++d)
            {
                c[d] = length * indices[d];
            }
            return c;
        }
    };

    // Interval<int, long long> (interval.hpp:51-254): [start, end) with step 1;
    // index + x is the storage index of cell x
    struct Interval
    {
        int start, end;
        long long index;
        int step = 1;

        int size() const
        {
            return end - start;
        }
    };

    template <class Config>
    class MRMesh
    {
      public:

        static constexpr std::size_t dim = Config::dim;

        MRMesh() = default;

        MRMesh(int min_level, int max_level, int stencil_radius, int prediction_radius, int graduation_width,
               const std::array<bool, dim>& periodic = {})
            : m_min(min_level)
            , m_max(max_level)
        {
            int per[3] = {0, 0, 0};
            for (std::size_t d = 0; d < dim; ++d)
            {
                per[d] = periodic[d] ? 1 : 0;
            }
            sg_mesh_t h = nullptr;
            detail::check(sg_mesh_create_periodic(static_cast<int>(dim), min_level, max_level, stencil_radius, prediction_radius, graduation_width,
                                                  per, &h),
                          "MRMesh");
            m_h = std::shared_ptr<sg_mesh_s>(h, [](sg_mesh_t p) { sg_mesh_destroy(p); });
        }

        // deprecated constructor of the README (mr/mesh.hpp:166-181)
        MRMesh(const Box<double, dim>&, std::size_t min_level, std::size_t max_level)
            : MRMesh(static_cast<int>(min_level), static_cast<int>(max_level), 1, Config::prediction_stencil_radius, 1)
        {
        }

        sg_mesh_t handle() const
        {
            return m_h.get();
        }

        std::size_t min_level() const
        {
            return static_cast<std::size_t>(m_min);
        }

        std::size_t max_level() const
        {
            return static_cast<std::size_t>(m_max);
        }

        double cell_length(std::size_t level) const
        {
            return 1.0 / static_cast<double>(1 << level);
        }

        double min_cell_length() const
        {
            return cell_length(max_level());
        }

        std::size_t nb_cells() const
        {
            long long nc = 0, nr = 0;
            detail::check(sg_mesh_counts(handle(), &nc, &nr), "nb_cells");
            return static_cast<std::size_t>(nr);
        }

        std::size_t nb_leaf_cells() const
        {
            long long nc = 0, nr = 0;
            detail::check(sg_mesh_counts(handle(), &nc, &nr), "nb_cells");
            return static_cast<std::size_t>(nc);
        }

        // MRMeshId (mr/mesh.hpp:25-33)
        enum class mesh_id_t : int
        {
            cells            = SG_CELLS,
            cells_and_ghosts = SG_CELLS_AND_GHOSTS,
            proj_cells       = SG_PROJ_CELLS,
            union_cells      = SG_UNION_CELLS,
            all_cells        = SG_REFERENCE,
            reference        = SG_REFERENCE
        };

        // mesh.nb_cells(mesh_id) (mesh.hpp:530-550)
        std::size_t nb_cells(mesh_id_t id) const
        {
            if (id == mesh_id_t::cells)
            {
                return nb_leaf_cells();
            }
            if (id == mesh_id_t::reference)
            {
                return nb_cells();
            }
            std::size_t n = 0;
            std::vector<Interval> iv;
            std::vector<std::array<int, dim - 1>> yz;
            for (int l = 0; l <= m_max; ++l)
            {
                intervals(static_cast<int>(id), static_cast<std::size_t>(l), iv, yz);
                for (const auto& i : iv)
                {
                    n += static_cast<std::size_t>(i.size());
                }
            }
            return n;
        }

        // mesh[mesh_id]: the cell set of one id, for for_each_interval / for_each_cell
        struct IdView
        {
            static constexpr std::size_t dim = MRMesh::dim;
            const MRMesh* mesh;
            mesh_id_t id;
        };

        IdView operator[](mesh_id_t id) const
        {
            return {this, id};
        }

        std::vector<Cell<dim>> cells() const
        {
            const std::size_t n = nb_leaf_cells();
            std::vector<int> level(n), coords(n * dim);
            std::vector<long long> index(n);
            detail::check(sg_mesh_get_cells(handle(), level.data(), coords.data(), index.data(), static_cast<long long>(n)), "cells");
            std::vector<Cell<dim>> out(n);
            for (std::size_t k = 0; k < n; ++k)
            {
                out[k].level = static_cast<std::size_t>(level[k]);
                for (std::size_t d = 0; d < dim; ++d)
                {
                    out[k].indices[d] = coords[k * dim + d];
                }
                out[k].index  = index[k];
                out[k].length = cell_length(out[k].level);
            }
            return out;
        }

        // the intervals of a mesh id at a level, rows in for_each_interval order
        // (z outer, y inner); yz[k] holds the dim-1 other coordinates of interval k
        void intervals(int mesh_id, std::size_t level, std::vector<Interval>& iv, std::vector<std::array<int, dim - 1>>& yz) const
        {
            long long n = 0;
            detail::check(sg_mesh_count_intervals(handle(), mesh_id, static_cast<int>(level), &n), "intervals");
            std::vector<long long> rec(static_cast<std::size_t>(n) * (dim + 2));
            if (n > 0)
            {
                detail::check(sg_mesh_get_intervals(handle(), mesh_id, static_cast<int>(level), rec.data(), n), "intervals");
            }
            iv.resize(static_cast<std::size_t>(n));
            yz.resize(static_cast<std::size_t>(n));
            for (long long k = 0; k < n; ++k)
            {
                const long long* r = rec.data() + k * (dim + 2);
                iv[k]              = {static_cast<int>(r[0]), static_cast<int>(r[1]), r[dim + 1]};
                for (std::size_t d = 0; d + 1 < dim; ++d)
                {
                    yz[k][d] = static_cast<int>(r[2 + d]);
                }
            }
        }

        // storage index of cell (x, yz) of the reference mesh at a level, -1 if absent
        // (find / get_index, algorithm.hpp:391-467 and level_cell_array.hpp:669-743)
        long long find(std::size_t level, int x, const std::array<int, dim - 1>& yz) const
        {
            const auto& lv = reference_rows(level);
            auto it        = lv.find(yz);
            if (it == lv.end())
            {
                return -1;
            }
            for (const Interval& i : it->second)
            {
                if (x >= i.start && x < i.end)
                {
                    return i.index + x;
                }
            }
            return -1;
        }

      private:

        // reference-mesh rows of a level, cached for the current mesh version
        const std::map<std::array<int, dim - 1>, std::vector<Interval>>& reference_rows(std::size_t level) const
        {
            unsigned long long version = 0;
            detail::check(sg_mesh_version(handle(), &version), "find");
            if (m_rows.size() <= level || m_rows_version != version)
            {
                m_rows.assign(m_max + 1, {});
                for (int l = 0; l <= m_max; ++l)
                {
                    std::vector<Interval> iv;
                    std::vector<std::array<int, dim - 1>> yz;
                    intervals(SG_REFERENCE, static_cast<std::size_t>(l), iv, yz);
                    for (std::size_t k = 0; k < iv.size(); ++k)
                    {
                        m_rows[static_cast<std::size_t>(l)][yz[k]].push_back(iv[k]);
                    }
                }
                m_rows_version = version;
            }
            return m_rows[level];
        }

        std::shared_ptr<sg_mesh_s> m_h;
        int m_min = 0, m_max = 0;
        mutable std::vector<std::map<std::array<int, dim - 1>, std::vector<Interval>>> m_rows;
        mutable unsigned long long m_rows_version = 0;
    };

    namespace mra
    {
        template <class Cfg>
        auto make_empty_mesh(const Cfg&)
        {
            return MRMesh<Cfg>();
        }

        template <class Cfg>
        auto make_mesh(const Box<double, Cfg::dim>&, const Cfg& cfg)
        {
            return MRMesh<Cfg>(static_cast<int>(cfg.min_level()), static_cast<int>(cfg.max_level()), cfg.parsed_stencil_radius(),
                               Cfg::prediction_stencil_radius, static_cast<int>(cfg.graduation_width()), cfg.periodic());
        }
    }

    template <class Mesh>
    class ScalarField;

    // host mirror of u.array(): downloaded on demand, uploaded when dirty
    class FieldArray
    {
      public:

        std::vector<double> values;
        bool valid = false;
        bool dirty = false;
    };

    // unp1 = u - dt * op(u): op is upwind(a, u) or a make_convection_upwind operator; Field is a
    // scalar or a vector field, evaluated on the device when assigned to unp1
    template <class Field>
    struct UpwindOp
    {
        const Field* u;
        std::array<double, Field::dim> a;
        int scheme = SG_UPWIND_OP;
    };

    template <class Field>
    struct ScaledUpwind
    {
        const Field* u;
        std::array<double, Field::dim> a;
        double dt;
        int scheme;
    };

    template <class Field>
    struct UpwindExpr // u - dt * upwind(a, u)
    {
        const Field* u;
        std::array<double, Field::dim> a;
        double dt;
        int scheme;
    };

    template <class Mesh>
    class ScalarField
    {
      public:

        static constexpr std::size_t dim    = Mesh::dim;
        static constexpr std::size_t n_comp = 1;
        using mesh_t                        = Mesh;

        ScalarField(std::string name, Mesh& mesh)
            : m_mesh(&mesh)
            , m_name(std::move(name))
        {
            sg_field_t h = nullptr;
            detail::check(sg_field_create(mesh.handle(), m_name.c_str(), &h), "make_scalar_field");
            m_h = std::shared_ptr<sg_field_s>(h, [](sg_field_t p) { sg_field_destroy(p); });
        }

        sg_field_t handle() const
        {
            return m_h.get();
        }

        Mesh& mesh() const
        {
            return *m_mesh;
        }

        const std::string& name() const
        {
            return m_name;
        }

        // u.fill(value) (field/access_base.hpp:63-66): every reference cell, on the device
        void fill(double value)
        {
            m_host.dirty = false;
            m_host.valid = false;
            detail::check(sg_field_fill(handle(), value), "fill");
        }

        // host mirror access (for_each_cell initialisation, inspection)
        double& operator[](const Cell<dim>& cell)
        {
            pull();
            m_host.dirty = true;
            return m_host.values[static_cast<std::size_t>(cell.index)];
        }

        double operator[](const Cell<dim>& cell) const
        {
            const_cast<ScalarField*>(this)->pull();
            return m_host.values[static_cast<std::size_t>(cell.index)];
        }

        // u(level, i, j[, k]): the value of a reference cell (field_base.hpp, access through
        // get_index, algorithm.hpp:391-467); std::out_of_range for a cell outside the reference mesh
        template <class... T>
        double& operator()(std::size_t level, int i, T... yz)
        {
            static_assert(sizeof...(T) == dim - 1, "u(level, i, j[, k])");
            const long long e = m_mesh->find(level, i, {static_cast<int>(yz)...});
            if (e < 0)
            {
                throw std::out_of_range("samurai_gb300: u(level, i, ...) outside the reference mesh");
            }
            pull();
            m_host.dirty = true;
            return m_host.values[static_cast<std::size_t>(e)];
        }

        template <class... T>
        double operator()(std::size_t level, int i, T... yz) const
        {
            return (*const_cast<ScalarField*>(this))(level, i, yz...);
        }

        void resize()
        {
        }

        // u.array(): swapping arrays swaps the device storage
        ScalarField& array()
        {
            return *this;
        }

        // push pending host writes before any GPU computation
        void sync_to_device()
        {
            if (m_host.dirty)
            {
                detail::check(sg_field_upload(handle(), m_host.values.data(), static_cast<long long>(m_host.values.size())), "upload");
                m_host.dirty = false;
            }
            m_host.valid = false;
        }

        ScalarField& operator=(const UpwindExpr<ScalarField>& e)
        {
            const_cast<ScalarField*>(e.u)->sync_to_device();
            detail::check(sg_upwind(e.u->handle(), handle(), e.a.data(), e.dt, e.scheme), "upwind");
            m_host.valid = false;
            return *this;
        }

        // the scalar fields a call of the C ABI takes for this field
        void append_handles(std::vector<sg_field_t>& out) const
        {
            out.push_back(handle());
        }

        void set_dirichlet(const std::vector<double>& values)
        {
            if (values.size() > 1)
            {
                throw std::invalid_argument("make_bc: the number of constant values should be equal to the number of components");
            }
            detail::check(sg_field_set_dirichlet(handle(), values.empty() ? 0. : values[0]), "make_bc");
        }

        void update_ghost()
        {
            sync_to_device();
            detail::check(sg_update_ghost_mr(handle()), "update_ghost_mr");
        }

        friend void swap(ScalarField& a, ScalarField& b)
        {
            a.sync_to_device();
            b.sync_to_device();
            detail::check(sg_field_swap(a.handle(), b.handle()), "swap");
        }

      private:

        void pull()
        {
            if (m_host.valid)
            {
                return;
            }
            m_host.values.resize(m_mesh->nb_cells());
            detail::check(sg_field_download(handle(), m_host.values.data(), static_cast<long long>(m_host.values.size())), "download");
            m_host.valid = true;
        }

        Mesh* m_mesh;
        std::string m_name;
        std::shared_ptr<sg_field_s> m_h;
        FieldArray m_host;
    };

    template <class value_t, class Mesh>
    auto make_scalar_field(const std::string& name, Mesh& mesh)
    {
        static_assert(std::is_same_v<value_t, double>, "samurai_gb300 fields are FP64");
        return ScalarField<Mesh>(name, mesh);
    }

    template <class Mesh, class F>
    auto for_each_cell(const Mesh& mesh, F&& f) -> decltype(mesh.cells(), void());

    // make_scalar_field<double>(name, mesh, init_value) and make_scalar_field<double>(name, mesh, f)
    // with f(center) (field/scalar_field.hpp:178-216)
    template <class value_t, class Mesh, class Init>
    auto make_scalar_field(const std::string& name, Mesh& mesh, Init&& init)
    {
        auto u = make_scalar_field<value_t>(name, mesh);
        if constexpr (std::is_invocable_v<Init, Coords<Mesh::dim>>)
        {
            u.fill(0.);
            for_each_cell(mesh, [&](const auto& cell) { u[cell] = init(cell.center()); });
        }
        else
        {
            u.fill(static_cast<double>(init));
        }
        return u;
    }

    // VectorField<Mesh, double, n_comp> (field/vector_field.hpp:134-216): n_comp scalar
    // component fields on the device; the host mirror keeps samurai's layout, the values of a
    // cell side by side (storage shape {size, n_comp})
    template <class Mesh, std::size_t n_comp_>
    class VectorField
    {
      public:

        static constexpr std::size_t dim    = Mesh::dim;
        static constexpr std::size_t n_comp = n_comp_;
        using mesh_t                        = Mesh;

        // v[cell]: the n_comp values of one cell in the host mirror
        class CellValues
        {
          public:

            explicit CellValues(double* p)
                : m_p(p)
            {
            }

            double& operator[](std::size_t c) const
            {
                return m_p[c];
            }

            double& operator()(std::size_t c) const
            {
                return m_p[c];
            }

            const CellValues& operator=(const std::array<double, n_comp>& v) const
            {
                for (std::size_t c = 0; c < n_comp; ++c)
                {
                    m_p[c] = v[c];
                }
                return *this;
            }

            const CellValues& operator=(double v) const
            {
                for (std::size_t c = 0; c < n_comp; ++c)
                {
                    m_p[c] = v;
                }
                return *this;
            }

          private:

            double* m_p;
        };

        VectorField(std::string name, Mesh& mesh)
            : m_mesh(&mesh)
            , m_name(std::move(name))
        {
            static_assert(n_comp >= 1 && n_comp <= SG_MAX_COMPONENTS, "samurai_gb300: 1 <= n_comp <= SG_MAX_COMPONENTS");
            sg_vfield_t h = nullptr;
            detail::check(sg_vector_field_create(mesh.handle(), m_name.c_str(), static_cast<int>(n_comp), &h), "make_vector_field");
            m_h = std::shared_ptr<sg_vfield_s>(h, [](sg_vfield_t p) { sg_vector_field_destroy(p); });
        }

        sg_vfield_t handle() const
        {
            return m_h.get();
        }

        Mesh& mesh() const
        {
            return *m_mesh;
        }

        CellValues operator[](const Cell<dim>& cell)
        {
            pull();
            m_host.dirty = true;
            return CellValues(m_host.values.data() + static_cast<std::size_t>(cell.index) * n_comp);
        }

        template <class... T>
        CellValues operator()(std::size_t level, int i, T... yz)
        {
            static_assert(sizeof...(T) == dim - 1, "v(level, i, j[, k])");
            const long long e = m_mesh->find(level, i, {static_cast<int>(yz)...});
            if (e < 0)
            {
                throw std::out_of_range("samurai_gb300: v(level, i, ...) outside the reference mesh");
            }
            pull();
            m_host.dirty = true;
            return CellValues(m_host.values.data() + static_cast<std::size_t>(e) * n_comp);
        }

        std::array<double, n_comp> operator[](const Cell<dim>& cell) const
        {
            const_cast<VectorField*>(this)->pull();
            std::array<double, n_comp> r;
            for (std::size_t c = 0; c < n_comp; ++c)
            {
                r[c] = m_host.values[static_cast<std::size_t>(cell.index) * n_comp + c];
            }
            return r;
        }

        void resize()
        {
        }

        VectorField& array()
        {
            return *this;
        }

        void sync_to_device()
        {
            if (m_host.dirty)
            {
                detail::check(sg_vector_field_upload(handle(), m_host.values.data(), static_cast<long long>(m_host.values.size())), "upload");
                m_host.dirty = false;
            }
            m_host.valid = false;
        }

        void append_handles(std::vector<sg_field_t>& out) const
        {
            for (std::size_t c = 0; c < n_comp; ++c)
            {
                sg_field_t f = nullptr;
                detail::check(sg_vector_field_component(handle(), static_cast<int>(c), &f), "component");
                out.push_back(f);
            }
        }

        void set_dirichlet(const std::vector<double>& values)
        {
            if (!values.empty() && values.size() != n_comp)
            {
                throw std::invalid_argument("make_bc: the number of constant values should be equal to the number of components");
            }
            std::array<double, n_comp> v{};
            for (std::size_t c = 0; c < values.size(); ++c)
            {
                v[c] = values[c];
            }
            detail::check(sg_vector_field_set_dirichlet(handle(), v.data()), "make_bc");
        }

        void update_ghost()
        {
            sync_to_device();
            detail::check(sg_vector_update_ghost_mr(handle()), "update_ghost_mr");
        }

        VectorField& operator=(const UpwindExpr<VectorField>& e)
        {
            const_cast<VectorField*>(e.u)->sync_to_device();
            detail::check(sg_vector_upwind(e.u->handle(), handle(), e.a.data(), e.dt, e.scheme), "upwind");
            m_host.valid = false;
            return *this;
        }

        friend void swap(VectorField& a, VectorField& b)
        {
            a.sync_to_device();
            b.sync_to_device();
            detail::check(sg_vector_field_swap(a.handle(), b.handle()), "swap");
        }

      private:

        void pull()
        {
            if (m_host.valid)
            {
                return;
            }
            m_host.values.resize(m_mesh->nb_cells() * n_comp);
            detail::check(sg_vector_field_download(handle(), m_host.values.data(), static_cast<long long>(m_host.values.size())), "download");
            m_host.valid = true;
        }

        Mesh* m_mesh;
        std::string m_name;
        std::shared_ptr<sg_vfield_s> m_h;
        FieldArray m_host;
    };

    // make_vector_field<double, n_comp>(name, mesh) and make_vector_field<n_comp>(name, mesh)
    // (field/vector_field.hpp:232-237, 278-283)
    template <class value_t, std::size_t n_comp, class Mesh>
    auto make_vector_field(const std::string& name, Mesh& mesh)
    {
        static_assert(std::is_same_v<value_t, double>, "samurai_gb300 fields are FP64");
        return VectorField<Mesh, n_comp>(name, mesh);
    }

    template <std::size_t n_comp, class Mesh>
    auto make_vector_field(const std::string& name, Mesh& mesh)
    {
        return VectorField<Mesh, n_comp>(name, mesh);
    }

    // README spelling make_field<double, n_comp>(name, mesh)
    template <class value_t, std::size_t n_comp, class Mesh>
    auto make_field(const std::string& name, Mesh& mesh)
    {
        if constexpr (n_comp == 1)
        {
            return make_scalar_field<value_t>(name, mesh);
        }
        else
        {
            return make_vector_field<value_t, n_comp>(name, mesh);
        }
    }

    template <std::size_t order = 1>
    struct Dirichlet
    {
        static_assert(order == 1, "samurai_gb300 implements Dirichlet<1>");
    };

    // make_bc<Dirichlet<1>>(u, v_0, .., v_{n_comp-1}) (bc/bc.hpp:752-800): one constant per component,
    // none for zeros
    template <class Bc, class Field, class... T>
    void make_bc(Field& u, T... values)
    {
        u.set_dirichlet(std::vector<double>{static_cast<double>(values)...});
    }

    template <class Mesh, class F>
    auto for_each_cell(const Mesh& mesh, F&& f) -> decltype(mesh.cells(), void())
    {
        for (auto& c : mesh.cells())
        {
            f(c);
        }
    }

    // for_each_interval(mesh[mesh_id], f) and for_each_cell(mesh[mesh_id], f) on any cell set of the mesh
    template <class View, class F>
    auto for_each_interval(const View& v, F&& f) -> decltype(v.mesh, v.id, void())
    {
        std::vector<Interval> iv;
        std::vector<std::array<int, View::dim - 1>> yz;
        for (std::size_t l = 0; l <= v.mesh->max_level(); ++l)
        {
            v.mesh->intervals(static_cast<int>(v.id), l, iv, yz);
            for (std::size_t k = 0; k < iv.size(); ++k)
            {
                f(l, iv[k], yz[k]);
            }
        }
    }

    template <class View, class F>
    auto for_each_cell(const View& v, F&& f) -> decltype(v.mesh, v.id, void())
    {
        for_each_interval(v,
                          [&](std::size_t level, const Interval& i, const std::array<int, View::dim - 1>& yz)
                          {
                              for (int x = i.start; x < i.end; ++x)
                              {
                                  Cell<View::dim> c;
                                  c.level      = level;
                                  c.indices[0] = x;
                                  for (std::size_t d = 1; d < View::dim; ++d)
                                  {
                                      c.indices[d] = yz[d - 1];
                                  }
                                  c.index  = i.index + x;
                                  c.length = v.mesh->cell_length(level);
                                  f(c);
                              }
                          });
    }

    // for_each_interval(mesh, f(level, i, index)) (algorithm.hpp:75-123) on the leaf cells: levels
    // ascending, rows with z outer and y inner; index holds the dim-1 other coordinates and
    // i.index + x is the storage index of cell x
    template <class Mesh, class F>
    auto for_each_interval(const Mesh& mesh, F&& f) -> decltype(mesh.min_level(), void())
    {
        std::vector<Interval> iv;
        std::vector<std::array<int, Mesh::dim - 1>> yz;
        for (std::size_t l = mesh.min_level(); l <= mesh.max_level(); ++l)
        {
            mesh.intervals(SG_CELLS, l, iv, yz);
            for (std::size_t k = 0; k < iv.size(); ++k)
            {
                f(l, iv[k], yz[k]);
            }
        }
    }

    class mra_config
    {
      public:

        mra_config& epsilon(double e)
        {
            m_eps = e;
            return *this;
        }

        double epsilon() const
        {
            return m_eps;
        }

        mra_config& regularity(double r)
        {
            m_reg = r;
            return *this;
        }

        double regularity() const
        {
            return m_reg;
        }

        // details divided by max |u| over the leaf cells (mr/rel_detail.hpp)
        mra_config& relative_detail(bool r)
        {
            m_rel = r;
            return *this;
        }

        bool relative_detail() const
        {
            return m_rel;
        }

      private:

        double m_eps = 1e-4, m_reg = 1.;
        bool m_rel   = false;
    };

    // make_MRAdapt(u, v, ...) (mr/adapt.hpp:96-203, 391-420): the details of all
    // its fields decide the mesh (a vector field contributes its components, in
    // order); a call may carry other fields along
    template <class Field, class... Fields>
    class Adapt
    {
      public:

        explicit Adapt(Field& u, Fields&... fields)
            : m_fields(&u, &fields...)
        {
        }

        template <class... Others>
        void operator()(const mra_config& cfg, Others&... others)
        {
            std::vector<sg_field_t> fs, os;
            std::apply(
                [&](auto*... f)
                {
                    ((f->sync_to_device(), f->append_handles(fs)), ...);
                },
                m_fields);
            ((others.sync_to_device(), others.append_handles(os)), ...);
            detail::check(sg_mesh_set_refine_boundary(std::get<0>(m_fields)->mesh().handle(), args::refine_boundary ? 1 : 0), "MRadaptation");
            const int rel = cfg.relative_detail() ? 1 : 0;
            if (fs.size() == 1 && os.empty())
            {
                detail::check(sg_adapt_ex(fs[0], cfg.epsilon(), cfg.regularity(), rel, &m_last), "MRadaptation");
            }
            else
            {
                detail::check(sg_adapt_fields(static_cast<int>(fs.size()), fs.data(), static_cast<int>(os.size()), os.data(), cfg.epsilon(),
                                              cfg.regularity(), rel, &m_last),
                              "MRadaptation");
            }
        }

        template <class... Others>
        void operator()(double eps, double regularity, Others&... others)
        {
            (*this)(mra_config().epsilon(eps).regularity(regularity), others...);
        }

        int last_harten_passes() const
        {
            return m_last;
        }

      private:

        std::tuple<Field*, Fields*...> m_fields;
        int m_last = 0;
    };

    template <class Field, class... Fields>
    auto make_MRAdapt(Field& u, Fields&... fields)
    {
        return Adapt<Field, Fields...>(u, fields...);
    }

    template <class Field, class... Fields>
    void update_ghost_mr(Field& u, Fields&... fields)
    {
        u.update_ghost();
        (fields.update_ghost(), ...);
    }

    template <class Field, class A>
    auto upwind(const A& a, const Field& u)
    {
        UpwindOp<Field> op{&u, {}};
        for (std::size_t d = 0; d < Field::dim; ++d)
        {
            op.a[d] = a[d];
        }
        return op;
    }

    template <class Field>
    ScaledUpwind<Field> operator*(double dt, const UpwindOp<Field>& op)
    {
        return {op.u, op.a, dt, op.scheme};
    }

    // VelocityVector<dim> (schemes/fv/operators/convection_lin.hpp:8-9)
    template <std::size_t dim>
    using VelocityVector = std::array<double, dim>;

    // make_convection_upwind<Field>(velocity) (schemes/fv/operators/convection_lin.hpp:16-89): the
    // conservative flux form; conv(u) is evaluated on the device inside unp1 = u - dt * conv(u)
    template <class Field>
    struct ConvectionUpwind
    {
        VelocityVector<Field::dim> velocity;

        auto operator()(const Field& u) const
        {
            UpwindOp<Field> op{&u, velocity, SG_CONVECTION};
            return op;
        }
    };

    template <class Field>
    ConvectionUpwind<Field> make_convection_upwind(const VelocityVector<Field::dim>& velocity)
    {
        return {velocity};
    }

    template <class Field>
    UpwindExpr<Field> operator-(const Field& u, const ScaledUpwind<Field>& s)
    {
        if (&u != s.u)
        {
            throw std::invalid_argument("samurai_gb300: u - dt * upwind(a, v) needs v == u");
        }
        return {&u, s.a, s.dt, s.scheme};
    }
    // save / dump / load (io/hdf5.hpp:1331-1350, io/restart.hpp:188-227, 425-495): HDF5 files written and
    // read by the library without libhdf5; load needs a mesh with the file's dimension and levels
    namespace detail
    {
        class IoList
        {
          public:

            IoList()
            {
                check(sg_io_create(&m_h), "io");
            }

            ~IoList()
            {
                sg_io_destroy(m_h);
            }

            IoList(const IoList&)            = delete;
            IoList& operator=(const IoList&) = delete;

            template <class Mesh>
            void add(ScalarField<Mesh>& f)
            {
                f.sync_to_device();
                check(sg_io_add_field(m_h, f.handle()), "io");
            }

            template <class Mesh, std::size_t n>
            void add(VectorField<Mesh, n>& f)
            {
                f.sync_to_device();
                check(sg_io_add_vector_field(m_h, f.handle()), "io");
            }

            sg_io_t handle() const
            {
                return m_h;
            }

          private:

            sg_io_t m_h = nullptr;
        };
    }

    template <class Cfg, class... T>
    void save(const std::filesystem::path& path, const std::string& filename, const MRMesh<Cfg>& mesh, const T&... fields)
    {
        detail::IoList l;
        (l.add(const_cast<T&>(fields)), ...);
        detail::check(sg_save(path.string().c_str(), filename.c_str(), mesh.handle(), l.handle()), "save");
    }

    template <class Cfg, class... T>
    void save(const std::string& filename, const MRMesh<Cfg>& mesh, const T&... fields)
    {
        save(std::filesystem::current_path(), filename, mesh, fields...);
    }

    template <class Cfg, class... T>
    void dump(const std::filesystem::path& path, const std::string& filename, const MRMesh<Cfg>& mesh, const T&... fields)
    {
        detail::IoList l;
        (l.add(const_cast<T&>(fields)), ...);
        detail::check(sg_dump(path.string().c_str(), filename.c_str(), mesh.handle(), l.handle()), "dump");
    }

    template <class Cfg, class... T>
    void dump(const std::string& filename, const MRMesh<Cfg>& mesh, const T&... fields)
    {
        dump(std::filesystem::current_path(), filename, mesh, fields...);
    }

    template <class Cfg, class... T>
    void load(const std::filesystem::path& path, const std::string& filename, MRMesh<Cfg>& mesh, T&... fields)
    {
        detail::IoList l;
        (l.add(fields), ...);
        detail::check(sg_load(path.string().c_str(), filename.c_str(), mesh.handle(), l.handle()), "load");
        (fields.sync_to_device(), ...); // the host mirrors are stale
    }

    template <class Cfg, class... T>
    void load(const std::string& filename, MRMesh<Cfg>& mesh, T&... fields)
    {
        load(std::filesystem::current_path(), filename, mesh, fields...);
    }
} // namespace samurai


namespace std
{
    // std::swap(u.array(), unp1.array())
    template <class Mesh>
    void swap(samurai::ScalarField<Mesh>& a, samurai::ScalarField<Mesh>& b)
    {
        swap(a, b);
    }

    template <class Mesh, std::size_t n_comp>
    void swap(samurai::VectorField<Mesh, n_comp>& a, samurai::VectorField<Mesh, n_comp>& b)
    {
        swap(a, b);
    }
}
