// VectorField (field/vector_field.hpp:28-233) over the scalar C ABI.
//
// A vector field of n_comp components is held on the device as n_comp scalar
// component fields of one mesh (component-major: each component is a dense
// FP64 slab, so every kernel of the path reads a component with the same
// coalesced accesses as a scalar field).  This is exact with respect to
// samurai's vector semantics on this path:
//  - make_MRAdapt(v): the detail field has v's n_comp components
//    (mr/adapt.hpp:86-95), the criteria test them together
//    (mr/criteria.hpp:45-107), and relative details divide each component by
//    its own max (mr/rel_detail.hpp:35-52) -- which is sg_adapt_fields over
//    the components, one detail component per component field;
//  - update_ghost_mr, update_fields, upwind and the flux form act component by
//    component with the same arithmetic as for a scalar field
//    (algorithm/update_ghost_mr.hpp, stencil_field.hpp:91-179);
//  - make_bc<Dirichlet<1>>(v, v_0, ..) gives each component its own value.
// Only the host layout of v.array() differs from a scalar field: samurai
// stores the n_comp values of a cell side by side (storage shape
// {nb_cells, n_comp}, field/vector_field.hpp:38), so element (k, c) of the
// host array is k * n_comp + c.
#include <cstdio>
#include <vector>

#include "../../include/samurai_gpu.h"
#include "sg_ctx.cuh"

#include "sg_handles.cuh"


namespace
{
    int vfail(const char* msg)
    {
        sg::set_last_error(msg, nullptr);
        return SG_ERR_ARG;
    }

    bool same_shape(sg_vfield_t a, sg_vfield_t b)
    {
        return a && b && a->mesh == b->mesh && a->comp.size() == b->comp.size();
    }

    // element k of component c in the host layout of v.array() / v[cell]
    inline size_t at(const sg_vfield_s& v, long long k, size_t c)
    {
        return static_cast<size_t>(k) * v.comp.size() + c;
    }

    long long count_of(sg_vfield_t v, bool cells)
    {
        long long nc = 0, nr = 0;
        if (sg_mesh_counts(v->mesh, &nc, &nr))
        {
            return -1;
        }
        return cells ? nc : nr;
    }

    // host copy in or out of the components, one scalar call per component
    template <class Scalar>
    int move_host(sg_vfield_t v, double* values, long long n, bool cells, bool upload, Scalar scalar, const char* what)
    {
        if (!v || !values)
        {
            return vfail(what);
        }
        const long long nb = count_of(v, cells);
        if (nb < 0)
        {
            return SG_ERR_CUDA;
        }
        const size_t nc = v->comp.size();
        if (n != nb * static_cast<long long>(nc))
        {
            return vfail(upload ? "sg_vector_field upload: n must be n_comp times the mesh size"
                                : "sg_vector_field download: n must be n_comp times the mesh size");
        }
        std::vector<double> one(static_cast<size_t>(nb));
        for (size_t c = 0; c < nc; ++c)
        {
            if (upload)
            {
                for (long long k = 0; k < nb; ++k)
                {
                    one[static_cast<size_t>(k)] = values[at(*v, k, c)];
                }
            }
            if (int st = scalar(v->comp[c], one.data(), nb))
            {
                return st;
            }
            if (!upload)
            {
                for (long long k = 0; k < nb; ++k)
                {
                    values[at(*v, k, c)] = one[static_cast<size_t>(k)];
                }
            }
        }
        return SG_OK;
    }
} // namespace

extern "C"
{
    int sg_vector_field_create(sg_mesh_t mesh, const char* name, int n_comp, sg_vfield_t* out)
    try
    {
        if (!mesh || !out || n_comp < 1 || n_comp > SG_MAX_COMPONENTS)
        {
            return vfail("sg_vector_field_create: need a mesh, 1 <= n_comp <= SG_MAX_COMPONENTS and an output handle");
        }
        sg_vfield_s* v = new (std::nothrow) sg_vfield_s();
        if (!v)
        {
            sg::set_last_error("sg_vector_field_create: out of host memory", nullptr);
            return SG_ERR_CAPACITY;
        }
        v->mesh = mesh;
        v->name = name ? name : "";
        for (int c = 0; c < n_comp; ++c)
        {
            char nm[256];
            std::snprintf(nm, sizeof(nm), "%s_%d", name ? name : "", c);
            sg_field_t f = nullptr;
            if (int st = sg_field_create(mesh, nm, &f))
            {
                sg_vector_field_destroy(v);
                return st;
            }
            v->comp.push_back(f);
        }
        *out = v;
        return SG_OK;
    }
    SG_API_CATCH(sg_vector_field_create)

    int sg_vector_field_destroy(sg_vfield_t v)
    try
    {
        if (v)
        {
            for (auto* f : v->comp)
            {
                sg_field_destroy(f);
            }
            delete v;
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_vector_field_destroy)

    int sg_vector_field_n_comp(sg_vfield_t v, int* n_comp)
    try
    {
        if (!v || !n_comp)
        {
            return vfail("sg_vector_field_n_comp: null argument");
        }
        *n_comp = static_cast<int>(v->comp.size());
        return SG_OK;
    }
    SG_API_CATCH(sg_vector_field_n_comp)

    int sg_vector_field_component(sg_vfield_t v, int c, sg_field_t* out)
    try
    {
        if (!v || !out || c < 0 || c >= static_cast<int>(v->comp.size()))
        {
            return vfail("sg_vector_field_component: no such component");
        }
        *out = v->comp[static_cast<size_t>(c)];
        return SG_OK;
    }
    SG_API_CATCH(sg_vector_field_component)

    int sg_vector_field_set_dirichlet(sg_vfield_t v, const double* values)
    try
    {
        if (!v || !values)
        {
            return vfail("sg_vector_field_set_dirichlet: null argument");
        }
        for (size_t c = 0; c < v->comp.size(); ++c)
        {
            if (int st = sg_field_set_dirichlet(v->comp[c], values[c]))
            {
                return st;
            }
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_vector_field_set_dirichlet)

    int sg_vector_field_upload(sg_vfield_t v, const double* values, long long n)
    try
    {
        return move_host(v, const_cast<double*>(values), n, false, true, sg_field_upload, "sg_vector_field_upload: null argument");
    }
    SG_API_CATCH(sg_vector_field_upload)

    int sg_vector_field_download(sg_vfield_t v, double* values, long long n)
    try
    {
        return move_host(v, values, n, false, false, sg_field_download, "sg_vector_field_download: null argument");
    }
    SG_API_CATCH(sg_vector_field_download)

    int sg_vector_field_set_cells(sg_vfield_t v, const double* values, long long n)
    try
    {
        return move_host(v, const_cast<double*>(values), n, true, true, sg_field_set_cells, "sg_vector_field_set_cells: null argument");
    }
    SG_API_CATCH(sg_vector_field_set_cells)

    int sg_vector_field_get_cells(sg_vfield_t v, double* values, long long n)
    try
    {
        return move_host(v, values, n, true, false, sg_field_get_cells, "sg_vector_field_get_cells: null argument");
    }
    SG_API_CATCH(sg_vector_field_get_cells)

    int sg_vector_field_swap(sg_vfield_t a, sg_vfield_t b)
    try
    {
        if (!same_shape(a, b) || a == b)
        {
            return vfail("sg_vector_field_swap: need two distinct vector fields of one mesh with the same n_comp");
        }
        for (size_t c = 0; c < a->comp.size(); ++c)
        {
            if (int st = sg_field_swap(a->comp[c], b->comp[c]))
            {
                return st;
            }
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_vector_field_swap)

    int sg_vector_adapt(sg_vfield_t v, double eps, double regularity, int relative_detail, int* n_harten)
    try
    {
        if (!v)
        {
            return vfail("sg_vector_adapt: null field");
        }
        return sg_adapt_fields(static_cast<int>(v->comp.size()), v->comp.data(), 0, nullptr, eps, regularity, relative_detail, n_harten);
    }
    SG_API_CATCH(sg_vector_adapt)

    int sg_vector_update_ghost_mr(sg_vfield_t v)
    try
    {
        if (!v)
        {
            return vfail("sg_vector_update_ghost_mr: null field");
        }
        return sg_update_ghost_mr_fields(static_cast<int>(v->comp.size()), v->comp.data());
    }
    SG_API_CATCH(sg_vector_update_ghost_mr)

    int sg_vector_upwind(sg_vfield_t u, sg_vfield_t unp1, const double* a, double dt, int scheme)
    try
    {
        if (!same_shape(u, unp1) || u == unp1 || !a)
        {
            return vfail("sg_vector_upwind: need two distinct vector fields of one mesh with the same n_comp, and a velocity");
        }
        for (size_t c = 0; c < u->comp.size(); ++c)
        {
            if (int st = sg_upwind(u->comp[c], unp1->comp[c], a, dt, scheme))
            {
                return st;
            }
        }
        return SG_OK;
    }
    SG_API_CATCH(sg_vector_upwind)
}
