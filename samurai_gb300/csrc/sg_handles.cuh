// Opaque handle types of the C ABI (include/samurai_gpu.h).
#pragma once

#include <exception>
#include <new>

#include "../../include/samurai_gpu.h"
#include "sg_ctx.cuh"

namespace sg
{
    void set_last_error(const char* msg, const char* detail);
}

// The handler of every C entry point's function-try-block: no C++ exception (a host allocation that fails,
// a library throw) leaves the C ABI; it becomes a status code and sg_last_error().
#define SG_API_CATCH(fn)                                                                                                   \
    catch (const std::bad_alloc&)                                                                                          \
    {                                                                                                                      \
        sg::set_last_error(#fn ": out of host memory", nullptr);                                                          \
        return SG_ERR_CAPACITY;                                                                                            \
    }                                                                                                                      \
    catch (const std::exception& e)                                                                                        \
    {                                                                                                                      \
        sg::set_last_error(#fn ": ", e.what());                                                                            \
        return SG_ERR_ARG;                                                                                                 \
    }                                                                                                                      \
    catch (...)                                                                                                            \
    {                                                                                                                      \
        sg::set_last_error(#fn ": unexpected exception", nullptr);                                                        \
        return SG_ERR_ARG;                                                                                                 \
    }

struct sg_mesh_s
{
    sg::Ctx ctx;
    double* staging     = nullptr; // compact host<->device staging (nb_ref doubles)
    long long staging_n = 0;
    // fields created on the mesh and not yet destroyed: sg_mesh_destroy of a mesh that still has fields
    // only marks it, and the last sg_field_destroy frees it, so that no destruction order touches freed memory
    long long attached = 0;
    bool destroyed     = false;
};

struct sg_field_s
{
    sg_mesh_s* mesh = nullptr;
    sg::DeviceField f;
};

// VectorField<mesh, double, n_comp> (field/vector_field.hpp:134-216): n_comp
// scalar component fields on one mesh
struct sg_vfield_s
{
    sg_mesh_s* mesh = nullptr;
    std::string name;
    std::vector<sg_field_s*> comp;
};
