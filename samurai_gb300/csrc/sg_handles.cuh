// Opaque handle types of the C ABI (include/samurai_gpu.h).
#pragma once

#include "../../include/samurai_gpu.h"
#include "sg_ctx.cuh"

struct sg_mesh_s
{
    sg::Ctx ctx;
    double* staging     = nullptr; // compact host<->device staging (nb_ref doubles)
    long long staging_n = 0;
};

struct sg_field_s
{
    sg_mesh_s* mesh = nullptr;
    sg::DeviceField f;
};
