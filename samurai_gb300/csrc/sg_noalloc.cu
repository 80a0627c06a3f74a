// sg_field_download_noalloc: u.array() to host memory without allocating.
//
// sg_field_download gathers the dense field into samurai's compact
// numbering through a staging buffer that it allocates (and grows) with
// cudaMalloc.  Some callers cannot let a library allocate device memory: a
// host program whose device memory is entirely reserved by another allocator
// (a framework's caching pool, a fixed budget per process) gets
// cudaErrorMemoryAllocation at an arbitrary point, and a real-time loop must
// not pay for an allocation on its path.  This variant gathers into a
// file-scope device array instead, so it allocates nothing on any path.
//
// Limits and behaviour:
//  - the array holds SG_NOALLOC_MAX_CELLS doubles (16 MiB); every GPU that
//    loads the library holds it until the process exits, and a larger mesh
//    is rejected with SG_ERR_CAPACITY;
//  - the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current, once per device; make
//    that first call before any stream capture;
//  - the device current at the call must be the one the mesh was created on
//    (SG_ERR_ARG otherwise), since the address looked up is that of the
//    current device's copy of the array;
//  - every call shares the one array and leaves its contents behind; each
//    call overwrites the n entries it returns, so nothing needs clearing, but
//    calls that overlap on the GPU (several host threads or meshes at once)
//    race on the array.
#include <cstdio>
#include <mutex>

#include "sg_handles.cuh"

namespace sg
{
    void set_last_error(const char* msg, const char* detail);
}

namespace
{
    constexpr long long SG_NOALLOC_MAX_CELLS = 1LL << 21;
    constexpr int MAX_DEVICES                = 64;

    __device__ __align__(256) double g_download_scratch[SG_NOALLOC_MAX_CELLS];

    std::mutex g_setup_mutex;
    double* g_scratch_ptr[MAX_DEVICES] = {};

    // reported through sg_last_error(); writing the text allocates nothing
    int noalloc_fail(int code, const char* msg, const char* detail = "")
    {
        sg::set_last_error(msg, detail);
        return code;
    }

    // device address of the array on the mesh's device, looked up once per device; that device must be the
    // current one, since the address belongs to the current device's copy of the array
    int scratch_for_device(int mesh_device, double** out)
    {
        int dev       = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess)
        {
            return noalloc_fail(SG_ERR_CUDA, "sg_field_download_noalloc: cudaGetDevice: ", cudaGetErrorString(e));
        }
        if (dev != mesh_device)
        {
            return noalloc_fail(SG_ERR_ARG, "sg_field_download_noalloc: the current device is not the one the mesh was created on");
        }
        if (dev < 0 || dev >= MAX_DEVICES)
        {
            return noalloc_fail(SG_ERR_ARG, "sg_field_download_noalloc: device ordinal beyond 63");
        }
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_ptr[dev])
        {
            void* p = nullptr;
            e       = cudaGetSymbolAddress(&p, g_download_scratch);
            if (e != cudaSuccess || !p)
            {
                return noalloc_fail(SG_ERR_CUDA, "sg_field_download_noalloc: cudaGetSymbolAddress: ", cudaGetErrorString(e));
            }
            g_scratch_ptr[dev] = static_cast<double*>(p);
        }
        *out = g_scratch_ptr[dev];
        return SG_OK;
    }
}

extern "C" int sg_field_download_noalloc(sg_field_t field, double* values, long long n)
try
{
    if (!field || !values)
    {
        return noalloc_fail(SG_ERR_ARG, "sg_field_download_noalloc: null argument");
    }
    sg::Ctx& c        = field->mesh->ctx;
    sg::DeviceMesh& m = c.m();
    if (!m.host_valid)
    {
        cudaError_t e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess)
        {
            return noalloc_fail(SG_ERR_CUDA, "sg_field_download_noalloc: ", cudaGetErrorString(e));
        }
        m.nb_ref     = m.h_lo[0];
        m.nb_cells   = m.h_lo[2];
        m.host_valid = true;
    }
    if (n != m.nb_ref)
    {
        return noalloc_fail(SG_ERR_ARG, "sg_field_download_noalloc: size differs from the reference mesh");
    }
    if (n > SG_NOALLOC_MAX_CELLS)
    {
        return noalloc_fail(SG_ERR_CAPACITY, "sg_field_download_noalloc: the reference mesh exceeds the static staging array of 2^21 cells; "
                                             "use sg_field_download");
    }
    double* scratch = nullptr;
    if (int st = scratch_for_device(c.device, &scratch))
    {
        return st;
    }
    cudaError_t e = sg::launch_gather(c, m, field->f.data, scratch);
    if (e == cudaSuccess)
    {
        e = cudaMemcpyAsync(values, scratch, static_cast<size_t>(n) * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    }
    int fault = 0;
    if (e == cudaSuccess)
    {
        e = sg::read_device_error(c, &fault); // synchronises the stream
    }
    if (e != cudaSuccess)
    {
        return noalloc_fail(SG_ERR_CUDA, "sg_field_download_noalloc: ", cudaGetErrorString(e));
    }
    if (fault)
    {
        return noalloc_fail(SG_ERR_STATE, "sg_field_download_noalloc: a kernel addressed a cell outside the stored level box (invalid mesh)");
    }
    return SG_OK;
}
SG_API_CATCH(sg_field_download_noalloc)
