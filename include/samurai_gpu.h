/*
 * C ABI of the GB300-native samurai MR advection path (libsamurai_gpu.so).
 *
 * samurai (hpc-maths/samurai v0.33.0) is a header-only C++ library with no
 * FFI of its own; its "interface" for this path is the set of C++ calls a
 * user program makes.  Each entry point below replaces one of them, cited
 * next to it (paths relative to the samurai source tree).  The C++ drop-in
 * header include/samurai_gb300/samurai.hpp and the Python package samurai_gb300 are
 * thin layers over these functions.
 *
 * Conventions
 *  - every call returns 0 (SG_OK) or a status code; sg_last_error() gives a
 *    message for the calling thread.  No call aborts the process.
 *  - host arrays are plain pointers with explicit sizes; field values in
 *    host arrays use samurai's storage numbering of the reference mesh
 *    (interval.index + x, level_cell_array.hpp:727-743).
 *  - one mesh owns one CUDA stream; calls on a mesh are issued in order on
 *    that stream by one host thread.
 *  - a mesh may be destroyed before or after its fields: its memory goes
 *    with the last of them.  An IO list (sg_io_t) and a batch borrow the
 *    fields given to them, which must outlive them; an adjoint copies what
 *    it needs at creation.
 *  - there is no CPU fallback: without a usable sm_103a device every call
 *    that computes returns SG_ERR_CUDA.
 */
#ifndef SAMURAI_GPU_H
#define SAMURAI_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sg_mesh_s* sg_mesh_t;
typedef struct sg_field_s* sg_field_t;

enum sg_status
{
    SG_OK           = 0,
    SG_ERR_ARG      = 1,
    SG_ERR_CUDA     = 2,
    SG_ERR_CAPACITY = 3,
    SG_ERR_STATE    = 4,
    SG_ERR_NOTFOUND = 5
};

/* MRMeshId (mr/mesh.hpp:25-33) */
enum sg_mesh_id
{
    SG_CELLS            = 0,
    SG_CELLS_AND_GHOSTS = 1,
    SG_PROJ_CELLS       = 2,
    SG_UNION_CELLS      = 3,
    SG_REFERENCE        = 4
};

/* upwind variants */
enum sg_scheme
{
    SG_UPWIND_OP = 0, /* unp1 = u - dt * samurai::upwind(a, u)  (stencil_field.hpp:91-179, demos/FiniteVolume/advection_2d.cpp:144) */
    SG_README    = 1, /* the README for_each_interval lambda    (README.md:144-153) */
    SG_CONVECTION = 2 /* unp1 = u - dt * conv(u), conv = samurai::make_convection_upwind<Field>(a): the conservative flux
                         form with level-jump interfaces (schemes/fv/operators/convection_lin.hpp:16-89,
                         schemes/fv/flux_based/explicit_flux_based_scheme__lin_hom.hpp:39-319) */
};

const char* sg_last_error(void);
int sg_version(int* major, int* minor);

/* Mesh on the unit box, uniform at max_level: samurai::mra::make_mesh(box, mesh_config<dim, prediction_radius>()
 * .min_level().max_level().max_stencil_radius().graduation_width()) (mr/mesh.hpp:511-518, mesh_config.hpp:16-433),
 * also the deprecated MRMesh<MRConfig<dim>>(box, min_level, max_level) (mr/mesh.hpp:166-181). */
int sg_mesh_create(int dim, int min_level, int max_level, int max_stencil_radius, int prediction_radius, int graduation_width,
                   sg_mesh_t* out);
/* the same with mesh_config<dim>().periodic({periodic[0], .., periodic[dim-1]}) (mesh_config.hpp): periodic axes have no
 * boundary; the mesh wraps around them (mr/mesh.hpp:276-368) and the ghost update copies across them
 * (algorithm/update_periodic.hpp).  periodic may be NULL (no periodic axis).  The flux form (SG_CONVECTION) and the
 * adjoint are not available on meshes with a periodic axis. */
int sg_mesh_create_periodic(int dim, int min_level, int max_level, int max_stencil_radius, int prediction_radius, int graduation_width,
                            const int* periodic, sg_mesh_t* out);
int sg_mesh_destroy(sg_mesh_t mesh);
/* mesh.nb_cells(mesh_id_t::cells) and mesh.nb_cells() (= reference size) (mesh.hpp:530-550) */
int sg_mesh_counts(sg_mesh_t mesh, long long* nb_cells, long long* nb_reference);
/* for_each_cell(mesh, f) (algorithm.hpp:301-363): leaf cells in samurai order with their storage index */
int sg_mesh_get_cells(sg_mesh_t mesh, int* level, int* coords, long long* index, long long capacity);
/* LevelCellArray intervals of mesh[id][level] (level_cell_array.hpp:68-256): records (start, end, y[, z], index) */
int sg_mesh_count_intervals(sg_mesh_t mesh, int mesh_id, int level, long long* n);
int sg_mesh_get_intervals(sg_mesh_t mesh, int mesh_id, int level, long long* out, long long capacity);
/* MRMesh(cl, cfg) from a leaf-cell list (mr/mesh.hpp:152-158); fields keep their storage but their values are void */
int sg_mesh_set_cells(sg_mesh_t mesh, long long n, const int* level, const int* coords);
/* the mesh's CUDA stream (cudaStream_t) for interop */
int sg_mesh_stream(sg_mesh_t mesh, void** stream);
int sg_mesh_synchronize(sg_mesh_t mesh);
/* kernel launches issued on the mesh since the last reset (instrumentation) */
int sg_mesh_launch_count(sg_mesh_t mesh, int reset, long long* count);
/* a number that changes whenever the mesh's cells change (adaptation, sg_mesh_set_cells, sg_load): host caches of
 * the mesh (intervals, cell lists) are current while it stays the same */
int sg_mesh_version(sg_mesh_t mesh, unsigned long long* version);

/* args::refine_boundary, samurai's --refine-boundary flag (arguments.hpp:26, 67; mr/adapt.hpp:341-346): when set,
 * every Harten pass of this mesh tags keep the leaves of max_level within max_stencil_radius cells of the domain
 * boundary (keep_boundary_refined, mr/adapt.hpp:245-274), so the boundary stays refined at max_level.  Off by default,
 * as in samurai; it applies to the adaptations of this mesh (a process-wide flag in samurai). */
int sg_mesh_set_refine_boundary(sg_mesh_t mesh, int enable);

/* Without a samurai counterpart: how an adaptation runs.  enable = 1: the whole of sg_adapt / sg_adapt_fields (and
 * of sg_step) is one captured graph in which each Harten pass, the second half of a pass (new mesh, update_fields)
 * and the graduation iterations run under device-side conditions (conditional graph nodes), with one host
 * synchronisation at the end; enable = 0 (the default, unless the launch-shape cache chose otherwise): pass by pass,
 * one captured graph per half pass and the host reading the fixed-point test after each pass.  Both give the same
 * results; the named timers and the kernel trace use the pass-by-pass path while they are on. */
int sg_mesh_set_adapt_graph(sg_mesh_t mesh, int enable);

/* Without a samurai counterpart: the launch-shape autotuner.  Times sg_step(u, unp1, eps, regularity, a, dt, scheme)
 * over `steps` steps from the problem's current state under candidate launch shapes (threads per block of the FP64
 * list kernels, grid limit of the word launches, level sizes up to which the ghost-update and tag-finalisation
 * chains run in one block, the adaptation path of sg_mesh_set_adapt_graph, two levels per launch in the
 * tag-finalisation chain), each step after an untimed 256 MiB
 * write that empties the L2 (a scratch array held during the call), keeps the fastest on the mesh and caches it for
 * this device and level range (later meshes start from it; SG_TUNE_FILE names a file that keeps the cache across
 * processes; the SG_BLOCK, SG_MAX_BLOCKS, SG_FUSE_WORDS*, SG_GRAPHED_ADAPT, SG_LEVEL_PAIRS environment variables
 * override it).  The
 * problem is left in the state it had.  default_ms / tuned_ms receive the step time under the starting and the
 * chosen shape. */
int sg_autotune(sg_field_t u, sg_field_t unp1, double eps, double regularity, const double* a, double dt, int scheme, int steps,
                double* default_ms, double* tuned_ms);
/* the mesh's launch shape: threads per block, grid limit (blocks of 8 warps), one-block chain limits in words per
 * level of the mesh, field and tag-finalisation chains, 1 when the adaptation runs as one graph with conditional
 * nodes (0: pass by pass), 1 when the tag-finalisation chain takes two levels per launch; any pointer may be NULL */
int sg_launch_shape(sg_mesh_t mesh, int* block, long long* max_blocks, long long* fuse_mesh_words, long long* fuse_field_words,
                    long long* fuse_max_words, int* graphed_adapt, int* level_pairs);

/* samurai's named timers (timers.hpp:111-1036, printed with --timers): CUDA-event timers per phase.
 * ids: 0 mesh adaptation, 1 ghost update, 2 detail computation, 3 tag cells, 4 tag finalization,
 * 5 mesh update, 6 make_graduation, 7 mesh construction, 8 fields update, 9 field expressions (upwind). */
int sg_timers_enable(sg_mesh_t mesh, int enable);
int sg_timers_get(sg_mesh_t mesh, int timer_id, double* total_ms, long long* calls);
int sg_timers_reset(sg_mesh_t mesh);

/* Instrumentation without a samurai counterpart: a per-launch trace of the mesh's kernels.  While on
 * (sg_kernel_trace(mesh, 1)), every kernel launch on the mesh's stream is followed by an event (inside
 * captured launch sequences too), and the time from the previous event to it is that launch's share of
 * the timeline.  sg_kernel_trace(mesh, 0) stops; sg_kernel_trace_read then returns, for entry i (0, 1, ...;
 * SG_ERR_NOTFOUND past the last), a kernel name, its launches and their summed time in ms, in order of first
 * launch.  *valid is 0 when one captured sequence ran twice in the window (trace one step at a time). */
int sg_kernel_trace(sg_mesh_t mesh, int enable);
int sg_kernel_trace_read(sg_mesh_t mesh, int i, const char** name, long long* launches, double* ms, int* valid);

/* Instrumentation without a samurai counterpart: the device's FP64 rate (non-fused adds and multiplies
 * per second, in GFLOP/s), measured by a throughput probe kernel.  The FP64 pipe bounds this path on GB300. */
int sg_device_fp64_rate(double* gflops);

/* samurai::make_scalar_field<double>(name, mesh) (field/scalar_field.hpp:173-216) */
int sg_field_create(sg_mesh_t mesh, const char* name, sg_field_t* out);
int sg_field_destroy(sg_field_t field);
/* samurai::make_bc<samurai::Dirichlet<1>>(u, value) (bc/bc.hpp:786-800, bc/dirichlet.hpp:22-29) */
int sg_field_set_dirichlet(sg_field_t field, double value);
/* u.array() in the reference numbering, host memory (n = nb_reference) */
int sg_field_upload(sg_field_t field, const double* values, long long n);
int sg_field_download(sg_field_t field, double* values, long long n);
/* the same with device memory (n = nb_reference), e.g. torch tensors */
int sg_field_upload_device(sg_field_t field, const double* dvalues, long long n);
int sg_field_download_device(sg_field_t field, double* dvalues, long long n);
/* u[cell] for the leaf cells in for_each_cell order (n = nb_cells); other entries become 0 on upload */
int sg_field_set_cells(sg_field_t field, const double* values, long long n);
int sg_field_get_cells(sg_field_t field, double* values, long long n);
/* u.fill(value) (field/field_base.hpp): every reference cell, ghosts included */
int sg_field_fill(sg_field_t field, double value);
/* std::swap(u.array(), unp1.array()) (demos/FiniteVolume/advection_2d.cpp:146) */
int sg_field_swap(sg_field_t a, sg_field_t b);

/* auto MRadaptation = samurai::make_MRAdapt(u); MRadaptation(mra_config().epsilon(eps).regularity(reg))
 * (mr/adapt.hpp:147-203, 391-420); n_harten receives the number of Harten passes */
int sg_adapt(sg_field_t u, double eps, double regularity, int* n_harten);
/* one Harten pass (mr/adapt.hpp:276-389); converged = 1 at the fixed point */
int sg_harten(sg_field_t u, int ite, double eps, double regularity, int* converged);
/* the same with mra_config().relative_detail(relative_detail): details divided by max |u| over the leaf cells
   (mr/adapt.hpp:319-322, mr/rel_detail.hpp:75-111) */
int sg_adapt_ex(sg_field_t u, double eps, double regularity, int relative_detail, int* n_harten);
int sg_harten_ex(sg_field_t u, int ite, double eps, double regularity, int relative_detail, int* converged);
/* auto MRadaptation = samurai::make_MRAdapt(f_0, .., f_{n-1}); MRadaptation(mra_config, o_0, .., o_{n_other-1})
   (mr/adapt.hpp:96-203): the details of the n fields (one component each) decide the mesh, a cell being coarsened
   when every component is small and refined when one is large (mr/criteria.hpp:45-107); the n fields and the
   n_other fields are carried to the new mesh (update_ghost_mr of the others first, mr/adapt.hpp:383-385).
   All fields live on one mesh. */
int sg_adapt_fields(int n, const sg_field_t* fields, int n_other, const sg_field_t* others, double eps, double regularity,
                    int relative_detail, int* n_harten);
/* samurai::update_ghost_mr(f_0, .., f_{n-1}) (algorithm/update_ghost_mr.hpp:261-270) */
int sg_update_ghost_mr_fields(int n, const sg_field_t* fields);
/* samurai::update_ghost_mr(u) (algorithm/update_ghost_mr.hpp:261-270) */
int sg_update_ghost_mr(sg_field_t u);
/* unp1 = u - dt * samurai::upwind(a, u) on mesh[cells] (a has dim entries), or one of the other schemes above */
int sg_upwind(sg_field_t u, sg_field_t unp1, const double* a, double dt, int scheme);
/* One iteration of the demo's time loop (demos/FiniteVolume/advection_2d.cpp:140-147): MRadaptation(eps, regularity),
   samurai::update_ghost_mr(u), unp1 = u - dt * scheme(a, u), std::swap(u.array(), unp1.array()).  The same results as
   the four calls; the whole step is one captured CUDA graph (passes and buffers decided on the device) with one host
   synchronisation.  n_harten receives the adaptation's Harten passes. */
int sg_step(sg_field_t u, sg_field_t unp1, double eps, double regularity, const double* a, double dt, int scheme, int* n_harten);
/* detail and tag fields of the last Harten pass, reference numbering (n = nb_reference) */
int sg_detail_download(sg_field_t u, double* values, long long n);
int sg_tag_download(sg_field_t u, unsigned char* values, long long n);

/* VectorField<mesh, double, n_comp>: samurai::make_vector_field<double, n_comp>(name, mesh)
 * (field/vector_field.hpp:134-237).  Held on the device as n_comp scalar component fields of the mesh; every scalar
 * call accepts a component (sg_vector_field_component), so make_MRAdapt(v, u)(cfg) is sg_adapt_fields over v's
 * components followed by u (the detail of several fields lists their components in order, mr/adapt.hpp:74-95).
 * Host arrays keep samurai's layout, the values of a cell side by side: element (k, c) at k * n_comp + c
 * (storage shape {size, n_comp}, field/vector_field.hpp:38).  1 <= n_comp <= SG_MAX_COMPONENTS. */
enum
{
    SG_MAX_COMPONENTS = 16
};
typedef struct sg_vfield_s* sg_vfield_t;
int sg_vector_field_create(sg_mesh_t mesh, const char* name, int n_comp, sg_vfield_t* out);
int sg_vector_field_destroy(sg_vfield_t v);
int sg_vector_field_n_comp(sg_vfield_t v, int* n_comp);
int sg_vector_field_component(sg_vfield_t v, int c, sg_field_t* out);
/* samurai::make_bc<samurai::Dirichlet<1>>(v, values[0], .., values[n_comp-1]) (bc/bc.hpp:752-800) */
int sg_vector_field_set_dirichlet(sg_vfield_t v, const double* values);
/* v.array() in the reference numbering (n = n_comp * nb_reference) */
int sg_vector_field_upload(sg_vfield_t v, const double* values, long long n);
int sg_vector_field_download(sg_vfield_t v, double* values, long long n);
/* v[cell] for the leaf cells in for_each_cell order (n = n_comp * nb_cells) */
int sg_vector_field_set_cells(sg_vfield_t v, const double* values, long long n);
int sg_vector_field_get_cells(sg_vfield_t v, double* values, long long n);
/* std::swap(v.array(), vnp1.array()) */
int sg_vector_field_swap(sg_vfield_t a, sg_vfield_t b);
/* make_MRAdapt(v)(mra_config().epsilon(eps).regularity(reg).relative_detail(relative_detail)) (mr/adapt.hpp:147-203) */
int sg_vector_adapt(sg_vfield_t v, double eps, double regularity, int relative_detail, int* n_harten);
/* samurai::update_ghost_mr(v) (algorithm/update_ghost_mr.hpp:261-270) */
int sg_vector_update_ghost_mr(sg_vfield_t v);
/* unp1 = u - dt * samurai::upwind(a, u) component by component (stencil_field.hpp:91-179), or another scheme */
int sg_vector_upwind(sg_vfield_t u, sg_vfield_t unp1, const double* a, double dt, int scheme);

/* Output and restart files (io/hdf5.hpp, io/restart.hpp), written and read without libhdf5.  A field list
 * (sg_io_t) names the fields of a call in order, as the variadic fields... of samurai's functions. */
typedef struct sg_io_s* sg_io_t;
int sg_io_create(sg_io_t* out);
int sg_io_destroy(sg_io_t io);
int sg_io_add_field(sg_io_t io, sg_field_t field);
int sg_io_add_vector_field(sg_io_t io, sg_vfield_t field);
/* samurai::save(path, filename, mesh, fields...) (io/hdf5.hpp:1331-1336): <path>/<filename>.h5 holding
 * /mesh/points, /mesh/connectivity (corner ids in order of first appearance over for_each_cell, io/hdf5.hpp:85-144)
 * and /mesh/fields/<name> (<name>_<c> per component of a vector field), and <path>/<filename>.xdmf.
 * fields may be NULL; path NULL or "" is the current directory. */
int sg_save(const char* path, const char* filename, sg_mesh_t mesh, sg_io_t fields);
/* samurai::dump(path, filename, mesh, fields...) (io/restart.hpp:188-201): the leaf CellArray and the fields */
int sg_dump(const char* path, const char* filename, sg_mesh_t mesh, sg_io_t fields);
/* dimension and levels of a restart file, to create the mesh that sg_load fills */
int sg_restart_levels(const char* path, const char* filename, int* dim, int* min_level, int* max_level);
/* samurai::load(path, filename, mesh, fields...) (io/restart.hpp:425-463): the mesh becomes the file's leaf cells
 * (MRMesh(ca, cfg)) and each field gets its leaf values; the mesh must have the file's dimension and levels
 * (samurai recreates it with them). */
int sg_load(const char* path, const char* filename, sg_mesh_t mesh, sg_io_t fields);

/* u.array() to host memory without allocating anything (no counterpart in the reference: samurai has no
 * C interface).  For callers that cannot let a library allocate device memory, e.g. a process whose device
 * memory is reserved by another allocator.  Same output as sg_field_download, through a static 16 MiB device
 * array instead of an allocated staging buffer: meshes beyond 2^21 reference cells are rejected with
 * SG_ERR_CAPACITY.  The first call on a device sets the array up (make it before any stream capture); calls
 * share the array, so calls that overlap on the GPU race. */
int sg_field_download_noalloc(sg_field_t field, double* values, long long n);

/* Batched mode: n independent problems (u[k], unp1[k] on a mesh of their own, meshes may differ in dimension and
 * levels) advanced together.  samurai has no batched API: the calls below stand for a user's loop over problems
 * that makes, for each k, the calls of the time loop of demos/FiniteVolume/advection_2d.cpp:140-147.  The
 * instances run concurrently on their own streams, driven by n_threads host threads (instance k on thread
 * k mod n_threads); results are those of the serial calls on each instance.  Per-instance arrays: eps[k],
 * regularity[k], dt[k], a[3k .. 3k+dim-1] (stride 3 whatever the dimension), n_harten[k] (may be NULL). */
typedef struct sg_batch_s* sg_batch_t;
int sg_batch_create(int n, const sg_field_t* u, const sg_field_t* unp1, int n_threads, sg_batch_t* out);
int sg_batch_destroy(sg_batch_t batch);
int sg_batch_size(sg_batch_t batch, int* n);
/* MRadaptation_k(eps[k], regularity[k]) for every k (mr/adapt.hpp:147-203) */
int sg_batch_adapt(sg_batch_t batch, const double* eps, const double* regularity, int* n_harten);
/* samurai::update_ghost_mr(u[k]) for every k (algorithm/update_ghost_mr.hpp:261-270) */
int sg_batch_update_ghost_mr(sg_batch_t batch);
/* unp1[k] = u[k] - dt[k] * samurai::upwind(a_k, u[k]) for every k (stencil_field.hpp:91-179) */
int sg_batch_upwind(sg_batch_t batch, const double* a, const double* dt, int scheme);
/* std::swap(u[k].array(), unp1[k].array()) for every k */
int sg_batch_swap(sg_batch_t batch);
/* one time step of every instance: adapt, update_ghost_mr, upwind, swap (advection_2d.cpp:140-147) */
int sg_batch_step(sg_batch_t batch, const double* eps, const double* regularity, const double* a, const double* dt, int scheme,
                  int* n_harten);
int sg_batch_synchronize(sg_batch_t batch);

/* Without a samurai counterpart: the batch's launch-shape autotuner.  Times `steps` batched steps (sg_batch_step)
 * from the instances' current state under candidate shapes (the level size, in words, up to which every instance's
 * ghost-update, tag-finalisation and mesh chains run their levels in one block; the threads per block of their FP64
 * list kernels), each from the same saved state and each step after an untimed 256 MiB write that empties the L2;
 * keeps the fastest and leaves every instance's mesh and values as they were.  default_ms / tuned_ms receive the
 * batched step time under the starting and the chosen shape. */
int sg_batch_autotune(sg_batch_t batch, const double* eps, const double* regularity, const double* a, const double* dt, int scheme,
                      int steps, double* default_ms, double* tuned_ms);
/* the batch's launch shape: one-block chain limit in words per level, threads per block (0: each instance's own) */
int sg_batch_launch_shape(sg_batch_t batch, long long* fuse_words, int* block);

/* Discrete adjoint of the time loop (no counterpart in samurai, which has no derivatives).  The loop of
 * demos/FiniteVolume/advection_2d.cpp:140-147 (MRadaptation(eps, regularity); update_ghost_mr; upwind; swap)
 * is recorded with its mesh sequence; derivatives are those of the loop on the recorded meshes (adaptation
 * decisions are piecewise constant).  Fields are leaf values in for_each_cell order (algorithm.hpp:301-363):
 * u0 on the initial mesh (the leaf cells of u when the adjoint is created), uT on the final mesh.  The dense
 * field is checkpointed every checkpoint_every steps; the backward pass recomputes each segment from its
 * checkpoint.  a has dim entries; ga receives dim entries.  The leaf-value arrays u0, uT, gT and g0 may be host
 * memory or device memory of the mesh's GPU (told apart by unified addressing); device inputs must be complete
 * before the call, and every call returns with its outputs written. */
typedef struct sg_adjoint_s* sg_adjoint_t;
int sg_adjoint_create(sg_field_t u, int checkpoint_every, sg_adjoint_t* out);
int sg_adjoint_destroy(sg_adjoint_t adj);
/* leaf counts of the initial and final meshes and the number of recorded steps */
int sg_adjoint_counts(sg_adjoint_t adj, long long* n0, long long* nT, int* n_steps);
/* leaf cells (level, dim coordinates) of the initial (which = 0) or final (which = 1) mesh */
int sg_adjoint_cells(sg_adjoint_t adj, int which, int* level, int* coords, long long n);
/* forward with adaptation from u0: n_steps of the loop, recording meshes and checkpoints */
int sg_adjoint_record(sg_adjoint_t adj, const double* u0, int n_steps, double eps, double regularity, const double* a, double dt, int scheme,
                      long long* nT);
/* uT of the last forward (record or replay) */
int sg_adjoint_final(sg_adjoint_t adj, double* uT, long long nT);
/* the recorded steps on the recorded meshes from u0 with velocity a; uT may be NULL */
int sg_adjoint_replay(sg_adjoint_t adj, const double* u0, const double* a, double* uT);
/* reverse pass at the last forward: gT = dJ/duT gives g0 = dJ/du0 and ga = dJ/da */
int sg_adjoint_backward(sg_adjoint_t adj, const double* gT, double* g0, double* ga);

#ifdef __cplusplus
}
#endif

#endif /* SAMURAI_GPU_H */
