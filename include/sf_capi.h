/*
 * sf_capi.h -- C ABI of the GB300-native coupled SPH-DEM seepage-flow substep.
 *
 * One opaque handle owns the device state of one or more independent scenes
 * (a single scene is the reference's CudaSFSystem; several scenes are the
 * batched ensemble). Every entry point returns an sf_status, never throws and
 * never traps; the text of the last failure is available from
 * sf_last_error_string().
 *
 * Reference interfaces each entry point replaces (paths are inside the
 * sph_seepage_flows project):
 *   sf_create            CudaSFParticles ctor (seepage_flows_cuda/include/kiri_pbs_cuda/particle/cuda_sf_particles.cuh:131-165),
 *                        CudaBoundaryParticles ctor (include/kiri_pbs_cuda/particle/cuda_boundary_particles.cuh:29-36),
 *                        CudaGNSearcher / CudaGNBoundarySearcher ctors (src/kiri_pbs_cuda/searcher/cuda_neighbor_searcher.cu:19-62,118-123),
 *                        CudaWCSphSFSolver ctor (include/kiri_pbs_cuda/solver/seepageflow/cuda_wcsph_sf_solver.cuh:22-32),
 *                        CudaSFSystem ctor incl. boundary volume (src/kiri_pbs_cuda/system/cuda_sf_system.cu:17-64,121-136)
 *   sf_step              CudaBaseSystem::UpdateSystem (src/kiri_pbs_cuda/system/cuda_base_system.cu:29-56)
 *                        -> CudaSFSystem::OnUpdateSolver (src/kiri_pbs_cuda/system/cuda_sf_system.cu:66-119)
 *   sf_num_substeps      CudaBaseSystem::GetNumOfSubTimeSteps (include/kiri_pbs_cuda/system/cuda_base_system.cuh:36)
 *   sf_frame_adaptive    the adaptive frame loop of seepage_flows/src/seepageflow/main.cpp:235-247
 *   sf_get_field         CudaSFParticles::Get*Ptr getters (include/kiri_pbs_cuda/particle/cuda_sf_particles.cuh:170-190)
 *   sf_get_fields / sf_set_fields  several of those fields in one call (no reference counterpart)
 *   sf_get_cell_table    CudaGNBaseSearcher::GetCellStart / GetGridSize (include/kiri_pbs_cuda/searcher/cuda_neighbor_searcher.cuh:35-44)
 *   sf_export_bgeo       ExportBgeoFileCUDA (seepage_flows/include/kiri_utils.h:364-448) with a handle's particle arrays
 *   sf_export_bgeo_device ExportBgeoFileCUDA itself (device arrays in the reference's layout)
 *   sf_read_bgeo         ReadBgeoFileForGPU (seepage_flows/include/kiri_utils.h:252-302)
 *   sf_add_sph_particles CudaSFParticles::AddSphParticles (src/kiri_pbs_cuda/particle/cuda_sf_particles.cu:50-68)
 *   sf_run_stage         the protected per-pass methods of CudaSphSFSolver (src/kiri_pbs_cuda/solver/seepage_flow/cuda_sph_sf_solver.cu:20-402)
 *   sf_substeps_fixed    fixed-substep mode of main.cpp:250-258 (no reference counterpart for the graph capture)
 *   sf_reset_order       no reference counterpart (creation order back, for repeatable runs from a reset state)
 *   sf_create_batched    no reference counterpart (independent scenes in one launch)
 *   sf_adjoint_run       no reference counterpart (reverse-mode gradient of a trajectory loss)
 *   sf_set_adjoint_seed_scale  no reference counterpart (range of the adjoint's FP32 cotangents)
 *   sf_autotune          no reference counterpart (list capacity and block sizes of the passes)
 *   sf_set_density_staging / sf_get_density_staging  no reference counterpart (shared-memory staging of the density pass's candidates)
 *   sf_get_list_capacity no reference counterpart (neighbour list capacity and its growth)
 *
 * Threading: handles are independent; one handle must not be used from two
 * host threads at once. All work is issued on the stream given at creation.
 */
#ifndef SF_CAPI_H
#define SF_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SF_CAPI_VERSION 1

typedef int32_t sf_status;
enum {
    SF_OK = 0,
    SF_ERR_INVALID = 1,     /* bad argument, size or parameter */
    SF_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    SF_ERR_CAPACITY = 3,    /* particle count would exceed the capacity */
    SF_ERR_DEVICE = 4,      /* the device error word is set (see sf_check_error) */
    SF_ERR_NO_DEVICE = 5,   /* no CUDA device is visible */
    SF_ERR_UNSUPPORTED = 6  /* request not supported by the library */
};

/* CudaSphSolverType (include/kiri_pbs_cuda/data/cuda_sph_params.h:19-24) */
enum { SF_SOLVER_SPH = 0, SF_SOLVER_WCSPH = 1 };
/* CudaSeepageflowType (include/kiri_pbs_cuda/data/cuda_seepageflow_params.h:19-23) */
enum { SF_TYPE_SF = 0, SF_TYPE_MULTI_SF = 1 };
/* particle labels (include/kiri_pbs_cuda/solver/seepageflow/cuda_sph_sf_solver_gpu.cuh:434) */
enum { SF_LABEL_WATER = 0, SF_LABEL_SAND = 1 };

/* CudaSeepageflowParams (include/kiri_pbs_cuda/data/cuda_seepageflow_params.h:25-69), field for field. */
typedef struct sf_params {
    float sph_mass, sph_density, sph_particle_radius, sph_kernel_radius;
    float sph_stiff, sph_visc, sph_nu, sph_bnu;
    float dem_mass, dem_density, dem_particle_radius, dem_kernel_radius;
    float dem_young, dem_poisson, dem_tan_friction_angle, dem_damping;
    float sf_c0, sf_csat, sf_cmc, sf_cmc_p, sf_cd;
    float sf_a0, sf_asat, sf_amc, sf_amc_p;
    float sf_dry_sand_color[3];
    float sf_wet_sand_color[3];
    float gravity[3];
    float dt;
    int32_t solver_type; /* SF_SOLVER_* */
    int32_t sf_type;     /* SF_TYPE_* */
} sf_params;

/* CudaBoundaryParams (include/kiri_pbs_cuda/data/cuda_boundary_params.h:19-27). The grid of
 * the fluid and boundary searchers is lowest_point, kernel_radius and grid_size. */
typedef struct sf_boundary_params {
    float kernel_radius;
    float lowest_point[3];
    float highest_point[3];
    float world_size[3];
    float world_center[3];
    int32_t grid_size[3];
} sf_boundary_params;

/* CudaWCSphSFSolver ctor arguments (cuda_wcsph_sf_solver.cuh:22-32) and the
 * fixed CFL factors (cuda_wcsph_sf_solver.cuh:59-60). */
typedef struct sf_solver_params {
    float negative_scale;        /* default 0 */
    float time_step_limit_scale; /* default 3 */
    float speed_of_sound;        /* default 100 */
} sf_solver_params;

/* Host-side initial state of one scene (the vectors handed to the
 * CudaSFParticles and CudaBoundaryParticles ctors). vel, cda0asat and amcamcp
 * may be NULL (zero-filled, as the reference's cudaMemset-cleared arrays). */
typedef struct sf_scene_init {
    int64_t n;
    const float* pos;        /* n*3 */
    const float* vel;        /* n*3 or NULL */
    const float* col;        /* n*3 */
    const int32_t* label;    /* n, SF_LABEL_* */
    const float* mass;       /* n, > 0 */
    const float* radius;     /* n */
    const float* cda0asat;   /* n*3 or NULL */
    const float* amcamcp;    /* n*2 or NULL */
    int64_t nb;
    const float* bpos;       /* nb*3 */
    const int32_t* blabel;   /* nb (0 = world wall, 1 = scene shape) */
} sf_scene_init;

/* Per-particle fields, named after the reference getters. */
enum {
    SF_FIELD_POS = 0,            /* f32 x3 */
    SF_FIELD_VEL = 1,            /* f32 x3 */
    SF_FIELD_ACC = 2,            /* f32 x3 */
    SF_FIELD_COL = 3,            /* f32 x3 */
    SF_FIELD_LABEL = 4,          /* i32 */
    SF_FIELD_RADIUS = 5,         /* f32 */
    SF_FIELD_MASS = 6,           /* f32 */
    SF_FIELD_DENSITY = 7,        /* f32 */
    SF_FIELD_PRESSURE = 8,       /* f32 */
    SF_FIELD_VOIDAGE = 9,        /* f32 */
    SF_FIELD_SATURATION = 10,    /* f32 */
    SF_FIELD_MAX_SATURATION = 11,/* f32 */
    SF_FIELD_AVG_FLOW = 12,      /* f32 x3 */
    SF_FIELD_AVG_DRAG = 13,      /* f32 x3 (sand; 0 for water) */
    SF_FIELD_ADHESION = 14,      /* f32 x3 (water) */
    SF_FIELD_AVG_ADHESION = 15,  /* f32 x3 (water; 0 for sand) */
    SF_FIELD_CDA0ASAT = 16,      /* f32 x3 */
    SF_FIELD_AMCAMCP = 17,       /* f32 x2 */
    SF_FIELD_ID = 18,            /* i32: creation index of the particle */
    SF_FIELD_KEY = 19,           /* i32: scene-local cell key of the last sort */
    SF_FIELD_NEIGHBORS = 20,     /* i32: particles within the interaction reach at the last
                                    density pass, the particle itself included */
    SF_FIELD_COUNT = 21,
    SF_BFIELD_POS = 32,          /* f32 x3, boundary particles in sorted order */
    SF_BFIELD_LABEL = 33,        /* i32 */
    SF_BFIELD_VOLUME = 34        /* f32 (Akinci volume) */
};

/* Element order of sf_get_field / sf_set_field. */
enum {
    SF_ORDER_SORTED = 0, /* current cell-sorted order: what the reference getters return */
    SF_ORDER_ID = 1      /* creation order (index = particle id) */
};

/* Passes that sf_run_stage runs, in substep order. */
enum {
    SF_STAGE_SORT = 0,              /* hash, stable radix sort by cell, reorder, cell tables */
    SF_STAGE_DENSITY = 1,           /* density + Tait/linear pressure */
    SF_STAGE_AVGFLOW = 2,           /* average flow, fluid voidage, saturation */
    SF_STAGE_VOIDAGE_ADHESION = 3,  /* sand voidage, water adhesion, wet-sand colour; also each
                                       water particle's rho / voidage and pressure term, which the
                                       momentum stages read (set density, pressure or voidage
                                       before this stage, not after it) */
    SF_STAGE_SAND_MOMENTUM = 4,     /* acc = g + sand forces; average drag */
    SF_STAGE_WATER_MOMENTUM = 5,    /* acc = g + water forces; max |acc| */
    SF_STAGE_INTEGRATE = 6,         /* CFL dt, damping, Euler, water clamp, next keys */
    SF_STAGE_COUNT = 7
};

/* Bits of the device error word. */
enum {
    SF_DEVERR_NONFINITE = 1u << 0,  /* NaN/Inf in a position or acceleration */
    SF_DEVERR_KEY_RANGE = 1u << 1,  /* a cell key outside the scene's grid */
    SF_DEVERR_CELL_TABLE = 1u << 2, /* cell table inconsistent with the sort */
    SF_DEVERR_TIMEOUT = 1u << 3     /* a bounded device wait gave up */
};

typedef struct sf_handle sf_handle;

/* Library identification; usable without a GPU. */
const char* sf_version(void);
int32_t sf_capi_version(void);

/* Number of visible CUDA devices (0 when none). */
int32_t sf_device_count(void);

/* Create a single-scene handle. capacity >= init->n bounds later emitter growth.
 * stream is a cudaStream_t (NULL = the legacy default stream). */
sf_status sf_create(const sf_params* params, const sf_boundary_params* bparams,
                    const sf_solver_params* sparams, const sf_scene_init* init,
                    int64_t capacity, void* stream, sf_handle** out);

/* Create a handle over n_scenes independent scenes (arrays of n_scenes entries);
 * every substep of the handle advances all scenes in the same launches. */
sf_status sf_create_batched(int32_t n_scenes, const sf_params* params,
                            const sf_boundary_params* bparams, const sf_solver_params* sparams,
                            const sf_scene_init* inits, const int64_t* capacities,
                            void* stream, sf_handle** out);

sf_status sf_destroy(sf_handle* h);

/* Replace the parameters of one scene (the reference reads its global params
 * at every UpdateSystem call). */
sf_status sf_set_params(sf_handle* h, int32_t scene, const sf_params* params);
sf_status sf_get_params(const sf_handle* h, int32_t scene, sf_params* params);

/* One reference substep of every scene: UpdateSystem(render_interval) with the
 * CFL sub-step count (WCSPH) or render_interval/params.dt (SPH) and
 * dt = render_interval / N_sub. n_substeps_out (scene 0's N_sub) and ms_out
 * (elapsed device time) may be NULL. */
sf_status sf_step(sf_handle* h, float render_interval, int64_t* n_substeps_out, float* ms_out);

/* n substeps of every scene at a fixed dt, replayed from captured CUDA graphs.
 * Calls of up to 64 substeps return without waiting for the GPU. Longer calls
 * wait, after each block of 64 substeps, until the block before it has run
 * (the GPU keeps the newer block queued), so that the neighbour lists can grow
 * within the call (see sf_get_list_capacity). */
sf_status sf_substeps_fixed(sf_handle* h, float dt, int64_t n);

/* Puts every scene's particles back in creation order (slot = particle id),
 * no reference counterpart. The sort of the next substep is stable, so its
 * order among the particles of a cell (and with it the FP32 order of every
 * neighbour sum) follows the order before it: a state reset by particle id
 * (sf_set_field with SF_ORDER_ID) after this call repeats a fresh handle's
 * run bit for bit, where without it the previous run's order would carry
 * over. The cell tables are invalid until the next substep. */
sf_status sf_reset_order(sf_handle* h);

/* One frame of the reference adaptive loop: while remaining > 1e-6:
 * sf_step(remaining); remaining -= remaining / N_sub. Single-scene handles only. */
sf_status sf_frame_adaptive(sf_handle* h, float render_interval, int64_t* n_calls_out);

/* Run one pass of the substep (parity testing; the reference's per-pass
 * solver methods). time_arg is the render interval when adaptive != 0, else dt. */
sf_status sf_run_stage(sf_handle* h, int32_t stage, float time_arg, int32_t adaptive);

/* Copy a field of one scene to dst (device pointer when dst_on_device, else
 * host). count = number of particles (or boundary particles for SF_BFIELD_*)
 * to copy; must equal the scene's live count. */
sf_status sf_get_field(sf_handle* h, int32_t scene, int32_t field, int32_t order,
                       void* dst, int64_t count, int32_t dst_on_device);
sf_status sf_set_field(sf_handle* h, int32_t scene, int32_t field, int32_t order,
                       const void* src, int64_t count, int32_t src_on_device);

/* Several fields of one scene in one call: the copies of fields[k] to / from
 * dsts[k] / srcs[k] are queued back to back and the call waits once (for host
 * buffers), instead of once per field. Same rules per field as sf_get_field /
 * sf_set_field. */
sf_status sf_get_fields(sf_handle* h, int32_t scene, int32_t n_fields, const int32_t* fields, int32_t order,
                        void* const* dsts, int64_t count, int32_t dst_on_device);
sf_status sf_set_fields(sf_handle* h, int32_t scene, int32_t n_fields, const int32_t* fields, int32_t order,
                        const void* const* srcs, int64_t count, int32_t src_on_device);

/* Cell start table of one scene (which = 0 particles, 1 boundary), as
 * scene-relative offsets: G+1 entries, entry G = the scene's count. */
sf_status sf_get_cell_table(sf_handle* h, int32_t scene, int32_t which, int64_t* dst, int64_t count);

/* Houdini classic .bgeo files (the format the reference reads and writes
 * through partio). The export writes folder_path/file_name.bgeo (creating
 * the folder) with the point attributes position, Cd (float 3), pscale
 * (float 1) and label (int 1), one point per particle:
 *   sf_export_bgeo: one scene of a handle, in the current (cell-sorted)
 *     order, as the reference exports its particle arrays after a frame;
 *   sf_export_bgeo_device: n particles from device arrays in the reference's
 *     layout (float3 positions and colours, float radii, size_t labels),
 *     issued on `stream` (NULL: the default stream); errors go to
 *     sf_last_error_string(NULL).
 * The records are packed big-endian on the GPU; both calls return after the
 * file is written. */
sf_status sf_export_bgeo(sf_handle* h, int32_t scene, const char* folder_path, const char* file_name);
sf_status sf_export_bgeo_device(const char* folder_path, const char* file_name, const float* pos3, const float* col3,
                                const float* radius, const uint64_t* labels, int64_t n, void* stream);

/* Reads the points of a .bgeo file as ReadBgeoFileForGPU does: 4 floats per
 * point (x, y, z, pscale), pscale 0.01 when the file has no float pscale
 * attribute, y and z swapped when flip_yz. Host only (no GPU work). With
 * xyzs_out == NULL it only stores the point count in *n_out; otherwise
 * capacity (points) must hold them all. Errors go to sf_last_error_string(NULL). */
sf_status sf_read_bgeo(const char* path, int32_t flip_yz, float* xyzs_out, int64_t capacity, int64_t* n_out);
sf_status sf_get_grid(const sf_handle* h, int32_t scene, int32_t grid_size[3], int64_t* n_cells);

sf_status sf_size(const sf_handle* h, int32_t scene, int64_t* n, int64_t* capacity);
sf_status sf_num_scenes(const sf_handle* h, int32_t* n_scenes);
sf_status sf_num_substeps(sf_handle* h, int32_t scene, int64_t* n_sub);

/* Append water particles (CudaSFParticles::AddSphParticles). Returns
 * SF_ERR_CAPACITY (and adds nothing) when size + n >= capacity, as the
 * reference does. */
sf_status sf_add_sph_particles(sf_handle* h, int32_t scene, const float* pos3, int64_t n,
                               const float col[3], const float vel[3], float mass, float radius);

/* Read and clear the device error word (SF_DEVERR_* bits). */
sf_status sf_check_error(sf_handle* h, uint32_t* flags);

/* Wait for all work of the handle. */
sf_status sf_synchronize(sf_handle* h);

/* Number of kernel launches the handle has issued so far (graph replays count
 * every kernel node). */
sf_status sf_launch_count(const sf_handle* h, int64_t* launches);

/* Neighbour list capacity (entries per particle) and how many times the
 * handle has grown it (no reference counterpart: the reference walks the 27
 * cells in every pass). A density pass that finds a particle's list full
 * records the particle's neighbour count; the particle's later passes walk the
 * stencil instead (same results, slower). sf_step, sf_substeps_fixed and
 * sf_adjoint_run read those records once the GPU has reached them and
 * re-allocate the lists for the largest count + 25% + 8, a multiple of 32 up
 * to 256. Any pointer may be NULL. */
sf_status sf_get_list_capacity(const sf_handle* h, int32_t* capacity, int64_t* growths);

/* Launch configuration of the passes: threads per block (32, 64, 128 or 256)
 * for every tuned pass, and the particles each thread handles (1); 0 keeps a
 * value. Takes effect at the next substep (captured graphs are dropped). */
sf_status sf_set_tuning(sf_handle* h, int32_t block_size, int32_t items_per_thread);

/* Threads per particle of the neighbour passes and of the adjoint pair
 * kernels (no reference counterpart): 1, 2, 4 or 8, or 0 for the automatic
 * choice (doubled up to 8 while fewer than 2048 threads per SM would run,
 * i.e. 1 for large scenes). The density, average-flow and voidage/adhesion
 * results and the neighbour lists are the same for every value; the
 * momentum sums are grouped differently (FP32 rounding only). Takes effect
 * at the next substep (captured graphs are dropped). */
sf_status sf_set_lanes(sf_handle* h, int32_t lanes);

/* Shared-memory staging of the density pass (no reference counterpart), for
 * one thread per particle: 1 makes each block copy the stencil columns of its
 * particles' one or two (x, y) cell columns into shared memory and test every
 * candidate from there (blocks spanning more columns, or with more candidates
 * than 14 per thread, walk global memory); 0 walks global memory. Lists and
 * results are identical either way; sf_autotune times both. Takes effect at
 * the next substep (captured graphs are dropped). */
sf_status sf_set_density_staging(sf_handle* h, int32_t staged);
sf_status sf_get_density_staging(const sf_handle* h, int32_t* staged);

/* Autotuner (no reference counterpart). Sizes the neighbour lists for the
 * current state (list capacity = largest neighbour count + 25%, a multiple of
 * 32 in [64, 256]; sf_create does this once for the initial state), then
 * times on the current state, with CUDA events: the radix sort with 8, 4, 2
 * and 1 keys per thread (tile size) and with 8-bit or wider digits, and, for
 * 1, 2, 4 and 8 threads per
 * particle, each neighbour pass with 64, 128 and 256 threads per block
 * (density, average flow, voidage/adhesion, sand momentum, water momentum;
 * the integrator keeps its size; with one thread per particle the density
 * pass with and without its shared-memory staging); it keeps the fastest sort tiles and the
 * lane count with the smallest sum of its passes' best times, with those
 * block sizes. The state is not advanced. block_sizes_out (6 entries, in
 * that pass order then the integrator) and list_capacity_out may be NULL;
 * sf_get_tuning reads every choice back. */
sf_status sf_autotune(sf_handle* h, float dt, int32_t* block_sizes_out, int32_t* list_capacity_out);

/* The current launch configuration (no reference counterpart): block sizes
 * (6 entries, as sf_autotune), threads per particle of the neighbour passes,
 * keys per thread of the radix sort tiles and bits per radix digit (8, or
 * 9-11 where wider digits save a pass). Any pointer may be NULL. */
sf_status sf_get_tuning(const sf_handle* h, int32_t* block_sizes_out, int32_t* lanes_out, int32_t* sort_items_out,
                        int32_t* sort_digit_bits_out);

/* Text of the last error on this handle (or of the last failed create when h is NULL). */
const char* sf_last_error_string(const sf_handle* h);

/* Gradient of a trajectory loss by reverse-mode differentiation (no reference
 * counterpart: the reference has no adjoint).
 *
 * Runs n_substeps substeps of every scene at the fixed dt from the current
 * state (the same trajectory sf_substeps_fixed computes), evaluates per scene
 *     L = (1 / N_sand) * sum over sand particles of |x_T - target|^2
 * and back-propagates it through every substep. The substeps of one segment
 * of checkpoint_every substeps are stored as they run (neighbour lists and
 * intermediate fields, about 0.7 KB per particle slot and substep); earlier
 * segments keep only a checkpoint of their starting state (76 bytes per slot)
 * and are recomputed once in the reverse sweep. checkpoint_every >= n_substeps
 * stores the whole trajectory and recomputes nothing (fastest); smaller values
 * trade one extra forward pass for memory.
 *
 * Arrays are scene-major over the handle's scenes and ordered by particle id
 * within a scene (the creation order), 3 floats per particle:
 *   target_pos       in:  sum(n) * 3 target positions (water entries unused)
 *   loss_out         out: n_scenes losses
 *   grad_params_out  out: n_scenes * 3: dL/d tan(friction angle), dL/d capillary
 *                         scale (a factor on c0, cmc, csat), dL/d permeability
 *                         scale (a factor on cd), each at its current value   (may be NULL)
 *   grad_pos0_out    out: sum(n) * 3: dL/d initial positions                    (may be NULL)
 *   grad_vel0_out    out: sum(n) * 3: dL/d initial velocities                   (may be NULL)
 *   ms_out           out: [forward ms, reverse ms] of device time               (may be NULL)
 * All pointers are host memory. On return the handle holds the final state
 * x_T, v_T; the per-substep fields (density, pressure, ...) hold the values of
 * the first substep until the next substep runs. The push-out of water from
 * shape-boundary particles (label 1) is held constant in the gradient. */
sf_status sf_adjoint_run(sf_handle* h, float dt, int64_t n_substeps, int64_t checkpoint_every,
                         const float* target_pos, float* loss_out, float* grad_params_out,
                         float* grad_pos0_out, float* grad_vel0_out, float* ms_out);

/* Seed scale of one scene's adjoint (no reference counterpart). The reverse
 * sweep of sf_adjoint_run carries its cotangents in FP32, and over long
 * horizons they grow exponentially (contact and liquid-bridge stiffness,
 * the stiff Tait pressure) until they overflow. With scale s the scene's
 * cotangents are seeded with s x dL/dx_T, so every cotangent of the sweep is
 * s times the unscaled one, and sf_adjoint_run divides s out of the returned
 * gradients in FP64. A power of two changes no rounding: the gradients equal
 * the unscaled ones bit for bit wherever neither overflows nor reaches the
 * subnormal range. scale must be finite and > 0; the default is 1; it is kept
 * until set again (sf_set_params leaves it). */
sf_status sf_set_adjoint_seed_scale(sf_handle* h, int32_t scene, float scale);

/* Allocation-free cell sort (no counterpart in the reference; its neighbour
 * searcher allocates its buffers in the CudaGNSearcher constructor).
 *
 * The sort stage of a single-scene handle without a handle and without any
 * device allocation: cell keys of n positions (Pos2GridHash on `grid`), a
 * stable radix sort and the cell-start table. Scratch lives in a static
 * device array sized for at most SF_NOALLOC_MAX_PARTICLES particles
 * (about 4.5 MB per device); larger n is rejected with SF_ERR_INVALID.
 *   pos_dev             in:  n * 3 floats, device memory
 *   perm_out_dev        out: n ints, device: perm[i] = input index of the
 *                            i-th particle in cell order (stable)
 *   cell_start_out_dev  out: G + 1 ints, device, G = grid cells:
 *                            first sorted index with cell >= c; entry G = n
 *   stream              the CUDA stream to use (NULL = the legacy default stream)
 * Every call copies a flag word to host memory and waits for its stream
 * before returning, and returns SF_ERR_DEVICE when a position is not finite;
 * the output buffers then hold unspecified values. The first call on a
 * device looks up the scratch address (cudaGetSymbolAddress), which may load
 * the module: make the first call before any stream capture. The lookup is
 * repeated when the cached address no longer belongs to the device (after
 * cudaDeviceReset). Calls that overlap on the GPU (two streams or host
 * threads) share the scratch and race: serialise them. Errors are reported
 * by sf_last_error_string(NULL). */
#define SF_NOALLOC_MAX_PARTICLES 262144
sf_status sf_cell_sort_noalloc(const sf_boundary_params* grid, const float* pos_dev, int64_t n,
                               int32_t* perm_out_dev, int32_t* cell_start_out_dev, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SF_CAPI_H */
