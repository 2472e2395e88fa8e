/* vfs_cuda.h — C ABI of the GB300-native WCSPH step (VkFluidSim's WCSPHWithBoundaryModel).
 *
 * Plain C types only: host pointers, sizes, an opaque handle and an int status. No call throws.
 * Every entry point names the reference interface it replaces (paths are relative to the
 * VkFluidSim source tree). One handle serves one host thread at a time; work is enqueued on the
 * handle's CUDA stream (vfs_model_set_stream) and host-visible results are returned after the
 * stream has been synchronised.
 *
 * Vectors on the host are packed float3 (12 bytes per particle, the reference's scalar layout).
 * Particle arrays are in the model's current (sorted) order; ids[] map them back to the order in
 * which they were first set (the reference permutes positions and velocities in place every
 * substep and keeps no ids: src/models/model.cpp:210-223).
 */
#ifndef VFS_CUDA_H
#define VFS_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference aborts through VK_CHECK, src/gfx/common.h:20-29) ---- */
#define VFS_OK 0
#define VFS_ERR_INVALID_ARGUMENT 1
#define VFS_ERR_CUDA 2
#define VFS_ERR_OUT_OF_MEMORY 3
#define VFS_ERR_IO 4
#define VFS_ERR_PARSE 5
#define VFS_ERR_CAPACITY 6
#define VFS_ERR_DEVICE_CHECK 7 /* a kernel reported an error word (e.g. look-back timeout) */
#define VFS_ERR_NOT_READY 8

typedef struct vfs_model vfs_model;

/* SimulationParameters, src/simulation.h:10-13 (defaults g = (0,-9.81,0), h = 0.2,
 * src/simulation.cpp:20-27). */
typedef struct vfs_sim_params {
    float gravity[3];
    float smooth_radius;
} vfs_sim_params;

/* SPHModel::Parameters, src/models/model.h:14-21 (gfx::BoundingBox is {size, pos},
 * src/gfx/mesh.h:13-16). n_particles is the model capacity. */
typedef struct vfs_sph_params {
    float time_scale;
    int32_t iterations;
    int32_t n_particles;
    float fixed_dt;
    float target_density;
    float bbox_size[3];
    float bbox_pos[3];
} vfs_sph_params;

/* WCSPHWithBoundaryModel::Parameters, src/models/wcsph_with_boundary_model.h:26-33
 * (defaults 1e4, 1000, 7, 0.01: src/models/wcsph_with_boundary_model.cpp:27-36). */
typedef struct vfs_wcsph_params {
    float wall_stiffness;
    float stiffness;
    float expoent;
    float viscosity_strenght;
} vfs_wcsph_params;

/* WCSPHWithBoundaryModel::BoundaryObjectInfo, src/models/wcsph_with_boundary_model.h:16-24:
 * transform = inverse of the object's world matrix, rotation = mat4 of its rotation, both glm
 * column-major (element (row r, column c) at [c*4 + r]); the grids are host arrays of
 * resolution[0]*resolution[1]*resolution[2] floats indexed x + nx*(y + ny*z) and are copied. */
typedef struct vfs_boundary_object {
    float transform[16];
    float rotation[16];
    float box_size[3];
    float box_pos[3];
    uint32_t resolution[3];
    const float* sdf_grid;
    const float* volume_map_grid;
} vfs_boundary_object;

/* An analytic boundary shape whose SDF grid and volume map the library builds on the GPU, in
 * place of the reference's OBJ mesh -> MeshSDF -> GenerateVolumeMap chain
 * (src/scenes/generic_scene.cpp:88-124, src/util/volume_map.cpp:9-54). The placement fields are
 * the scene JSON's boundaryObjects[] keys (src/util/scene_loader.cpp:75-111). */
#define VFS_SHAPE_SPHERE 0    /* params[0] = radius */
#define VFS_SHAPE_BOX 1       /* params[0..2] = half extents, solid */
#define VFS_SHAPE_CONTAINER 2 /* params[0..2] = half extents, fluid inside (inverted box) */
typedef struct vfs_analytic_object {
    int32_t shape;
    double params[3];
    float position[3];
    float rotation_angle_deg;
    float rotation_axis[3];
    float scale[3];
    uint32_t resolution[3];
} vfs_analytic_object;

/* A triangle-mesh boundary object: GenericScene's ObjectDef (src/scenes/generic_scene.h) with the
 * mesh given as an OBJ file (its last object, polygons triangulated as fans; LoadObjMesh,
 * src/util/mesh_loader.cpp) or as arrays (obj_path NULL). */
typedef struct vfs_mesh_object {
    const char* obj_path;
    const float* vertices;      /* n_vertices x 3 */
    uint32_t n_vertices;
    const uint32_t* triangles;  /* n_triangles x 3 vertex indices */
    uint32_t n_triangles;
    float position[3];
    float rotation_angle_deg;
    float rotation_axis[3];
    float scale[3];
    uint32_t resolution[3];
} vfs_mesh_object;

/* Thread-local message of the last failing call on this thread. */
const char* vfs_last_error(void);
/* Library version string. */
const char* vfs_version(void);
/* Number of CUDA devices visible to the library (0 when there is none or no driver). */
int vfs_device_count(void);

/* ---- model lifecycle: SPHModel / WCSPHWithBoundaryModel (src/models/model.h:58-64) ---- */

/* WCSPHWithBoundaryModel(sph, wcsph) + Init (src/models/wcsph_with_boundary_model.cpp:39-79,
 * src/models/model.cpp:82-98): allocates every device buffer for sph->n_particles particles. */
int vfs_model_create(const vfs_sim_params* sim, const vfs_sph_params* sph,
                     const vfs_wcsph_params* wcsph, vfs_model** out);
/* SPHModel::Clear (src/models/model.cpp:102-111). */
int vfs_model_destroy(vfs_model* m);
/* The CUDA stream (a cudaStream_t passed as void*) all later work is enqueued on; NULL selects
 * the handle's own non-blocking stream. */
int vfs_model_set_stream(vfs_model* m, void* stream);
/* Simulation::SetGlobalParameters (src/simulation.cpp:47-51) and the parameter edits of
 * DrawDebugUI (src/models/model.cpp:236-263, wcsph_with_boundary_model.cpp:119-141). Any
 * argument may be NULL. n_particles is ignored (the capacity is fixed at create). */
int vfs_model_set_parameters(vfs_model* m, const vfs_sim_params* sim, const vfs_sph_params* sph,
                             const vfs_wcsph_params* wcsph);
int vfs_model_get_parameters(const vfs_model* m, vfs_sim_params* sim, vfs_sph_params* sph,
                             vfs_wcsph_params* wcsph);
uint32_t vfs_model_num_particles(const vfs_model* m);

/* GenericScene::AddBoundaryObject + CreateBoundaryObjectBuffer
 * (src/scenes/generic_scene.cpp:88-145), from prepared grids. */
int vfs_model_add_boundary_object(vfs_model* m, const vfs_boundary_object* obj);
/* The same from an analytic shape: SDF grid and 16^3-point Gauss-Legendre volume map are
 * generated on the GPU over the shape's box grown by a margin of 8h
 * (MeshSDF::Build, src/util/mesh_sdf.cpp:28-44, with margin 8h from generic_scene.cpp:100). */
int vfs_model_add_analytic_object(vfs_model* m, const vfs_analytic_object* obj);
/* The same for a triangle mesh (GenericScene::AddBoundaryObject, src/scenes/generic_scene.cpp:89-124):
 * the SDF grid holds the mesh's signed distance (nearest triangle through a BVH, sign from
 * angle-weighted pseudonormals; SignedDistanceToMesh, src/util/geometry.cpp:267-328) at the nodes
 * of the mesh bounds grown by 8h, and the volume map integrates it, both on the GPU. */
int vfs_model_add_mesh_object(vfs_model* m, const vfs_mesh_object* obj);
uint32_t vfs_model_num_boundary_objects(const vfs_model* m);
/* Reads back boundary object idx: matrices and box into *info (grid pointers set to NULL), and
 * the grids into sdf_out / vm_out when they are not NULL. */
int vfs_model_get_boundary_object(const vfs_model* m, uint32_t idx, vfs_boundary_object* info,
                                  float* sdf_out, float* vm_out);

/* ---- state: SPHModel::SetParticleState / SetParticlesInBox / CopyDataBuffers ---- */

/* SetParticleState (src/models/model.h:77-81, model.cpp:139-147): writes count particles at
 * offset (count < 0: all from offset); densities of those particles are zeroed. ids are set to
 * offset + i. An upload of every particle keeps the model's candidate lists usable when the
 * particles stay near the positions the slots held (a host round trip of the model's own
 * state); an upload of part of the scene leaves them to be rebuilt. */
int vfs_model_set_particle_state(vfs_model* m, const float* pos, const float* vel,
                                 uint32_t offset, int64_t count);
/* SetParticlesInBox in Compact mode (src/models/model.cpp:117-137, 35-66): a lattice with
 * spacing cbrt(1 / target_density), zero velocity. mode 1 (Random) draws uniform positions from
 * a seeded generator (the reference seeds from std::random_device). */
int vfs_model_set_particles_in_box(vfs_model* m, const float box_size[3], const float box_pos[3],
                                   uint32_t offset, int64_t count, int32_t mode, uint64_t seed);
/* SPHModel::CopyDataBuffers (src/models/model.cpp:158-170), into host arrays; any may be NULL.
 * acc is the acceleration of the last substep (recorded only while field recording is on). */
int vfs_model_copy_data_buffers(vfs_model* m, float* pos, float* vel, float* dens, float* acc);
/* One host round trip: SetParticleState of every particle from pos / vel (both NULL: keep the
 * state), `substeps` substeps, then CopyDataBuffers into pos_out / vel_out / dens_out (any may be
 * NULL), with a single wait at the end, as the reference's frame records Step and
 * CopyDataBuffers into one command buffer (src/models/model.cpp:158-170) behind its staged
 * SetParticleState (model.cpp:139-147). When every given output is page-locked, the last
 * substep writes them itself (its density pass the densities, its force pass positions and
 * velocities), so the read-back overlaps those passes; otherwise the outputs are packed after the
 * substeps. Results equal those of the three separate calls.
 * Single-scene models only. */
int vfs_model_step_host(vfs_model* m, const float* pos, const float* vel, int32_t substeps,
                        float* pos_out, float* vel_out, float* dens_out);
int vfs_model_get_ids(vfs_model* m, uint32_t* ids);
/* Neighbour arrays of the last substep: SpatialHash keys / sorted_indices / spatial_offsets
 * (src/compute/spatial_hash.h:15-17; offsets hold N for empty keys). Any may be NULL. */
int vfs_model_get_neighbor_arrays(vfs_model* m, uint32_t* keys, uint32_t* sorted_indices,
                                  uint32_t* offsets);
/* Boundary density Psi_b and gradient of the last substep (VolumeMapBuffers,
 * src/models/wcsph_with_boundary_model.cpp:19-22). */
int vfs_model_get_boundary_fields(vfs_model* m, float* boundary_density,
                                  float* boundary_gradient);
/* Keep the per-particle acceleration of every substep for copy_data_buffers (off by default:
 * the fused force pass otherwise never stores it). */
int vfs_model_record_fields(vfs_model* m, int32_t enable);

/* ---- stepping: WCSPHWithBoundaryModel::Step (src/models/wcsph_with_boundary_model.cpp:81-117) */

/* One Simulation::Step: `iterations` substeps of dt = time_scale * fixed_dt / iterations. */
int vfs_model_step(vfs_model* m);
/* count substeps. */
int vfs_model_substeps(vfs_model* m, int32_t count);
/* Capture each substep as a CUDA graph (default on). */
int vfs_model_use_graph(vfs_model* m, int32_t enable);
/* Waits for the stream and reads the device error word; VFS_ERR_DEVICE_CHECK if set. */
int vfs_model_synchronize(vfs_model* m);
/* count substeps without graphs, with events between passes; phase_ms[6] receives the mean
 * milliseconds per substep of: keys+moved flags, radix sort+merge, cell ranges+reorder, density,
 * force+integrate, and a sixth slot with nothing enqueued between its events (the event overhead
 * alone: the sort scratch is cleared by the cell pass). */
int vfs_model_profile_substeps(vfs_model* m, int32_t count, float* phase_ms);
/* Sort tuning: digit width in bits (4..8) and items per thread of a onesweep tile (8, 12, 16). */
int vfs_model_set_sort_config(vfs_model* m, int32_t digit_bits, int32_t tile_items);
int vfs_model_get_sort_config(const vfs_model* m, int32_t* digit_bits, int32_t* tile_items,
                              int32_t* passes);
/* Neighbour-list slots per particle (default 128, range [16, 4096], 4 bytes per particle each).
 * A particle with more in-range neighbours makes the force pass walk its candidates again and a
 * differentiable rollout fail with VFS_ERR_CAPACITY, so dense scenes want more slots. Results do
 * not depend on the capacity. The getter returns -1 for a NULL handle. */
int vfs_model_set_neighbor_capacity(vfs_model* m, int32_t slots);
int32_t vfs_model_get_neighbor_capacity(const vfs_model* m);
/* Candidate lists with a skin (Verlet lists). At a build, each particle lists the particles within
 * h (1 + skin); until some particle of the scene has moved more than h skin / 2 since then
 * (checked every substep from the current positions, so state set by any route is seen), a
 * particle whose list was built from 125 provably distinct cell keys sums the list instead of
 * walking the 27 buckets of CalculateDensities (wcsph_with_boundary_model.slang:153-197). The
 * in-range sets are the reference's; the sums follow the visiting order of the last build. Lists
 * that go stale within 12 substeps of their build (a build substep costs about two walks) make
 * the scene wait up to 256 substeps before building again (it walks meanwhile), so the lists pay
 * off where the fastest particle moves less than about h skin / 24 per substep and cost a few
 * percent where particles move faster. skin in [0, 0.5],
 * default 0.05; 0 walks the buckets every substep. Models of up to ~39,000 particles (three lanes
 * per particle in the density pass) and models whose lists do not fit in device memory (224 bytes
 * per particle) have no lists; the getter then reports 0. */
int vfs_model_set_skin(vfs_model* m, float skin);
int vfs_model_get_skin(const vfs_model* m, float* skin);
/* Block-per-cell staging in the density pass's bucket walk (CalculateDensities,
 * wcsph_with_boundary_model.slang:153-197): a warp whose particles share one row of
 * cells loads the 3 x 3 rows of cells around it into shared memory once and tests every staged
 * particle against each of its own, instead of each thread walking its 27 buckets from global
 * memory. Results are bit-identical either way. Off by default; the autotuner's choice
 * (vfs_tune_config.walk_staging) turns it on for workloads where it is faster. */
int vfs_model_set_walk_staging(vfs_model* m, int32_t enable);
/* Number of list builds so far (synchronises the handle's stream). */
int vfs_model_get_skin_builds(vfs_model* m, uint32_t* builds);
/* Device pointers of the current state: float4 (x, y, z, id bits) and (vx, vy, vz, 0). They stay
 * valid for the model's lifetime. Positions and velocities written through them (ordered with
 * the model's stream) are what the next substep steps: every substep recomputes each particle's
 * key from its position, as UpdateSpatialHash does. */
int vfs_model_device_state(vfs_model* m, void** pos4, void** vel4);

/* ---- headless state export (the "record particle positions" roadmap item, README.md:30, in
 * place of the render hand-off SPHModel::CopyDataBuffers, src/models/model.cpp:158-170) ----
 * A snapshot is `<prefix>.bin` (positions f32[N][3], velocities f32[N][3], densities f32[N], each
 * indexed by particle id, little-endian, back to back) and `<prefix>.json` (format
 * "vkfluidsim_gb300.state" version 1: offsets, shapes, substep count, simulation parameters). */
int vfs_model_export_state(vfs_model* m, const char* path_prefix);
/* Loads a snapshot of the same particle count (positions and velocities, ids = file order). */
int vfs_model_import_state(vfs_model* m, const char* path_prefix);
/* Runs `substeps` substeps, writing a snapshot `<prefix>_f<frame, 6 digits>` every `every`
 * substeps; file writes overlap the following substeps (two pinned buffers, a writer thread). */
int vfs_model_record(vfs_model* m, int32_t substeps, int32_t every, const char* path_prefix);

/* ---- headless rendering (the particle pass of src/gui/scene_renderer.cpp:101-109 and
 * assets/shaders/draw/particles_3d.slang, into a host RGBA8 image instead of a swapchain) ----
 * model_view, proj: column-major 4x4 (glm layout), as the reference's Particle3DDrawPipeline push
 * constants. Each particle is a screen-facing quad of side quad_side (view units; the reference
 * draws 0.15) shaded as a sphere impostor: colour = IDL Mac-style colour map of |v| / v_max
 * (reference 6.5) times max(0, n . normalize(0, 1, 1)), depth of view + depth_radius * n
 * (reference 0.15), nearest wins (LESS_OR_EQUAL). rgba: width * height * 4 bytes, row 0 at NDC
 * y = -1; depth (optional): width * height floats, 1 where no particle. */
int vfs_model_render_particles(vfs_model* m, const float* model_view, const float* proj,
                               int32_t width, int32_t height, float quad_side, float depth_radius,
                               float v_max, uint8_t* rgba, float* depth);

/* ---- density field and density raymarch (assets/shaders/draw/raymarch.slang as drawn by
 * DensityRaymarchDrawPipeline::Draw, src/pipelines/raymarch_pipeline.cpp:62-115; an extension
 * for the field: the reference raymarches a precomputed 3D grid) ----
 * vfs_model_density_grid: SPH density sum_j m W(|x - x_j|) of the current particles at the nodes
 * of a regular grid over [lo, hi] (node (i, j, k) at lo + (i, j, k) (hi - lo) / (res - 1); res[a]
 * = 1 puts one node at lo[a]), stored x fastest: grid[(k res[1] + j) res[0] + i]. grid: device,
 * page-locked or pageable memory, res[0] res[1] res[2] floats. Float atomics: the sums' last
 * bits vary from run to run. */
int vfs_model_density_grid(vfs_model* m, const float* lo, const float* hi, const int32_t* res,
                           float* grid);
/* Raymarches the scalar field (res[0] x res[1] x res[2] floats, x fastest, host or device memory)
 * occupying the box center +- half_extent, the reference placing it at 0 +- field_size, and
 * alpha-blends the result over rgba (width * height float4 RGBA, row 0 at NDC y = -1, in/out,
 * host or device memory). Per pixel: start on the box face the camera sees first (the exit face
 * when the camera is inside), then at most n_steps steps of `step` world units while inside the
 * box, adding step * colormap(d * color_scale) * d * emission, colormap = IDL Mac style with
 * alpha 1 and d the trilinear, wrap-around sample of the field (texel centres at (i + 0.5) / n).
 * The sum is clamped to [0, 1] and blended: rgb = s.rgb s.a + dst.rgb (1 - s.a),
 * a = s.a + dst.a (1 - s.a). Reference values: step 0.05, n_steps 1000, color_scale 5,
 * emission 200. view, proj: column-major 4x4 (glm layout). */
int vfs_render_density_raymarch(const float* field, const int32_t* res, const float* center,
                                const float* half_extent, const float* view, const float* proj,
                                int32_t width, int32_t height, float step, int32_t n_steps,
                                float color_scale, float emission, float* rgba);

/* ---- autotuner (an extension: the reference's dispatch sizes are fixed in its shaders'
 * numthreads, e.g. assets/shaders/simulation/wcsph_with_boundary_model.slang:92) ----
 * Launch shapes of one substep. None changes any result: the sort is stable for every digit
 * width, and each particle's sums are accumulated by one thread in the same order for every
 * block shape. */
typedef struct vfs_tune_config {
    int32_t sort_digit_bits; /* 4..8 (the tuner tries 6, 7, 8) */
    int32_t sort_tile_items; /* 8, 12 or 16 keys per thread of a onesweep tile */
    int32_t nbr_block;       /* neighbour passes: threads per block ... */
    int32_t nbr_min_blocks;  /* ... and minimum resident blocks per SM: 128x6, 128x8, 96x8, 64x12 */
    int32_t cell_block;      /* keys per block of the cell-range / reorder kernel: 128, 256, 512 */
    int32_t force_block;     /* force pass: threads per block and minimum resident blocks per */
    int32_t force_min_blocks;/* SM, the same four shapes; 0, 0 = the neighbour passes' shape */
    int32_t walk_staging;    /* block-per-cell staging of the density walk: 1 on, 0 off */
} vfs_tune_config;
/* Times every candidate of each stage (sort, neighbour passes, cell ranges) for `repeats`
 * substeps from the model's current state, keeps the fastest, and restores the state (the
 * neighbour arrays then need a new substep). With use_cache, a choice cached in this process for
 * the same device and workload size is applied without timing. `chosen` may be NULL. */
int vfs_model_autotune(vfs_model* m, int32_t repeats, int32_t use_cache, vfs_tune_config* chosen);
int vfs_model_set_tune_config(vfs_model* m, const vfs_tune_config* c);
int vfs_model_get_tune_config(vfs_model* m, vfs_tune_config* c);
/* The process-wide cache of autotuner choices, as a text file (one line per workload key). */
int vfs_tune_cache_save(const char* path);
int vfs_tune_cache_load(const char* path);
int vfs_tune_cache_clear(void);

/* ---- batches: many independent scenes advanced by one launch per pass ----
 * Each scene is a complete reference simulation (its own parameters, particle count N_s = its
 * hash-table size, boundary objects). Scene s owns particles and keys [off_s, off_s + N_s): its
 * keys are off_s + HashCell3D % N_s, so one stable sort of all keys yields every scene's own stable
 * sort and results equal those of one vfs_model per scene. Scene arguments index [0, n_scenes);
 * offsets, ids and neighbour arrays are scene-local. */
typedef struct vfs_batch vfs_batch;
int vfs_batch_create(int32_t n_scenes, const vfs_sim_params* sims, const vfs_sph_params* sphs,
                     const vfs_wcsph_params* wcsphs, vfs_batch** out);
int vfs_batch_destroy(vfs_batch* b);
int32_t vfs_batch_num_scenes(const vfs_batch* b);
uint32_t vfs_batch_num_particles(const vfs_batch* b, int32_t scene);
int vfs_batch_set_stream(vfs_batch* b, void* stream);
int vfs_batch_set_scene_parameters(vfs_batch* b, int32_t scene, const vfs_sim_params* sim,
                                   const vfs_sph_params* sph, const vfs_wcsph_params* wcsph);
int vfs_batch_add_boundary_object(vfs_batch* b, int32_t scene, const vfs_boundary_object* obj);
int vfs_batch_add_analytic_object(vfs_batch* b, int32_t scene, const vfs_analytic_object* obj);
int vfs_batch_add_mesh_object(vfs_batch* b, int32_t scene, const vfs_mesh_object* obj);
int vfs_batch_get_boundary_object(const vfs_batch* b, int32_t scene, uint32_t idx,
                                  vfs_boundary_object* info, float* sdf_out, float* vm_out);
int vfs_batch_set_particle_state(vfs_batch* b, int32_t scene, const float* pos, const float* vel,
                                 uint32_t offset, int64_t count);
int vfs_batch_copy_data_buffers(vfs_batch* b, int32_t scene, float* pos, float* vel, float* dens,
                                float* acc);
int vfs_batch_get_ids(vfs_batch* b, int32_t scene, uint32_t* ids);
int vfs_batch_get_neighbor_arrays(vfs_batch* b, int32_t scene, uint32_t* keys,
                                  uint32_t* sorted_indices, uint32_t* offsets);
int vfs_batch_get_boundary_fields(vfs_batch* b, int32_t scene, float* boundary_density,
                                  float* boundary_gradient);
int vfs_batch_record_fields(vfs_batch* b, int32_t enable);
/* count substeps of every scene (each with its own dt). */
int vfs_batch_substeps(vfs_batch* b, int32_t count);
int vfs_batch_use_graph(vfs_batch* b, int32_t enable);
int vfs_batch_synchronize(vfs_batch* b);
int vfs_batch_profile_substeps(vfs_batch* b, int32_t count, float* phase_ms);
int vfs_batch_set_sort_config(vfs_batch* b, int32_t digit_bits, int32_t tile_items);
int vfs_batch_set_neighbor_capacity(vfs_batch* b, int32_t slots);
int vfs_batch_set_skin(vfs_batch* b, float skin);
int vfs_batch_set_walk_staging(vfs_batch* b, int32_t enable);
int vfs_batch_get_skin(const vfs_batch* b, float* skin);
int vfs_batch_get_skin_builds(vfs_batch* b, uint32_t scene, uint32_t* builds);
int vfs_batch_export_state(vfs_batch* b, int32_t scene, const char* path_prefix);
int vfs_batch_import_state(vfs_batch* b, int32_t scene, const char* path_prefix);
/* As vfs_model_record; the snapshots are `<prefix>_s<scene>_f<frame>`. */
int vfs_batch_record(vfs_batch* b, int32_t substeps, int32_t every, const char* path_prefix);
int vfs_batch_render_particles(vfs_batch* b, int32_t scene, const float* model_view,
                               const float* proj, int32_t width, int32_t height, float quad_side,
                               float depth_radius, float v_max, uint8_t* rgba, float* depth);
int vfs_batch_density_grid(vfs_batch* b, int32_t scene, const float* lo, const float* hi,
                           const int32_t* res, float* grid);
int vfs_batch_autotune(vfs_batch* b, int32_t repeats, int32_t use_cache, vfs_tune_config* chosen);
int vfs_batch_set_tune_config(vfs_batch* b, const vfs_tune_config* c);
int vfs_batch_get_tune_config(vfs_batch* b, vfs_tune_config* c);

/* ---- differentiable rollouts (an extension: the reference has no differentiation) ----
 * A rollout advances a single-scene model `steps` substeps from its current state, keeping the
 * state every `checkpoint_every` substeps. The backward pass recomputes each segment from its
 * checkpoint (keeping that segment's sorted inputs, permutations, density products and neighbour
 * lists on the device) and runs the adjoint kernels of integration, force, EOS, density and the
 * volume-map terms in reverse. Gradients are by particle id (the order state was first set in):
 * dl_dx_final / dl_dv_final (3N floats, either may be NULL) seed d loss / d final state; dl_dv0 and
 * dl_dx0 receive d loss / d initial velocities and positions; dl_dparams[0..1] receive
 * d loss / d viscosity_strenght and d loss / d stiffness. Neighbour lists longer than 128 entries
 * make the backward pass fail with VFS_ERR_CAPACITY. */
typedef struct vfs_rollout vfs_rollout;
int vfs_rollout_create(vfs_model* m, int32_t steps, int32_t checkpoint_every, vfs_rollout** out);
int vfs_rollout_destroy(vfs_rollout* r);
int vfs_rollout_forward(vfs_rollout* r);
int vfs_rollout_backward(vfs_rollout* r, const float* dl_dx_final, const float* dl_dv_final,
                         float* dl_dv0, float* dl_dx0, double* dl_dparams);

/* ---- scene: LoadScene / GenericScene (src/util/scene_loader.cpp:113-140,
 * src/scenes/generic_scene.cpp:10-57) ---- */

/* Parses a scene JSON, creates the model (N = sum of fluid-block sizes), adds its boundary
 * objects (resourcePath resolved against resources_dir) and spawns the fluid blocks
 * (GenericScene::Reset). */
int vfs_scene_load(const char* json_path, const char* resources_dir, vfs_model** out);
/* GenericScene::Reset (src/scenes/generic_scene.cpp:42-57): re-spawns the fluid blocks of a
 * model created by vfs_scene_load. */
int vfs_scene_reset(vfs_model* m);

/* ---- spatial-hash compute primitives on device buffers (enqueued on `stream`, a cudaStream_t
 * passed as void*; NULL is the legacy default stream; no host synchronisation) ---- */

/* GPUCountSort::Run (src/compute/sort.cpp:107-143, sort.slang:13-55): sorts the n (key, item)
 * pairs in place by key, stably; items are first set to 0..n-1 (ClearCounts), so on return
 * items[] is the sorting permutation and keys[] the sorted keys. Keys must be <= max_value.
 * Temporary buffers come from the stream-ordered allocator. */
int vfs_sort_pairs(uint32_t* items, uint32_t* keys, uint32_t n, uint32_t max_value, void* stream);
/* Status of the pair sorts (vfs_sort_pairs, vfs_sort_pairs_noalloc) enqueued on the current device
 * since the previous status call: synchronises `stream`, returns the OR of their device error
 * words in *err_word (may be NULL) and clears it. VFS_ERR_DEVICE_CHECK when a sort's bounded
 * look-back wait timed out (that sort's output is invalid), else VFS_OK. The sorts themselves
 * return without synchronising, so their device errors surface here. The reference's counting
 * sort (src/compute/sort.cpp:107-143) has no wait that can fail, hence no counterpart. */
int vfs_sort_pairs_status(void* stream, uint32_t* err_word);
/* Signed distances (double) of n_points points (x, y, z floats) to a triangle mesh, computed on
 * the GPU exactly as the mesh objects' SDF grids are (the primitive behind them). */
int vfs_mesh_signed_distance(const float* vertices, uint32_t n_vertices, const uint32_t* triangles,
                             uint32_t n_triangles, const float* points, uint32_t n_points,
                             double* distances);

/* ---- failure detection ----
 * Self-test of the radix sort's decoupled look-back wait (the sort's counterpart of the
 * reference's global-atomic scan, src/compute/sort.cpp:57-86, which has no wait to fail). 32
 * threads each wait on a predecessor tile's status word, with the same bounded-poll code the sort
 * uses. With predecessor_published = 0 nothing ever publishes: after spin_limit polls (1..2^20)
 * each sets the timeout bit of the error word and returns, and the call returns
 * VFS_ERR_DEVICE_CHECK with err_word = 1 while the CUDA context stays usable. With 1, the
 * predecessor has published prefix b + 1 for digit b: exclusive[b] = b + 1 and VFS_OK. */
int vfs_selftest_lookback(int32_t predecessor_published, int32_t spin_limit, uint32_t* err_word,
                          uint32_t* exclusive);

/* The same sort without any allocation, for callers that cannot allocate device memory: code in
 * a frame loop or inside a host framework that owns the GPU memory budget, where a cudaMalloc
 * could synchronise the device, fragment the host's pool or break a stream capture. This entry
 * point has no counterpart in the reference. Its temporaries live in one fixed device array of
 * 2.3 MB that every GPU loading the library holds until the process exits; n above
 * VFS_SORT_NOALLOC_MAX_PAIRS is rejected with VFS_ERR_CAPACITY. The first call on each device
 * looks up that array's device address (cudaGetSymbolAddress) and should come before any stream
 * capture. All calls share the array, so calls whose work overlaps on the GPU (other streams,
 * other threads) race; serialise them on one stream. Errors of the sort itself are reported by
 * vfs_sort_pairs_status, as for vfs_sort_pairs. */
#define VFS_SORT_NOALLOC_MAX_PAIRS 262144u
int vfs_sort_pairs_noalloc(uint32_t* items, uint32_t* keys, uint32_t n, uint32_t max_value,
                           void* stream);
/* SpatialOffset::Run with init (src/compute/sort.cpp:155-176, spatial_offsets.slang:10-31):
 * offsets[k] = first index of key k in sorted_keys, or n when k is absent. */
int vfs_spatial_offsets(const uint32_t* sorted_keys, uint32_t* offsets, uint32_t n, void* stream);
/* BufferReorder::Reorder (src/compute/sort.cpp:206-219, reorder.slang:11-19) on packed float3:
 * dst[i] = src[sorted_indices[i]]; src and dst must not alias (the reference copies back). */
int vfs_reorder_float3(const uint32_t* sorted_indices, const float* src, float* dst, uint32_t n,
                       void* stream);

/* ---- seeded synthetic inputs (counter-based generator; identical on every host) ---- */

/* Jittered lattice: positions origin + spacing * (i + 0.5, j + 0.5, k + 0.5) + U(-jitter,
 * +jitter) * spacing per component, i fastest. */
int vfs_generate_lattice(const uint32_t dims[3], const float origin[3], float spacing,
                         float jitter, uint64_t seed, float* pos_out);
/* n_uniform points uniform in [lo, hi) followed by n_blob Gaussian points around center. */
int vfs_generate_uniform_blob(uint64_t n_uniform, const float lo[3], const float hi[3],
                              uint64_t n_blob, const float center[3], float sigma, uint64_t seed,
                              float* pos_out);
/* Smooth velocity field: sum of `modes` random Fourier modes, scaled so the largest speed over
 * the given positions equals amplitude. */
int vfs_generate_fourier_velocity(uint64_t n, const float* pos, int32_t modes, float amplitude,
                                  uint64_t seed, float* vel_out);

#ifdef __cplusplus
}
#endif

#endif /* VFS_CUDA_H */
