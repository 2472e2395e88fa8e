// Host-side state behind the vfs_model / vfs_batch handles (C++ only).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "vfs_cuda.h"
#include "vfs_internal.h"

namespace vfs {

int fail(int code, const std::string& msg);
std::string last_error_message();  // this thread's last error

struct ObjectStore {
    vfs_boundary_object info;  // grid pointers cleared; grids live on the device
    float* d_sdf = nullptr;
    float* d_vm = nullptr;
};

// One fluid block of a scene (GenericScene::FluidBlock, src/scenes/generic_scene.h:15-18).
struct FluidBlock {
    uint32_t size[3];
    float pos[3];
};

// One independent simulation: the reference's scene + model parameters, its boundary objects and
// its slice [off, off + n) of the particle and key arrays.
struct SceneHost {
    vfs_sim_params sim{};
    vfs_sph_params sph{};
    vfs_wcsph_params wcsph{};
    uint32_t n = 0;
    uint32_t off = 0;
    std::vector<ObjectStore> objects;
    std::vector<FluidBlock> blocks;  // set by vfs_scene_load for vfs_scene_reset
    SceneParams params{};
};

// The engine behind both handles: a plain model is one scene, a batch is many advanced together.
struct Model {
    std::vector<SceneHost> scenes;
    uint32_t n = 0;  // particles of all scenes

    cudaStream_t stream = nullptr;
    bool own_stream = false;

    float4* pos[2] = {nullptr, nullptr};
    float4* vel[2] = {nullptr, nullptr};
    int cur = 0;
    uint32_t* keys = nullptr;
    uint32_t* keys_alt = nullptr;
    uint32_t* vals = nullptr;
    uint32_t* vals_alt = nullptr;
    uint32_t* skeys = nullptr;  // sorted keys of the last substep (sk_buf)
    uint32_t* sperm = nullptr;  // sorted_indices of the last substep (sp_buf)
    uint32_t* sk_buf = nullptr;   // merge output: sorted keys
    uint32_t* sp_buf = nullptr;   // merge output: sorted_indices
    uint32_t* pkeys = nullptr;    // previous substep's sorted keys (all ones in a fresh model)
    uint32_t* moved = nullptr;       // 2 ceil(n/32) + 1 words: moved bitmask, moved count before each word
    uint32_t* cell_guess = nullptr;  // per cell block: its bound in the sorted keys last substep
    uint32_t* cell_scan = nullptr;
    float4* aux = nullptr;
    float4* rec = nullptr;  // 2 float4 per particle: the force pass's neighbour records
    float4* bnd = nullptr;
    float4* acc = nullptr;
    uint32_t* nbr = nullptr;        // nbr_cap slot-major neighbour lists
    uint32_t nbr_cap = kNbrCap;     // slots per particle (longer lists fall back to a walk)
    uint32_t* nbr_count = nullptr;  // list length per particle
    SkinLists skin{};               // candidate lists with a skin (absent in three-lane mode)
    float skin_fraction = 0.05f;    // skin / h; 0 turns the lists off
    // Every id is a different slot's (true from creation; an upload of part of a scene can
    // repeat ids). While it holds, an upload of a whole scene moves each slot's build index to
    // the slot's new id, so a host round trip of the model's own state keeps its skin lists.
    bool ids_unique = true;
    float* stage = nullptr;         // 32 bytes per particle of host-transfer staging
    uint32_t* scratch = nullptr;
    size_t scratch_words = 0;
    uint32_t* err = nullptr;
    uint32_t* err_host = nullptr;  // pinned copy of the error word read by check_device
    uint32_t* walk_sched = nullptr;  // two words: the density walk's run counter (zero between launches)
    HostOut host_out{};              // set only while step_host enqueues its last substep
    cudaEvent_t cells_wait = nullptr;  // set only while step_host enqueues its first substep
    cudaStream_t io_stream = nullptr;  // step_host's velocity upload (created on first use)
    cudaEvent_t io_ev[2] = {nullptr, nullptr};
    // step_host with page-locked inputs: the next substep's key pass reads the positions from
    // this device alias of the host array, and its velocity upload (from keys_host_vel) starts
    // after that pass. Set by enqueue_set_state, taken by the next enqueue_substep.
    const float* keys_host_pos = nullptr;
    const float* keys_host_vel = nullptr;
    bool keys_host_remap = false;  // that pass also moves the build indices (skin.b_next)
    // step_host's one-substep round trip through page-locked buffers, captured once per set of
    // buffers (host pointers and their device aliases) and replayed.
    cudaGraphExec_t host_graph = nullptr;
    const void* host_graph_key[11] = {};
    SceneParams* d_scenes = nullptr;   // batched launches: the scene table
    uint16_t* d_scene_of = nullptr;    // batched launches: scene id per particle
    DevObject* d_objects = nullptr;    // boundary objects of all scenes
    size_t d_objects_cap = 0;

    int digit_bits = 8;
    int tile_items = 16;
    SortConfig sc{};
    SortScratch sort_scratch{};
    KernelConfig kc{};
    StepLaunch launch{};

    bool record = false;
    uint64_t substeps_done = 0;  // substeps run by run_substeps (the snapshot sidecar's counter)
    bool use_graph = true;
    bool stepped = false;
    cudaGraphExec_t graph_exec = nullptr;

    ~Model();
    int init();
    int refresh_params();
    void invalidate_graph();
    int alloc_sort_scratch();
    int alloc_skin();
    int invalidate_skin();
    SkinLists active_skin() const;
    int enqueue_substep(cudaEvent_t* ev);
    int run_substeps(int count);
    int check_device();
    // Scene-relative state I/O (offset and ids are scene-local).
    int set_state(uint32_t scene, const float* pos3, const float* vel3, uint32_t offset,
                  int64_t count);
    // set_state without the final wait (the conversion kernel may still be reading host memory).
    int enqueue_set_state(uint32_t scene, const float* pos3, const float* vel3, uint32_t offset,
                          int64_t count, cudaStream_t vel_stream = nullptr);
    // The velocities' upload on vel_stream after the work queued on the model's stream so far:
    // io_ev[0] there, the DMA into the staging buffer and the conversion, io_ev[1] when done.
    int enqueue_vel_upload(const SceneHost& sh, uint32_t offset, uint64_t cnt, const float* vel3,
                           cudaStream_t vel_stream);
    int move_build_indices(const uint32_t* b_next, uint32_t off, uint64_t cnt);
    // set_state of every particle (when pos3 / vel3 are given), `count` substeps and get_state,
    // with one wait at the end; outputs in page-locked memory come from the last substep's
    // density pass (densities) and force pass (positions, velocities).
    int step_host(const float* pos3, const float* vel3, int32_t count, float* pos_out,
                  float* vel_out, float* dens_out);
    int ensure_io_stream();
    void set_host_out(const HostOut& ho);
    int get_state(uint32_t scene, float* pos3, float* vel3, float* dens, uint32_t* ids);
    int get_acc(uint32_t scene, float* acc3);
    int get_neighbors(uint32_t scene, uint32_t* keys, uint32_t* perm, uint32_t* offsets);
    int get_boundary(uint32_t scene, float* bdens, float* bgrad);
    int add_object(uint32_t scene, const vfs_boundary_object& src, const float* d_sdf,
                   const float* d_vm);
    int add_analytic(uint32_t scene, const vfs_analytic_object& a);
    int add_mesh(uint32_t scene, const vfs_mesh_object& a);
};

// Builds a model of the given scenes (sizes from each sph.n_particles) and allocates it.
int create_model(const std::vector<SceneHost>& scenes, Model** out);

// Runs `count` substeps with events between the passes; phase_ms[6] = mean ms of keys, sort,
// cells+reorder, density, force, clear.
// The address under which this device's kernels reach buffer p: page-locked host memory, or
// device and managed memory of this device; null for pageable host memory.
void* device_alias(const void* p);
int profile_phases(Model& m, int32_t count, float* phase_ms);
int set_sort_config(Model& m, int32_t digit_bits, int32_t tile_items);
int set_neighbor_capacity(Model& m, int32_t slots);
int set_skin(Model& m, float skin);
float get_skin(const Model& m);
int get_skin_builds(Model& m, uint32_t scene, uint32_t* builds);

}  // namespace vfs

struct vfs_model;
vfs::Model* vfs_model_impl(vfs_model* h);
struct vfs_batch;
vfs::Model* vfs_batch_impl(vfs_batch* h);
