// Host-side model state behind the vfs_model handle (C++ only).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "vfs_cuda.h"
#include "vfs_internal.h"

namespace vfs {

int fail(int code, const std::string& msg);

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

struct Model {
    vfs_sim_params sim{};
    vfs_sph_params sph{};
    vfs_wcsph_params wcsph{};
    uint32_t n = 0;

    cudaStream_t stream = nullptr;
    bool own_stream = false;

    float4* pos[2] = {nullptr, nullptr};
    float4* vel[2] = {nullptr, nullptr};
    int cur = 0;
    uint32_t* keys = nullptr;
    uint32_t* keys_alt = nullptr;
    uint32_t* vals = nullptr;
    uint32_t* vals_alt = nullptr;
    uint32_t* skeys = nullptr;  // sorted keys of the last substep (aliases keys / keys_alt)
    uint32_t* sperm = nullptr;  // sorted_indices of the last substep (aliases vals / vals_alt)
    uint32_t* cell_scan = nullptr;
    float4* aux = nullptr;
    float4* bnd = nullptr;
    float4* acc = nullptr;
    uint32_t* nbr = nullptr;        // kNbrCap slot-major neighbour lists
    uint32_t* nbr_count = nullptr;  // list length per particle
    float* stage = nullptr;  // 32 bytes per particle of host-transfer staging
    uint32_t* scratch = nullptr;
    size_t scratch_words = 0;
    uint32_t* err = nullptr;

    int digit_bits = 8;
    int tile_items = 16;
    SortConfig sc{};
    SortScratch sort_scratch{};
    StepParams params{};

    std::vector<ObjectStore> objects;
    std::vector<FluidBlock> blocks;  // set by vfs_scene_load for vfs_scene_reset

    bool record = false;
    bool use_graph = true;
    bool stepped = false;
    cudaGraphExec_t graph_exec = nullptr;

    ~Model();
    int init();
    void refresh_params();
    void invalidate_graph();
    int alloc_sort_scratch();
    int enqueue_substep(cudaEvent_t* ev);
    int run_substeps(int count);
    int check_device();
    int set_state(const float* pos3, const float* vel3, uint32_t offset, int64_t count);
    int get_state(float* pos3, float* vel3, float* dens, uint32_t* ids);
    int add_object(const vfs_boundary_object& src, const float* d_sdf, const float* d_vm);
    int add_analytic(const vfs_analytic_object& a);
};

}  // namespace vfs

struct vfs_model;
vfs::Model* vfs_model_impl(vfs_model* h);
