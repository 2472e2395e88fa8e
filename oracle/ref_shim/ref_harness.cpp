// Host driver of the reference's own step shaders compiled as C++ (test infrastructure).
//
// It includes oracle/_ref/ref_shaders_gen.cpp, which oracle/ref_build.py generates from the
// reference's Slang sources, and runs their entry points in the order of the reference's host
// code. A dispatch of G groups of 256 threads runs ids 0..n-1 (every entry returns early for larger
// ids except CalculateBoundaryVolume, whose writes past n the reference leaves unguarded and which
// runs ids below n only). The counting sort's two atomic passes (CalculateCounts, ScatterOutputs)
// run their ids in index order on one host thread, so the sort is stable; every other entry writes
// only its own id's outputs and runs its ids across the host's threads (OpenMP), and the scan's
// workgroups run on separate host threads, each as cooperative fibers:
//   WCSPHWithBoundaryModel::Step        src/models/wcsph_with_boundary_model.cpp:81-117
//   SPHModel::RunSpatialHash            src/models/model.cpp:210-223
//   SpatialHash::Run                    src/compute/spatial_hash.cpp:52-63
//   GPUCountSort::Run / GPUScan::Run    src/compute/sort.cpp:107-143 / 57-86
//   SpatialOffset::Run (init)           src/compute/sort.cpp:155-176
//   BufferReorder::Reorder / Copyback   src/compute/sort.cpp:206-227
//   SPHModel::CalcKernelCoefficients    src/models/model.cpp:225-234
// Boundary objects are given as the reference's GenericScene packs them
// (src/scenes/generic_scene.cpp:125-145): the inverse of the object transform and its rotation
// as glm (column-major) 4x4 matrices, the SDF grid box, resolution, SDF and volume-map grids.
#include "ref_shaders_gen.cpp"

#include <omp.h>

#include <cstring>
#include <vector>

namespace {

struct RefParams {  // same field order as the oracle's parameter block
    float gravity[3];
    float smooth_radius;
    float time_scale;
    int32_t iterations;
    float fixed_dt;
    float target_density;
    float bbox_size[3];
    float bbox_pos[3];
    float wall_stiffness;
    float stiffness;
    float expoent;
    float viscosity_strenght;
};

template <class T>
ref_ptr<T> view(std::vector<T>& v) {
    ref_ptr<T> r;
    r.p = v.data();
    r.n = v.size();
    return r;
}

struct Object {
    float4x4 transform, rotation;
    prog_wcsph::BoundingBox box;
    uint3 res;
    std::vector<float> sdf, vm;
};

struct Model {
    RefParams prm;
    uint32_t n;
    std::vector<float3> pos, vel, acc, bgrad, pos_tmp, vel_tmp;
    std::vector<float> dens, bdens;
    std::vector<uint> keys, indices, offsets, sorted_items, sorted_keys, counts;
    std::vector<std::vector<uint>> group_sums;  // GPUScan's per-level group-sum buffers
    std::vector<Object> objects;
    std::vector<prog_wcsph::wcsph_model::BoundaryObjectInfo> infos;
};

float4x4 from_glm(const float* m) {  // column-major 16 floats -> rows
    float4x4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r.m[i][j] = m[4 * j + i];
    return r;
}

// ---------------------------------------------------------------- dispatch helpers
// Ids in index order on the calling thread (the sort's atomic passes).
template <class F>
void each_in_order(uint32_t n, F f) {
    for (uint32_t id = 0; id < n; id++) f(id);
}

// Ids whose writes are disjoint, across the host's threads.
template <class F>
void each(uint32_t n, F f) {
#pragma omp parallel for schedule(static)
    for (int64_t id = 0; id < (int64_t)n; id++) f((uint32_t)id);
}

thread_local prog_scan::Constants g_scan_k;
thread_local uint g_scan_group;
void scan_block_thread(int t) {
    prog_scan::ScanBlock(g_scan_group * 256u + (uint)t, (uint)t, g_scan_group, g_scan_k);
}

// GPUScan::Run: exclusive scan of `elements` in place, recursing on the group sums.
void gpu_scan(Model& m, std::vector<uint>& elements, size_t level) {
    const uint count = (uint)elements.size();
    const uint num_groups = (uint)__builtin_ceil((double)((float)count / 2.0f / 256.0f));
    // All levels exist up front, so a recursive call never moves the caller's buffer.
    if (m.group_sums.size() < 16) m.group_sums.resize(16);
    std::vector<uint>& sums = m.group_sums[level];
    sums.assign(num_groups, 0u);
    prog_scan::Constants k;
    k.elements = view(elements);
    k.group_sums = view(sums);
    k.item_count = count;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t g = 0; g < (int64_t)num_groups; g++) {
        g_scan_k = k;
        g_scan_group = (uint)g;
        slang_shim::run_group(256, scan_block_thread);
    }
    if (num_groups > 1) {
        gpu_scan(m, sums, level + 1);
        k.group_sums = view(m.group_sums[level]);
        each(num_groups * 256u, [&](uint id) { prog_scan::ScanCombine(id, id / 256u, k); });
    }
}

void run_spatial_hash(Model& m) {
    const uint n = m.n;
    // SpatialHash::Run: UpdateSpatialHash with cell_size = smooth_radius.
    prog_hash::ubo.cell_size = m.prm.smooth_radius;
    prog_hash::ubo.spatial_keys = view(m.keys);
    prog_hash::PushConstants hp;
    hp.positions = view(m.pos);
    hp.n_particles = n;
    each(n, [&](uint id) { prog_hash::UpdateSpatialHash(id, hp); });
    // GPUCountSort::Run(items = spatial_indices, keys = spatial_keys, max_value = n - 1).
    prog_sort::Constants sk;
    sk.input_items = view(m.indices);
    sk.input_keys = view(m.keys);
    sk.sorted_items = view(m.sorted_items);
    sk.sorted_keys = view(m.sorted_keys);
    sk.counts = view(m.counts);
    sk.item_count = n;
    each(n, [&](uint id) { prog_sort::ClearCounts(id, sk); });
    each_in_order(n, [&](uint id) { prog_sort::CalculateCounts(id, sk); });
    gpu_scan(m, m.counts, 0);
    each_in_order(n, [&](uint id) { prog_sort::ScatterOutputs(id, sk); });
    each(n, [&](uint id) { prog_sort::CopyBack(id, sk); });
    // SpatialOffset::Run with init.
    prog_offsets::Constants ok;
    ok.sorted_keys = view(m.keys);
    ok.offsets = view(m.offsets);
    ok.num_inputs = n;
    each(n, [&](uint id) { prog_offsets::InitOffsets(id, ok); });
    each(n, [&](uint id) { prog_offsets::CalculateOffsets(id, ok); });
    // BufferReorder::Reorder (positions, velocities) and Copyback.
    prog_reorder::ReorderPushConstants rk;
    rk.sorted_indices = view(m.indices);
    rk.n = n;
    rk.buffer = view(m.pos);
    rk.sort_target = view(m.pos_tmp);
    each(n, [&](uint id) { prog_reorder::Reorder(id, rk); });
    rk.buffer = view(m.vel);
    rk.sort_target = view(m.vel_tmp);
    each(n, [&](uint id) { prog_reorder::Reorder(id, rk); });
    m.pos = m.pos_tmp;
    m.vel = m.vel_tmp;
}

// Binds the model's buffers and parameters to the step program's uniform blocks (the
// descriptor updates of SPHModel::UpdateAllUniforms and WCSPHWithBoundaryModel::Init).
void bind(Model& m) {
    using namespace prog_wcsph;
    const float r = m.prm.smooth_radius;
    const float pi = 3.14159265358979323846f;  // glm::pi<float>()
    simulation::parameters.gravity = float3(m.prm.gravity[0], m.prm.gravity[1], m.prm.gravity[2]);
    simulation::parameters.smooth_radius = r;
    sph_model::kernel_coeff.spiky_pow3_scale = 15.0f / (pi * (float)__builtin_pow((double)r, 6.0));
    sph_model::kernel_coeff.spiky_pow2_scale = 15.0f / (2.0f * pi * (float)__builtin_pow((double)r, 5.0));
    sph_model::kernel_coeff.spiky_pow3_diff_scale = 45.0f / (pi * (float)__builtin_pow((double)r, 6.0));
    sph_model::kernel_coeff.spiky_pow2_diff_scale = 15.0f / (pi * (float)__builtin_pow((double)r, 5.0));
    sph_model::kernel_coeff.cubic_spline_scale = 8.0f / (pi * (float)__builtin_pow((double)r, 3.0));
    sph_model::kernel_coeff.grad_cubic_spline_scale = 48.0f / (pi * (float)__builtin_pow((double)r, 4.0));
    sph_model::parameters.time_scale = m.prm.time_scale;
    sph_model::parameters.iterations = m.prm.iterations;
    sph_model::parameters.n_particles = (int)m.n;
    sph_model::parameters.fixed_dt = m.prm.fixed_dt;
    sph_model::parameters.target_density = m.prm.target_density;
    sph_model::parameters.bounding_box.size = float3(m.prm.bbox_size[0], m.prm.bbox_size[1], m.prm.bbox_size[2]);
    sph_model::parameters.bounding_box.pos = float3(m.prm.bbox_pos[0], m.prm.bbox_pos[1], m.prm.bbox_pos[2]);
    sph_model::spatial_hash.spatial_keys = view(m.keys);
    sph_model::spatial_hash.spatial_offsets = view(m.offsets);
    sph_model::spatial_hash.sorted_indices = view(m.indices);
    sph_model::buffers.positions = view(m.pos);
    sph_model::buffers.velocities = view(m.vel);
    sph_model::buffers.densities = view(m.dens);
    sph_model::buffers.accelerations = view(m.acc);
    m.infos.clear();
    for (Object& o : m.objects) {
        wcsph_model::BoundaryObjectInfo info;
        info.transform = o.transform;
        info.rotation = o.rotation;
        info.box = o.box;
        info.sdf_grid = view(o.sdf);
        info.volume_map_grid = view(o.vm);
        info.resolution = o.res;
        m.infos.push_back(info);
    }
    wcsph_model::parameters.wall_stiffness = m.prm.wall_stiffness;
    wcsph_model::parameters.stiffness = m.prm.stiffness;
    wcsph_model::parameters.expoent = m.prm.expoent;
    wcsph_model::parameters.viscosity_strenght = m.prm.viscosity_strenght;
    wcsph_model::parameters.boundary_objects = view(m.infos);
    wcsph_model::parameters.n_boundary_objects = (uint)m.infos.size();
    wcsph_model::volume_map_buffers.boundary_density = view(m.bdens);
    wcsph_model::volume_map_buffers.boundary_gradient = view(m.bgrad);
}

// WCSPHWithBoundaryModel::Step.
void step(Model& m) {
    using namespace prog_wcsph;
    PushConstants push;
    push.time = 0.0f;
    push.dt = m.prm.time_scale * m.prm.fixed_dt / (float)m.prm.iterations;
    push.n_particles = m.n;
    const uint n = m.n;
    for (int it = 0; it < m.prm.iterations; it++) {
        bind(m);
        each(n, [&](uint id) { ExternalAccel(id, push); });
        run_spatial_hash(m);
        bind(m);  // Copyback refilled the position and velocity buffers
        each(n, [&](uint id) { CalculateBoundaryVolume(id, push); });
        each(n, [&](uint id) { CalculateDensities(id, push); });
        each(n, [&](uint id) { CalculatePressureAccel(id, push); });
        each(n, [&](uint id) { CalculateViscousAccel(id, push); });
        each(n, [&](uint id) { UpdatePositions(id, push); });
    }
}

void copy3(std::vector<float3>& dst, const float* src) {
    for (size_t i = 0; i < dst.size(); i++) dst[i] = float3(src[3 * i], src[3 * i + 1], src[3 * i + 2]);
}
void out3(const std::vector<float3>& src, float* dst) {
    if (!dst) return;
    for (size_t i = 0; i < src.size(); i++) {
        dst[3 * i] = src[i].x;
        dst[3 * i + 1] = src[i].y;
        dst[3 * i + 2] = src[i].z;
    }
}

}  // namespace

extern "C" {

void* vfs_ref_create(const RefParams* p, uint32_t n) {
    if (!p || n == 0) return nullptr;
    Model* m = new Model();
    m->prm = *p;
    m->n = n;
    for (auto* v : {&m->pos, &m->vel, &m->acc, &m->bgrad, &m->pos_tmp, &m->vel_tmp}) v->assign(n, float3());
    m->dens.assign(n, 0.0f);
    m->bdens.assign(n, 0.0f);
    for (auto* v : {&m->keys, &m->indices, &m->offsets, &m->sorted_items, &m->sorted_keys, &m->counts})
        v->assign(n, 0u);
    return m;
}

void vfs_ref_destroy(void* h) { delete static_cast<Model*>(h); }

void vfs_ref_set_threads(int threads) {
    if (threads > 0) omp_set_num_threads(threads);
}

int vfs_ref_get_threads() { return omp_get_max_threads(); }

int vfs_ref_add_object(void* h, const float* transform, const float* rotation, const float* box_size,
                       const float* box_pos, const uint32_t* res, const float* sdf, const float* vm) {
    Model* m = static_cast<Model*>(h);
    if (!m || !transform || !rotation || !box_size || !box_pos || !res || !sdf || !vm) return 1;
    Object o;
    o.transform = from_glm(transform);
    o.rotation = from_glm(rotation);
    o.box.size = float3(box_size[0], box_size[1], box_size[2]);
    o.box.pos = float3(box_pos[0], box_pos[1], box_pos[2]);
    o.res = uint3(res[0], res[1], res[2]);
    const size_t cnt = (size_t)res[0] * res[1] * res[2];
    o.sdf.assign(sdf, sdf + cnt);
    o.vm.assign(vm, vm + cnt);
    m->objects.push_back(std::move(o));
    return 0;
}

void vfs_ref_set_state(void* h, const float* pos, const float* vel) {
    Model* m = static_cast<Model*>(h);
    copy3(m->pos, pos);
    copy3(m->vel, vel);
}

void vfs_ref_step(void* h, int count) {
    Model* m = static_cast<Model*>(h);
    for (int i = 0; i < count; i++) step(*m);
}

void vfs_ref_get(void* h, float* pos, float* vel, float* dens, float* acc, float* bdens, float* bgrad,
                 uint32_t* keys, uint32_t* indices, uint32_t* offsets) {
    Model* m = static_cast<Model*>(h);
    out3(m->pos, pos);
    out3(m->vel, vel);
    out3(m->acc, acc);
    out3(m->bgrad, bgrad);
    if (dens) std::memcpy(dens, m->dens.data(), m->n * sizeof(float));
    if (bdens) std::memcpy(bdens, m->bdens.data(), m->n * sizeof(float));
    if (keys) std::memcpy(keys, m->keys.data(), m->n * sizeof(uint32_t));
    if (indices) std::memcpy(indices, m->indices.data(), m->n * sizeof(uint32_t));
    if (offsets) std::memcpy(offsets, m->offsets.data(), m->n * sizeof(uint32_t));
}

}  // extern "C"
