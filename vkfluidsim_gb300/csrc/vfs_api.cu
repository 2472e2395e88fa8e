// Host runtime behind include/vfs_cuda.h: the GB300 counterpart of VkFluidSim's SPHModel /
// WCSPHWithBoundaryModel host classes (src/models/model.cpp, wcsph_with_boundary_model.cpp) and
// of the compute primitives they drive (src/compute/spatial_hash.cpp, sort.cpp).
//
// The reference records 20 dispatches and 2 buffer copies per substep, each behind a full
// compute barrier. Here one substep is keys+moved flags, 2-4 onesweep passes over the particles
// whose cell changed, merge, cells+reorder, density and force on one stream, with no memset
// (the cell pass clears the sort scratch for the next substep), captured once as a CUDA graph and
// replayed. State ping-pongs between two float4 buffer pairs: the reorder writes the
// sorted copy into the spare pair and the force pass writes the integrated state back into the
// original pair, so the substep is graph-stable.
//
// One engine serves one scene (vfs_model) or many independent scenes (vfs_batch): scene s owns
// particles and keys [off_s, off_s + n_s) with key = off_s + HashCell3D % n_s, so one stable sort
// of all keys sorts every scene by its own keys, one cell-range array serves all scenes, and every
// pass is one launch over all scenes.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "vfs_cuda.h"
#include "vfs_internal.h"
#include "vfs_model.h"
#include "vfs_mesh.h"
#include "vfs_volume_map.h"

namespace vfs {

thread_local std::string g_last_error;
std::string last_error_message() { return g_last_error; }

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

#define VFS_CUDA_TRY(expr)                                                               \
    do {                                                                                 \
        cudaError_t e_ = (expr);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return ::vfs::fail(VFS_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace {

constexpr uint32_t kIoBlock = 256;

// SetParticleState's layout conversion: packed float3 records (host memory mapped into the
// device's address space, or a device staging copy) to the float4 state. A block moves its
// 256 records through shared memory, so every warp reads 128 contiguous bytes. Positions (with
// the ids and the zeroed densities) and velocities are converted when their source is given, so
// the two halves can run on different streams. With b_next (an upload of a whole scene while
// every id is a different slot's), the build index of the particle each slot held is stored
// under the slot's new id, read before the slot is overwritten.
__global__ void __launch_bounds__(kIoBlock)
    k_expand_state(uint32_t offset, uint32_t count, const float* __restrict__ pos3,
                   const float* __restrict__ vel3, float4* __restrict__ pos,
                   float4* __restrict__ vel, float4* __restrict__ aux,
                   const uint32_t* __restrict__ b_of_id, uint32_t* __restrict__ b_next,
                   uint32_t n_ids) {
    __shared__ float s_p[3 * kIoBlock], s_v[3 * kIoBlock];
    const uint32_t base = blockIdx.x * kIoBlock, t = threadIdx.x;
    const uint32_t m = min(kIoBlock, count - base);
    const size_t b3 = 3 * (size_t)base;
    for (uint32_t k = t; k < 3 * m; k += kIoBlock) {
        if (pos3) s_p[k] = pos3[b3 + k];
        if (vel3) s_v[k] = vel3[b3 + k];
    }
    __syncthreads();
    if (t >= m) return;
    const uint32_t d = offset + base + t;
    if (pos3) {
        if (b_next) {
            const uint32_t old = __float_as_uint(pos[d].w);
            b_next[d] = old < n_ids ? b_of_id[old] : 0u;
        }
        pos[d] = make_float4(s_p[3 * t], s_p[3 * t + 1], s_p[3 * t + 2], __uint_as_float(d));
        aux[d].z = 0.0f;  // SetParticleState zeroes the densities it covers (model.cpp:146)
    }
    if (vel3) vel[d] = make_float4(s_v[3 * t], s_v[3 * t + 1], s_v[3 * t + 2], 0.0f);
}

// Packs particles [start, start + n) into float3 / float arrays (any of them may be null);
// ids become scene-local. The float3 arrays are written through shared memory, 128 contiguous
// bytes per warp store, so host-mapped outputs receive whole lines.
__global__ void __launch_bounds__(kIoBlock)
    k_compact_state(uint32_t n, uint32_t start, const float4* __restrict__ pos,
                    const float4* __restrict__ vel, const float4* __restrict__ aux,
                    float* __restrict__ pos3, float* __restrict__ vel3,
                    float* __restrict__ dens, uint32_t* __restrict__ ids) {
    __shared__ float s_p[3 * kIoBlock], s_v[3 * kIoBlock];
    const uint32_t base = blockIdx.x * kIoBlock, t = threadIdx.x;
    const uint32_t m = min(kIoBlock, n - base);
    if (t < m) {
        const uint32_t i = start + base + t;
        const float4 p = pos[i];
        const float4 v = vel[i];
        s_p[3 * t] = p.x;
        s_p[3 * t + 1] = p.y;
        s_p[3 * t + 2] = p.z;
        s_v[3 * t] = v.x;
        s_v[3 * t + 1] = v.y;
        s_v[3 * t + 2] = v.z;
        if (dens) dens[base + t] = aux[i].z;
        if (ids) ids[base + t] = __float_as_uint(p.w) - start;
    }
    __syncthreads();
    const size_t b3 = 3 * (size_t)base;
    for (uint32_t k = t; k < 3 * m; k += kIoBlock) {
        if (pos3) pos3[b3 + k] = s_p[k];
        if (vel3) vel3[b3 + k] = s_v[k];
    }
}


// Scene id of every particle of a batched model.
__global__ void k_fill_scene_of(const uint32_t* __restrict__ scene_off, uint32_t n_scenes,
                                uint32_t total, uint16_t* __restrict__ scene_of) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    uint32_t lo = 0, hi = n_scenes;  // last scene with scene_off[s] <= i
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (scene_off[mid] <= i)
            lo = mid;
        else
            hi = mid;
    }
    scene_of[i] = (uint16_t)lo;
}

double pi_d() { return 3.14159265358979323846; }

// Gauss-Legendre rule on [-1, 1] by Newton iteration on the Legendre recurrence.
void gauss_legendre_nodes(int n, double* x, double* w) {
    for (int i = 0; i < n; i++) {
        double z = std::cos(pi_d() * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; k++) {
                const double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = pk;
            }
            const double dp = n * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= n; k++) {
            const double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
            p0 = p1;
            p1 = pk;
        }
        const double dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[i] = -z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

// 4x4 double matrices, column-major like glm.
struct M4 {
    double a[16];
};
M4 m4_identity() {
    M4 m{};
    m.a[0] = m.a[5] = m.a[10] = m.a[15] = 1.0;
    return m;
}
M4 m4_mul(const M4& A, const M4& B) {
    M4 C{};
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) {
            double s = 0.0;
            for (int k = 0; k < 4; k++) s += A.a[k * 4 + r] * B.a[c * 4 + k];
            C.a[c * 4 + r] = s;
        }
    return C;
}
bool m4_inverse(const M4& M, M4& out) {
    // Gauss-Jordan on a row-major copy.
    double a[4][8];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            a[r][c] = M.a[c * 4 + r];
            a[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int col = 0; col < 4; col++) {
        int piv = col;
        for (int r = col + 1; r < 4; r++)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (std::fabs(a[piv][col]) < 1e-300) return false;
        if (piv != col)
            for (int c = 0; c < 8; c++) std::swap(a[piv][c], a[col][c]);
        const double inv = 1.0 / a[col][col];
        for (int c = 0; c < 8; c++) a[col][c] *= inv;
        for (int r = 0; r < 4; r++) {
            if (r == col) continue;
            const double f = a[r][col];
            for (int c = 0; c < 8; c++) a[r][c] -= f * a[col][c];
        }
    }
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) out.a[c * 4 + r] = a[r][c + 4];
    return true;
}

// Rotation of `angle_deg` about `axis` (the scene JSON's rotation {angle, axis},
// src/util/scene_loader.cpp:83-88), as a column-major 4x4.
M4 m4_rotation(float angle_deg, const float axis[3]) {
    M4 m = m4_identity();
    const double ax = axis[0], ay = axis[1], az = axis[2];
    const double len = std::sqrt(ax * ax + ay * ay + az * az);
    if (angle_deg == 0.0f || len == 0.0) return m;
    const double x = ax / len, y = ay / len, z = az / len;
    const double t = (double)angle_deg * pi_d() / 180.0;
    const double c = std::cos(t), s = std::sin(t), C = 1.0 - c;
    const double R[3][3] = {{c + x * x * C, x * y * C - z * s, x * z * C + y * s},
                            {y * x * C + z * s, c + y * y * C, y * z * C - x * s},
                            {z * x * C - y * s, z * y * C + x * s, c + z * z * C}};
    for (int r = 0; r < 3; r++)
        for (int cc = 0; cc < 3; cc++) m.a[cc * 4 + r] = R[r][cc];
    return m;
}

void to_rowmajor34(const float* colmajor16, float* out12) {
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) out12[4 * r + c] = colmajor16[c * 4 + r];
}

}  // namespace

// Derives one scene's per-substep constants from its parameter blocks with the reference's float
// expressions (src/models/model.cpp:225-234; wcsph_with_boundary_model.slang:39-41, 322-323;
// src/models/wcsph_with_boundary_model.cpp:84-89).
static void derive_scene_params(const SceneHost& sh, SceneParams& p) {
    const float r = sh.sim.smooth_radius;
    const float pi_f = 3.14159265358979323846f;
    p.n = sh.n;
    p.off = sh.off;
    p.mod_magic = sh.n >= 1 ? (UINT64_MAX / (uint64_t)sh.n + 1ull) : 0ull;
    p.h = r;
    p.h2 = r * r;
    p.inv_h = 1.0f / r;
    p.cubic = 8.0f / (pi_f * (float)std::pow(r, 3));
    const float grad_scale = 48.0f / (pi_f * (float)std::pow(r, 4));
    p.grad_over_h = grad_scale / r;
    p.mass = sh.sph.target_density * (0.8f * powf(r, 3.0f) / 8.0f);
    p.rho0 = sh.sph.target_density;
    p.stiffness = sh.wcsph.stiffness;
    p.expoent = sh.wcsph.expoent;
    p.visc_scale = 2.0f * (3.0f + 2.0f) * sh.wcsph.viscosity_strenght;
    p.visc_eps = 0.01f * p.h2;
    p.wall_k = sh.wcsph.wall_stiffness;
    p.dt = sh.sph.time_scale * sh.sph.fixed_dt / (float)sh.sph.iterations;
    p.gx = sh.sim.gravity[0];
    p.gy = sh.sim.gravity[1];
    p.gz = sh.sim.gravity[2];
    for (int a = 0; a < 3; a++) {
        p.lo[a] = sh.sph.bbox_pos[a];
        p.hi[a] = sh.sph.bbox_pos[a] + sh.sph.bbox_size[a];
    }
    p.grad_eps = 0.1f * r;
    p.bnd_eighth = 0.125f * r;
    p.bnd_half = 0.5f * r;
    p.nbr_cap = kNbrCap;
    p.skin_r2 = p.skin_half2 = p.skin_lim = 0.0f;  // set by refresh_params when lists are on
    p.n_objects = (uint32_t)sh.objects.size();
    p.objects = nullptr;
}

static void to_dev_object(const ObjectStore& o, DevObject& d) {
    to_rowmajor34(o.info.transform, d.T);
    to_rowmajor34(o.info.rotation, d.R);
    for (int a = 0; a < 3; a++) {
        d.box_pos[a] = o.info.box_pos[a];
        d.box_size[a] = o.info.box_size[a];
        d.res[a] = o.info.resolution[a];
    }
    d.sdf = o.d_sdf;
    d.vm = o.d_vm;
}

// Rebuilds every scene's constants, the device object table and (batched) the scene table.
int Model::refresh_params() {
    std::vector<DevObject> objs;
    for (SceneHost& sh : scenes) {
        derive_scene_params(sh, sh.params);
        sh.params.nbr_cap = nbr_cap;
        if (skin.list && skin_fraction > 0.0f) {
            const float r = sh.params.h * (1.0f + skin_fraction), half = 0.5f * sh.params.h * skin_fraction;
            sh.params.skin_r2 = r * r;
            sh.params.skin_half2 = half * half;
            sh.params.skin_lim = (1.0f + skin_fraction) * (1.0f + skin_fraction) * 1.002f;
        }
        for (const ObjectStore& o : sh.objects) {
            DevObject d{};
            to_dev_object(o, d);
            objs.push_back(d);
        }
    }
    if (objs.size() > d_objects_cap) {
        if (d_objects) cudaFree(d_objects);
        d_objects = nullptr;
        d_objects_cap = 0;
        VFS_CUDA_TRY(cudaMalloc(&d_objects, objs.size() * sizeof(DevObject)));
        d_objects_cap = objs.size();
    }
    if (!objs.empty())
        VFS_CUDA_TRY(cudaMemcpy(d_objects, objs.data(), objs.size() * sizeof(DevObject),
                                cudaMemcpyHostToDevice));
    size_t base = 0;
    std::vector<SceneParams> table;
    for (SceneHost& sh : scenes) {
        sh.params.objects = sh.params.n_objects ? d_objects + base : nullptr;
        base += sh.params.n_objects;
        table.push_back(sh.params);
    }
    if (scenes.size() > 1)
        VFS_CUDA_TRY(cudaMemcpy(d_scenes, table.data(), table.size() * sizeof(SceneParams),
                                cudaMemcpyHostToDevice));
    launch.total = n;
    launch.n_scenes = (uint32_t)scenes.size();
    launch.scenes = d_scenes;
    launch.scene_of = d_scene_of;
    launch.one = scenes.empty() ? SceneParams{} : scenes[0].params;
    invalidate_graph();
    return invalidate_skin();  // h or the skin may have changed
}

void Model::invalidate_graph() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
    if (host_graph) cudaGraphExecDestroy(host_graph);
    host_graph = nullptr;
}

// The host outputs of the next substep enqueued: densities from the density pass (final there,
// while the host link is idle), positions and velocities from the force pass.
void Model::set_host_out(const HostOut& ho) {
    launch.host_dens = ho.dens;
    host_out = ho;
    host_out.dens = nullptr;
}

int Model::ensure_io_stream() {
    if (io_stream) return VFS_OK;
    VFS_CUDA_TRY(cudaStreamCreateWithFlags(&io_stream, cudaStreamNonBlocking));
    VFS_CUDA_TRY(cudaEventCreateWithFlags(&io_ev[0], cudaEventDisableTiming));
    VFS_CUDA_TRY(cudaEventCreateWithFlags(&io_ev[1], cudaEventDisableTiming));
    return VFS_OK;
}

int Model::alloc_sort_scratch() {
    sc = make_sort_config(n, digit_bits, tile_items);
    const size_t words = sort_scratch_words(sc);
    // Sized exactly for the configuration (a fresh buffer on every change), so every
    // configuration lays its regions out the same way whatever ran before it.
    if (words != scratch_words) {
        if (scratch) cudaFree(scratch);
        scratch = nullptr;
        VFS_CUDA_TRY(cudaMalloc(&scratch, words * sizeof(uint32_t)));
        scratch_words = words;
    }
    VFS_CUDA_TRY(cudaStreamSynchronize(stream));
    VFS_CUDA_TRY(cudaMemset(scratch, 0, words * sizeof(uint32_t)));
    sort_scratch.ghist = scratch;
    sort_scratch.counters = scratch + (size_t)sc.passes * sc.bins;
    sort_scratch.status = sort_scratch.counters + sc.passes;
    sort_scratch.mcount = sort_scratch.status + (size_t)sc.passes * sc.tiles * sc.bins;
    sort_scratch.dstatus = sort_scratch.mcount + 1;
    sort_scratch.err = err;
    invalidate_graph();
    return VFS_OK;
}

// Enqueues one substep (the body of WCSPHWithBoundaryModel::Step's loop,
// src/models/wcsph_with_boundary_model.cpp:93-116) for every scene. ExternalAccel needs no pass:
// the force kernel starts its accumulator at g.
int Model::enqueue_substep(cudaEvent_t* ev) {
    cudaStream_t s = stream;
    const int c = cur, o = 1 - cur;
    // Page-locked positions of a host round trip (enqueue_set_state left them): read by the key
    // pass itself, the velocities' upload queued behind it. Taken here, whatever returns below.
    const float* host_pos = keys_host_pos;
    const float* host_vel = keys_host_vel;
    uint32_t* const host_b_next = host_pos && keys_host_remap ? skin.b_next : nullptr;
    keys_host_pos = keys_host_vel = nullptr;
    keys_host_remap = false;
    if (ev) VFS_CUDA_TRY(cudaEventRecord(ev[0], s));
    // The sort scratch is zero here: zeroed when allocated and by every substep's cell pass.
    if (ev) VFS_CUDA_TRY(cudaEventRecord(ev[1], s));
    // Incremental stable sort: keys + the particles whose key changed (compacted into keys/vals),
    // a sort of those alone (count on the device), a merge with the rest.
    const SkinLists sk = active_skin();
    VFS_CUDA_TRY(launch_keys_delta(launch, pos[c], pkeys, keys, vals, moved, sc, sort_scratch, s,
                                   host_pos, pos[c], aux, skin.b_of_id, host_b_next));
    if (host_pos) {
        int rc = move_build_indices(host_b_next, 0, n);
        if (rc) return rc;
        rc = enqueue_vel_upload(scenes[0], 0, n, host_vel, io_stream);
        if (rc) return rc;
    }
    if (ev) VFS_CUDA_TRY(cudaEventRecord(ev[2], s));
    uint32_t *mk = nullptr, *mi = nullptr;
    VFS_CUDA_TRY(launch_sort(n, sc, sort_scratch, keys, keys_alt, vals, vals_alt, &mk, &mi, s,
                             /*vals_given=*/true, sort_scratch.mcount));
    VFS_CUDA_TRY(launch_merge(n, pkeys, moved, sort_scratch.mcount, mk, mi, sk_buf, sp_buf, s));
    skeys = sk_buf;
    sperm = sp_buf;
    if (ev) VFS_CUDA_TRY(cudaEventRecord(ev[3], s));
    // Velocities still on their way from the host (a host round trip's first substep): the cell
    // and density passes run without them, and their sorted copy and the force records' velocity
    // half follow once they have arrived, before the force pass.
    struct DeferOff {  // the flag holds for these two passes only, whatever returns
        StepLaunch& l;
        ~DeferOff() { l.defer_vel = false; }
    } defer_off{launch};
    launch.defer_vel = cells_wait != nullptr;
    VFS_CUDA_TRY(launch_cells_reorder(launch, n, skeys, sperm, cell_scan, pos[c], vel[c], pos[o], vel[o],
                                      scratch, (uint32_t)sort_scratch_words(sc), pkeys, cell_guess,
                                      sk, kc, s));
    if (ev) VFS_CUDA_TRY(cudaEventRecord(ev[4], s));
    VFS_CUDA_TRY(launch_density(launch, pos[o], vel[o], rec, cell_scan, aux, bnd, nbr, nbr_count, sk,
                                walk_sched, kc, s));
    launch.defer_vel = false;
    if (cells_wait) {
        VFS_CUDA_TRY(cudaStreamWaitEvent(s, cells_wait, 0));
        VFS_CUDA_TRY(launch_vel_records(n, sperm, stage + 3 * (size_t)n, vel[o], aux, rec, s));
    }
    if (ev) VFS_CUDA_TRY(cudaEventRecord(ev[5], s));
    VFS_CUDA_TRY(launch_force(launch, pos[o], vel[o], aux, rec, bnd, cell_scan, nbr, nbr_count, pos[c],
                              vel[c], record ? acc : nullptr, sk, kc, s, host_out));
    if (ev) VFS_CUDA_TRY(cudaEventRecord(ev[6], s));
    return VFS_OK;
}

int Model::run_substeps(int count) {
    if (count < 0) return fail(VFS_ERR_INVALID_ARGUMENT, "substep count must be >= 0");
    if (n == 0 || count == 0) return VFS_OK;
    if (!use_graph) {
        for (int i = 0; i < count; i++) {
            const int rc = enqueue_substep(nullptr);
            if (rc) return rc;
        }
        stepped = true;
        substeps_done += (uint64_t)count;
        return VFS_OK;
    }
    if (!graph_exec) {
        cudaGraph_t g = nullptr;
        VFS_CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_substep(nullptr);
        cudaError_t e = cudaStreamEndCapture(stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return fail(VFS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&graph_exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            graph_exec = nullptr;
            return fail(VFS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        }
    }
    for (int i = 0; i < count; i++) VFS_CUDA_TRY(cudaGraphLaunch(graph_exec, stream));
    stepped = true;
    substeps_done += (uint64_t)count;
    return VFS_OK;
}

int Model::check_device() {
    // The error word rides the stream into pinned memory, so one synchronisation covers both.
    VFS_CUDA_TRY(cudaMemcpyAsync(err_host, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
    VFS_CUDA_TRY(cudaStreamSynchronize(stream));
    const uint32_t e = *err_host;
    if (e) return fail(VFS_ERR_DEVICE_CHECK, "device error word set: " + std::to_string(e) +
                                                 (e & kErrLookbackTimeout ? " (look-back timeout)" : ""));
    return VFS_OK;
}

Model::~Model() {
    invalidate_graph();
    cudaFree(pos[0]);
    cudaFree(pos[1]);
    cudaFree(vel[0]);
    cudaFree(vel[1]);
    cudaFree(keys);
    cudaFree(keys_alt);
    cudaFree(vals);
    cudaFree(vals_alt);
    cudaFree(cell_scan);
    cudaFree(aux);
    cudaFree(rec);
    cudaFree(sk_buf);
    cudaFree(sp_buf);
    cudaFree(pkeys);
    cudaFree(moved);
    cudaFree(cell_guess);
    cudaFree(bnd);
    cudaFree(acc);
    cudaFree(stage);
    cudaFree(nbr);
    cudaFree(nbr_count);
    cudaFree(skin.list);
    cudaFree(skin.count);
    cudaFree(skin.x_build);
    cudaFree(skin.b_of_id);
    cudaFree(skin.b_next);
    cudaFree(skin.xcur);
    cudaFree(skin.stale);
    cudaFree(skin.ctl);
    cudaFree(skin.queue);
    cudaFree(skin.seg_n);
    cudaFree(skin.wcount);
    cudaFree(scratch);
    cudaFree(err);
    cudaFree(walk_sched);
    if (io_ev[0]) cudaEventDestroy(io_ev[0]);
    if (io_ev[1]) cudaEventDestroy(io_ev[1]);
    if (io_stream) cudaStreamDestroy(io_stream);
    if (err_host) cudaFreeHost(err_host);
    cudaFree(d_scenes);
    cudaFree(d_scene_of);
    cudaFree(d_objects);
    for (auto& sh : scenes)
        for (auto& o : sh.objects) {
            cudaFree(o.d_sdf);
            cudaFree(o.d_vm);
        }
    if (own_stream && stream) cudaStreamDestroy(stream);
}

int Model::init() {
    uint64_t total = 0;
    for (SceneHost& sh : scenes) {
        sh.off = (uint32_t)total;
        sh.n = (uint32_t)sh.sph.n_particles;
        total += sh.n;
    }
    if (total > kMaxParticles) return fail(VFS_ERR_CAPACITY, "more than 2^30 particles in total");
    n = (uint32_t)total;
    const size_t N = n ? n : 1;
    VFS_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    own_stream = true;
    for (int b = 0; b < 2; b++) {
        VFS_CUDA_TRY(cudaMalloc(&pos[b], N * sizeof(float4)));
        VFS_CUDA_TRY(cudaMalloc(&vel[b], N * sizeof(float4)));
    }
    VFS_CUDA_TRY(cudaMalloc(&keys, N * 4));
    VFS_CUDA_TRY(cudaMalloc(&keys_alt, N * 4));
    VFS_CUDA_TRY(cudaMalloc(&vals, N * 4));
    VFS_CUDA_TRY(cudaMalloc(&vals_alt, N * 4));
    VFS_CUDA_TRY(cudaMalloc(&cell_scan, (N + 1) * 4));
    VFS_CUDA_TRY(cudaMalloc(&sk_buf, N * 4));
    VFS_CUDA_TRY(cudaMalloc(&sp_buf, N * 4));
    VFS_CUDA_TRY(cudaMalloc(&pkeys, N * 4));
    VFS_CUDA_TRY(cudaMemset(pkeys, 0xFF, N * 4));  // sorted, and no key equals it: all moved
    VFS_CUDA_TRY(cudaMalloc(&moved, (2 * ((N + 31) / 32) + 1) * 4));
    VFS_CUDA_TRY(cudaMalloc(&cell_guess, (N / 128 + 2) * 4));
    VFS_CUDA_TRY(cudaMemset(cell_guess, 0, (N / 128 + 2) * 4));
    VFS_CUDA_TRY(cudaMalloc(&aux, N * sizeof(float4)));
    VFS_CUDA_TRY(cudaMalloc(&rec, 2 * N * sizeof(float4)));
    VFS_CUDA_TRY(cudaMalloc(&bnd, N * sizeof(float4)));
    VFS_CUDA_TRY(cudaMalloc(&acc, N * sizeof(float4)));
    VFS_CUDA_TRY(cudaMalloc(&stage, N * 32));
    VFS_CUDA_TRY(cudaMalloc(&nbr, N * nbr_cap * sizeof(uint32_t)));
    VFS_CUDA_TRY(cudaMalloc(&nbr_count, N * sizeof(uint32_t)));
    VFS_CUDA_TRY(cudaMalloc(&err, 4));
    VFS_CUDA_TRY(cudaMemset(err, 0, 4));
    VFS_CUDA_TRY(cudaMalloc(&walk_sched, 2 * sizeof(uint32_t)));
    VFS_CUDA_TRY(cudaMemset(walk_sched, 0, 2 * sizeof(uint32_t)));
    VFS_CUDA_TRY(cudaMallocHost(&err_host, 4));
    for (int b = 0; b < 2; b++) {
        VFS_CUDA_TRY(cudaMemset(pos[b], 0, N * sizeof(float4)));
        VFS_CUDA_TRY(cudaMemset(vel[b], 0, N * sizeof(float4)));
    }
    VFS_CUDA_TRY(cudaMemset(aux, 0, N * sizeof(float4)));
    VFS_CUDA_TRY(cudaMemset(bnd, 0, N * sizeof(float4)));
    VFS_CUDA_TRY(cudaMemset(acc, 0, N * sizeof(float4)));
    VFS_CUDA_TRY(cudaMemset(keys, 0, N * 4));
    VFS_CUDA_TRY(cudaMemset(cell_scan, 0, (N + 1) * 4));
    if (scenes.size() > 1) {
        VFS_CUDA_TRY(cudaMalloc(&d_scenes, scenes.size() * sizeof(SceneParams)));
        VFS_CUDA_TRY(cudaMalloc(&d_scene_of, N * sizeof(uint16_t)));
        std::vector<uint32_t> off(scenes.size() + 1);
        for (size_t k = 0; k < scenes.size(); k++) off[k] = scenes[k].off;
        off[scenes.size()] = n;
        uint32_t* d_off = nullptr;
        VFS_CUDA_TRY(cudaMalloc(&d_off, off.size() * 4));
        VFS_CUDA_TRY(cudaMemcpy(d_off, off.data(), off.size() * 4, cudaMemcpyHostToDevice));
        if (n) k_fill_scene_of<<<(n + 255) / 256, 256>>>(d_off, (uint32_t)scenes.size(), n, d_scene_of);
        VFS_CUDA_TRY(cudaGetLastError());
        VFS_CUDA_TRY(cudaDeviceSynchronize());
        cudaFree(d_off);
    }
    skeys = keys;
    sperm = vals;
    int rc = alloc_sort_scratch();
    if (rc) return rc;
    // Initial ids: slot index.
    std::vector<float4> init(N);
    for (size_t i = 0; i < N; i++) {
        uint32_t id = (uint32_t)i;
        float f;
        std::memcpy(&f, &id, 4);
        init[i] = make_float4(0.f, 0.f, 0.f, f);
    }
    VFS_CUDA_TRY(cudaMemcpy(pos[cur], init.data(), N * sizeof(float4), cudaMemcpyHostToDevice));
    rc = alloc_skin();
    if (rc) return rc;
    return refresh_params();
}

// Candidate lists with a skin, 228 bytes per particle. Three-lane (small) models do not use them,
// and a model too large for them on this device runs without (every particle walks its buckets).
int Model::alloc_skin() {
    if (n == 0 || planes_mode(n)) return VFS_OK;
    const size_t N = n;
    SkinLists s{};
    s.cap = kSkinCap;
    if (cudaMalloc(&s.list, N * s.cap * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&s.count, N * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&s.x_build, N * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&s.b_of_id, N * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&s.b_next, N * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&s.xcur, N * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&s.stale, scenes.size() * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&s.ctl, scenes.size() * kSkinCtl * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&s.queue, N * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&s.seg_n, ((N + 127) / 128) * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&s.wcount, sizeof(uint32_t)) != cudaSuccess) {
        cudaGetLastError();  // out of memory is not sticky: clear it and go on without lists
        cudaFree(s.list);
        cudaFree(s.count);
        cudaFree(s.x_build);
        cudaFree(s.b_of_id);
        cudaFree(s.b_next);
        cudaFree(s.xcur);
        cudaFree(s.stale);
        cudaFree(s.ctl);
        cudaFree(s.queue);
        cudaFree(s.seg_n);
        cudaFree(s.wcount);
        return VFS_OK;
    }
    VFS_CUDA_TRY(cudaMemset(s.count, 0, N * sizeof(uint32_t)));
    VFS_CUDA_TRY(cudaMemset(s.b_of_id, 0, N * sizeof(uint32_t)));  // any index below n until a build
    VFS_CUDA_TRY(cudaMemset(s.stale, 0, scenes.size() * sizeof(uint32_t)));
    VFS_CUDA_TRY(cudaMemset(s.wcount, 0, sizeof(uint32_t)));
    skin = s;
    return invalidate_skin();
}

// Every list is rebuilt by the next substep: the build positions are set far away (3.4e38), so
// every scene's displacement check fails, and the build policy starts over (builds counted from
// zero, no wait).
int Model::invalidate_skin() {
    if (!skin.x_build) return VFS_OK;
    VFS_CUDA_TRY(cudaMemsetAsync(skin.x_build, 0x7F, (size_t)n * sizeof(float4), stream));
    std::vector<uint32_t> ctl(scenes.size() * kSkinCtl, 0u);
    for (size_t s = 0; s < scenes.size(); s++) ctl[s * kSkinCtl + kCtlAllow] = 1u;
    VFS_CUDA_TRY(cudaMemcpyAsync(skin.ctl, ctl.data(), ctl.size() * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice, stream));
    VFS_CUDA_TRY(cudaStreamSynchronize(stream));  // ctl is a local
    return VFS_OK;
}

// The lists the passes use: none when switched off.
SkinLists Model::active_skin() const {
    return skin_fraction > 0.0f ? skin : SkinLists{};
}

int create_model(const std::vector<SceneHost>& scenes, Model** out) {
    *out = nullptr;
    Model* m = new Model();
    m->scenes = scenes;
    const int rc = m->init();
    if (rc) {
        delete m;
        return rc;
    }
    *out = m;
    return VFS_OK;
}

// The address under which this device's kernels reach host buffer p: page-locked host memory
// (cudaHostAlloc / cudaHostRegister, mapped under unified addressing) or device and managed
// memory of this device. Null for pageable memory, which goes through a staging copy.
void* device_alias(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    int dev = -1;
    cudaGetDevice(&dev);
    if (a.type == cudaMemoryTypeHost) return a.devicePointer;
    if ((a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == dev)
        return a.devicePointer;
    return nullptr;
}

int Model::set_state(uint32_t scene, const float* pos3, const float* vel3, uint32_t offset,
                     int64_t count) {
    const int rc = enqueue_set_state(scene, pos3, vel3, offset, count);
    if (rc) return rc;
    VFS_CUDA_TRY(cudaStreamSynchronize(stream));
    return VFS_OK;
}

int Model::step_host(const float* pos3, const float* vel3, int32_t count, float* pos_out,
                     float* vel_out, float* dens_out) {
    if (count < 1) return fail(VFS_ERR_INVALID_ARGUMENT, "step_host needs at least one substep");
    if (!pos3 != !vel3) return fail(VFS_ERR_INVALID_ARGUMENT, "pos and vel must both be given or both be NULL");
    if (scenes.size() != 1) return fail(VFS_ERR_INVALID_ARGUMENT, "step_host steps a single-scene model");
    HostOut ho;
    ho.pos3 = static_cast<float*>(device_alias(pos_out));
    ho.vel3 = static_cast<float*>(device_alias(vel_out));
    ho.dens = static_cast<float*>(device_alias(dens_out));
    const bool fused = n > 0 && ho.any() && (!pos_out || ho.pos3) && (!vel_out || ho.vel3) &&
                       (!dens_out || ho.dens);
    int remaining = count;
    const void* in_p = pos3 ? device_alias(pos3) : nullptr;
    const void* in_v = vel3 ? device_alias(vel3) : nullptr;
    if (fused && count == 1 && in_p && in_v && use_graph) {
        // The frame loop's case: one substep between a page-locked upload and read-back. The
        // sequence below (the upload, the velocities on the side stream, the substep with its
        // host outputs) is captured once for this set of buffers and replayed as one graph. The
        // graph either moves the build indices with the upload or not (ids_unique at capture),
        // so a change of ids_unique captures again.
        const void* key[11] = {pos3, vel3, pos_out, vel_out, dens_out, in_p, in_v,
                               ho.pos3, ho.vel3, ho.dens,
                               reinterpret_cast<const void*>((uintptr_t)ids_unique)};
        if (!host_graph || std::memcmp(key, host_graph_key, sizeof key) != 0) {
            if (host_graph) cudaGraphExecDestroy(host_graph);
            host_graph = nullptr;
            int rc = ensure_io_stream();
            if (rc) return rc;
            cudaGraph_t g = nullptr;
            VFS_CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            rc = enqueue_set_state(0, pos3, vel3, 0, -1, io_stream);
            if (rc == VFS_OK) {
                cells_wait = io_ev[1];
                set_host_out(ho);
                rc = enqueue_substep(nullptr);
                cells_wait = nullptr;
                set_host_out(HostOut{});
            }
            cudaError_t e = cudaStreamEndCapture(stream, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (e != cudaSuccess) return fail(VFS_ERR_CUDA, std::string("host-step capture: ") + cudaGetErrorString(e));
            e = cudaGraphInstantiate(&host_graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                host_graph = nullptr;
                return fail(VFS_ERR_CUDA, std::string("host-step instantiate: ") + cudaGetErrorString(e));
            }
            std::memcpy(host_graph_key, key, sizeof key);
        }
        VFS_CUDA_TRY(cudaGraphLaunch(host_graph, stream));
        ids_unique = true;  // the replayed upload set every id to its slot
        stepped = true;
        substeps_done += 1;
        return check_device();
    }
    if (pos3 && n > 0) {
        // Positions on the model's stream; velocities, first read by the cell pass, on a side
        // stream after them (so after all work queued before), their upload overlapping the key
        // and sort passes. The first substep is launched directly and waits for them before its
        // cell pass.
        int rc = ensure_io_stream();
        if (rc) return rc;
        rc = enqueue_set_state(0, pos3, vel3, 0, -1, io_stream);
        if (rc) return rc;
        cells_wait = io_ev[1];
        if (fused && count == 1) set_host_out(ho);
        rc = enqueue_substep(nullptr);
        cells_wait = nullptr;
        set_host_out(HostOut{});
        if (rc) return rc;
        stepped = true;
        substeps_done += 1;
        if (--remaining == 0) return fused ? check_device() : get_state(0, pos_out, vel_out, dens_out, nullptr);
    }
    int rc = run_substeps(fused ? remaining - 1 : remaining);
    if (rc) return rc;
    if (!fused) return get_state(0, pos_out, vel_out, dens_out, nullptr);
    // The last substep launched directly (not from the graph), its density and force passes also
    // writing the page-locked outputs: the read-back overlaps the passes instead of following them.
    set_host_out(ho);
    rc = enqueue_substep(nullptr);
    set_host_out(HostOut{});
    if (rc) return rc;
    stepped = true;
    substeps_done += 1;
    return check_device();
}

int Model::enqueue_set_state(uint32_t scene, const float* pos3, const float* vel3,
                             uint32_t offset, int64_t count, cudaStream_t vel_stream) {
    if (!vel_stream) vel_stream = stream;
    if (scene >= scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    const SceneHost& sh = scenes[scene];
    if (offset > sh.n) return fail(VFS_ERR_INVALID_ARGUMENT, "offset beyond the scene's particle count");
    const uint64_t cnt = count < 0 ? (uint64_t)(sh.n - offset) : (uint64_t)count;
    if (offset + cnt > sh.n)
        return fail(VFS_ERR_CAPACITY, "offset + count exceeds the scene's particle count");
    if (cnt == 0) return VFS_OK;
    if (!pos3 || !vel3) return fail(VFS_ERR_INVALID_ARGUMENT, "pos and vel must not be NULL");
    // The skin lists across the upload (see ids_unique): a whole scene's build indices follow
    // its slots to their new ids; after part of a scene ids may repeat, and nothing is moved
    // (the cell pass's displacement check then finds the lists stale).
    const bool whole = offset == 0 && cnt == sh.n;
    uint32_t* const b_next = whole && ids_unique ? skin.b_next : nullptr;
    if (!whole) ids_unique = false;
    else if (scenes.size() == 1) ids_unique = true;
    // Page-locked inputs are read by the conversion kernel itself (over NVLink-C2C on GB300);
    // pageable ones are copied into the staging buffer first.
    const float* sp = static_cast<const float*>(device_alias(pos3));
    if (!sp) {
        VFS_CUDA_TRY(cudaMemcpyAsync(stage, pos3, cnt * 12, cudaMemcpyHostToDevice, stream));
        sp = stage;
    }
    const unsigned blocks = (unsigned)((cnt + kIoBlock - 1) / kIoBlock);
    float* const vel_stage = stage + 3 * (size_t)n;
    if (vel_stream == stream) {
        const float* sv = static_cast<const float*>(device_alias(vel3));
        if (!sv) {
            VFS_CUDA_TRY(cudaMemcpyAsync(vel_stage, vel3, cnt * 12, cudaMemcpyHostToDevice, stream));
            sv = vel_stage;
        }
        k_expand_state<<<blocks, kIoBlock, 0, stream>>>(sh.off + offset, (uint32_t)cnt, sp, sv,
                                                         pos[cur], vel[cur], aux, skin.b_of_id,
                                                         b_next, n);
        VFS_CUDA_TRY(cudaGetLastError());
        return move_build_indices(b_next, sh.off, cnt);
    } else if (sp != stage && scenes.size() == 1 && whole) {
        // Positions first, alone on the host link, read by the next substep's key pass itself
        // (the upload and the key arithmetic overlap); the velocities follow after that pass.
        keys_host_pos = sp;
        keys_host_vel = vel3;
        keys_host_remap = b_next != nullptr;
        return VFS_OK;
    } else {
        // Positions first, alone on the host link; the velocities follow on the side stream.
        k_expand_state<<<blocks, kIoBlock, 0, stream>>>(sh.off + offset, (uint32_t)cnt, sp, nullptr,
                                                         pos[cur], vel[cur], aux, skin.b_of_id,
                                                         b_next, n);
        VFS_CUDA_TRY(cudaGetLastError());
        const int rc = move_build_indices(b_next, sh.off, cnt);
        if (rc) return rc;
        return enqueue_vel_upload(sh, offset, cnt, vel3, vel_stream);
    }
}

// The build indices an upload stored under the new ids of slots [off, off + cnt) (b_next, or
// nothing to do when null) replace the old mapping there.
int Model::move_build_indices(const uint32_t* b_next, uint32_t off, uint64_t cnt) {
    if (!b_next || cnt == 0) return VFS_OK;
    VFS_CUDA_TRY(cudaMemcpyAsync(skin.b_of_id + off, b_next + off, cnt * sizeof(uint32_t),
                                 cudaMemcpyDeviceToDevice, stream));
    return VFS_OK;
}

int Model::enqueue_vel_upload(const SceneHost& sh, uint32_t offset, uint64_t cnt, const float* vel3,
                              cudaStream_t vel_stream) {
    // By DMA into the staging buffer (a copy engine, so the velocities move while the key, sort
    // and later passes keep every SM busy); io_ev[1] marks them done. The substep's
    // k_vel_records reads them there (packed float3 in slot order) by the sort's permutation.
    float* const vel_stage = stage + 3 * (size_t)n;
    VFS_CUDA_TRY(cudaEventRecord(io_ev[0], stream));
    VFS_CUDA_TRY(cudaStreamWaitEvent(vel_stream, io_ev[0], 0));
    VFS_CUDA_TRY(cudaMemcpyAsync(vel_stage + 3 * ((size_t)sh.off + offset), vel3, cnt * 12,
                                 cudaMemcpyHostToDevice, vel_stream));
    VFS_CUDA_TRY(cudaEventRecord(io_ev[1], vel_stream));
    return VFS_OK;
}

int Model::get_state(uint32_t scene, float* pos3, float* vel3, float* dens, uint32_t* ids) {
    if (scene >= scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    const SceneHost& sh = scenes[scene];
    if (sh.n == 0) return VFS_OK;
    // Page-locked outputs are written by the packing kernel itself; the others through staging.
    float* dp = static_cast<float*>(device_alias(pos3));
    float* dv = static_cast<float*>(device_alias(vel3));
    float* dd = static_cast<float*>(device_alias(dens));
    uint32_t* di = static_cast<uint32_t*>(device_alias(ids));
    float* sp = pos3 && !dp ? stage : nullptr;
    float* sv = vel3 && !dv ? stage + 3 * (size_t)n : nullptr;
    float* sd = dens && !dd ? stage + 6 * (size_t)n : nullptr;
    uint32_t* si = ids && !di ? reinterpret_cast<uint32_t*>(stage + 7 * (size_t)n) : nullptr;
    k_compact_state<<<(sh.n + kIoBlock - 1) / kIoBlock, kIoBlock, 0, stream>>>(
        sh.n, sh.off, pos[cur], vel[cur], aux, dp ? dp : sp, dv ? dv : sv, dd ? dd : sd,
        di ? di : si);
    VFS_CUDA_TRY(cudaGetLastError());
    if (sp) VFS_CUDA_TRY(cudaMemcpyAsync(pos3, sp, (size_t)sh.n * 12, cudaMemcpyDeviceToHost, stream));
    if (sv) VFS_CUDA_TRY(cudaMemcpyAsync(vel3, sv, (size_t)sh.n * 12, cudaMemcpyDeviceToHost, stream));
    if (sd) VFS_CUDA_TRY(cudaMemcpyAsync(dens, sd, (size_t)sh.n * 4, cudaMemcpyDeviceToHost, stream));
    if (si) VFS_CUDA_TRY(cudaMemcpyAsync(ids, si, (size_t)sh.n * 4, cudaMemcpyDeviceToHost, stream));
    return check_device();
}

int Model::get_acc(uint32_t scene, float* acc3) {
    if (scene >= scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    const SceneHost& sh = scenes[scene];
    if (!acc3 || sh.n == 0) return VFS_OK;
    int rc = check_device();
    if (rc) return rc;
    std::vector<float4> a(sh.n);
    VFS_CUDA_TRY(cudaMemcpy(a.data(), acc + sh.off, (size_t)sh.n * sizeof(float4), cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < sh.n; i++) {
        acc3[3 * i] = a[i].x;
        acc3[3 * i + 1] = a[i].y;
        acc3[3 * i + 2] = a[i].z;
    }
    return VFS_OK;
}

int Model::get_neighbors(uint32_t scene, uint32_t* keys_out, uint32_t* perm_out, uint32_t* offs_out) {
    if (scene >= scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    if (!stepped) return fail(VFS_ERR_NOT_READY, "no substep has run yet");
    const SceneHost& sh = scenes[scene];
    if (sh.n == 0) return VFS_OK;
    uint32_t* off = reinterpret_cast<uint32_t*>(stage);
    VFS_CUDA_TRY(launch_offsets(sh.n, sh.off, cell_scan, off, stream));
    if (keys_out)
        VFS_CUDA_TRY(cudaMemcpyAsync(keys_out, skeys + sh.off, (size_t)sh.n * 4, cudaMemcpyDeviceToHost, stream));
    if (perm_out)
        VFS_CUDA_TRY(cudaMemcpyAsync(perm_out, sperm + sh.off, (size_t)sh.n * 4, cudaMemcpyDeviceToHost, stream));
    if (offs_out) VFS_CUDA_TRY(cudaMemcpyAsync(offs_out, off, (size_t)sh.n * 4, cudaMemcpyDeviceToHost, stream));
    const int rc = check_device();
    if (rc) return rc;
    for (uint32_t i = 0; i < sh.n; i++) {  // scene-local keys and indices
        if (keys_out) keys_out[i] -= sh.off;
        if (perm_out) perm_out[i] -= sh.off;
    }
    return VFS_OK;
}

int Model::get_boundary(uint32_t scene, float* bdens, float* bgrad) {
    if (scene >= scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    const SceneHost& sh = scenes[scene];
    if (sh.n == 0) return VFS_OK;
    int rc = check_device();
    if (rc) return rc;
    std::vector<float4> b(sh.n);
    VFS_CUDA_TRY(cudaMemcpy(b.data(), bnd + sh.off, (size_t)sh.n * sizeof(float4), cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < sh.n; i++) {
        if (bdens) bdens[i] = b[i].w;
        if (bgrad) {
            bgrad[3 * i] = b[i].x;
            bgrad[3 * i + 1] = b[i].y;
            bgrad[3 * i + 2] = b[i].z;
        }
    }
    return VFS_OK;
}

int Model::add_object(uint32_t scene, const vfs_boundary_object& src, const float* d_sdf_in,
                      const float* d_vm_in) {
    if (scene >= scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    SceneHost& sh = scenes[scene];
    if (sh.objects.size() >= (size_t)kMaxObjects)
        return fail(VFS_ERR_CAPACITY, "at most " + std::to_string(kMaxObjects) + " boundary objects per scene");
    for (int a = 0; a < 3; a++)
        if (src.resolution[a] < 2) return fail(VFS_ERR_INVALID_ARGUMENT, "grid resolution must be >= 2 per axis");
    ObjectStore o;
    o.info = src;
    o.info.sdf_grid = nullptr;
    o.info.volume_map_grid = nullptr;
    const size_t cnt = (size_t)src.resolution[0] * src.resolution[1] * src.resolution[2];
    if (!d_sdf_in && (!src.sdf_grid || !src.volume_map_grid))
        return fail(VFS_ERR_INVALID_ARGUMENT, "sdf_grid and volume_map_grid must not be NULL");
    VFS_CUDA_TRY(cudaMalloc(&o.d_sdf, cnt * 4));
    VFS_CUDA_TRY(cudaMalloc(&o.d_vm, cnt * 4));
    const cudaMemcpyKind kind = d_sdf_in ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    VFS_CUDA_TRY(cudaMemcpyAsync(o.d_sdf, d_sdf_in ? d_sdf_in : src.sdf_grid, cnt * 4, kind, stream));
    VFS_CUDA_TRY(cudaMemcpyAsync(o.d_vm, d_vm_in ? d_vm_in : src.volume_map_grid, cnt * 4, kind, stream));
    VFS_CUDA_TRY(cudaStreamSynchronize(stream));
    sh.objects.push_back(o);
    return refresh_params();
}

int Model::add_analytic(uint32_t scene, const vfs_analytic_object& a) {
    if (scene >= scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    if (a.shape < 0 || a.shape > 2) return fail(VFS_ERR_INVALID_ARGUMENT, "unknown analytic shape");
    for (int k = 0; k < 3; k++)
        if (a.resolution[k] < 2) return fail(VFS_ERR_INVALID_ARGUMENT, "grid resolution must be >= 2 per axis");
    const float h = scenes[scene].sim.smooth_radius;
    // Object matrix: translate * rotate * scale (gfx::Transform::Matrix, src/gfx/transform.cpp:33-45).
    M4 T = m4_identity();
    T.a[12] = a.position[0];
    T.a[13] = a.position[1];
    T.a[14] = a.position[2];
    const M4 R = m4_rotation(a.rotation_angle_deg, a.rotation_axis);
    M4 S = m4_identity();
    for (int k = 0; k < 3; k++) S.a[k * 5] = (a.scale[k] == 0.0f) ? 1.0 : (double)a.scale[k];
    const M4 W = m4_mul(m4_mul(T, R), S);
    M4 Wi;
    if (!m4_inverse(W, Wi)) return fail(VFS_ERR_INVALID_ARGUMENT, "object transform is singular");
    vfs_boundary_object info{};
    for (int k = 0; k < 16; k++) {
        info.transform[k] = (float)Wi.a[k];
        info.rotation[k] = (float)R.a[k];
    }
    // MeshSDF::Build box: shape AABB grown by tolerance (0) + margin (8h), in float
    // (src/util/mesh_sdf.cpp:28-44, src/scenes/generic_scene.cpp:100).
    const float margin = (float)(8.0 * (double)h);
    float lo[3], hi[3];
    for (int k = 0; k < 3; k++) {
        const double e = a.shape == 0 ? a.params[0] : a.params[k];
        lo[k] = (float)-e;
        hi[k] = (float)e;
        info.box_size[k] = (hi[k] - lo[k]) + 2.0f * margin;
        info.box_pos[k] = lo[k] - margin;
        info.resolution[k] = a.resolution[k];
    }
    VolumeMapParams vp{};
    vp.shape = a.shape;
    for (int k = 0; k < 3; k++) vp.prm[k] = a.params[k];
    vp.h = h;
    for (int k = 0; k < 3; k++) {
        vp.res[k] = a.resolution[k];
        vp.dmin[k] = info.box_pos[k];
        const float dmax = info.box_pos[k] + info.box_size[k];
        vp.step[k] = (double)((dmax - vp.dmin[k]) / (float)(a.resolution[k] - 1u));
    }
    vp.qn = 16;
    gauss_legendre_nodes(vp.qn, vp.gx, vp.gw);
    vp.c0 = 0.5 * (double)(h - (-h));
    vp.c1 = 0.5 * (double)(h + (-h));
    for (int k = 0; k < vp.qn; k++) vp.gxf[k] = (float)(vp.c0 * vp.gx[k] + vp.c1);
    const double hd = (double)h;
    vp.w_factor = 8.0 / (pi_d() * hd * hd * hd);
    vp.full_ball = volume_map_full_ball(vp);
    const size_t cnt = (size_t)a.resolution[0] * a.resolution[1] * a.resolution[2];
    float *d_sdf = nullptr, *d_vm = nullptr;
    VFS_CUDA_TRY(cudaMalloc(&d_sdf, cnt * 4));
    VFS_CUDA_TRY(cudaMalloc(&d_vm, cnt * 4));
    cudaError_t e = launch_volume_map(vp, d_sdf, d_vm, stream);
    if (e != cudaSuccess) {
        cudaFree(d_sdf);
        cudaFree(d_vm);
        return fail(VFS_ERR_CUDA, std::string("volume map: ") + cudaGetErrorString(e));
    }
    const int rc = add_object(scene, info, d_sdf, d_vm);
    cudaFree(d_sdf);
    cudaFree(d_vm);
    return rc;
}

namespace {

// Device copy of a host mesh; free() releases it.
struct MeshUpload {
    MeshDev dev{};
    void* blocks[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    void free() {
        for (void*& b : blocks) {
            if (b) cudaFree(b);
            b = nullptr;
        }
    }
};

template <typename T>
std::vector<T> rows4(const std::vector<T>& v, size_t width) {
    std::vector<T> out(v.size() / width * 4, T(0));
    for (size_t r = 0; r < v.size() / width; r++)
        for (size_t c = 0; c < width; c++) out[4 * r + c] = v[width * r + c];
    return out;
}

int upload_mesh(const MeshHost& mh, MeshUpload& up) {
    const auto pos4 = rows4(mh.pos, 3);
    const auto tri4 = rows4(mh.tri, 3);
    const auto tn4 = rows4(mh.tri_normal, 3);
    const auto en4 = rows4(mh.edge_normal, 3);
    const auto vn4 = rows4(mh.vertex_normal, 3);
    const void* src[6] = {pos4.data(), tri4.data(), tn4.data(), en4.data(), vn4.data(), mh.nodes.data()};
    const size_t bytes[6] = {pos4.size() * 4, tri4.size() * 4, tn4.size() * 4, en4.size() * 4,
                             vn4.size() * 4, mh.nodes.size() * sizeof(BvhNode)};
    for (int k = 0; k < 6; k++) {
        cudaError_t e = cudaMalloc(&up.blocks[k], bytes[k]);
        if (e == cudaSuccess) e = cudaMemcpy(up.blocks[k], src[k], bytes[k], cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            up.free();
            return fail(VFS_ERR_CUDA, std::string("mesh upload: ") + cudaGetErrorString(e));
        }
    }
    up.dev.pos = static_cast<const float4*>(up.blocks[0]);
    up.dev.tri = static_cast<const uint4*>(up.blocks[1]);
    up.dev.tri_normal = static_cast<const float4*>(up.blocks[2]);
    up.dev.edge_normal = static_cast<const float4*>(up.blocks[3]);
    up.dev.vertex_normal = static_cast<const float4*>(up.blocks[4]);
    up.dev.nodes = static_cast<const BvhNode*>(up.blocks[5]);
    return VFS_OK;
}

}  // namespace

// GenericScene::AddBoundaryObject for an OBJ mesh (src/scenes/generic_scene.cpp:89-124): the mesh
// SDF box is the mesh bounds grown by tolerance 0 + margin 8h (MeshSDF::Init/Build,
// src/util/mesh_sdf.cpp:14-44), the SDF grid holds the mesh's signed distance at the nodes and the
// volume map integrates it (GenerateVolumeMap, src/util/volume_map.cpp:9-54), both on the GPU.
int Model::add_mesh(uint32_t scene, const vfs_mesh_object& a) {
    if (scene >= scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    for (int k = 0; k < 3; k++)
        if (a.resolution[k] < 2) return fail(VFS_ERR_INVALID_ARGUMENT, "grid resolution must be >= 2 per axis");
    std::vector<float> pos;
    std::vector<uint32_t> tri;
    std::string err;
    if (a.obj_path) {
        if (!load_obj(a.obj_path, pos, tri, err)) return fail(VFS_ERR_IO, err);
    } else {
        if (!a.vertices || !a.triangles) return fail(VFS_ERR_INVALID_ARGUMENT, "mesh without an OBJ path or arrays");
        pos.assign(a.vertices, a.vertices + 3 * (size_t)a.n_vertices);
        tri.assign(a.triangles, a.triangles + 3 * (size_t)a.n_triangles);
    }
    MeshHost mh;
    if (!build_mesh(pos, tri, mh, err)) return fail(VFS_ERR_INVALID_ARGUMENT, "mesh: " + err);
    const float h = scenes[scene].sim.smooth_radius;
    M4 T = m4_identity();
    T.a[12] = a.position[0];
    T.a[13] = a.position[1];
    T.a[14] = a.position[2];
    const M4 R = m4_rotation(a.rotation_angle_deg, a.rotation_axis);
    M4 S = m4_identity();
    for (int k = 0; k < 3; k++) S.a[k * 5] = (a.scale[k] == 0.0f) ? 1.0 : (double)a.scale[k];
    const M4 W = m4_mul(m4_mul(T, R), S);
    M4 Wi;
    if (!m4_inverse(W, Wi)) return fail(VFS_ERR_INVALID_ARGUMENT, "object transform is singular");
    vfs_boundary_object info{};
    for (int k = 0; k < 16; k++) {
        info.transform[k] = (float)Wi.a[k];
        info.rotation[k] = (float)R.a[k];
    }
    const float margin = (float)(0.0 + 8.0 * (double)h);
    for (int k = 0; k < 3; k++) {
        info.box_size[k] = (mh.hi[k] - mh.lo[k]) + 2.0f * margin;
        info.box_pos[k] = mh.lo[k] - margin;
        info.resolution[k] = a.resolution[k];
    }
    VolumeMapParams vp{};
    vp.h = h;
    for (int k = 0; k < 3; k++) {
        vp.res[k] = a.resolution[k];
        vp.dmin[k] = info.box_pos[k];
        const float dmax = info.box_pos[k] + info.box_size[k];
        vp.step[k] = (double)((dmax - vp.dmin[k]) / (float)(a.resolution[k] - 1u));
    }
    vp.qn = 16;
    gauss_legendre_nodes(vp.qn, vp.gx, vp.gw);
    vp.c0 = 0.5 * (double)(h - (-h));
    vp.c1 = 0.5 * (double)(h + (-h));
    for (int k = 0; k < vp.qn; k++) vp.gxf[k] = (float)(vp.c0 * vp.gx[k] + vp.c1);
    const double hd = (double)h;
    vp.w_factor = 8.0 / (pi_d() * hd * hd * hd);
    vp.full_ball = volume_map_full_ball(vp);
    MeshUpload up;
    int rc = upload_mesh(mh, up);
    if (rc) return rc;
    const size_t cnt = (size_t)a.resolution[0] * a.resolution[1] * a.resolution[2];
    float *d_sdf = nullptr, *d_vm = nullptr;
    cudaError_t e = cudaMalloc(&d_sdf, cnt * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d_vm, cnt * 4);
    if (e == cudaSuccess) e = launch_mesh_volume_map(vp, up.dev, d_sdf, d_vm, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    up.free();
    if (e != cudaSuccess) {
        if (d_sdf) cudaFree(d_sdf);
        if (d_vm) cudaFree(d_vm);
        return fail(VFS_ERR_CUDA, std::string("mesh volume map: ") + cudaGetErrorString(e));
    }
    rc = add_object(scene, info, d_sdf, d_vm);
    cudaFree(d_sdf);
    cudaFree(d_vm);
    return rc;
}

int profile_phases(Model& m, int32_t count, float* phase_ms) {
    if (!phase_ms || count < 1) return fail(VFS_ERR_INVALID_ARGUMENT, "bad argument");
    for (int k = 0; k < 6; k++) phase_ms[k] = 0.0f;
    if (m.n == 0) return VFS_OK;
    cudaEvent_t ev[7];
    for (int k = 0; k < 7; k++) VFS_CUDA_TRY(cudaEventCreate(&ev[k]));
    // Event pairs in enqueue order: an empty pair (event overhead), keys, sort, cells+reorder,
    // density, force.
    double acc_ms[6] = {0, 0, 0, 0, 0, 0};
    int rc = VFS_OK;
    for (int it = 0; it < count && rc == VFS_OK; it++) {
        rc = m.enqueue_substep(ev);
        if (rc) break;
        cudaError_t e = cudaEventSynchronize(ev[6]);
        if (e != cudaSuccess) {
            rc = fail(VFS_ERR_CUDA, cudaGetErrorString(e));
            break;
        }
        for (int k = 0; k < 6; k++) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
            acc_ms[k] += ms;
        }
    }
    for (int k = 0; k < 7; k++) cudaEventDestroy(ev[k]);
    m.stepped = true;
    if (rc) return rc;
    // Reported order: keys, sort, cells+reorder, density, force, clear.
    phase_ms[0] = (float)(acc_ms[1] / count);
    phase_ms[1] = (float)(acc_ms[2] / count);
    phase_ms[2] = (float)(acc_ms[3] / count);
    phase_ms[3] = (float)(acc_ms[4] / count);
    phase_ms[4] = (float)(acc_ms[5] / count);
    phase_ms[5] = (float)(acc_ms[0] / count);
    return m.check_device();
}

static int set_stream(Model& m, void* stream) {
    cudaStreamSynchronize(m.stream);
    if (m.own_stream && m.stream) cudaStreamDestroy(m.stream);
    m.own_stream = false;
    m.stream = nullptr;
    if (stream) {
        m.stream = (cudaStream_t)stream;
    } else {
        VFS_CUDA_TRY(cudaStreamCreateWithFlags(&m.stream, cudaStreamNonBlocking));
        m.own_stream = true;
    }
    m.invalidate_graph();
    return VFS_OK;
}

// Neighbour-list slots per particle: lists longer than this make the force pass walk the
// candidates again (and a differentiable rollout fail), so dense scenes want more slots; each slot
// costs 4 bytes per particle.
int set_neighbor_capacity(Model& m, int32_t slots) {
    if (slots < 16 || slots > 4096) return fail(VFS_ERR_INVALID_ARGUMENT, "neighbour capacity must be in [16, 4096]");
    VFS_CUDA_TRY(cudaStreamSynchronize(m.stream));
    const size_t N = m.n ? m.n : 1;
    uint32_t* fresh = nullptr;
    VFS_CUDA_TRY(cudaMalloc(&fresh, N * (size_t)slots * sizeof(uint32_t)));
    cudaFree(m.nbr);
    m.nbr = fresh;
    m.nbr_cap = (uint32_t)slots;
    m.invalidate_graph();
    m.stepped = false;
    return m.refresh_params();
}

int set_skin(Model& m, float skin) {
    if (!(skin >= 0.0f && skin <= 0.5f)) return fail(VFS_ERR_INVALID_ARGUMENT, "skin must be in [0, 0.5]");
    m.skin_fraction = skin;
    return m.refresh_params();  // new constants and graph; every list is rebuilt
}

float get_skin(const Model& m) { return m.skin.list ? m.skin_fraction : 0.0f; }

int get_skin_builds(Model& m, uint32_t scene, uint32_t* builds) {
    if (scene >= m.scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    *builds = 0;
    if (!m.skin.ctl) return VFS_OK;
    VFS_CUDA_TRY(cudaMemcpyAsync(m.err_host, m.skin.ctl + scene * kSkinCtl + kCtlBuilds, sizeof(uint32_t),
                                 cudaMemcpyDeviceToHost, m.stream));
    VFS_CUDA_TRY(cudaStreamSynchronize(m.stream));
    *builds = *m.err_host;
    return VFS_OK;
}

int set_sort_config(Model& m, int32_t digit_bits, int32_t tile_items) {
    if (digit_bits < 4 || digit_bits > 8) return fail(VFS_ERR_INVALID_ARGUMENT, "digit_bits must be in [4, 8]");
    if (tile_items != 8 && tile_items != 12 && tile_items != 16)
        return fail(VFS_ERR_INVALID_ARGUMENT, "tile_items must be 8, 12 or 16");
    VFS_CUDA_TRY(cudaStreamSynchronize(m.stream));
    m.digit_bits = digit_bits;
    m.tile_items = tile_items;
    return m.alloc_sort_scratch();
}

static int validate(const vfs_sim_params* sim, const vfs_sph_params* sph) {
    if (sim && !(sim->smooth_radius > 0.0f)) return fail(VFS_ERR_INVALID_ARGUMENT, "smooth_radius must be > 0");
    if (sph && sph->iterations < 1) return fail(VFS_ERR_INVALID_ARGUMENT, "iterations must be >= 1");
    if (sph && !(sph->target_density > 0.0f)) return fail(VFS_ERR_INVALID_ARGUMENT, "target_density must be > 0");
    if (sph && (sph->n_particles < 0 || (uint64_t)sph->n_particles > kMaxParticles))
        return fail(VFS_ERR_CAPACITY, "n_particles must be in [0, 2^30]");
    return VFS_OK;
}

static int set_scene_parameters(Model& m, uint32_t scene, const vfs_sim_params* sim,
                                const vfs_sph_params* sph, const vfs_wcsph_params* wc) {
    if (scene >= m.scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    int rc = validate(sim, nullptr);
    if (rc) return rc;
    if (sph && sph->iterations < 1) return fail(VFS_ERR_INVALID_ARGUMENT, "iterations must be >= 1");
    if (sph && !(sph->target_density > 0.0f)) return fail(VFS_ERR_INVALID_ARGUMENT, "target_density must be > 0");
    SceneHost& sh = m.scenes[scene];
    if (sim) sh.sim = *sim;
    if (sph) {
        const int32_t keep = sh.sph.n_particles;
        sh.sph = *sph;
        sh.sph.n_particles = keep;
    }
    if (wc) sh.wcsph = *wc;
    VFS_CUDA_TRY(cudaStreamSynchronize(m.stream));
    return m.refresh_params();
}

}  // namespace vfs

using vfs::fail;
using vfs::Model;

extern "C" {

struct vfs_model {
    Model* m = nullptr;
    ~vfs_model() { delete m; }
};

struct vfs_batch {
    Model* m = nullptr;
    ~vfs_batch() { delete m; }
};

}  // extern "C"

vfs::Model* vfs_model_impl(vfs_model* h) { return h ? h->m : nullptr; }
vfs::Model* vfs_batch_impl(vfs_batch* h) { return h ? h->m : nullptr; }

#define VFS_HANDLE(h)                                                    \
    if (!(h) || !(h)->m) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL handle"); \
    Model& m = *(h)->m

extern "C" {

const char* vfs_last_error(void) { return vfs::g_last_error.c_str(); }
const char* vfs_version(void) { return "vkfluidsim_gb300 0.2 (sm_103a)"; }

int vfs_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// ---------------------------------------------------------------- single-scene model

int vfs_model_create(const vfs_sim_params* sim, const vfs_sph_params* sph,
                     const vfs_wcsph_params* wcsph, vfs_model** out) {
    try {
        if (!sim || !sph || !wcsph || !out) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
        *out = nullptr;
        int rc = vfs::validate(sim, sph);
        if (rc) return rc;
        std::vector<vfs::SceneHost> scenes(1);
        scenes[0].sim = *sim;
        scenes[0].sph = *sph;
        scenes[0].wcsph = *wcsph;
        vfs::Model* m = nullptr;
        rc = vfs::create_model(scenes, &m);
        if (rc) return rc;
        vfs_model* h = new vfs_model();
        h->m = m;
        *out = h;
        return VFS_OK;
    } catch (const std::exception& e) {
        return fail(VFS_ERR_OUT_OF_MEMORY, e.what());
    }
}

int vfs_model_destroy(vfs_model* h) {
    delete h;
    return VFS_OK;
}

int vfs_model_set_stream(vfs_model* h, void* stream) {
    VFS_HANDLE(h);
    return vfs::set_stream(m, stream);
}

int vfs_model_set_parameters(vfs_model* h, const vfs_sim_params* sim, const vfs_sph_params* sph,
                             const vfs_wcsph_params* wc) {
    VFS_HANDLE(h);
    return vfs::set_scene_parameters(m, 0, sim, sph, wc);
}

int vfs_model_get_parameters(const vfs_model* h, vfs_sim_params* sim, vfs_sph_params* sph,
                             vfs_wcsph_params* wc) {
    VFS_HANDLE(h);
    if (sim) *sim = m.scenes[0].sim;
    if (sph) *sph = m.scenes[0].sph;
    if (wc) *wc = m.scenes[0].wcsph;
    return VFS_OK;
}

uint32_t vfs_model_num_particles(const vfs_model* h) { return h && h->m ? h->m->n : 0u; }

int vfs_model_add_boundary_object(vfs_model* h, const vfs_boundary_object* obj) {
    VFS_HANDLE(h);
    if (!obj) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL object");
    return m.add_object(0, *obj, nullptr, nullptr);
}

int vfs_model_add_analytic_object(vfs_model* h, const vfs_analytic_object* obj) {
    VFS_HANDLE(h);
    if (!obj) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL object");
    return m.add_analytic(0, *obj);
}

int vfs_model_add_mesh_object(vfs_model* h, const vfs_mesh_object* obj) {
    VFS_HANDLE(h);
    if (!obj) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL object");
    return m.add_mesh(0, *obj);
}

int vfs_mesh_signed_distance(const float* vertices, uint32_t n_vertices, const uint32_t* triangles,
                             uint32_t n_triangles, const float* points, uint32_t n_points,
                             double* distances) {
    if (!vertices || !triangles || (n_points && (!points || !distances)))
        return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    std::vector<float> pos(vertices, vertices + 3 * (size_t)n_vertices);
    std::vector<uint32_t> tri(triangles, triangles + 3 * (size_t)n_triangles);
    vfs::MeshHost mh;
    std::string err;
    if (!vfs::build_mesh(pos, tri, mh, err)) return fail(VFS_ERR_INVALID_ARGUMENT, "mesh: " + err);
    if (n_points == 0) return VFS_OK;
    vfs::MeshUpload up;
    int rc = vfs::upload_mesh(mh, up);
    if (rc) return rc;
    float* dp = nullptr;
    double* dd = nullptr;
    cudaError_t e = cudaMalloc(&dp, (size_t)n_points * 12);
    if (e == cudaSuccess) e = cudaMalloc(&dd, (size_t)n_points * 8);
    if (e == cudaSuccess) e = cudaMemcpy(dp, points, (size_t)n_points * 12, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = vfs::launch_mesh_distance(up.dev, dp, n_points, dd, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(distances, dd, (size_t)n_points * 8, cudaMemcpyDeviceToHost);
    up.free();
    if (dp) cudaFree(dp);
    if (dd) cudaFree(dd);
    if (e != cudaSuccess) return fail(VFS_ERR_CUDA, std::string("mesh distance: ") + cudaGetErrorString(e));
    return VFS_OK;
}

uint32_t vfs_model_num_boundary_objects(const vfs_model* h) {
    return h && h->m ? (uint32_t)h->m->scenes[0].objects.size() : 0u;
}

static int get_object(const Model& m, uint32_t scene, uint32_t idx, vfs_boundary_object* info,
                      float* sdf_out, float* vm_out) {
    if (scene >= m.scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    const auto& objs = m.scenes[scene].objects;
    if (idx >= objs.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "object index out of range");
    const vfs::ObjectStore& o = objs[idx];
    if (info) *info = o.info;
    const size_t cnt = (size_t)o.info.resolution[0] * o.info.resolution[1] * o.info.resolution[2];
    if (sdf_out) VFS_CUDA_TRY(cudaMemcpy(sdf_out, o.d_sdf, cnt * 4, cudaMemcpyDeviceToHost));
    if (vm_out) VFS_CUDA_TRY(cudaMemcpy(vm_out, o.d_vm, cnt * 4, cudaMemcpyDeviceToHost));
    return VFS_OK;
}

int vfs_model_get_boundary_object(const vfs_model* h, uint32_t idx, vfs_boundary_object* info,
                                  float* sdf_out, float* vm_out) {
    VFS_HANDLE(h);
    return get_object(m, 0, idx, info, sdf_out, vm_out);
}

int vfs_model_set_particle_state(vfs_model* h, const float* pos, const float* vel,
                                 uint32_t offset, int64_t count) {
    VFS_HANDLE(h);
    return m.set_state(0, pos, vel, offset, count);
}

int vfs_model_step_host(vfs_model* h, const float* pos, const float* vel, int32_t substeps,
                        float* pos_out, float* vel_out, float* dens_out) {
    VFS_HANDLE(h);
    return m.step_host(pos, vel, substeps, pos_out, vel_out, dens_out);
}

int vfs_model_copy_data_buffers(vfs_model* h, float* pos, float* vel, float* dens, float* acc) {
    VFS_HANDLE(h);
    const int rc = m.get_state(0, pos, vel, dens, nullptr);
    if (rc) return rc;
    return m.get_acc(0, acc);
}

int vfs_model_get_ids(vfs_model* h, uint32_t* ids) {
    VFS_HANDLE(h);
    if (!ids) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL ids");
    return m.get_state(0, nullptr, nullptr, nullptr, ids);
}

int vfs_model_get_neighbor_arrays(vfs_model* h, uint32_t* keys, uint32_t* sorted_indices,
                                  uint32_t* offsets) {
    VFS_HANDLE(h);
    return m.get_neighbors(0, keys, sorted_indices, offsets);
}

int vfs_model_get_boundary_fields(vfs_model* h, float* bdens, float* bgrad) {
    VFS_HANDLE(h);
    return m.get_boundary(0, bdens, bgrad);
}

int vfs_model_record_fields(vfs_model* h, int32_t enable) {
    VFS_HANDLE(h);
    m.record = enable != 0;
    m.invalidate_graph();
    return VFS_OK;
}

int vfs_model_step(vfs_model* h) {
    VFS_HANDLE(h);
    return m.run_substeps(m.scenes[0].sph.iterations);
}

int vfs_model_substeps(vfs_model* h, int32_t count) {
    VFS_HANDLE(h);
    return m.run_substeps(count);
}

int vfs_model_use_graph(vfs_model* h, int32_t enable) {
    VFS_HANDLE(h);
    m.use_graph = enable != 0;
    m.invalidate_graph();
    return VFS_OK;
}

int vfs_model_synchronize(vfs_model* h) {
    VFS_HANDLE(h);
    return m.check_device();
}

int vfs_model_profile_substeps(vfs_model* h, int32_t count, float* phase_ms) {
    VFS_HANDLE(h);
    return vfs::profile_phases(m, count, phase_ms);
}

int vfs_model_set_sort_config(vfs_model* h, int32_t digit_bits, int32_t tile_items) {
    VFS_HANDLE(h);
    return vfs::set_sort_config(m, digit_bits, tile_items);
}

int vfs_model_set_neighbor_capacity(vfs_model* h, int32_t slots) {
    VFS_HANDLE(h);
    return vfs::set_neighbor_capacity(m, slots);
}

int vfs_model_set_skin(vfs_model* h, float skin) {
    VFS_HANDLE(h);
    return vfs::set_skin(m, skin);
}

int vfs_model_set_walk_staging(vfs_model* h, int32_t enable) {
    VFS_HANDLE(h);
    m.kc.walk_staging = enable != 0;
    m.invalidate_graph();
    return VFS_OK;
}

int vfs_model_get_skin_builds(vfs_model* h, uint32_t* builds) {
    VFS_HANDLE(h);
    if (!builds) return vfs::fail(VFS_ERR_INVALID_ARGUMENT, "NULL output");
    return vfs::get_skin_builds(m, 0, builds);
}

int vfs_model_get_skin(const vfs_model* h, float* skin) {
    if (!h || !h->m || !skin) return vfs::fail(VFS_ERR_INVALID_ARGUMENT, "NULL handle or output");
    *skin = vfs::get_skin(*h->m);
    return VFS_OK;
}

int32_t vfs_model_get_neighbor_capacity(const vfs_model* h) {
    return (h && h->m) ? (int32_t)h->m->nbr_cap : -1;
}

int vfs_model_get_sort_config(const vfs_model* h, int32_t* digit_bits, int32_t* tile_items,
                              int32_t* passes) {
    VFS_HANDLE(h);
    if (digit_bits) *digit_bits = m.sc.digit_bits;
    if (tile_items) *tile_items = m.sc.tile / 256;
    if (passes) *passes = m.sc.passes;
    return VFS_OK;
}

int vfs_model_device_state(vfs_model* h, void** pos4, void** vel4) {
    VFS_HANDLE(h);
    if (pos4) *pos4 = m.pos[m.cur];
    if (vel4) *vel4 = m.vel[m.cur];
    return VFS_OK;
}

// ---------------------------------------------------------------- batches of scenes

int vfs_batch_create(int32_t n_scenes, const vfs_sim_params* sims, const vfs_sph_params* sphs,
                     const vfs_wcsph_params* wcsphs, vfs_batch** out) {
    try {
        if (!sims || !sphs || !wcsphs || !out) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
        *out = nullptr;
        if (n_scenes < 1 || (uint32_t)n_scenes > vfs::kMaxScenes)
            return fail(VFS_ERR_CAPACITY, "n_scenes must be in [1, 65535]");
        std::vector<vfs::SceneHost> scenes((size_t)n_scenes);
        for (int32_t s = 0; s < n_scenes; s++) {
            const int rc = vfs::validate(&sims[s], &sphs[s]);
            if (rc) return fail(rc, "scene " + std::to_string(s) + ": " + vfs::g_last_error);
            scenes[s].sim = sims[s];
            scenes[s].sph = sphs[s];
            scenes[s].wcsph = wcsphs[s];
        }
        vfs::Model* m = nullptr;
        const int rc = vfs::create_model(scenes, &m);
        if (rc) return rc;
        vfs_batch* h = new vfs_batch();
        h->m = m;
        *out = h;
        return VFS_OK;
    } catch (const std::exception& e) {
        return fail(VFS_ERR_OUT_OF_MEMORY, e.what());
    }
}

int vfs_batch_destroy(vfs_batch* h) {
    delete h;
    return VFS_OK;
}

int32_t vfs_batch_num_scenes(const vfs_batch* h) {
    return h && h->m ? (int32_t)h->m->scenes.size() : 0;
}

uint32_t vfs_batch_num_particles(const vfs_batch* h, int32_t scene) {
    if (!h || !h->m || scene < 0 || (size_t)scene >= h->m->scenes.size()) return 0u;
    return h->m->scenes[scene].n;
}

int vfs_batch_set_stream(vfs_batch* h, void* stream) {
    VFS_HANDLE(h);
    return vfs::set_stream(m, stream);
}

int vfs_batch_set_scene_parameters(vfs_batch* h, int32_t scene, const vfs_sim_params* sim,
                                   const vfs_sph_params* sph, const vfs_wcsph_params* wc) {
    VFS_HANDLE(h);
    return vfs::set_scene_parameters(m, (uint32_t)scene, sim, sph, wc);
}

int vfs_batch_add_boundary_object(vfs_batch* h, int32_t scene, const vfs_boundary_object* obj) {
    VFS_HANDLE(h);
    if (!obj) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL object");
    return m.add_object((uint32_t)scene, *obj, nullptr, nullptr);
}

int vfs_batch_add_analytic_object(vfs_batch* h, int32_t scene, const vfs_analytic_object* obj) {
    VFS_HANDLE(h);
    if (!obj) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL object");
    return m.add_analytic((uint32_t)scene, *obj);
}

int vfs_batch_add_mesh_object(vfs_batch* h, int32_t scene, const vfs_mesh_object* obj) {
    VFS_HANDLE(h);
    if (!obj || scene < 0) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL object or negative scene");
    return m.add_mesh((uint32_t)scene, *obj);
}

int vfs_batch_get_boundary_object(const vfs_batch* h, int32_t scene, uint32_t idx,
                                  vfs_boundary_object* info, float* sdf_out, float* vm_out) {
    VFS_HANDLE(h);
    return get_object(m, (uint32_t)scene, idx, info, sdf_out, vm_out);
}

int vfs_batch_set_particle_state(vfs_batch* h, int32_t scene, const float* pos, const float* vel,
                                 uint32_t offset, int64_t count) {
    VFS_HANDLE(h);
    return m.set_state((uint32_t)scene, pos, vel, offset, count);
}

int vfs_batch_copy_data_buffers(vfs_batch* h, int32_t scene, float* pos, float* vel, float* dens,
                                float* acc) {
    VFS_HANDLE(h);
    const int rc = m.get_state((uint32_t)scene, pos, vel, dens, nullptr);
    if (rc) return rc;
    return m.get_acc((uint32_t)scene, acc);
}

int vfs_batch_get_ids(vfs_batch* h, int32_t scene, uint32_t* ids) {
    VFS_HANDLE(h);
    if (!ids) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL ids");
    return m.get_state((uint32_t)scene, nullptr, nullptr, nullptr, ids);
}

int vfs_batch_get_neighbor_arrays(vfs_batch* h, int32_t scene, uint32_t* keys,
                                  uint32_t* sorted_indices, uint32_t* offsets) {
    VFS_HANDLE(h);
    return m.get_neighbors((uint32_t)scene, keys, sorted_indices, offsets);
}

int vfs_batch_get_boundary_fields(vfs_batch* h, int32_t scene, float* bdens, float* bgrad) {
    VFS_HANDLE(h);
    return m.get_boundary((uint32_t)scene, bdens, bgrad);
}

int vfs_batch_record_fields(vfs_batch* h, int32_t enable) {
    VFS_HANDLE(h);
    m.record = enable != 0;
    m.invalidate_graph();
    return VFS_OK;
}

int vfs_batch_substeps(vfs_batch* h, int32_t count) {
    VFS_HANDLE(h);
    return m.run_substeps(count);
}

int vfs_batch_use_graph(vfs_batch* h, int32_t enable) {
    VFS_HANDLE(h);
    m.use_graph = enable != 0;
    m.invalidate_graph();
    return VFS_OK;
}

int vfs_batch_synchronize(vfs_batch* h) {
    VFS_HANDLE(h);
    return m.check_device();
}

int vfs_batch_profile_substeps(vfs_batch* h, int32_t count, float* phase_ms) {
    VFS_HANDLE(h);
    return vfs::profile_phases(m, count, phase_ms);
}

int vfs_batch_set_neighbor_capacity(vfs_batch* h, int32_t slots) {
    VFS_HANDLE(h);
    return vfs::set_neighbor_capacity(m, slots);
}

int vfs_batch_set_walk_staging(vfs_batch* h, int32_t enable) {
    VFS_HANDLE(h);
    m.kc.walk_staging = enable != 0;
    m.invalidate_graph();
    return VFS_OK;
}

int vfs_batch_set_skin(vfs_batch* h, float skin) {
    VFS_HANDLE(h);
    return vfs::set_skin(m, skin);
}

int vfs_batch_get_skin_builds(vfs_batch* h, uint32_t scene, uint32_t* builds) {
    VFS_HANDLE(h);
    if (!builds) return vfs::fail(VFS_ERR_INVALID_ARGUMENT, "NULL output");
    return vfs::get_skin_builds(m, scene, builds);
}

int vfs_batch_get_skin(const vfs_batch* h, float* skin) {
    if (!h || !h->m || !skin) return vfs::fail(VFS_ERR_INVALID_ARGUMENT, "NULL handle or output");
    *skin = vfs::get_skin(*h->m);
    return VFS_OK;
}

int vfs_batch_set_sort_config(vfs_batch* h, int32_t digit_bits, int32_t tile_items) {
    VFS_HANDLE(h);
    return vfs::set_sort_config(m, digit_bits, tile_items);
}

}  // extern "C"
