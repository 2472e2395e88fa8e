// Headless state export: device -> file snapshots of a model's particle state, the counterpart of
// the reference's render hand-off (SPHModel::CopyDataBuffers, src/models/model.cpp:158-170, read by
// src/gui/scene_renderer.cpp:52-55) and of the "record particle positions" item of its roadmap
// (README.md:30).
//
// A snapshot is two files: `<prefix>.bin` holds positions f32[N][3], velocities f32[N][3] and
// densities f32[N], each indexed by particle id, little-endian and back to back; `<prefix>.json`
// describes them (offsets, shapes, the substep count, the simulation parameters). One kernel
// scatters the sorted state by id into the model's staging buffer in exactly the file's layout,
// so a snapshot is one device->host copy. The recorder overlaps stepping with file writes: frames
// alternate between two pinned host buffers and a writer thread saves each one once its copy has
// completed.

#include <cuda_runtime.h>

#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "vfs_cuda.h"
#include "vfs_internal.h"
#include "vfs_model.h"

#define VFS_EXP_TRY(expr)                                                                \
    do {                                                                                 \
        cudaError_t e_ = (expr);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return ::vfs::fail(VFS_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace vfs {

namespace {

// out = [pos (3n) | vel (3n) | dens (n)], each indexed by the scene-local particle id.
__global__ void k_state_by_id(uint32_t n, uint32_t start, const float4* __restrict__ pos,
                              const float4* __restrict__ vel, const float4* __restrict__ aux,
                              float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[start + i];
    const uint32_t id = __float_as_uint(p.w) - start;
    if (id >= n) return;  // ids are a permutation of [0, n)
    const float4 v = vel[start + i];
    float* op = out + 3 * (size_t)id;
    float* ov = out + 3 * (size_t)n + 3 * (size_t)id;
    op[0] = p.x;
    op[1] = p.y;
    op[2] = p.z;
    ov[0] = v.x;
    ov[1] = v.y;
    ov[2] = v.z;
    out[6 * (size_t)n + id] = aux[start + i].z;
}

std::string json_floats(const float* v, int k) {
    std::string s = "[";
    char b[32];
    for (int i = 0; i < k; i++) {
        std::snprintf(b, sizeof(b), "%s%.9g", i ? ", " : "", (double)v[i]);
        s += b;
    }
    return s + "]";
}

std::string base_name(const std::string& path) {
    const size_t k = path.find_last_of('/');
    return k == std::string::npos ? path : path.substr(k + 1);
}

std::string sidecar(const SceneHost& sh, uint64_t substeps, const std::string& bin_name) {
    const size_t n = sh.n;
    const vfs_sim_params& sim = sh.sim;
    const vfs_sph_params& sph = sh.sph;
    const vfs_wcsph_params& wc = sh.wcsph;
    const double dt = (double)sph.time_scale * (double)sph.fixed_dt / (double)sph.iterations;
    char buf[4096];
    std::snprintf(
        buf, sizeof(buf),
        "{\n"
        "  \"format\": \"vkfluidsim_gb300.state\",\n"
        "  \"version\": 1,\n"
        "  \"binary\": \"%s\",\n"
        "  \"particles\": %zu,\n"
        "  \"order\": \"particle id\",\n"
        "  \"substeps\": %llu,\n"
        "  \"time\": %.17g,\n"
        "  \"arrays\": {\n"
        "    \"positions\": {\"dtype\": \"<f4\", \"shape\": [%zu, 3], \"offset\": 0},\n"
        "    \"velocities\": {\"dtype\": \"<f4\", \"shape\": [%zu, 3], \"offset\": %zu},\n"
        "    \"densities\": {\"dtype\": \"<f4\", \"shape\": [%zu], \"offset\": %zu}\n"
        "  },\n"
        "  \"parameters\": {\n"
        "    \"gravity\": %s, \"smooth_radius\": %.9g,\n"
        "    \"time_scale\": %.9g, \"iterations\": %d, \"fixed_dt\": %.9g, \"target_density\": %.9g,\n"
        "    \"bbox_size\": %s, \"bbox_pos\": %s,\n"
        "    \"wall_stiffness\": %.9g, \"stiffness\": %.9g, \"expoent\": %.9g, \"viscosity_strenght\": %.9g\n"
        "  }\n"
        "}\n",
        bin_name.c_str(), n, (unsigned long long)substeps, dt * (double)substeps, n, n, 12 * n, n,
        24 * n, json_floats(sim.gravity, 3).c_str(), (double)sim.smooth_radius,
        (double)sph.time_scale, sph.iterations, (double)sph.fixed_dt, (double)sph.target_density,
        json_floats(sph.bbox_size, 3).c_str(), json_floats(sph.bbox_pos, 3).c_str(),
        (double)wc.wall_stiffness, (double)wc.stiffness, (double)wc.expoent,
        (double)wc.viscosity_strenght);
    return buf;
}

int write_files(const std::string& prefix, const SceneHost& sh, uint64_t substeps,
                const float* data) {
    const std::string bin = prefix + ".bin";
    FILE* f = std::fopen(bin.c_str(), "wb");
    if (!f) return fail(VFS_ERR_IO, "cannot write " + bin);
    const size_t words = 7 * (size_t)sh.n;
    const bool ok = std::fwrite(data, 4, words, f) == words;
    if (std::fclose(f) != 0 || !ok) return fail(VFS_ERR_IO, "cannot write " + bin);
    const std::string js = prefix + ".json";
    FILE* g = std::fopen(js.c_str(), "w");
    if (!g) return fail(VFS_ERR_IO, "cannot write " + js);
    const std::string text = sidecar(sh, substeps, base_name(bin));
    const bool ok2 = std::fputs(text.c_str(), g) >= 0;
    if (std::fclose(g) != 0 || !ok2) return fail(VFS_ERR_IO, "cannot write " + js);
    return VFS_OK;
}

// Enqueues the by-id scatter of scene `scene` into the staging buffer and its copy to `host`.
int enqueue_snapshot(Model& m, uint32_t scene, float* host) {
    const SceneHost& sh = m.scenes[scene];
    if (sh.n == 0) return VFS_OK;
    k_state_by_id<<<(sh.n + 255) / 256, 256, 0, m.stream>>>(sh.n, sh.off, m.pos[m.cur],
                                                           m.vel[m.cur], m.aux, m.stage);
    VFS_EXP_TRY(cudaGetLastError());
    VFS_EXP_TRY(cudaMemcpyAsync(host, m.stage, 28 * (size_t)sh.n, cudaMemcpyDeviceToHost, m.stream));
    return VFS_OK;
}

// Minimal reader of the sidecar written above: the value of a top-level integer key.
bool json_int(const std::string& text, const char* key, unsigned long long* out) {
    const std::string k = std::string("\"") + key + "\"";
    const size_t p = text.find(k);
    if (p == std::string::npos) return false;
    const size_t c = text.find(':', p + k.size());
    if (c == std::string::npos) return false;
    return std::sscanf(text.c_str() + c + 1, " %llu", out) == 1;
}

}  // namespace

int export_state(Model& m, uint32_t scene, const char* prefix) {
    if (!prefix) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL path prefix");
    if (scene >= m.scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    const SceneHost& sh = m.scenes[scene];
    std::vector<float> host(7 * (size_t)sh.n);
    int rc = enqueue_snapshot(m, scene, host.data());
    if (rc) return rc;
    rc = m.check_device();
    if (rc) return rc;
    return write_files(prefix, sh, m.substeps_done, host.data());
}

int import_state(Model& m, uint32_t scene, const char* prefix) {
    if (!prefix) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL path prefix");
    if (scene >= m.scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    const SceneHost& sh = m.scenes[scene];
    const std::string js = std::string(prefix) + ".json";
    FILE* g = std::fopen(js.c_str(), "r");
    if (!g) return fail(VFS_ERR_IO, "cannot read " + js);
    std::string text;
    char buf[4096];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), g)) > 0) text.append(buf, got);
    std::fclose(g);
    unsigned long long n = 0, version = 0;
    if (text.find("\"vkfluidsim_gb300.state\"") == std::string::npos || !json_int(text, "version", &version) ||
        version != 1 || !json_int(text, "particles", &n))
        return fail(VFS_ERR_PARSE, js + " is not a version-1 state sidecar");
    if (n != sh.n)
        return fail(VFS_ERR_INVALID_ARGUMENT, js + " holds " + std::to_string(n) +
                                                  " particles, the scene has " + std::to_string(sh.n));
    const std::string bin = std::string(prefix) + ".bin";
    FILE* f = std::fopen(bin.c_str(), "rb");
    if (!f) return fail(VFS_ERR_IO, "cannot read " + bin);
    std::vector<float> data(7 * (size_t)n);
    const size_t words = std::fread(data.data(), 4, data.size(), f);
    std::fclose(f);
    if (words != data.size()) return fail(VFS_ERR_PARSE, bin + " is shorter than its sidecar says");
    const int rc = m.set_state(scene, data.data(), data.data() + 3 * n, 0, (int64_t)n);
    if (rc) return rc;
    unsigned long long steps = 0;
    if (json_int(text, "substeps", &steps)) m.substeps_done = steps;
    return VFS_OK;
}

// Runs `substeps` substeps and writes a snapshot of every scene every `every` substeps, named
// `<prefix>_f<frame>` (batches: `<prefix>_s<scene>_f<frame>`), frame 0 being the state after the
// first `every` substeps. File writes overlap the following substeps.
int record(Model& m, int32_t substeps, int32_t every, const char* prefix) {
    if (!prefix) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL path prefix");
    if (substeps < 0 || every < 1) return fail(VFS_ERR_INVALID_ARGUMENT, "need substeps >= 0, every >= 1");
    const int frames = substeps / every;
    const bool batch = m.scenes.size() > 1;
    const size_t bytes = 28 * (size_t)m.n;
    float* pinned[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    int rc = VFS_OK;
    for (int b = 0; b < 2 && rc == VFS_OK; b++) {
        if (cudaMallocHost(&pinned[b], bytes > 0 ? bytes : 4) != cudaSuccess ||
            cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming) != cudaSuccess)
            rc = fail(VFS_ERR_OUT_OF_MEMORY, "recorder: pinned host buffers");
    }
    // Writer thread: saves a frame once its copy has completed.
    struct Job {
        int frame = -1;
        uint64_t steps = 0;
    };
    std::mutex mu;
    std::condition_variable cv;
    Job pending[2];
    bool busy[2] = {false, false};
    bool stop = false;
    int writer_rc = VFS_OK;
    std::string writer_err;
    std::thread writer([&] {
        int next = 0;
        while (true) {
            Job job;
            const int b = next & 1;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return busy[b] || stop; });
                if (!busy[b]) return;
                job = pending[b];
            }
            int r = cudaEventSynchronize(done[b]) == cudaSuccess ? VFS_OK : VFS_ERR_CUDA;
            size_t off = 0;
            for (size_t s = 0; s < m.scenes.size() && r == VFS_OK; s++) {
                const SceneHost& sh = m.scenes[s];
                char name[64];
                if (batch)
                    std::snprintf(name, sizeof(name), "_s%zu_f%06d", s, job.frame);
                else
                    std::snprintf(name, sizeof(name), "_f%06d", job.frame);
                r = write_files(std::string(prefix) + name, sh, job.steps, pinned[b] + off);
                off += 7 * (size_t)sh.n;
            }
            std::lock_guard<std::mutex> lk(mu);
            if (r != VFS_OK && writer_rc == VFS_OK) {
                writer_rc = r;
                writer_err = last_error_message();
            }
            busy[b] = false;
            next++;
            cv.notify_all();
        }
    });
    for (int f = 0; f < frames && rc == VFS_OK; f++) {
        rc = m.run_substeps(every);
        if (rc) break;
        const int b = f & 1;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return !busy[b]; });
            if (writer_rc) break;
        }
        size_t off = 0;
        for (size_t s = 0; s < m.scenes.size() && rc == VFS_OK; s++) {
            rc = enqueue_snapshot(m, (uint32_t)s, pinned[b] + off);
            off += 7 * (size_t)m.scenes[s].n;
        }
        if (rc == VFS_OK && cudaEventRecord(done[b], m.stream) != cudaSuccess)
            rc = fail(VFS_ERR_CUDA, "recorder: event record failed");
        if (rc) break;
        std::lock_guard<std::mutex> lk(mu);
        pending[b] = Job{f, m.substeps_done};
        busy[b] = true;
        cv.notify_all();
    }
    if (rc == VFS_OK && substeps % every) {
        rc = m.run_substeps(substeps % every);
    }
    {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return !busy[0] && !busy[1]; });
        stop = true;
        cv.notify_all();
    }
    writer.join();
    for (int b = 0; b < 2; b++) {
        if (pinned[b]) cudaFreeHost(pinned[b]);
        if (done[b]) cudaEventDestroy(done[b]);
    }
    if (rc) return rc;
    if (writer_rc) return fail(writer_rc, writer_err);
    return m.check_device();
}

}  // namespace vfs

using vfs::fail;

extern "C" {

int vfs_model_export_state(vfs_model* h, const char* path_prefix) {
    vfs::Model* m = vfs_model_impl(h);
    if (!m) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL model");
    return vfs::export_state(*m, 0, path_prefix);
}

int vfs_model_import_state(vfs_model* h, const char* path_prefix) {
    vfs::Model* m = vfs_model_impl(h);
    if (!m) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL model");
    return vfs::import_state(*m, 0, path_prefix);
}

int vfs_model_record(vfs_model* h, int32_t substeps, int32_t every, const char* path_prefix) {
    vfs::Model* m = vfs_model_impl(h);
    if (!m) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL model");
    return vfs::record(*m, substeps, every, path_prefix);
}

int vfs_batch_export_state(vfs_batch* h, int32_t scene, const char* path_prefix) {
    vfs::Model* m = vfs_batch_impl(h);
    if (!m || scene < 0) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL batch or negative scene");
    return vfs::export_state(*m, (uint32_t)scene, path_prefix);
}

int vfs_batch_import_state(vfs_batch* h, int32_t scene, const char* path_prefix) {
    vfs::Model* m = vfs_batch_impl(h);
    if (!m || scene < 0) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL batch or negative scene");
    return vfs::import_state(*m, (uint32_t)scene, path_prefix);
}

int vfs_batch_record(vfs_batch* h, int32_t substeps, int32_t every, const char* path_prefix) {
    vfs::Model* m = vfs_batch_impl(h);
    if (!m) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL batch");
    return vfs::record(*m, substeps, every, path_prefix);
}

}  // extern "C"
