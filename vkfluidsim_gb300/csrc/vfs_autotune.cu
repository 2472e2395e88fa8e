// Project-written autotuner for the substep's launch shapes (the reference has no counterpart: its
// dispatch sizes are fixed in the shaders' numthreads). It chooses, per model or batch:
//   * the radix sort's digit width (6, 7 or 8 bits) and items per thread (8, 12 or 16),
//   * the neighbour passes' block shape (threads per block x minimum resident blocks per SM),
//   * the cells-per-block of the cell-range / reorder kernel (128, 256 or 512 keys),
//   * whether the density walk stages a warp's row of cells in shared memory (block-per-cell
//     staging; it helps where walking warps share rows and the per-thread walk prunes little).
// None of these changes any result: the sort is stable whatever its digits, and every particle's
// sums are accumulated by one thread in the same order whatever the block shape. Candidates are
// timed with CUDA events on the model's stream from the same saved state (restored before every
// candidate and at the end), one stage at a time, each stage by the phases it affects. Choices are
// cached per process under a key of the device and the workload's size, and the cache can be saved
// to and loaded from a text file.

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "vfs_cuda.h"
#include "vfs_internal.h"
#include "vfs_model.h"

#define VFS_TUNE_TRY(expr)                                                               \
    do {                                                                                 \
        cudaError_t e_ = (expr);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return ::vfs::fail(VFS_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace vfs {

namespace {

struct Shape {
    int threads, min_blocks;
};
constexpr Shape kShapes[kNumNbrShapes] = {{128, 6}, {128, 8}, {96, 8}, {64, 12}};

std::mutex g_cache_mu;
std::map<std::string, vfs_tune_config> g_cache;

vfs_tune_config current(const Model& m) {
    vfs_tune_config c{};
    c.sort_digit_bits = m.digit_bits;
    c.sort_tile_items = m.tile_items;
    c.nbr_block = kShapes[m.kc.nbr_shape].threads;
    c.nbr_min_blocks = kShapes[m.kc.nbr_shape].min_blocks;
    c.cell_block = m.kc.cell_block;
    c.force_block = kShapes[m.kc.force_shape].threads;
    c.force_min_blocks = kShapes[m.kc.force_shape].min_blocks;
    c.walk_staging = m.kc.walk_staging;
    return c;
}

int shape_of(int threads, int min_blocks) {
    for (int k = 0; k < kNumNbrShapes; k++)
        if (kShapes[k].threads == threads && kShapes[k].min_blocks == min_blocks) return k;
    return -1;
}

// Device, particle count, scene count and a fingerprint of the scenes' sizes and radii.
std::string tune_key(const Model& m) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, dev);
    uint64_t f = 1469598103934665603ull;
    auto mix = [&](uint64_t v) {
        f ^= v;
        f *= 1099511628211ull;
    };
    for (const SceneHost& s : m.scenes) {
        mix(s.n);
        uint32_t hb;
        std::memcpy(&hb, &s.sim.smooth_radius, 4);
        mix(hb);
    }
    char buf[256];
    std::snprintf(buf, sizeof(buf), "sm%d%d_%dsms_n%u_s%zu_%016llx", prop.major, prop.minor,
                  prop.multiProcessorCount, m.n, m.scenes.size(), (unsigned long long)f);
    return buf;
}

}  // namespace

int apply_tune_config(Model& m, const vfs_tune_config& c) {
    const int shape = shape_of(c.nbr_block, c.nbr_min_blocks);
    if (shape < 0)
        return fail(VFS_ERR_INVALID_ARGUMENT,
                    "neighbour block shape must be 128x6, 128x8, 96x8 or 64x12 (threads x blocks/SM)");
    const int fshape = c.force_block == 0 && c.force_min_blocks == 0
                           ? shape
                           : shape_of(c.force_block, c.force_min_blocks);
    if (fshape < 0)
        return fail(VFS_ERR_INVALID_ARGUMENT,
                    "force block shape must be 128x6, 128x8, 96x8 or 64x12, or 0x0 for the neighbour shape");
    if (c.cell_block != 128 && c.cell_block != 256 && c.cell_block != 512)
        return fail(VFS_ERR_INVALID_ARGUMENT, "cell_block must be 128, 256 or 512");
    if (c.walk_staging != 0 && c.walk_staging != 1)
        return fail(VFS_ERR_INVALID_ARGUMENT, "walk_staging must be 0 or 1");
    if (c.sort_digit_bits != m.digit_bits || c.sort_tile_items != m.tile_items) {
        const int rc = set_sort_config(m, c.sort_digit_bits, c.sort_tile_items);
        if (rc) return rc;
    }
    VFS_TUNE_TRY(cudaStreamSynchronize(m.stream));
    m.kc.nbr_shape = shape;
    m.kc.force_shape = fshape;
    m.kc.cell_block = c.cell_block;
    m.kc.walk_staging = c.walk_staging;
    m.invalidate_graph();
    return VFS_OK;
}

vfs_tune_config get_tune_config(const Model& m) { return current(m); }

int autotune(Model& m, int repeats, bool use_cache, vfs_tune_config* chosen) {
    if (repeats < 1) return fail(VFS_ERR_INVALID_ARGUMENT, "repeats must be >= 1");
    if (m.n == 0) {
        if (chosen) *chosen = current(m);
        return VFS_OK;
    }
    const std::string key = tune_key(m);
    if (use_cache) {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        auto it = g_cache.find(key);
        if (it != g_cache.end()) {
            const int rc = apply_tune_config(m, it->second);
            if (rc == VFS_OK && chosen) *chosen = it->second;
            return rc;
        }
    }
    const size_t bytes = (size_t)m.n * sizeof(float4);
    float4* save_pos = nullptr;
    float4* save_vel = nullptr;
    VFS_TUNE_TRY(cudaMalloc(&save_pos, bytes));
    if (cudaMalloc(&save_vel, bytes) != cudaSuccess) {
        cudaFree(save_pos);
        return fail(VFS_ERR_CUDA, "autotune: out of device memory for the saved state");
    }
    int rc = VFS_OK;
    auto copy = [&](float4* dp, const float4* sp, float4* dv, const float4* sv) {
        if (rc) return;
        if (cudaMemcpyAsync(dp, sp, bytes, cudaMemcpyDeviceToDevice, m.stream) != cudaSuccess ||
            cudaMemcpyAsync(dv, sv, bytes, cudaMemcpyDeviceToDevice, m.stream) != cudaSuccess)
            rc = fail(VFS_ERR_CUDA, "autotune: state copy failed");
    };
    copy(save_pos, m.pos[m.cur], save_vel, m.vel[m.cur]);
    const bool keep_record = m.record;
    m.record = false;
    // Mean phase times of `repeats` substeps from the saved state under configuration c.
    auto measure = [&](const vfs_tune_config& c, float* ph) {
        if (rc) return;
        rc = apply_tune_config(m, c);
        for (int pass = 0; pass < 2 && rc == VFS_OK; pass++) {  // pass 0 warms up
            copy(m.pos[m.cur], save_pos, m.vel[m.cur], save_vel);
            if (rc == VFS_OK) rc = profile_phases(m, pass == 0 ? 1 : repeats, ph);
        }
    };
    vfs_tune_config best = current(m);
    float ph[6];
    // Stage 1: sort digits and items (keys + sort phases: the key pass builds the digit histograms).
    {
        float best_t = 1e30f;
        vfs_tune_config c = best;
        for (int bits : {8, 7, 6})
            for (int items : {16, 12, 8}) {
                c.sort_digit_bits = bits;
                c.sort_tile_items = items;
                measure(c, ph);
                if (rc) break;
                if (ph[0] + ph[1] < best_t) {
                    best_t = ph[0] + ph[1];
                    best.sort_digit_bits = bits;
                    best.sort_tile_items = items;
                }
            }
    }
    // The walk kernel's shape and staging matter only in substeps that walk (no lists, a stale
    // scene, a list build); while a scene's lists are current it returns at once, and a
    // comparison there would pick by noise. So stages 2 and 3 run with the lists off (every
    // substep walks); they are switched back on afterwards, and rebuilt by the next substep.
    const float keep_skin = m.skin_fraction;
    if (rc == VFS_OK && keep_skin > 0.0f) rc = set_skin(m, 0.0f);
    // Stage 2: block shapes of the density and force passes (independent kernels, one sweep).
    if (rc == VFS_OK) {
        float best_d = 1e30f, best_f = 1e30f;
        vfs_tune_config c = best;
        for (int k = 0; k < kNumNbrShapes && rc == VFS_OK; k++) {
            c.nbr_block = c.force_block = kShapes[k].threads;
            c.nbr_min_blocks = c.force_min_blocks = kShapes[k].min_blocks;
            measure(c, ph);
            if (rc) break;
            if (ph[3] < best_d) {
                best_d = ph[3];
                best.nbr_block = c.nbr_block;
                best.nbr_min_blocks = c.nbr_min_blocks;
            }
            if (ph[4] < best_f) {
                best_f = ph[4];
                best.force_block = c.force_block;
                best.force_min_blocks = c.force_min_blocks;
            }
        }
    }
    // Stage 3: staging of the density walk, with the chosen density shape.
    if (rc == VFS_OK) {
        float best_t = 1e30f;
        vfs_tune_config c = best;
        for (int st : {0, 1}) {
            c.walk_staging = st;
            measure(c, ph);
            if (rc) break;
            if (ph[3] < best_t) {
                best_t = ph[3];
                best.walk_staging = st;
            }
        }
    }
    if (keep_skin > 0.0f) {
        const int rs = set_skin(m, keep_skin);
        if (rc == VFS_OK) rc = rs;
    }
    // Stage 4: cells per block of the cell-range / reorder kernel.
    if (rc == VFS_OK) {
        float best_t = 1e30f;
        vfs_tune_config c = best;
        for (int cb : {256, 128, 512}) {
            c.cell_block = cb;
            measure(c, ph);
            if (rc) break;
            if (ph[2] < best_t) {
                best_t = ph[2];
                best.cell_block = cb;
            }
        }
    }
    if (rc == VFS_OK) rc = apply_tune_config(m, best);
    copy(m.pos[m.cur], save_pos, m.vel[m.cur], save_vel);
    if (rc == VFS_OK && cudaStreamSynchronize(m.stream) != cudaSuccess)
        rc = fail(VFS_ERR_CUDA, "autotune: stream error");
    cudaFree(save_pos);
    cudaFree(save_vel);
    m.record = keep_record;
    m.stepped = false;  // the neighbour arrays are not those of a step taken by the caller
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        g_cache[key] = best;
    }
    if (chosen) *chosen = best;
    return VFS_OK;
}

int tune_cache_save(const char* path) {
    if (!path) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL path");
    std::lock_guard<std::mutex> lk(g_cache_mu);
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(VFS_ERR_IO, std::string("cannot write ") + path);
    std::fprintf(f, "# vkfluidsim_gb300 tune cache: key digit_bits tile_items nbr_block nbr_min_blocks "
                    "cell_block force_block force_min_blocks walk_staging\n");
    for (const auto& kv : g_cache)
        std::fprintf(f, "%s %d %d %d %d %d %d %d %d\n", kv.first.c_str(), kv.second.sort_digit_bits,
                     kv.second.sort_tile_items, kv.second.nbr_block, kv.second.nbr_min_blocks,
                     kv.second.cell_block, kv.second.force_block, kv.second.force_min_blocks,
                     kv.second.walk_staging);
    const bool ok = std::fclose(f) == 0;
    return ok ? VFS_OK : fail(VFS_ERR_IO, std::string("cannot write ") + path);
}

int tune_cache_load(const char* path) {
    if (!path) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL path");
    FILE* f = std::fopen(path, "r");
    if (!f) return fail(VFS_ERR_IO, std::string("cannot read ") + path);
    std::lock_guard<std::mutex> lk(g_cache_mu);
    char line[512];
    int rc = VFS_OK;
    while (std::fgets(line, sizeof(line), f)) {
        if (line[0] == '#' || line[0] == '\n') continue;
        char key[256];
        vfs_tune_config c{};
        // Lines of 6 values (no force shape) take the neighbour shape for the force pass; lines
        // without the walk-staging value (6 or 8 values) walk per thread.
        c.walk_staging = 0;
        const int got = std::sscanf(line, "%255s %d %d %d %d %d %d %d %d", key, &c.sort_digit_bits,
                                    &c.sort_tile_items, &c.nbr_block, &c.nbr_min_blocks,
                                    &c.cell_block, &c.force_block, &c.force_min_blocks,
                                    &c.walk_staging);
        if (got == 6) {
            c.force_block = c.nbr_block;
            c.force_min_blocks = c.nbr_min_blocks;
        }
        if ((got != 6 && got != 8 && got != 9) || shape_of(c.nbr_block, c.nbr_min_blocks) < 0 ||
            shape_of(c.force_block, c.force_min_blocks) < 0 || c.sort_digit_bits < 4 ||
            c.sort_digit_bits > 8 || (c.walk_staging != 0 && c.walk_staging != 1)) {
            rc = fail(VFS_ERR_PARSE, std::string("bad tune cache line in ") + path);
            break;
        }
        g_cache[key] = c;
    }
    std::fclose(f);
    return rc;
}

void tune_cache_clear() {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    g_cache.clear();
}

}  // namespace vfs

using vfs::fail;

extern "C" {

int vfs_model_autotune(vfs_model* h, int32_t repeats, int32_t use_cache, vfs_tune_config* chosen) {
    vfs::Model* m = vfs_model_impl(h);
    if (!m) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL model");
    return vfs::autotune(*m, repeats, use_cache != 0, chosen);
}

int vfs_model_set_tune_config(vfs_model* h, const vfs_tune_config* c) {
    vfs::Model* m = vfs_model_impl(h);
    if (!m || !c) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    return vfs::apply_tune_config(*m, *c);
}

int vfs_model_get_tune_config(vfs_model* h, vfs_tune_config* c) {
    vfs::Model* m = vfs_model_impl(h);
    if (!m || !c) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    *c = vfs::get_tune_config(*m);
    return VFS_OK;
}

int vfs_batch_autotune(vfs_batch* h, int32_t repeats, int32_t use_cache, vfs_tune_config* chosen) {
    vfs::Model* m = vfs_batch_impl(h);
    if (!m) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL batch");
    return vfs::autotune(*m, repeats, use_cache != 0, chosen);
}

int vfs_batch_set_tune_config(vfs_batch* h, const vfs_tune_config* c) {
    vfs::Model* m = vfs_batch_impl(h);
    if (!m || !c) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    return vfs::apply_tune_config(*m, *c);
}

int vfs_batch_get_tune_config(vfs_batch* h, vfs_tune_config* c) {
    vfs::Model* m = vfs_batch_impl(h);
    if (!m || !c) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    *c = vfs::get_tune_config(*m);
    return VFS_OK;
}

int vfs_tune_cache_save(const char* path) { return vfs::tune_cache_save(path); }
int vfs_tune_cache_load(const char* path) { return vfs::tune_cache_load(path); }
int vfs_tune_cache_clear(void) {
    vfs::tune_cache_clear();
    return VFS_OK;
}

}  // extern "C"
