// The reference's spatial-hash compute primitives as standalone C-ABI calls on device buffers:
//   GPUCountSort::Run  (src/compute/sort.cpp:107-143)  -> vfs_sort_pairs
//   SpatialOffset::Run (src/compute/sort.cpp:155-176)  -> vfs_spatial_offsets
//   BufferReorder      (src/compute/sort.cpp:185-227)  -> vfs_reorder_float3
// They run on the caller's stream and return without synchronising it.
#include <cuda_runtime.h>

#include <string>

#include "vfs_cuda.h"
#include "vfs_internal.h"
#include "vfs_model.h"

namespace vfs {
namespace {

#define VFS_PRIM_TRY(expr)                                                                   \
    do {                                                                                     \
        cudaError_t e_ = (expr);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return ::vfs::fail(VFS_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// InitOffsets + CalculateOffsets, assets/shaders/simulation/spatial_hash/spatial_offsets.slang:10-31.
__global__ void k_init_offsets(uint32_t* __restrict__ offsets, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) offsets[i] = n;
}

__global__ void k_calc_offsets(const uint32_t* __restrict__ sorted_keys,
                               uint32_t* __restrict__ offsets, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t key = sorted_keys[i];
    const uint32_t prev = i == 0u ? n : sorted_keys[i - 1];
    if (key != prev && key < n) offsets[key] = i;
}

// Reorder, assets/shaders/simulation/spatial_hash/reorder.slang:11-19, on packed float3.
__global__ void k_reorder_float3(const uint32_t* __restrict__ idx, const float* __restrict__ src,
                                 float* __restrict__ dst, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t s = idx[i];
    if (s >= n) return;
    dst[3 * (size_t)i] = src[3 * (size_t)s];
    dst[3 * (size_t)i + 1] = src[3 * (size_t)s + 1];
    dst[3 * (size_t)i + 2] = src[3 * (size_t)s + 2];
}

// Error bits of every pair sort on this device since the last vfs_sort_pairs_status: each sort's
// own error word (its look-back timeouts) is OR-ed in after its passes. A fixed device word, so
// the no-allocation sort can report through it too.
__device__ uint32_t g_sort_status;

__global__ void k_sort_status_accumulate(const uint32_t* __restrict__ err) {
    const uint32_t e = *err;
    if (e) atomicOr(&g_sort_status, e);
}

}  // namespace

// Enqueues a stable sort of (keys, index) with caller-provided scratch: tmp_keys / tmp_items
// (n words each) and `scratch` of sort_scratch_words(sc) words plus one error word.
int enqueue_sort_pairs(uint32_t* items, uint32_t* keys, uint32_t n, const SortConfig& sc,
                       uint32_t* tmp_keys, uint32_t* tmp_items, uint32_t* scratch,
                       cudaStream_t s) {
    SortScratch scr;
    scr.ghist = scratch;
    scr.counters = scratch + (size_t)sc.passes * sc.bins;
    scr.status = scr.counters + sc.passes;
    scr.err = scratch + sort_scratch_words(sc);
    VFS_PRIM_TRY(cudaMemsetAsync(scratch, 0, (sort_scratch_words(sc) + 1) * sizeof(uint32_t), s));
    VFS_PRIM_TRY(launch_digit_hist(keys, n, sc, scr.ghist, s));
    uint32_t* sk = nullptr;
    uint32_t* sp = nullptr;
    VFS_PRIM_TRY(launch_sort(n, sc, scr, keys, tmp_keys, items, tmp_items, &sk, &sp, s));
    if (sk != keys) VFS_PRIM_TRY(cudaMemcpyAsync(keys, sk, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    if (sp != items)
        VFS_PRIM_TRY(cudaMemcpyAsync(items, sp, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    k_sort_status_accumulate<<<1, 1, 0, s>>>(scr.err);
    VFS_PRIM_TRY(cudaGetLastError());
    return VFS_OK;
}

}  // namespace vfs

using vfs::fail;

extern "C" {

int vfs_sort_pairs(uint32_t* items, uint32_t* keys, uint32_t n, uint32_t max_value, void* stream) {
    if (n == 0) return VFS_OK;
    if (!items || !keys) return fail(VFS_ERR_INVALID_ARGUMENT, "items and keys must not be NULL");
    if (n > vfs::kMaxParticles) return fail(VFS_ERR_CAPACITY, "n must be <= 2^30");
    cudaStream_t s = (cudaStream_t)stream;
    const vfs::SortConfig sc = vfs::make_sort_config(n, 8, 16, vfs::key_bits_for(max_value));
    const size_t words = vfs::sort_scratch_words(sc) + 1;
    uint32_t *tk = nullptr, *ti = nullptr, *scratch = nullptr;
    VFS_PRIM_TRY(cudaMallocAsync(&tk, (size_t)n * 4, s));
    VFS_PRIM_TRY(cudaMallocAsync(&ti, (size_t)n * 4, s));
    VFS_PRIM_TRY(cudaMallocAsync(&scratch, words * 4, s));
    const int rc = vfs::enqueue_sort_pairs(items, keys, n, sc, tk, ti, scratch, s);
    cudaFreeAsync(tk, s);
    cudaFreeAsync(ti, s);
    cudaFreeAsync(scratch, s);
    return rc;
}

int vfs_sort_pairs_status(void* stream, uint32_t* err_word) {
    cudaStream_t s = (cudaStream_t)stream;
    VFS_PRIM_TRY(cudaStreamSynchronize(s));
    uint32_t e = 0u;
    const uint32_t zero = 0u;
    VFS_PRIM_TRY(cudaMemcpyFromSymbol(&e, vfs::g_sort_status, sizeof(e)));
    VFS_PRIM_TRY(cudaMemcpyToSymbol(vfs::g_sort_status, &zero, sizeof(zero)));
    if (err_word) *err_word = e;
    if (e) return fail(VFS_ERR_DEVICE_CHECK, "pair sort error word set: " + std::to_string(e) +
                                                 " (look-back timeout; the sorted output is invalid)");
    return VFS_OK;
}

int vfs_spatial_offsets(const uint32_t* sorted_keys, uint32_t* offsets, uint32_t n, void* stream) {
    if (n == 0) return VFS_OK;
    if (!sorted_keys || !offsets) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL buffer");
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned blocks = (n + 255u) / 256u;
    vfs::k_init_offsets<<<blocks, 256, 0, s>>>(offsets, n);
    vfs::k_calc_offsets<<<blocks, 256, 0, s>>>(sorted_keys, offsets, n);
    VFS_PRIM_TRY(cudaGetLastError());
    return VFS_OK;
}

int vfs_reorder_float3(const uint32_t* sorted_indices, const float* src, float* dst, uint32_t n,
                       void* stream) {
    if (n == 0) return VFS_OK;
    if (!sorted_indices || !src || !dst || src == dst)
        return fail(VFS_ERR_INVALID_ARGUMENT, "NULL or aliased buffer");
    vfs::k_reorder_float3<<<(n + 255u) / 256u, 256, 0, (cudaStream_t)stream>>>(sorted_indices, src,
                                                                             dst, n);
    VFS_PRIM_TRY(cudaGetLastError());
    return VFS_OK;
}

int vfs_selftest_lookback(int32_t predecessor_published, int32_t spin_limit, uint32_t* err_word,
                          uint32_t* exclusive) {
    if (spin_limit < 1 || spin_limit > (1 << 20))
        return fail(VFS_ERR_INVALID_ARGUMENT, "spin_limit must be in [1, 2^20]");
    uint32_t* d = nullptr;
    VFS_PRIM_TRY(cudaMalloc(&d, 97 * sizeof(uint32_t)));  // status 2 x 32, exclusive 32, error word
    uint32_t h[33];
    cudaError_t e = cudaMemset(d, 0, 97 * sizeof(uint32_t));
    if (e == cudaSuccess)
        e = vfs::launch_lookback_selftest(predecessor_published != 0, (uint32_t)spin_limit, d, d + 96,
                                          nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(h, d + 64, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return fail(VFS_ERR_CUDA, cudaGetErrorString(e));
    if (exclusive)
        for (int b = 0; b < 32; b++) exclusive[b] = h[b];
    if (err_word) *err_word = h[32];
    if (h[32]) return fail(VFS_ERR_DEVICE_CHECK, "device error word set: " + std::to_string(h[32]) +
                                                     " (look-back timeout)");
    return VFS_OK;
}

}  // extern "C"
