// vfs_sort_pairs_noalloc: the stable pair sort of vfs_sort_pairs for callers that cannot allocate
// device memory — code running in a frame loop or inside a host framework that owns the GPU's
// memory budget (a cudaMalloc there can synchronise the device, fragment the host's pool, or break
// a stream capture). Its scratch is the fixed array below, reserved once per device when the
// library's module loads and kept until the process exits.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "vfs_cuda.h"
#include "vfs_internal.h"
#include "vfs_model.h"

namespace vfs {
namespace {

constexpr uint32_t kNoAllocPairs = VFS_SORT_NOALLOC_MAX_PAIRS;
constexpr uint32_t kNoAllocTile = 256u * 16u;  // onesweep tile of make_sort_config(.., 8, 16, ..)
constexpr uint32_t kNoAllocTiles = (kNoAllocPairs + kNoAllocTile - 1u) / kNoAllocTile;
// Digit histograms + tile counters + look-back status words + the key pass's words
// (unused by a pair sort, but part of sort_scratch_words) + the error word, for any key width.
constexpr size_t kNoAllocSortWords = (size_t)kMaxSortPasses * kMaxSortBins + kMaxSortPasses +
                                     (size_t)kMaxSortPasses * kNoAllocTiles * kMaxSortBins + 2 +
                                     (kNoAllocPairs + 1023u) / 1024u + 1;
// Two temporaries of kNoAllocPairs words (keys, items) followed by the sort scratch: 2.3 MB.
constexpr size_t kNoAllocWords = 2 * (size_t)kNoAllocPairs + kNoAllocSortWords;

// Host code never dereferences this name: on the host it is only a stand-in for the symbol, and
// the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
uint32_t* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device, looked up once per device.
int scratch_address(uint32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(VFS_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(VFS_ERR_CAPACITY, "device ordinal beyond 63");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(VFS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch_addr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch_addr[dev];
    return VFS_OK;
}

}  // namespace
}  // namespace vfs

extern "C" int vfs_sort_pairs_noalloc(uint32_t* items, uint32_t* keys, uint32_t n,
                                      uint32_t max_value, void* stream) {
    using namespace vfs;
    if (n == 0) return VFS_OK;
    if (!items || !keys) return fail(VFS_ERR_INVALID_ARGUMENT, "items and keys must not be NULL");
    if (n > kNoAllocPairs)
        return fail(VFS_ERR_CAPACITY, "vfs_sort_pairs_noalloc sorts at most " +
                                          std::to_string(kNoAllocPairs) + " pairs (got " +
                                          std::to_string(n) + ")");
    const SortConfig sc = make_sort_config(n, 8, 16, key_bits_for(max_value));
    if (sort_scratch_words(sc) + 1 > kNoAllocSortWords)
        return fail(VFS_ERR_CAPACITY, "sort configuration exceeds the static scratch");
    uint32_t* base = nullptr;
    const int rc = scratch_address(&base);
    if (rc) return rc;
    // enqueue_sort_pairs zeroes the histogram / status / error words the previous call left.
    return enqueue_sort_pairs(items, keys, n, sc, base, base + kNoAllocPairs,
                              base + 2 * (size_t)kNoAllocPairs, (cudaStream_t)stream);
}
