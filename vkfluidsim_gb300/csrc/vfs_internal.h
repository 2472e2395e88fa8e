// Internal structures shared by the host runtime and the sm_103a kernels of the WCSPH step.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vfs {

constexpr int kMaxObjects = 8;      // boundary objects per scene
constexpr uint32_t kMaxScenes = 65535;  // scene ids are 16-bit
constexpr int kMaxSortPasses = 4;   // 32-bit keys at >= 8-bit digits
constexpr int kMaxSortBins = 256;   // digit width <= 8 bits
constexpr uint32_t kFlagAggregate = 1u << 30;
constexpr uint32_t kFlagPrefix = 2u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1u;
constexpr uint32_t kMaxParticles = 1u << 30;
constexpr uint32_t kNbrCap = 128;  // neighbour-list slots per particle (overflow falls back)
// nbr_count[i] holds the list length in its low 25 bits, particle i's cell coordinates mod 4 in
// bits 25-26 (x), 27-28 (y), 29-30 (z), and in the top bit whether its 27 neighbour cells have 27
// distinct keys (then every in-range neighbour appears once in its list).
constexpr uint32_t kNbrDistinct = 0x80000000u;
constexpr uint32_t kNbrCountMask = 0x01FFFFFFu;
constexpr uint32_t kNbrCellShift = 25;

__host__ __device__ inline uint32_t nbr_word(uint32_t listed, uint32_t cx, uint32_t cy, uint32_t cz,
                                             bool distinct) {
    return (listed < kNbrCountMask ? listed : kNbrCountMask) | ((cx & 3u) << kNbrCellShift) |
           ((cy & 3u) << (kNbrCellShift + 2)) | ((cz & 3u) << (kNbrCellShift + 4)) |
           (distinct ? kNbrDistinct : 0u);
}

// For two particles within h of each other (cells at most 2 apart per axis): are their cells
// adjacent (at most 1 apart on every axis)? Decided from the cell residues of their words.
__host__ __device__ inline bool nbr_cells_adjacent(uint32_t a, uint32_t b) {
    bool adj = true;
    for (uint32_t s = kNbrCellShift; s < kNbrCellShift + 6; s += 2)
        adj = adj && (((a >> s) - (b >> s)) & 3u) != 2u;
    return adj;
}

// Error bits of the per-model device error word.
constexpr uint32_t kErrLookbackTimeout = 1u;

// One volume-map boundary object as the kernels read it
// (WCSPHWithBoundaryModel::BoundaryObjectInfo, src/models/wcsph_with_boundary_model.h:16-24):
// the glm column-major matrices are stored row-major 3x4 (the fourth row of both is (0,0,0,1)).
struct DevObject {
    float T[12];  // world -> object-local affine (inverse of the object transform)
    float R[12];  // rotation applied to the local normal, with w = 1 as the shader does
    float box_pos[3];
    float box_size[3];
    uint32_t res[3];
    const float* sdf;
    const float* vm;
};

// Per-scene, per-substep constants. Derived on the host once, from the same float expressions the
// reference host and shaders use (src/models/model.cpp:225-234, wcsph_with_boundary_model.slang:39-41).
// A scene owns particles [off, off + n) and keys [off, off + n): key = off + HashCell3D % n.
struct SceneParams {
    uint32_t n;          // particles of the scene = its hash-table size
    uint32_t off;        // first particle index and first key of the scene
    uint64_t mod_magic;  // ceil(2^64 / n): hash % n by multiply-high
    float h, h2, inv_h;
    float cubic;        // 8 / (pi h^3)
    float grad_over_h;  // 48 / (pi h^4) / h (the shader's extra 1/h)
    float mass;         // rho0 * 0.8 h^3 / 8
    float rho0, stiffness, expoent;
    float visc_scale;   // 2 (d + 2) nu with d = 3
    float visc_eps;     // 0.01 h^2
    float wall_k, dt;
    float gx, gy, gz;
    float lo[3], hi[3];
    float grad_eps;     // 0.1 h (GradientVector)
    float bnd_eighth;   // 0.125 h
    float bnd_half;     // 0.5 h
    uint32_t nbr_cap;   // neighbour-list slots per particle
    float skin_r2;      // (h (1 + skin))^2: radius of the candidate lists (0: no lists)
    float skin_half2;   // (h skin / 2)^2: displacement since the last build that forces a rebuild
    float skin_lim;     // (1 + skin)^2 x 1.002: cell pruning limit of the list build, in h^2
    uint32_t n_objects;
    const DevObject* objects;  // device array of n_objects
};

// What every pass of one substep needs: a single scene passed inline, or (batched) a device table
// of scenes with the scene id of every particle.
struct StepLaunch {
    uint32_t total;              // particles of all scenes
    uint32_t n_scenes;
    const SceneParams* scenes;   // device, n_scenes entries (batched launches)
    const uint16_t* scene_of;    // device, scene id per particle (batched launches)
    SceneParams one;             // the scene of a single-scene launch
    float* host_dens = nullptr;  // page-locked host array (its device address): the density pass
                                 // also writes each particle's density there, in slot order
    bool defer_vel = false;      // velocities still on their way from the host: the cell pass
                                 // leaves them unsorted and the density pass leaves the force
                                 // records' velocity half to launch_vel_records
};

// Scratch of one onesweep sort: global digit histograms, tile counters, look-back status words.
struct SortScratch {
    uint32_t* ghist;     // [passes][bins]
    uint32_t* counters;  // [passes]
    uint32_t* status;    // [passes][tiles][bins]
    uint32_t* dstatus;   // key pass: each tile's moved count, then its exclusive prefix [delta_blocks]
    uint32_t* mcount;    // number of particles whose key changed [1]
    uint32_t* err;       // device error word
};

struct SortConfig {
    int digit_bits;  // 4..8
    int passes;
    int bins;
    int tile;        // elements per onesweep tile
    uint32_t tiles;
    uint32_t delta_blocks;  // tiles of the key pass (1024 particles each)
};

// ---- launch wrappers (vfs_kernels.cu) ----
// Number of bits needed to hold every key <= max_key (at least 1).
int key_bits_for(uint32_t max_key);
// key_bits <= 0: keys are spatial-hash keys, < n.
SortConfig make_sort_config(uint32_t n, int digit_bits, int tile_items, int key_bits = 0);

// Launch shapes of the neighbour passes: threads per block x minimum resident blocks per SM.
enum NbrShape : int { kNbr128x6 = 0, kNbr128x8 = 1, kNbr96x8 = 2, kNbr64x12 = 3, kNumNbrShapes = 4 };
// Candidate lists with a skin (Verlet lists). A build, in a density pass, lists for every particle
// the particles within h (1 + skin), in the reference's visiting order, under the particles' sorted
// indices of that substep (their build indices), and keeps each particle's position. Until some
// particle of the scene has moved more than h skin / 2 since then, every pair within h is in the
// lists, and a particle whose list is usable sums it instead of walking the 27 buckets (same
// in-range set, multiplicity one). The cell pass keeps `cur`, the current sorted index of every
// build index, checks every displacement against `x_build` and marks the scene stale; in a stale
// scene every particle walks, and the lists are rebuilt when the scene's build policy allows it.
// The force pass runs the policy: a stale scene walks at least one substep before it rebuilds;
// lists that went stale within kSkinMinLife substeps of their build, or a build that left fewer
// than half of the scene's lists usable, double the substeps it walks before the next build
// (from kSkinMinWait to kSkinMaxWait); longer-lived lists rebuild as soon as they go stale. A
// single scene whose last build left most lists unusable is walked in index order, as a stale
// one is, until its next build.
struct SkinLists {
    uint32_t* list = nullptr;     // slot-major: list[k * total + b] = build index of candidate k of b
    uint32_t* count = nullptr;    // per build index: list length, kSkinUsable when it can be summed
    float4* x_build = nullptr;    // per build index: position at the last build
    uint32_t* b_of_id = nullptr;  // per id: build index
    uint32_t* b_next = nullptr;   // a whole-scene upload's b_of_id under the new ids (id = slot:
                                  // the build index of the particle the slot held), copied back
    float4* xcur = nullptr;       // per build index: current position (x, y, z) and current sorted
                                  // index (w, as bits), written by the cell pass
    uint32_t* stale = nullptr;    // per scene: nonzero when some particle moved past h skin / 2
    uint32_t* ctl = nullptr;      // per scene, kSkinCtl words: the build policy's state (kCtl*)
    uint32_t* queue = nullptr;    // the particles the density pass walks this substep: those of
                                  // list block b at [128 b, 128 b + seg_n[b]), in index order
    uint32_t* seg_n = nullptr;    // per list block (128 particles): its walkers
    uint32_t* wcount = nullptr;   // single scene: walkers in `queue`, packed from 0 (one word)
    uint32_t cap = 0;             // slots per particle
};
constexpr uint32_t kSkinUsable = 1u << 31;
constexpr uint32_t kSkinCtl = 8;       // words of policy state per scene:
constexpr uint32_t kCtlAllow = 0;      //   a stale scene may rebuild this substep
constexpr uint32_t kCtlAge = 1;        //   substeps since the last build
constexpr uint32_t kCtlWait = 2;       //   stale substeps to walk before the next build
constexpr uint32_t kCtlBuilds = 3;     //   builds so far
constexpr uint32_t kCtlFresh = 4;      //   the lists of the last build have not gone stale yet
constexpr uint32_t kCtlSince = 5;      //   stale substeps since the lists went stale
constexpr uint32_t kCtlUsable = 6;     //   usable lists left by this substep's build
constexpr uint32_t kCtlPoor = 7;       //   the last build left fewer than half of them usable
constexpr uint32_t kSkinMinLife = 12;  // a build substep costs about two walks; a list pass saves ~0.45 of one
constexpr uint32_t kSkinMinWait = 8;
constexpr uint32_t kSkinMaxWait = 256;
constexpr uint32_t kSkinCap = 48;  // also the density walk's shared list, where a build is staged

// Launch shapes chosen per model (by default or by the autotuner); none changes any result.
struct KernelConfig {
    int nbr_shape = kNbr96x8;     // density pass (and the adjoint's recomputed forward)
    int force_shape = kNbr128x8;  // force pass (no shared memory: it takes the larger blocks)
    int cell_block = 256;  // keys per block of the cell-range / reorder kernel: 128, 256 or 512
    int walk_staging = 0;  // density walk: warps whose particles share a row of cells stage it
                           // (off by default: the autotuner turns it on where it is faster)
};
size_t sort_scratch_words(const SortConfig& c);

// Per-pass digit histograms of caller-provided keys.
cudaError_t launch_digit_hist(const uint32_t* keys, uint32_t n, const SortConfig& sc,
                              uint32_t* ghist, cudaStream_t s);
// Incremental sort, pass 1 (flags, compaction, and a tile scan above 4M particles): keys, moved flags
// (key != pkeys[i]) as a bitmask bits[0, W) with the moved count before each word in bits[W, 2W]
// (W = ceil(n / 32)), the moved (key, index) pairs compacted in index order, their digit
// histograms, and the moved count in scr.mcount. host3 (a single scene only): the positions are
// read from that page-locked packed float3 array instead, and stored into pos_out (= pos) as the
// state upload stores them (id = slot, the densities in aux zeroed; with b_next, each slot's
// old id's build index stored under its new id, b_next[slot] = b_of_id[old id]).
cudaError_t launch_keys_delta(const StepLaunch& L, const float4* pos, const uint32_t* pkeys,
                              uint32_t* mkeys, uint32_t* midx, uint32_t* bits,
                              const SortConfig& sc, const SortScratch& scr, cudaStream_t s,
                              const float* host3 = nullptr, float4* pos_out = nullptr,
                              float4* aux = nullptr, const uint32_t* b_of_id = nullptr,
                              uint32_t* b_next = nullptr);
// Incremental sort, last pass: merge of the unmoved particles with the sorted moved ones into the
// stable sort of all (key, index) pairs.
cudaError_t launch_merge(uint32_t n, const uint32_t* pkeys, const uint32_t* bits,
                         const uint32_t* mcount, const uint32_t* mk, const uint32_t* mi,
                         uint32_t* out_keys, uint32_t* out_perm, cudaStream_t s);
// Stable LSD onesweep over sc.passes digits; returns the buffers holding sorted keys / perm.
// vals_given: `vals` holds the values to carry (else the values are the indices); n_dev: an
// optional device-side count (<= n) of elements to sort (the digit histograms must match it).
cudaError_t launch_sort(uint32_t n, const SortConfig& sc, const SortScratch& scratch,
                        uint32_t* keys, uint32_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                        uint32_t** sorted_keys, uint32_t** sorted_perm, cudaStream_t s,
                        bool vals_given = false, const uint32_t* n_dev = nullptr);
// cell_scan[k] = first sorted index with key >= k (k in [0, n]); gathers pos/vel by perm; zeroes
// zero[0, zero_words) (the sort scratch, for the next substep); copies skeys to pkeys_out (the next
// substep's previous sorted keys) when pkeys_out is not NULL. guess (n / 128 + 2 words, any
// contents) keeps each block's bound of the sorted keys as the next call's starting point; NULL
// searches from scratch. With skin lists (sk.cur set), also sk.cur[sk.b_of_id[id]] = sorted index
// for the ids in x.w, and flags every scene of L with a particle that moved more than h skin / 2
// since its list build.
// The sorted velocities and the force records' velocity half of a substep whose cell and density
// passes ran with StepLaunch::defer_vel, from the uploaded velocities (packed float3 in slot
// order, vel3): vel_out[i] = (vel3[perm[i]], 0), rec[2i + 1] = (that velocity, aux[i].y), the
// values those passes write otherwise.
cudaError_t launch_vel_records(uint32_t n, const uint32_t* perm, const float* vel3,
                               float4* vel_out, const float4* aux, float4* rec, cudaStream_t s);
cudaError_t launch_cells_reorder(const StepLaunch& L, uint32_t n, const uint32_t* skeys, const uint32_t* perm,
                                 uint32_t* cell_scan, const float4* pos_in, const float4* vel_in,
                                 float4* pos_out, float4* vel_out, uint32_t* zero,
                                 uint32_t zero_words, uint32_t* pkeys_out, uint32_t* guess,
                                 const SkinLists& sk, const KernelConfig& kc, cudaStream_t s);
// Failure-detection self-test of the sort's bounded look-back wait (d_work: 96 words).
cudaError_t launch_lookback_selftest(bool published, uint32_t spin_limit, uint32_t* d_work,
                                     uint32_t* err, cudaStream_t s);
// True when the density pass runs three lanes per particle: the model is small enough that one
// lane per particle would leave the GPU waiting on each thread's chain of loads (3 N threads
// still fit one wave at 768 threads per SM). The density pass's launch shape does not apply then.
bool planes_mode(uint32_t total);
// Boundary volume + density + EOS epilogue; writes each particle's neighbour list.
// Also writes rec[2i], rec[2i+1] = (x, y, z, p/rho^2), (v, m/max(rho, 1e-6)) for the force pass.
// With skin lists (sk.list set): sums the lists where they are usable and rebuilds flagged scenes.
// walk_sched: two device words, zero between launches (the walk kernel's run counter, put back to
// zero by its last warp).
cudaError_t launch_density(const StepLaunch& L, const float4* pos, const float4* vel, float4* rec,
                           const uint32_t* cell_scan, float4* aux, float4* bnd, uint32_t* nbr,
                           uint32_t* nbr_count, const SkinLists& sk, uint32_t* walk_sched,
                           const KernelConfig& kc, cudaStream_t s);
// Pressure + viscosity + wall + symplectic Euler over the density pass's neighbour lists; runs the
// skin lists' build policy and clears their flags (when sk.stale is set).
// Page-locked host arrays (device addresses of them) the force pass of a single scene writes its
// results into besides the state buffers: positions and velocities as float3, densities as float,
// in slot order (any may be null). Written through shared memory in whole 128-byte lines.
struct HostOut {
    float* pos3 = nullptr;
    float* vel3 = nullptr;
    float* dens = nullptr;
    bool any() const { return pos3 || vel3 || dens; }
};
cudaError_t launch_force(const StepLaunch& L, const float4* pos, const float4* vel,
                         const float4* aux, const float4* rec, const float4* bnd, const uint32_t* cell_scan,
                         const uint32_t* nbr, const uint32_t* nbr_count, float4* pos_out,
                         float4* vel_out, float4* acc_out, const SkinLists& sk,
                         const KernelConfig& kc, cudaStream_t s, const HostOut& ho = HostOut{});
// Stable in-place sort of (keys, items) with caller-provided temporaries (n words each) and
// sort scratch (sort_scratch_words(sc) + 1 words, zeroed here); items become the permutation.
int enqueue_sort_pairs(uint32_t* items, uint32_t* keys, uint32_t n, const SortConfig& sc,
                       uint32_t* tmp_keys, uint32_t* tmp_items, uint32_t* scratch,
                       cudaStream_t s);
// Scene-local spatial_offsets[k] = cell start - off, or n for empty keys (reference layout), for
// the scene owning keys [off, off + n).
cudaError_t launch_offsets(uint32_t n, uint32_t off, const uint32_t* cell_scan, uint32_t* offsets,
                           cudaStream_t s);

}  // namespace vfs
