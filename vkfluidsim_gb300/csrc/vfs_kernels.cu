// sm_103a kernels of one WCSPH-with-boundary substep (VkFluidSim's
// WCSPHWithBoundaryModel::Step, src/models/wcsph_with_boundary_model.cpp:81-117):
//
//   k_keys            key[i] = HashCell3D(floor(x_i / h)) % N  + per-pass digit histograms
//   k_onesweep        stable LSD radix pass of (key, index) with decoupled look-back
//   k_cells_reorder   cell_scan[] (lower bound of every key) + gather of x, v (and ids in x.w)
//   k_density         volume-map boundary terms + density + Tait EOS epilogue
//   k_force           pressure + viscosity + wall penalty + symplectic Euler
//
// Data layout: particle state is float4 SoA (x,y,z,id-bits) and (vx,vy,vz,0) in sorted order;
// per-particle density products aux = (p/rho^2, m/max(rho,1e-6), rho, p/rho0^2); boundary
// bnd = (grad Psi_b, Psi_b). All arrays are 16-byte aligned and read with 128-bit loads.
//
// The neighbour loops visit exactly the reference's candidate multiset in the reference's order:
// for each (dy, dz) the keys of cells (cx-1..cx+1) are usually consecutive (HashCell3D is
// x-linear inside a 50-cell block), and consecutive keys' buckets are adjacent in the sorted
// array, so the three buckets are one contiguous range [scan[kA], scan[kA+3]). When the three
// keys are not consecutive, each bucket is walked on its own. Duplicate keys among the 27 are
// walked as often as they occur, like wcsph_with_boundary_model.slang:166-190.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <climits>
#include <atomic>

#include "vfs_internal.h"

namespace vfs {
namespace {

// ---------------------------------------------------------------- hashing

// HashCell3D, assets/shaders/simulation/spatial_hash/spatial_hash_3d.slang:20-28.
__device__ __forceinline__ uint32_t hash_cell(uint32_t cx, uint32_t cy, uint32_t cz) {
    const uint32_t ux = cx + 25u, uy = cy + 25u, uz = cz + 25u;
    const uint32_t lx = ux % 50u, ly = uy % 50u, lz = uz % 50u;
    const uint32_t bx = ux / 50u, by = uy / 50u, bz = uz / 50u;
    const uint32_t block_hash = bx * 15823u + by * 9737333u + bz * 440817757u;
    return lx + 50u * (ly + 50u * lz) + block_hash;
}

// KeyFromHash (spatial_hash_3d.slang:30-32): hash % n, computed as the high word of
// (magic * hash mod 2^64) * n with magic = ceil(2^64 / n) (exact for 32-bit operands).
__device__ __forceinline__ uint32_t key_mod(uint32_t hash, uint64_t magic, uint32_t n) {
    const uint64_t low = magic * (uint64_t)hash;
    return (uint32_t)__umul64hi(low, (uint64_t)n);
}

// GetCell3D (spatial_hash_3d.slang:16-18): IEEE division, floor, saturating conversion.
__device__ __forceinline__ uint32_t cell_coord(float x, float h) {
    return (uint32_t)__float2int_rz(floorf(__fdiv_rn(x, h)));
}

// ---------------------------------------------------------------- SPH kernel

// CubicSpline (kernels_3d.slang:62-76) at q = r / h.
__device__ __forceinline__ float cubic_w(float q, float sigma) {
    if (q <= 1.0f) {
        if (q > 0.5f) {
            const float t = 1.0f - q;
            return sigma * 2.0f * (t * t * t);
        }
        const float q2 = q * q;
        const float q3 = q2 * q;
        return sigma * (6.0f * q3 - 6.0f * q2 + 1.0f);
    }
    return 0.0f;
}

// GradCubicSpline (kernels_3d.slang:78-91); sigma already carries the extra 1/h.
__device__ __forceinline__ float cubic_dw(float r, float q, float sigma) {
    if ((r > 1e-9f) && (q <= 1.0f)) {
        if (q > 0.5f) {
            const float t = 1.0f - q;
            return -sigma * (t * t);
        }
        return sigma * q * (3.0f * q - 2.0f);
    }
    return 0.0f;
}

// ---------------------------------------------------------------- volume-map sampling
// Written with round-to-nearest intrinsics, which the compiler never fuses, so the thresholds
// of CalculateBoundaryVolume (inside-box, 0 <= dist < h, volume > 0) evaluate bit-identically
// to an unfused IEEE restatement.

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsb(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdv(float a, float b) { return __fdiv_rn(a, b); }

// One axis of SampleGrid with the cell index clamped to [0, n-2] (linear extrapolation outside;
// the reference reads out of bounds there, wcsph_with_boundary_model.slang:51-66).
__device__ __forceinline__ void grid_axis(uint32_t n, float u, uint32_t& cell, float& chi) {
    const float x = fm(fsb((float)n, 1.0f), u);
    float f = floorf(x);
    const float hi = (float)(n - 2u);
    if (!(f >= 0.0f)) f = 0.0f;
    if (f > hi) f = hi;
    cell = (uint32_t)f;
    chi = fsb(fm(2.0f, fsb(x, f)), 1.0f);
}

// A point of a grid in SampleGrid's terms: per axis the clamped cell and chi = 2 frac - 1.
struct GridPoint {
    uint32_t cell[3];
    float chi[3];
};

// Index of a point's base corner (its cell's lowest corner) in the grid array.
__device__ __forceinline__ size_t grid_base(const uint32_t* n, const GridPoint& g) {
    return g.cell[0] + (size_t)n[0] * g.cell[1] + (size_t)n[0] * n[1] * g.cell[2];
}

// The 8 corner values of a point's cell, in the shader's offsets[8] order:
// (0,0,0) (0,1,0) (0,0,1) (0,1,1) (1,0,0) ...
__device__ __forceinline__ void grid_corners(const float* __restrict__ g, const uint32_t* n,
                                             const GridPoint& p, float c[8]) {
    const size_t b = grid_base(n, p), sy = n[0], sz = (size_t)n[0] * n[1];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int ox = i >> 2, oy = i & 1, oz = (i >> 1) & 1;
        c[i] = __ldg(g + b + ox + oy * sy + oz * sz);
    }
}

// SampleGrid's weighted sum over the corner values (wcsph_with_boundary_model.slang:51-66).
__device__ __forceinline__ float grid_interp(const float c[8], const GridPoint& p) {
    float val = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int ox = i >> 2, oy = i & 1, oz = (i >> 1) & 1;
        const float fx = fa(1.0f, fm(ox ? 1.0f : -1.0f, p.chi[0]));
        const float fy = fa(1.0f, fm(oy ? 1.0f : -1.0f, p.chi[1]));
        const float fz = fa(1.0f, fm(oz ? 1.0f : -1.0f, p.chi[2]));
        val = fa(val, fm(c[i], fm(fm(fx, fy), fz)));
    }
    return fdv(val, 8.0f);
}

// SampleGrid at normalised coordinates (u, v, w).
__device__ __forceinline__ float sample_grid(const float* __restrict__ g, const uint32_t* n,
                                             float u, float v, float w) {
    GridPoint p;
    grid_axis(n[0], u, p.cell[0], p.chi[0]);
    grid_axis(n[1], v, p.cell[1], p.chi[1]);
    grid_axis(n[2], w, p.cell[2], p.chi[2]);
    float c[8];
    grid_corners(g, n, p, c);
    return grid_interp(c, p);
}

__device__ __forceinline__ void to_uvw(const DevObject& o, float x, float y, float z, float& u,
                                       float& v, float& w) {
    u = fdv(fsb(x, o.box_pos[0]), o.box_size[0]);
    v = fdv(fsb(y, o.box_pos[1]), o.box_size[1]);
    w = fdv(fsb(z, o.box_pos[2]), o.box_size[2]);
}

// Row r of a row-major 3x4 matrix applied to (x, y, z, 1), summed left to right.
__device__ __forceinline__ float mat_row(const float* M, int r, float x, float y, float z) {
    return fa(fa(fa(fm(M[4 * r], x), fm(M[4 * r + 1], y)), fm(M[4 * r + 2], z)), M[4 * r + 3]);
}

// CalculateBoundaryVolume for one particle (wcsph_with_boundary_model.slang:102-151).
__device__ __forceinline__ void boundary_terms(const SceneParams& p, float px, float py, float pz,
                                               float& bd, float& bgx, float& bgy, float& bgz) {
    bd = 0.0f;
    bgx = bgy = bgz = 0.0f;
    for (uint32_t oi = 0; oi < p.n_objects; oi++) {
        const DevObject& o = p.objects[oi];
        const float lx = mat_row(o.T, 0, px, py, pz);
        const float ly = mat_row(o.T, 1, px, py, pz);
        const float lz = mat_row(o.T, 2, px, py, pz);
        const bool outside = lx < o.box_pos[0] || ly < o.box_pos[1] || lz < o.box_pos[2] ||
                             lx > fa(o.box_pos[0], o.box_size[0]) ||
                             ly > fa(o.box_pos[1], o.box_size[1]) ||
                             lz > fa(o.box_pos[2], o.box_size[2]);
        if (outside) continue;
        float u, v, w;
        to_uvw(o, lx, ly, lz, u, v, w);
        GridPoint g0;
        grid_axis(o.res[0], u, g0.cell[0], g0.chi[0]);
        grid_axis(o.res[1], v, g0.cell[1], g0.chi[1]);
        grid_axis(o.res[2], w, g0.cell[2], g0.chi[2]);
        float c0[8];
        grid_corners(o.sdf, o.res, g0, c0);
        const float dist = grid_interp(c0, g0);
        if (!(dist >= 0.0f && dist < p.h)) continue;
        const float volume = sample_grid(o.vm, o.res, u, v, w);
        if (!(volume > 0.0f)) continue;
        // GradientVector (slang:68-85): central differences of the SDF at +-0.1 h. A sample
        // moved along one axis shares the other two axes' coordinates with the centre (the same
        // operations on the same inputs), and the centre's corner values while it stays in the
        // centre's cell; the sums are formed exactly as SampleGrid forms them.
        const float e = p.grad_eps;
        const float lc[3] = {lx, ly, lz};
        float grad[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            float s2[2];
#pragma unroll
            for (int sgn = 0; sgn < 2; sgn++) {
                const float la = sgn == 0 ? fa(lc[a], e) : fsb(lc[a], e);
                GridPoint g = g0;
                grid_axis(o.res[a], fdv(fsb(la, o.box_pos[a]), o.box_size[a]), g.cell[a], g.chi[a]);
                if (g.cell[a] == g0.cell[a]) {
                    s2[sgn] = grid_interp(c0, g);
                } else {
                    float c[8];
                    grid_corners(o.sdf, o.res, g, c);
                    s2[sgn] = grid_interp(c, g);
                }
            }
            grad[a] = fdv(fsb(s2[0], s2[1]), fm(2.0f, e));
        }
        const float gx = grad[0], gy = grad[1], gz = grad[2];
        const float modn = __fsqrt_rn(fa(fa(fm(gx, gx), fm(gy, gy)), fm(gz, gz)));
        if (!(modn > 1e-9f)) continue;
        float nx = mat_row(o.R, 0, gx, gy, gz);
        float ny = mat_row(o.R, 1, gx, gy, gz);
        float nz = mat_row(o.R, 2, gx, gy, gz);
        nx = fdv(nx, modn);
        ny = fdv(ny, modn);
        nz = fdv(nz, modn);
        const float d = fmaxf(fa(dist, p.bnd_eighth), p.bnd_half);
        const float xbx = fsb(px, fm(d, nx)), xby = fsb(py, fm(d, ny)), xbz = fsb(pz, fm(d, nz));
        const float xx = fsb(px, xbx), xy = fsb(py, xby), xz = fsb(pz, xbz);
        const float r = __fsqrt_rn(fa(fa(fm(xx, xx), fm(xy, xy)), fm(xz, xz)));
        float ux = 0.0f, uy = 0.0f, uz = 0.0f;
        if (r > 0.0f) {
            ux = fdv(xx, r);
            uy = fdv(xy, r);
            uz = fdv(xz, r);
        }
        const float q = fdv(r, p.h);
        bd = fa(bd, fm(volume, cubic_w(q, p.cubic)));
        const float s = fm(volume, cubic_dw(r, q, p.grad_over_h));
        bgx = fa(bgx, fm(s, ux));
        bgy = fa(bgy, fm(s, uy));
        bgz = fa(bgz, fm(s, uz));
    }
}

// ---------------------------------------------------------------- neighbour ranges

// ---------------------------------------------------------------- scenes

// Parameters of the scene owning particle i: the inline scene of a single-scene launch, or the
// scene-table entry of a batched one.
template <bool kBatch>
__device__ __forceinline__ const SceneParams& scene_params(const StepLaunch& L, uint32_t i) {
    if constexpr (kBatch)
        return L.scenes[__ldg(L.scene_of + i)];
    else
        return L.one;
}

// ---------------------------------------------------------------- kernels


// Per-pass digit histograms of caller-provided keys (the histogram half of k_keys).
__global__ void __launch_bounds__(256) k_digit_hist(const uint32_t* __restrict__ keys, uint32_t n,
                                                    int passes, int digit_bits,
                                                    uint32_t* __restrict__ ghist) {
    __shared__ uint32_t s_h[kMaxSortPasses * kMaxSortBins];
    const int bins = 1 << digit_bits;
    const uint32_t mask = (uint32_t)bins - 1u;
    for (int e = threadIdx.x; e < passes * bins; e += blockDim.x) s_h[e] = 0u;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t key = keys[i];
        for (int ps = 0; ps < passes; ps++)
            atomicAdd(&s_h[ps * bins + ((key >> (ps * digit_bits)) & mask)], 1u);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < passes * bins; e += blockDim.x)
        if (s_h[e]) atomicAdd(&ghist[e], s_h[e]);
}

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) {
    return *(const volatile uint32_t*)p;
}
__device__ __forceinline__ void st_volatile(uint32_t* p, uint32_t v) { *(volatile uint32_t*)p = v; }

// Exclusive scan over a 256-thread block; returns the exclusive prefix and writes the total.
__device__ __forceinline__ uint32_t block_excl_scan256(uint32_t v, uint32_t* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < 8 ? s_warp[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < 8) s_warp[8 + lane] = wi - w;
    }
    __syncthreads();
    const uint32_t r = s_warp[8 + warp] + incl - v;
    __syncthreads();
    return r;
}

constexpr uint32_t kLookbackSpinLimit = 1u << 20;

// Decoupled look-back of tile `tile` for digit `bin`: sums the predecessors' published counts,
// walking back until a tile with an inclusive prefix. A predecessor that has published nothing is
// polled at most spin_limit times; then kErrLookbackTimeout is set in *err and the partial sum is
// returned (the caller's scatter is guarded, and the host reports the error word).
__device__ __forceinline__ uint32_t lookback_exclusive(const uint32_t* status, int bins,
                                                       uint32_t tile, int bin, uint32_t spin_limit,
                                                       uint32_t* err) {
    uint32_t excl = 0u;
    uint32_t t = tile - 1u;
    uint32_t spins = 0u;
    while (true) {
        const uint32_t s = ld_volatile(status + (size_t)t * bins + bin);
        const uint32_t flag = s & ~kCountMask;
        if (flag == 0u) {
            if (++spins > spin_limit) {
                atomicOr(err, kErrLookbackTimeout);
                break;
            }
            __nanosleep(32);
            continue;
        }
        excl += s & kCountMask;
        if (flag == kFlagPrefix || t == 0u) break;
        t--;
    }
    return excl;
}

// Failure-detection self-test of the look-back wait: thread b plays tile 1 of digit b over a
// status table whose tile 0 has published (prefix b + 1) or not (nothing). exclusive[b] gets the
// look-back result.
__global__ void k_lookback_selftest(const uint32_t* status, int bins, uint32_t spin_limit,
                                    uint32_t* exclusive, uint32_t* err) {
    const int b = threadIdx.x;
    if (b < bins) exclusive[b] = lookback_exclusive(status, bins, 1u, b, spin_limit, err);
}

// One stable LSD radix pass (onesweep: Adinets & Merrill 2022). Tiles are claimed in launch
// order through an atomic counter, so every predecessor of a tile is already resident and the
// bounded look-back always terminates; a timeout sets an error bit instead of hanging.
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK)
    k_onesweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
               uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint32_t n,
               int shift, int bins, const uint32_t* __restrict__ ghist,
               uint32_t* __restrict__ counter, uint32_t* __restrict__ status,
               uint32_t* __restrict__ err, const uint32_t* __restrict__ n_dev) {
    static_assert(BLOCK == 256, "block scan assumes 256 threads");
    constexpr int WARPS = BLOCK / 32;
    constexpr int TILE = BLOCK * ITEMS;
    // A device-side count (at most n) sorts only that prefix; the grid is sized for n and tiles
    // past the count leave at once (no later tile waits on them: tiles are claimed in order).
    if (n_dev) n = min(n, *n_dev);
    __shared__ uint32_t s_whist[WARPS][kMaxSortBins];
    __shared__ uint32_t s_dstart[kMaxSortBins];
    __shared__ uint32_t s_gofs[kMaxSortBins];
    __shared__ uint32_t s_keys[TILE];
    __shared__ uint32_t s_vals[TILE];
    __shared__ uint32_t s_scan[16];
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const uint32_t mask = (uint32_t)bins - 1u;
    if (tid == 0) s_tile = atomicAdd(counter, 1u);
    for (int e = tid; e < WARPS * kMaxSortBins; e += BLOCK) (&s_whist[0][0])[e] = 0u;
    // Global exclusive digit offsets of this pass.
    const uint32_t gcount = tid < bins ? __ldg(ghist + tid) : 0u;
    const uint32_t gbase = block_excl_scan256(gcount, s_scan);  // contains __syncthreads
    const uint32_t tile = s_tile;
    if ((uint64_t)tile * TILE >= n) return;  // block-uniform, after the last barrier of the scan
    const uint32_t base = tile * (uint32_t)TILE + (uint32_t)warp * ITEMS * 32u;
    const uint32_t lt_mask = (1u << lane) - 1u;

    uint32_t k[ITEMS], v[ITEMS], r[ITEMS];
#pragma unroll
    for (int it = 0; it < ITEMS; it++) {
        const uint32_t idx = base + it * 32u + lane;
        const bool valid = idx < n;
        k[it] = valid ? keys_in[idx] : 0u;
        v[it] = valid ? (vals_in ? vals_in[idx] : idx) : 0u;
    }
#pragma unroll
    for (int it = 0; it < ITEMS; it++) {
        const uint32_t idx = base + it * 32u + lane;
        const bool valid = idx < n;
        const uint32_t d = valid ? ((k[it] >> shift) & mask) : (uint32_t)bins;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t pre = __popc(peers & lt_mask);
        uint32_t prev = 0u;
        if (valid) prev = s_whist[warp][d];
        __syncwarp();
        if (valid && pre == 0u) s_whist[warp][d] = prev + __popc(peers);
        __syncwarp();
        r[it] = prev + pre;
    }
    __syncthreads();
    uint32_t cnt = 0u;
    if (tid < bins) {
        uint32_t run = 0u;
#pragma unroll
        for (int w = 0; w < WARPS; w++) {
            const uint32_t c = s_whist[w][tid];
            s_whist[w][tid] = run;
            run += c;
        }
        cnt = run;
    }
    const uint32_t dstart = block_excl_scan256(cnt, s_scan);
    if (tid < bins) {
        s_dstart[tid] = dstart;
        uint32_t* st = status + (size_t)tile * bins + tid;
        uint32_t excl = 0u;
        if (tile == 0u) {
            st_volatile(st, kFlagPrefix | cnt);
        } else {
            st_volatile(st, kFlagAggregate | cnt);
            excl = lookback_exclusive(status, bins, tile, tid, kLookbackSpinLimit, err);
            st_volatile(st, kFlagPrefix | ((excl + cnt) & kCountMask));
        }
        s_gofs[tid] = gbase + excl;
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < ITEMS; it++) {
        const uint32_t idx = base + it * 32u + lane;
        if (idx < n) {
            const uint32_t d = (k[it] >> shift) & mask;
            const uint32_t lpos = s_dstart[d] + s_whist[warp][d] + r[it];
            s_keys[lpos] = k[it];
            s_vals[lpos] = v[it];
        }
    }
    __syncthreads();
    const uint32_t tile_base = tile * (uint32_t)TILE;
    const uint32_t tile_n = min((uint32_t)TILE, n - tile_base);
    for (uint32_t i = tid; i < tile_n; i += BLOCK) {
        const uint32_t kk = s_keys[i];
        const uint32_t d = (kk >> shift) & mask;
        const uint32_t g = s_gofs[d] + (i - s_dstart[d]);
        if (g < n) {  // always true unless a look-back timed out (error word set)
            keys_out[g] = kk;
            vals_out[g] = s_vals[i];
        }
    }
}

// First index in sorted keys[0, n) whose key is >= c (n when none).
__device__ __forceinline__ uint32_t lower_bound_keys(const uint32_t* __restrict__ keys, uint32_t n,
                                                    uint32_t c) {
    uint32_t lo = 0u, hi = n;
    while (lo < hi) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if (keys[mid] < c)
            lo = mid + 1u;
        else
            hi = mid;
    }
    return lo;
}


// Block b owns keys [256 b, 256 b + 256) of cell_scan (n + 1 entries: cell_scan[k] is the first
// sorted index with key >= k, so bucket k is [cell_scan[k], cell_scan[k + 1])) and gathers the
// particles with sorted indices in the same range. Two binary searches bound the block's slice
// of the sorted keys; each element of the slice writes the entries between its predecessor's key
// and its own, which never leave the block's range, so no thread loops over more than 256
// entries however the keys cluster.
// First index in sorted keys[0, n) whose key is >= c, searched from guess g: a gallop away from g
// (doubling steps) brackets the answer, a binary search finishes it. A few loads when g is close
// (the previous substep's answer), about twice the plain search's otherwise; exact for any g.
__device__ __forceinline__ uint32_t lower_bound_near(const uint32_t* __restrict__ keys, uint32_t n,
                                                    uint32_t c, uint32_t g) {
    g = min(g, n);
    uint32_t lo, hi;
    if (g < n && keys[g] < c) {  // the answer lies in (g, n]
        lo = g + 1u;
        hi = lo;
        uint32_t step = 1u;
        while (hi < n && keys[hi] < c) {
            lo = hi + 1u;
            hi = (n - hi > step) ? hi + step : n;
            step <<= 1;
        }
    } else {  // the answer lies in [0, g]
        hi = g;
        lo = g;
        uint32_t step = 1u;
        while (lo > 0u && keys[lo - 1u] >= c) {
            hi = lo - 1u;
            lo = lo > step ? lo - step : 0u;
            step <<= 1;
        }
    }
    // Now (lo == 0 or keys[lo - 1] < c) and (hi == n or keys[hi] >= c).
    while (lo < hi) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if (keys[mid] < c)
            lo = mid + 1u;
        else
            hi = mid;
    }
    return lo;
}

template <uint32_t kCellBlock>
__global__ void __launch_bounds__(kCellBlock)
    k_cells_reorder(StepLaunch L, uint32_t n, const uint32_t* __restrict__ skeys,
                    const uint32_t* __restrict__ perm, uint32_t* __restrict__ scan,
                    const float4* __restrict__ pos_in, const float4* __restrict__ vel_in,
                    float4* __restrict__ pos_out, float4* __restrict__ vel_out,
                    uint32_t* __restrict__ zero, uint32_t zero_words,
                    uint32_t* __restrict__ pkeys_out, uint32_t* guess,
                    const uint32_t* __restrict__ b_of_id, float4* __restrict__ xcur,
                    const float4* __restrict__ x_build, uint32_t* __restrict__ stale,
                    const uint32_t* __restrict__ ctl) {
    __shared__ uint32_t s_lo, s_hi;
    // The sort is done with its scratch (histograms, tile counters, look-back status): clear it
    // for the next substep here instead of in a separate memset.
    for (uint32_t w = blockIdx.x * kCellBlock + threadIdx.x; w < zero_words; w += gridDim.x * kCellBlock)
        zero[w] = 0u;
    const uint32_t c0 = blockIdx.x * kCellBlock;
    const uint32_t c1 = min(c0 + kCellBlock, n + 1u);
    const uint32_t tid = threadIdx.x;
    // The block's slice of the sorted keys, searched from the previous substep's bounds (cell
    // boundaries move little per substep). guess[b] is block b's lower bound; block b reads its
    // neighbour's entry while that block may be rewriting it, and either value is a valid guess.
    if (tid == 0) {
        s_lo = guess ? lower_bound_near(skeys, n, c0, ((volatile uint32_t*)guess)[blockIdx.x])
                     : lower_bound_keys(skeys, n, c0);
        if (guess) guess[blockIdx.x] = s_lo;
    }
    if (tid == 32)
        s_hi = guess ? lower_bound_near(skeys, n, c1, ((volatile uint32_t*)guess)[blockIdx.x + 1])
                     : lower_bound_keys(skeys, n, c1);
    const uint32_t i = c0 + tid;
    bool exceed = false;  // skin lists: the particle moved past h skin / 2 since its list build
    uint32_t exceed_sc = 0u;
    if (i < n) {
        uint32_t src = perm[i];
        if (src >= n) src = i;  // only after a reported sort failure
        const float4 x = __ldg(pos_in + src);
        pos_out[i] = x;
        if (!L.defer_vel) vel_out[i] = __ldg(vel_in + src);
        if (xcur) {
            const uint32_t sc = L.n_scenes > 1 ? (uint32_t)__ldg(L.scene_of + i) : 0u;
            exceed_sc = sc;
            if (ctl[sc * kSkinCtl + kCtlFresh] == 0u) {
                // No build yet, or the last build's lists have gone stale: they stay unusable
                // until the next build, so the scene is stale without a displacement check, and
                // nothing reads its positions by build index.
                exceed = true;
            } else {
                // Skin lists: the particle's current position and sorted index under its build
                // index (the list pass gathers both with one load), and its displacement since
                // the build.
                const uint32_t id = __float_as_uint(x.w);
                const uint32_t bi = id < n ? __ldg(b_of_id + id) : n;
                if (bi < n) {
                    xcur[bi] = make_float4(x.x, x.y, x.z, __uint_as_float(i));
                    const float4 b = __ldg(x_build + bi);
                    const float dx = x.x - b.x, dy = x.y - b.y, dz = x.z - b.z;
                    const float lim = L.n_scenes > 1 ? L.scenes[sc].skin_half2 : L.one.skin_half2;
                    exceed = !(dx * dx + dy * dy + dz * dz <= lim);
                }
            }
        }
        if (pkeys_out) pkeys_out[i] = skeys[i];
    }
    // Stale scenes, one atomic per warp and scene at most (most particles of a fast scene exceed).
    if (xcur) {
        const uint32_t m = __ballot_sync(0xffffffffu, exceed);
        if (exceed) {
            const uint32_t g = __match_any_sync(m, exceed_sc);
            if ((tid & 31u) == (uint32_t)(__ffs(g) - 1) && ld_volatile(stale + exceed_sc) == 0u)
                atomicOr(stale + exceed_sc, 1u);
        }
    }
    __syncthreads();
    const uint32_t lo = s_lo, hi = max(s_lo, s_hi);
    if (lo == hi) {
        for (uint32_t c = c0 + tid; c < c1; c += kCellBlock) scan[c] = lo;
        return;
    }
    // The clamps keep writes inside [c0, c1) even if the keys were not sorted.
    for (uint32_t j = lo + tid; j < hi; j += kCellBlock) {
        const uint32_t k = min(skeys[j], c1 - 1u);
        const uint32_t start = j == lo ? c0 : max(skeys[j - 1] + 1u, c0);
        for (uint32_t c = start; c <= k; c++) scan[c] = j;
    }
    const uint32_t last = max(min(skeys[hi - 1u], c1 - 1u) + 1u, c0);
    for (uint32_t c = last + tid; c < c1; c += kCellBlock) scan[c] = hi;
}

__global__ void __launch_bounds__(256)
    k_offsets(uint32_t n, uint32_t off, const uint32_t* __restrict__ scan,
              uint32_t* __restrict__ offsets) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t a = scan[off + k], b = scan[off + k + 1];
    offsets[k] = b > a ? a - off : n;
}

// ---------------------------------------------------------------- neighbour passes
// Two phases per particle. Phase A walks every candidate of the 27 buckets with a cheap,
// branch-free distance test and appends the in-range ones to a per-thread list in shared memory
// (slot-major, so a warp's lanes hit consecutive banks). Phase B runs the kernel math over the
// compacted list. Without the split a warp pays the in-range path for almost every candidate
// (only ~15% of candidates are within h, but one of 32 lanes nearly always is). The list keeps
// candidate order, so the sums are accumulated in the reference's visiting order. A list that
// fills up (dense regions) is drained early and refilled.

constexpr int kListCap = 48;
constexpr int kDrainAt = kListCap - 4;  // a batch of four never overflows the list

// Squared distance, in units of h^2, from a particle at fraction f of its cell (along one axis)
// to the neighbour cell at offset d in {-1, 0, +1} along that axis.
__device__ __forceinline__ float face_dist2(uint32_t d, float f) {
    const float l = d == 0xFFFFFFFFu ? f : (d == 1u ? 1.0f - f : 0.0f);
    const float c = fmaxf(l, 0.0f);
    return c * c;
}

// Cells whose box lies farther than h from the particle hold no in-range candidate and are
// skipped, which cannot change any sum as long as no other of the 27 neighbour cells shares
// their key (a shared key would be walked once more by the reference). The 27 keys are distinct
// when the 3x3x3 block of cells lies inside one 50^3 hash block and its hashes do not wrap past
// 2^32 (they are then hmin + d with distinct d in [0, 5102]) and n > 5102; elsewhere nothing is
// skipped. The 2e-3 margin keeps the float cell fractions conservative.
constexpr float kPruneLimit = 1.002f;

// True when the 27 neighbour cells of (cx, cy, cz) provably have 27 distinct keys (see above).
__device__ __forceinline__ bool distinct_keys(const SceneParams& p, uint32_t cx, uint32_t cy,
                                              uint32_t cz) {
    const uint32_t h_lo = hash_cell(cx - 1u, cy - 1u, cz - 1u);
    const uint32_t h_hi = hash_cell(cx + 1u, cy + 1u, cz + 1u);
    return p.n > 5102u && (cx + 24u) / 50u == (cx + 26u) / 50u &&
           (cy + 24u) / 50u == (cy + 26u) / 50u && (cz + 24u) / 50u == (cz + 26u) / 50u &&
           h_hi >= h_lo;
}

// Walks the candidates of the 27 neighbour buckets of cell (cx, cy, cz) in the reference's order
// and calls visit(j, q) for each, with q = pos[j]; four positions are fetched per iteration and
// batch_end() runs after each group of at most four (where a full list is drained).
// Rows t_begin..t_end-1 only, when given (t = (dy + 1) + 3 (dz + 1)).
template <typename Visit, typename BatchEnd>
__device__ __forceinline__ void for_each_candidate(const SceneParams& p,
                                                   const uint32_t* __restrict__ scan,
                                                   const float4* __restrict__ pos,
                                                   const float4& xi, uint32_t cx, uint32_t cy,
                                                   uint32_t cz, Visit&& visit,
                                                   BatchEnd&& batch_end, int t_begin = 0,
                                                   int t_end = 9) {
    const bool interior = distinct_keys(p, cx, cy, cz);
    const float lim = interior ? kPruneLimit : 1e30f;
    const float fx = fmaf(-(float)(int)cx, p.h, xi.x) * p.inv_h;
    const float fy = fmaf(-(float)(int)cy, p.h, xi.y) * p.inv_h;
    const float fz = fmaf(-(float)(int)cz, p.h, xi.z) * p.inv_h;
    const float dxl = face_dist2(0xFFFFFFFFu, fx), dxr = face_dist2(1u, fx);
#pragma unroll 1
    for (int t = t_begin; t < t_end; t++) {
        const uint32_t dy = (uint32_t)(t % 3) - 1u, dz = (uint32_t)(t / 3) - 1u;
        const float dyz = face_dist2(dy, fy) + face_dist2(dz, fz);
        if (dyz > lim) continue;
        const bool skip_l = dyz + dxl > lim, skip_r = dyz + dxr > lim;
        const uint32_t ry = cy + dy, rz = cz + dz;
        const uint32_t hA = hash_cell(cx - 1u, ry, rz);
        const uint32_t kA = key_mod(hA, p.mod_magic, p.n);
        uint32_t b0, e0, b1 = 0u, e1 = 0u, b2 = 0u, e2 = 0u;
        int nseg = 1;
        // Cells cx-1..cx+1 share a hash block iff (cell + 25) / 50 agrees at both ends (this also
        // covers the wrap of cell + 25 at 2^32 near cell -26).
        const bool same_block = (cx + 24u) / 50u == (cx + 26u) / 50u && hA <= 0xFFFFFFFDu;
        const uint32_t* sc = scan + p.off;  // the scene's keys are off + local key
        if (same_block && kA + 2u < p.n) {
            // Buckets kA, kA+1, kA+2 are adjacent: one range, trimmed at either end.
            b0 = __ldg(sc + kA + (skip_l ? 1u : 0u));
            e0 = __ldg(sc + kA + (skip_r ? 2u : 3u));
        } else {
            const uint32_t kB = key_mod(hash_cell(cx, ry, rz), p.mod_magic, p.n);
            const uint32_t kC = key_mod(hash_cell(cx + 1u, ry, rz), p.mod_magic, p.n);
            b0 = __ldg(sc + kA);
            e0 = skip_l ? b0 : __ldg(sc + kA + 1u);
            b1 = __ldg(sc + kB);
            e1 = __ldg(sc + kB + 1u);
            nseg = 3;
            if (!skip_r) {
                b2 = __ldg(sc + kC);
                e2 = __ldg(sc + kC + 1u);
            }
        }
#pragma unroll 1
        for (int seg = 0; seg < nseg; seg++) {
            const uint32_t b = seg == 0 ? b0 : (seg == 1 ? b1 : b2);
            const uint32_t e = seg == 0 ? e0 : (seg == 1 ? e1 : e2);
            uint32_t j = b;
            const float4* pp = pos + b;
#pragma unroll 1
            for (; j + 4u <= e; j += 4u, pp += 4) {
                const float4 q0 = __ldg(pp), q1 = __ldg(pp + 1);
                const float4 q2 = __ldg(pp + 2), q3 = __ldg(pp + 3);
                visit(j, q0);
                visit(j + 1u, q1);
                visit(j + 2u, q2);
                visit(j + 3u, q3);
                batch_end();
            }
#pragma unroll 1
            for (; j < e; j++, pp++) visit(j, __ldg(pp));
            batch_end();
        }
    }
}

// |x_j - x_i|^2 as the density pass's in-range tests evaluate it, explicitly rounded so that the
// bucket walk and the skin lists decide every pair the same way.
__device__ __forceinline__ float in_range2(const float4& xi, const float4& xj) {
    const float dx = __fsub_rn(xj.x, xi.x), dy = __fsub_rn(xj.y, xi.y), dz = __fsub_rn(xj.z, xi.z);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// Along one axis, how many of the cells c-2..c+2 share the 50-cell hash block of c-2 (5 when all
// do). Five consecutive cells span at most two blocks: the short block before the 2^32 wrap of
// cell + 25 is 46 cells long.
__device__ __forceinline__ int first_block_cells(uint32_t c) {
    const uint32_t b0 = (c - 2u + 25u) / 50u;
    int n = 1;
#pragma unroll
    for (int t = 1; t < 5; t++) n += (c - 2u + (uint32_t)t + 25u) / 50u == b0 ? 1 : 0;
    return n;
}

// Whether box a (keys (ka + x + 50 y + 2500 z) mod n for x, y, z below its widths wa) and box b
// (keys from kb, widths wb) share a key: each key of a, minus kb modulo n, is one of b's offsets
// exactly when its digits in base 50 / 2500 lie below b's widths (every offset is < 5 + 50 * 5 +
// 2500 * 5 < n, so the decomposition is unique). Kept out of line: it runs for few particles, and
// inlined into the walk kernel it cost the 1M scene's list-building substep half again (density
// 0.94 ms against 0.60, same rule, same decisions).
__device__ __noinline__ bool boxes_share_a_key(uint32_t ka, uint32_t wax, uint32_t way, uint32_t waz,
                                               uint32_t kb, uint32_t wbx, uint32_t wby, uint32_t wbz,
                                               uint32_t n) {
#pragma unroll 1
    for (uint32_t z = 0; z < waz; z++)
#pragma unroll 1
        for (uint32_t y = 0; y < way; y++)
#pragma unroll 1
            for (uint32_t x = 0; x < wax; x++) {
                uint32_t key = ka + x + 50u * y + 2500u * z;
                if (key >= n) key -= n;  // ka < n and the offset is below n
                const uint32_t d = key >= kb ? key - kb : key + (n - kb);
                const uint32_t oz = d / 2500u, r = d - 2500u * oz, oy = r / 50u, ox = r - 50u * oy;
                if (ox < wbx && oy < wby && oz < wbz) return true;
            }
    return false;
}

// Box `slot` of the 5 x 5 x 5 block around (cx, cy, cz): bit 0 (1, 2) of the slot picks the
// cells of the block's first or second 50-cell hash block along x (y, z). Returns false when the
// slot is not a box of this block (the block lies in one hash block along that axis); otherwise
// its first key k, the span of its hashes (its last minus its first) and its widths, or wraps =
// true when its hashes wrap 2^32. Computed from the slot alone, so no per-box array is kept.
__device__ __forceinline__ bool key_box(const SceneParams& p, uint32_t cx, uint32_t cy, uint32_t cz,
                                        uint32_t fx, uint32_t fy, uint32_t fz, uint32_t slot,
                                        uint32_t& k, uint32_t& span, uint32_t w[3], bool& wraps) {
    const bool bx = slot & 1u, by = slot & 2u, bz = slot & 4u;
    if ((bx && fx == 5u) || (by && fy == 5u) || (bz && fz == 5u)) return false;
    const uint32_t x0 = bx ? fx : 0u, x1 = bx ? 4u : fx - 1u;
    const uint32_t y0 = by ? fy : 0u, y1 = by ? 4u : fy - 1u;
    const uint32_t z0 = bz ? fz : 0u, z1 = bz ? 4u : fz - 1u;
    const uint32_t lo = hash_cell(cx - 2u + x0, cy - 2u + y0, cz - 2u + z0);
    const uint32_t hi = hash_cell(cx - 2u + x1, cy - 2u + y1, cz - 2u + z1);
    wraps = hi < lo;
    k = key_mod(lo, p.mod_magic, p.n);
    span = hi - lo;
    w[0] = x1 - x0 + 1u;
    w[1] = y1 - y0 + 1u;
    w[2] = z1 - z0 + 1u;
    return true;
}

// True when the 125 cells around (cx, cy, cz) have distinct keys, so that a walk of their buckets
// meets every particle once. The block splits into at most eight boxes, one per hash block it
// touches; inside a box the hashes are hmin + lx + 50 ly + 2500 lz, so its keys lie in the
// circular interval [hmin mod n, hmin mod n + span] (span <= 10204) and are distinct when
// n > 10204 and the box's hashes do not wrap 2^32. Boxes whose intervals are disjoint modulo n
// share no key; boxes whose intervals overlap are compared key by key (boxes_share_a_key), so
// the answer is exact under those two conditions. Most blocks lie in one hash block (one box, no
// pair to compare); the boxes of a pair are recomputed from their slots rather than kept in a
// per-thread array, which would live in local memory.
__device__ __forceinline__ bool skin_keys_distinct(const SceneParams& p, uint32_t cx, uint32_t cy,
                                                   uint32_t cz) {
    if (p.n <= 10204u) return false;
    const uint32_t fx = (uint32_t)first_block_cells(cx), fy = (uint32_t)first_block_cells(cy),
                   fz = (uint32_t)first_block_cells(cz);
    uint32_t ka, sa, wa[3], kb, sb, wb[3];
    bool wraps;
#pragma unroll 1
    for (uint32_t a = 0; a < 8u; a++) {
        if (!key_box(p, cx, cy, cz, fx, fy, fz, a, ka, sa, wa, wraps)) continue;
        if (wraps) return false;
#pragma unroll 1
        for (uint32_t b = 0; b < a; b++) {
            if (!key_box(p, cx, cy, cz, fx, fy, fz, b, kb, sb, wb, wraps)) continue;
            const uint32_t ab = kb >= ka ? kb - ka : kb + (p.n - ka);  // (k_b - k_a) mod n
            const uint32_t ba = ka >= kb ? ka - kb : ka + (p.n - kb);
            if ((ab <= sa || ba <= sb) &&
                boxes_share_a_key(ka, wa[0], wa[1], wa[2], kb, wb[0], wb[1], wb[2], p.n))
                return false;
        }
    }
    return true;
}

// Squared distance, in h^2, from a particle at fraction f of its cell to the slab of cells at
// offset d in [-2, 2] along one axis.
__device__ __forceinline__ float slab_dist2(int d, float f) {
    const float l = d < 0 ? f + (float)(-d - 1) : (d > 0 ? (float)d - f : 0.0f);
    const float c = fmaxf(l, 0.0f);
    return c * c;
}

// The list build of a particle whose 125 keys are distinct: the sorted indices (this substep's,
// which become the build indices) of every particle within h (1 + skin), stored at out[k stride],
// from the 5x5x5 cells around (cx, cy, cz) whose boxes lie within that radius: planes dz and
// rows dy in increasing order, the cells of a row in increasing x as runs of consecutive keys (a
// run ends at a hash-block boundary; a run whose keys pass n - 1 continues at key 0) - the
// reference's visiting order restricted to its 27 cells. Returns the number found (ids past
// `cap` are not stored).
__device__ __forceinline__ uint32_t skin_walk(const SceneParams& p, const uint32_t* __restrict__ scan,
                                              const float4* __restrict__ pos, const float4& xi,
                                              uint32_t cx, uint32_t cy, uint32_t cz,
                                              uint32_t* __restrict__ out, size_t stride,
                                              uint32_t cap) {
    const float fx = fmaf(-(float)(int)cx, p.h, xi.x) * p.inv_h;
    const float fy = fmaf(-(float)(int)cy, p.h, xi.y) * p.inv_h;
    const float fz = fmaf(-(float)(int)cz, p.h, xi.z) * p.inv_h;
    const float lim = p.skin_lim;
    const uint32_t* sc = scan + p.off;
    uint32_t c = 0;
    auto walk = [&](uint32_t b, uint32_t e) {
#pragma unroll 1
        for (uint32_t j = b; j < e; j++) {
            const float4 xj = __ldg(pos + j);
            if (in_range2(xi, xj) <= p.skin_r2) {
                if (c < cap) out[c * stride] = j;
                c++;
            }
        }
    };
#pragma unroll 1
    for (int dz = -2; dz <= 2; dz++) {
        const float sz = slab_dist2(dz, fz);
        if (sz > lim) continue;
#pragma unroll 1
        for (int dy = -2; dy <= 2; dy++) {
            const float syz = sz + slab_dist2(dy, fy);
            if (syz > lim) continue;
            int xl = -2, xr = 2;  // cell 0 is always within the limit here
            while (xl < 0 && syz + slab_dist2(xl, fx) > lim) xl++;
            while (xr > 0 && syz + slab_dist2(xr, fx) > lim) xr--;
            const uint32_t ry = cy + (uint32_t)dy, rz = cz + (uint32_t)dz;
#pragma unroll 1
            for (int x = xl; x <= xr;) {
                const uint32_t bx = (cx + (uint32_t)x + 25u) / 50u;
                int xe = x;
                while (xe < xr && (cx + (uint32_t)(xe + 1) + 25u) / 50u == bx) xe++;
                const uint32_t k0 = key_mod(hash_cell(cx + (uint32_t)x, ry, rz), p.mod_magic, p.n);
                const uint32_t len = (uint32_t)(xe - x + 1);
                if (k0 + len <= p.n) {
                    walk(__ldg(sc + k0), __ldg(sc + k0 + len));
                } else {
                    walk(__ldg(sc + k0), __ldg(sc + p.n));
                    walk(__ldg(sc), __ldg(sc + (k0 + len - p.n)));
                }
                x = xe + 1;
            }
        }
    }
    return c;
}

// Threads per block of the density pass over the skin lists; the walk queue is kept in segments of
// one such block.
constexpr int kListBlock = 128;

// Particle i's density sum and neighbour list as the density pass builds them: add() takes one
// in-range neighbour, adds its W / sigma (explicitly rounded, so every launch shape and both the
// bucket walk and the skin lists give the same sums) and appends j to the list unless j == i.
struct DensitySum {
    float rho = 0.0f;
    uint32_t listed = 0;
    uint32_t* out;  // slot `listed` of i's list (slot-major, stride = particles)
    __device__ __forceinline__ void add(uint32_t i, const float4& xi, uint32_t j, const float4& xj,
                                        float inv_h, uint32_t cap, uint32_t stride) {
        add_r2(i, j, in_range2(xi, xj), inv_h, cap, stride);
    }
    // The same with r2 = in_range2(x_i, x_j) already computed (by the in-range test).
    __device__ __forceinline__ void add_r2(uint32_t i, uint32_t j, float r2, float inv_h,
                                           uint32_t cap, uint32_t stride) {
        const float r = r2 > 0.0f ? __fmul_rn(r2, rsqrtf(r2)) : 0.0f;
        // W(q) / sigma, branch-free: 2 (1-q)^3 above q = 1/2, 6q^3 - 6q^2 + 1 below, 0 past 1.
        const float q = __fmul_rn(r, inv_h);
        const float t = __fsub_rn(1.0f, q);
        const float w_out = __fmul_rn(__fmul_rn(__fmul_rn(t, t), t), 2.0f);
        const float q2 = __fmul_rn(q, q);
        const float w_in = __fmaf_rn(6.0f, __fmul_rn(q2, q), __fmaf_rn(-6.0f, q2, 1.0f));
        const float w = q <= 1.0f ? (q > 0.5f ? w_out : w_in) : 0.0f;
        rho = __fadd_rn(rho, w);
        if (j != i) {
            if (listed < cap) {
                *out = j;
                out += stride;
            }
            listed++;
        }
    }
};

// The per-particle end of the density pass: list length word, boundary terms, density, Tait EOS
// and the force pass's record of i.
__device__ __forceinline__ void density_finish(const SceneParams& p, uint32_t i, const float4& xi,
                                               const float4* __restrict__ vel, uint32_t cx,
                                               uint32_t cy, uint32_t cz, bool distinct,
                                               const DensitySum& d, float4* __restrict__ rec,
                                               float4* __restrict__ aux, float4* __restrict__ bnd,
                                               uint32_t* __restrict__ nbr_count,
                                               float* __restrict__ host_dens, bool defer_vel) {
    nbr_count[i] = nbr_word(d.listed, cx, cy, cz, distinct);
    float bd, bgx, bgy, bgz;
    boundary_terms(p, xi.x, xi.y, xi.z, bd, bgx, bgy, bgz);
    const float rho = p.mass * p.cubic * d.rho + p.rho0 * bd;  // the factor the sum leaves out
    const float pr = p.stiffness * (powf(fmaxf(rho, p.rho0) / p.rho0, p.expoent) - 1.0f);
    const float pd = rho > 0.0f ? pr / (rho * rho) : 0.0f;
    const float mr = p.mass / fmaxf(rho, 1e-6f);
    const float pb = rho > 0.0f ? pr / (p.rho0 * p.rho0) : 0.0f;
    aux[i] = make_float4(pd, mr, rho, pb);
    if (host_dens) host_dens[i] = rho;
    // The force pass's neighbour record of i: one 32-byte sector per gathered neighbour (the
    // velocity half later, from launch_vel_records, when the velocities arrive late).
    rec[2 * (size_t)i] = make_float4(xi.x, xi.y, xi.z, pd);
    if (!defer_vel) {
        const float4 vi = __ldg(vel + i);
        rec[2 * (size_t)i + 1] = make_float4(vi.x, vi.y, vi.z, mr);
    }
    bnd[i] = make_float4(bgx, bgy, bgz, bd);
}

// Block-per-cell staging of the neighbourhood, one warp at a time: when a warp's particles share
// one row of cells (same scene, same y and z cells, at most four consecutive x cells) and the
// 3 x 3 rows of cells around them (x from the first cell - 1 to the last + 1) lie in one 50^3 hash
// block whose keys do not wrap, every row of that union is one run of consecutive keys, hence one
// contiguous range of the sorted particles, and all of the union's keys are distinct (n > 5110:
// the union's hashes span at most 5105). The warp then stages each row's particles in shared
// memory 32 at a time and every lane tests all of them against its particle. Every in-range
// candidate of a particle lies in its own 27 cells, each of its 27 buckets is met once (distinct
// keys), and rows and candidates are met in the reference's visiting order, so the in-range
// sequence and hence the sum are exactly the bucket walk's. Returns false when the warp does not
// qualify; otherwise the union's first x cell's row keys start at index key_lo of the cell scan
// (the leader's scene offset included) and each row spans `width` keys. Warp-uniform: every test
// reads the leader's scene (an idle lane of a batched launch holds a slot of another scene), so
// all 32 lanes take the same branch and stage the same rows.
__device__ __forceinline__ bool warp_row_union(const SceneParams& p, bool act, bool ok, uint32_t cx,
                                               uint32_t cy, uint32_t cz, uint32_t sc,
                                               uint32_t& key_lo, uint32_t& width) {
    const uint32_t am = __ballot_sync(0xffffffffu, act);
    const int leader = __ffs(am) - 1;
    const uint32_t cy0 = __shfl_sync(0xffffffffu, cy, leader);
    const uint32_t cz0 = __shfl_sync(0xffffffffu, cz, leader);
    const uint32_t sc0 = __shfl_sync(0xffffffffu, sc, leader);
    const uint32_t n0 = __shfl_sync(0xffffffffu, p.n, leader);
    const uint32_t off0 = __shfl_sync(0xffffffffu, p.off, leader);
    const unsigned long long magic0 =
        __shfl_sync(0xffffffffu, (unsigned long long)p.mod_magic, leader);
    int lo = act ? (int)cx : INT_MAX, hi = act ? (int)cx : INT_MIN;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    const bool same = !act || (ok && cy == cy0 && cz == cz0 && sc == sc0);
    if (!__all_sync(0xffffffffu, same)) return false;
    if ((int64_t)hi - (int64_t)lo > 3 || n0 <= 5110u) return false;
    const uint32_t c0 = (uint32_t)lo - 1u, c1 = (uint32_t)hi + 1u;
    if ((c0 + 25u) / 50u != (c1 + 25u) / 50u || (cy0 + 24u) / 50u != (cy0 + 26u) / 50u ||
        (cz0 + 24u) / 50u != (cz0 + 26u) / 50u)
        return false;
    const uint32_t h_lo = hash_cell(c0, cy0 - 1u, cz0 - 1u);
    const uint32_t h_hi = hash_cell(c1, cy0 + 1u, cz0 + 1u);
    if (h_hi < h_lo) return false;  // the block's hashes wrap past 2^32
    const uint32_t k_lo = key_mod(h_lo, (uint64_t)magic0, n0);
    if ((uint64_t)k_lo + (h_hi - h_lo) >= n0) return false;  // keys wrap past n - 1
    key_lo = off0 + k_lo;
    width = c1 - c0 + 1u;
    return true;
}

// CalculateBoundaryVolume + CalculateDensities + the per-particle part of PressureFromDensityEOS
// (wcsph_with_boundary_model.slang:102-203), by the bucket walk. Besides the density products it
// writes particle i's neighbour list: every in-range j except i itself, in visiting order,
// slot-major (nbr[s * n + i], so a warp's lanes store and later load consecutive words), and its
// length in nbr_count[i] (a length above nbr_cap means the list overflowed and was truncated).
// Positions do not change before the force pass, so that list is exactly the force pass's
// neighbour set. Without skin lists every particle is walked, one per thread. With them, a
// batch's walkers are the queue k_density_list leaves (each list block's walkers in index order,
// so a stale scene is walked in index order); a single scene is walked here only when it is stale
// or its lists are mostly unusable (in index order; otherwise k_density_walkers takes its few
// walkers and this launch returns at its top). In a stale scene whose build policy allows it,
// every particle also builds its skin list. The launch is one resident wave whose warps claim
// runs of 32 slots. A warp whose particles share a row of cells walks the staged rows of
// warp_row_union; any other warp walks per thread (for_each_candidate).
template <bool kBatch, int kNbrBlock, int kMinBlocks, bool kStaging>
__global__ void __launch_bounds__(kNbrBlock, kMinBlocks)
    k_density(StepLaunch L, const float4* __restrict__ pos, const float4* __restrict__ vel,
              float4* __restrict__ rec, const uint32_t* __restrict__ scan,
              float4* __restrict__ aux, float4* __restrict__ bnd, uint32_t* __restrict__ nbr,
              uint32_t* __restrict__ nbr_count, SkinLists sk, uint32_t* __restrict__ sched) {
    static_assert(kSkinCap <= (uint32_t)kListCap, "a list build is staged in the shared list");
    static_assert(kNbrBlock % 32 == 0, "whole warps");
    static_assert(kListBlock % 32 == 0, "a warp's 32 slots lie in one list block");
    __shared__ uint32_t s_j[kListCap * kNbrBlock];
    // Each warp's 32 staged candidates (one placeholder element without staging, so that the
    // shared memory the per-thread walk does not use stays L1 for its candidate loads).
    __shared__ float4 s_stage[kStaging ? kNbrBlock : 1];
    const int tid = threadIdx.x;
    const uint32_t lane = (uint32_t)(tid & 31);
    // A single scene whose lists are current and mostly usable: k_density_list and
    // k_density_walkers cover every particle, and the whole launch returns here.
    if (!kBatch && sk.list && sk.stale[0] == 0u && sk.ctl[kCtlPoor] == 0u) return;
    // Every warp takes runs of 32 slots: first the run of its own index, then runs claimed from
    // the launch's counter (sched[0]), until none is left. Walks differ widely in length (the
    // queued walkers of a batch, the list builds of a stale scene), and a warp that finishes early
    // takes the next run. No lane leaves a run before the warp's collective steps: inactive lanes
    // carry act = false.
    const uint32_t runs = (L.total + 31u) / 32u;
    const uint32_t warps = gridDim.x * (uint32_t)(kNbrBlock / 32);
    uint32_t run = blockIdx.x * (uint32_t)(kNbrBlock / 32) + (uint32_t)(tid >> 5);
    for (; run < runs;) {
        const uint32_t t = run * 32u + lane;
        bool act = t < L.total;
        uint32_t i = act ? t : 0u, sc = 0u;
        bool rebuild = false;
        if (act && sk.list) {
            if (kBatch) {
                // Slot t of the queue: valid below its list block's count of walkers.
                if (t % kListBlock >= __ldg(sk.seg_n + t / kListBlock)) {
                    act = false;
                } else {
                    i = __ldg(sk.queue + t);
                    sc = (uint32_t)__ldg(L.scene_of + i);
                }
            } else if (sk.stale[0] == 0u && sk.ctl[kCtlPoor] == 0u) {
                act = false;  // k_density_walkers walks the single scene's queued particles
            }  // else a single scene that is stale or whose lists are mostly unusable: every
               // particle, in index order (no queue)
            rebuild = act && sk.stale[sc] != 0u && sk.ctl[sc * kSkinCtl + kCtlAllow] != 0u;
        }
        // The next run, claimed now so that the counter's latency hides behind this one.
        uint32_t next = 0u;
        if (lane == 0u) next = warps + atomicAdd(sched, 1u);
        next = __shfl_sync(0xffffffffu, next, 0);
        if (__ballot_sync(0xffffffffu, act) == 0u) {  // the whole warp is idle
            run = next;
            continue;
        }
        const SceneParams& p = scene_params<kBatch>(L, i);
        const float4 xi = act ? __ldg(pos + i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const uint32_t cx = cell_coord(xi.x, p.h), cy = cell_coord(xi.y, p.h), cz = cell_coord(xi.z, p.h);
        DensitySum d;
        d.out = nbr + i;
        uint32_t s_end = tid;  // shared-memory word one past the last kept candidate (stride kNbrBlock)
        // Scene constants used per candidate, in registers (a batched launch reads its scene's
        // parameters from a device table).
        const float s_inv_h = p.inv_h;
        const uint32_t s_nbr_cap = p.nbr_cap;
        auto drain = [&]() {
#pragma unroll 2
            for (uint32_t o = tid; o < s_end; o += kNbrBlock) {
                const uint32_t j = s_j[o];
                d.add(i, xi, j, __ldg(pos + j), s_inv_h, s_nbr_cap, L.total);
            }
            s_end = tid;
        };
        const bool distinct = distinct_keys(p, cx, cy, cz);
        const float h2 = p.h2;
        uint32_t c = 0;
        bool usable = false;
        uint32_t key_lo = 0u, width = 0u;
        if (kStaging && warp_row_union(p, act, !rebuild, cx, cy, cz, sc, key_lo, width)) {
            // The staged walk: branch-free append as below, candidates read from shared memory.
            // key_lo indexes the cell scan directly (the warp's scene offset included).
            float4* stage = s_stage + (tid & ~31);
#pragma unroll 1
            for (uint32_t r = 0; r < 9u; r++) {
                const uint32_t kA = key_lo + 50u * (r % 3u) + 2500u * (r / 3u);
                const uint32_t b = __ldg(scan + kA), e = __ldg(scan + kA + width);
#pragma unroll 1
                for (uint32_t jb = b; jb < e; jb += 32u) {
                    const uint32_t jl = jb + lane;
                    if (jl < e) stage[lane] = __ldg(pos + jl);
                    __syncwarp();
                    const uint32_t cnt = min(32u, e - jb);
#pragma unroll 4
                    for (uint32_t k = 0; k < cnt; k++) {
                        const float4 xj = stage[k];
                        s_j[s_end] = jb + k;
                        s_end += act && in_range2(xi, xj) <= h2 ? kNbrBlock : 0u;
                        if ((k & 3u) == 3u && s_end > tid + kDrainAt * kNbrBlock) drain();
                    }
                    if (s_end > tid + kDrainAt * kNbrBlock) drain();
                    __syncwarp();  // the next chunk overwrites the stage
                }
            }
            drain();
        } else if (act) {
            if (rebuild && skin_keys_distinct(p, cx, cy, cz)) {
                // A list build, staged in this thread's column of the shared list.
                c = skin_walk(p, scan, pos, xi, cx, cy, cz, s_j + tid, (size_t)kNbrBlock, sk.cap);
                usable = c <= sk.cap;
            }
            if (usable) {
                // The density from the staged list (its in-range members, in the visiting order),
                // then the list written out a slot at a time (a warp's lanes store consecutive words).
#pragma unroll 1
                for (uint32_t k = 0; k < c; k++) {
                    const uint32_t j = s_j[k * kNbrBlock + tid];
                    const float r2 = in_range2(xi, __ldg(pos + j));
                    if (r2 <= h2) d.add_r2(i, j, r2, s_inv_h, s_nbr_cap, L.total);
                }
#pragma unroll 1
                for (uint32_t k = 0; k < c; k++) sk.list[(size_t)k * L.total + i] = s_j[k * kNbrBlock + tid];
            } else {
                // Branch-free append: every candidate is stored at the list's end and kept only when
                // in range (the next one overwrites it otherwise). Lists are drained above kDrainAt,
                // so the slot index stays below kListCap.
                for_each_candidate(p, scan, pos, xi, cx, cy, cz, [&](uint32_t j, const float4& xj) {
                    s_j[s_end] = j;
                    s_end += in_range2(xi, xj) <= h2 ? kNbrBlock : 0u;
                }, [&]() {
                    if (s_end > tid + kDrainAt * kNbrBlock) drain();
                });
                drain();
            }
        }
        run = next;
        if (!act) continue;
        if (rebuild) {
            // This substep's sorted index becomes the particle's build index.
            sk.x_build[i] = xi;
            sk.b_of_id[__float_as_uint(xi.w)] = i;
            sk.count[i] = min(c, sk.cap) | (usable ? kSkinUsable : 0u);
            // The scene's usable lists, one atomic per warp and scene.
            const uint32_t g = __match_any_sync(__activemask(), sc);
            const uint32_t u = __ballot_sync(g, usable);
            if ((uint32_t)(tid & 31) == (uint32_t)(__ffs(g) - 1) && u)
                atomicAdd(sk.ctl + sc * kSkinCtl + kCtlUsable, (uint32_t)__popc(u));
        }
        density_finish(p, i, xi, vel, cx, cy, cz, distinct, d, rec, aux, bnd, nbr_count, L.host_dens,
                       L.defer_vel);
    }
    // The last warp out puts the counter back to zero for the next launch (every other warp has
    // made its last claim before it counts itself out).
    if (lane == 0u) {
        __threadfence();
        if (atomicAdd(sched + 1, 1u) == warps - 1u) {
            atomicExch(sched, 0u);
            atomicExch(sched + 1, 0u);
        }
    }
}

// The density pass over the skin lists: a particle of a scene that is not stale, whose list is
// usable, sums the in-range members of its list (the same in-range set as the walk: every
// pair within h was within h (1 + skin) at the build; each once: the particle has moved less than
// h / 4 since the build, so its 27 cells lie in the build's 5x5x5 block, whose keys were
// distinct), in the list's order. Every other particle goes to the queue for k_density.
// No shared memory: the pass is bound by its chains of dependent loads, so it runs at the
// occupancy its registers allow.
template <bool kBatch>
__global__ void __launch_bounds__(kListBlock, 10)
    k_density_list(StepLaunch L, const float4* __restrict__ pos, const float4* __restrict__ vel,
                   float4* __restrict__ rec, float4* __restrict__ aux, float4* __restrict__ bnd,
                   uint32_t* __restrict__ nbr, uint32_t* __restrict__ nbr_count, SkinLists sk) {
    const uint32_t i = blockIdx.x * kListBlock + threadIdx.x;
    // A single scene that is stale, or whose last build left most lists unusable: k_density walks
    // it in index order.
    if (!kBatch && (sk.stale[0] != 0u || sk.ctl[kCtlPoor] != 0u)) return;
    bool walk = false;
    if (i < L.total) {
        const SceneParams& p = scene_params<kBatch>(L, i);
        uint32_t c = 0u, row = 0u;
        walk = sk.stale[kBatch ? (uint32_t)__ldg(L.scene_of + i) : 0u] != 0u;
        // A particle of a stale scene only joins the queue: its position is not read.
        const float4 xi = walk ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : __ldg(pos + i);
        if (!walk) {
            row = __ldg(sk.b_of_id + __float_as_uint(xi.w));
            c = __ldg(sk.count + row);
            walk = (c & kSkinUsable) == 0u;
        }
        if (!walk) {
            const uint32_t cx = cell_coord(xi.x, p.h), cy = cell_coord(xi.y, p.h),
                           cz = cell_coord(xi.z, p.h);
            const uint32_t n_list = c & ~kSkinUsable;
            const float h2 = p.h2, s_inv_h = p.inv_h;
            const uint32_t s_nbr_cap = p.nbr_cap;
            DensitySum d;
            d.out = nbr + i;
            const size_t stride = L.total;
            const uint32_t* q = sk.list + row;
            uint32_t k = 0;
            // The next batch's build indices load while the current batch is resolved and summed.
            uint32_t jn[4];
            if (n_list >= 4u) {
#pragma unroll
                for (int u = 0; u < 4; u++) jn[u] = __ldg(q + u * stride);
            }
#pragma unroll 1
            for (; k + 4u <= n_list; k += 4u, q += 4 * stride) {
                uint32_t j[4];
                float4 xj[4];
#pragma unroll
                for (int u = 0; u < 4; u++) j[u] = jn[u];
                if (k + 8u <= n_list) {
#pragma unroll
                    for (int u = 0; u < 4; u++) jn[u] = __ldg(q + (4 + u) * stride);
                }
#pragma unroll
                for (int u = 0; u < 4; u++) xj[u] = __ldg(sk.xcur + j[u]);  // position, sorted index
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const float r2 = in_range2(xi, xj[u]);
                    if (r2 <= h2) d.add_r2(i, __float_as_uint(xj[u].w), r2, s_inv_h, s_nbr_cap, L.total);
                }
            }
#pragma unroll 1
            for (; k < n_list; k++, q += stride) {
                const float4 xj = __ldg(sk.xcur + __ldg(q));
                const float r2 = in_range2(xi, xj);
                if (r2 <= h2) d.add_r2(i, __float_as_uint(xj.w), r2, s_inv_h, s_nbr_cap, L.total);
            }
            density_finish(p, i, xi, vel, cx, cy, cz, distinct_keys(p, cx, cy, cz), d, rec, aux,
                           bnd, nbr_count, L.host_dens, L.defer_vel);
        }
    }
    // The walkers go to the queue in index order within the block: batched, to this block's
    // segment (k_density takes slot t below its segment's count); a single scene, packed from 0
    // in blocks claimed by one atomic each (k_density_walkers takes one walker per warp).
    __shared__ uint32_t s_cnt[kListBlock / 32];
    __shared__ uint32_t s_base;
    const uint32_t m = __ballot_sync(0xffffffffu, walk);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_cnt[warp] = (uint32_t)__popc(m);
    __syncthreads();
    uint32_t base = 0u, total = 0u;
#pragma unroll
    for (int w = 0; w < kListBlock / 32; w++) {
        base += w < warp ? s_cnt[w] : 0u;
        total += s_cnt[w];
    }
    if (kBatch) {
        base += blockIdx.x * kListBlock;
        if (threadIdx.x == 0) sk.seg_n[blockIdx.x] = total;
    } else {
        if (threadIdx.x == 0) s_base = total ? atomicAdd(sk.wcount, total) : 0u;
        __syncthreads();
        base += s_base;  // at most L.total walkers in all: the slots stay inside the queue
    }
    if (walk) sk.queue[base + (uint32_t)__popc(m & ((1u << lane) - 1u))] = i;
}

// W(|x_j - x_i|) / sigma with the density drain's explicitly rounded arithmetic, from
// r2 = in_range2(x_i, x_j).
__device__ __forceinline__ float w_over_sigma_r2(float r2, float inv_h) {
    const float r = r2 > 0.0f ? __fmul_rn(r2, rsqrtf(r2)) : 0.0f;
    const float q = __fmul_rn(r, inv_h);
    const float t = __fsub_rn(1.0f, q);
    const float w_out = __fmul_rn(__fmul_rn(__fmul_rn(t, t), t), 2.0f);
    const float q2 = __fmul_rn(q, q);
    const float w_in = __fmaf_rn(6.0f, __fmul_rn(q2, q), __fmaf_rn(-6.0f, q2, 1.0f));
    return q <= 1.0f ? (q > 0.5f ? w_out : w_in) : 0.0f;
}

// Warps per block of k_density_walkers.
constexpr int kWalkerWarps = 4;

// The density pass of a single scene's walkers (the particles k_density_list queued: no usable
// list this substep), one warp per walker, so a walker's ~280 candidates are tested 32 at a time
// instead of in one thread's chain of dependent loads. Lane r < 27 holds candidate segment r of
// the walk (row r / 3, part r % 3 of the rows of for_each_candidate: the same buckets, the same
// pruning), the segments' candidates are numbered in visiting order and taken in chunks of 32,
// and the in-range ones are summed in visiting order (every lane adds them one by one through
// shuffles) and listed in visiting order: exactly the sum and the list of the one-thread walk.
__global__ void __launch_bounds__(kWalkerWarps * 32)
    k_density_walkers(StepLaunch L, const float4* __restrict__ pos, const float4* __restrict__ vel,
                      float4* __restrict__ rec, const uint32_t* __restrict__ scan,
                      float4* __restrict__ aux, float4* __restrict__ bnd, uint32_t* __restrict__ nbr,
                      uint32_t* __restrict__ nbr_count, SkinLists sk) {
    if (sk.stale[0] != 0u || sk.ctl[kCtlPoor] != 0u) return;  // k_density walks every particle
    const uint32_t walkers = min(*sk.wcount, L.total);
    const int lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    const SceneParams& p = L.one;
    const uint32_t* sc = scan + p.off;
    for (uint32_t w = blockIdx.x * kWalkerWarps + (threadIdx.x >> 5); w < walkers;
         w += gridDim.x * kWalkerWarps) {
        const uint32_t i = __ldg(sk.queue + w);
        const float4 xi = __ldg(pos + i);
        const uint32_t cx = cell_coord(xi.x, p.h), cy = cell_coord(xi.y, p.h),
                       cz = cell_coord(xi.z, p.h);
        const bool distinct = distinct_keys(p, cx, cy, cz);
        // Segment r of the walk: [b, b + len).
        uint32_t b = 0u, len = 0u;
        if (lane < 27) {
            const float lim = distinct ? kPruneLimit : 1e30f;
            const float fx = fmaf(-(float)(int)cx, p.h, xi.x) * p.inv_h;
            const float fy = fmaf(-(float)(int)cy, p.h, xi.y) * p.inv_h;
            const float fz = fmaf(-(float)(int)cz, p.h, xi.z) * p.inv_h;
            const int t = lane / 3, part = lane % 3;
            const uint32_t dy = (uint32_t)(t % 3) - 1u, dz = (uint32_t)(t / 3) - 1u;
            const float dyz = face_dist2(dy, fy) + face_dist2(dz, fz);
            if (dyz <= lim) {
                const bool skip_l = dyz + face_dist2(0xFFFFFFFFu, fx) > lim;
                const bool skip_r = dyz + face_dist2(1u, fx) > lim;
                const uint32_t ry = cy + dy, rz = cz + dz;
                const uint32_t hA = hash_cell(cx - 1u, ry, rz);
                const uint32_t kA = key_mod(hA, p.mod_magic, p.n);
                const bool same_block = (cx + 24u) / 50u == (cx + 26u) / 50u && hA <= 0xFFFFFFFDu;
                uint32_t e = 0u;
                if (same_block && kA + 2u < p.n) {
                    if (part == 0) {
                        b = __ldg(sc + kA + (skip_l ? 1u : 0u));
                        e = __ldg(sc + kA + (skip_r ? 2u : 3u));
                    }
                } else if (part == 0) {
                    b = __ldg(sc + kA);
                    e = skip_l ? b : __ldg(sc + kA + 1u);
                } else if (part == 1) {
                    const uint32_t kB = key_mod(hash_cell(cx, ry, rz), p.mod_magic, p.n);
                    b = __ldg(sc + kB);
                    e = __ldg(sc + kB + 1u);
                } else if (!skip_r) {
                    const uint32_t kC = key_mod(hash_cell(cx + 1u, ry, rz), p.mod_magic, p.n);
                    b = __ldg(sc + kC);
                    e = __ldg(sc + kC + 1u);
                }
                len = e > b ? e - b : 0u;
            }
        }
        // Exclusive prefix of the segment lengths: the visiting-order number of each segment's
        // first candidate.
        uint32_t incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        const uint32_t start = incl - len;
        float rho = 0.0f;
        uint32_t listed = 0u;
        for (uint32_t base = 0; base < total; base += 32u) {
            const uint32_t f = base + (uint32_t)lane;
            // The segment holding candidate f: the last one starting at or before f.
            int r = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const uint32_t s_probe = __shfl_sync(0xffffffffu, start, (r + step) & 31);
                if (r + step < 27 && s_probe <= f) r += step;
            }
            const uint32_t rb = __shfl_sync(0xffffffffu, b, r);
            const uint32_t rs = __shfl_sync(0xffffffffu, start, r);
            const bool valid = f < total;
            const uint32_t j = rb + (f - rs);
            float4 xj = make_float4(0.f, 0.f, 0.f, 0.f);
            if (valid) xj = __ldg(pos + j);
            const float r2 = in_range2(xi, xj);
            const bool inr = valid && r2 <= p.h2;
            const float wv = inr ? w_over_sigma_r2(r2, p.inv_h) : 0.0f;
            uint32_t mask = __ballot_sync(0xffffffffu, inr);
            const uint32_t listm = __ballot_sync(0xffffffffu, inr && j != i);
            if (inr && j != i) {
                const uint32_t slot = listed + (uint32_t)__popc(listm & lt);
                if (slot < p.nbr_cap) nbr[(size_t)slot * L.total + i] = j;
            }
            listed += (uint32_t)__popc(listm);
            while (mask) {
                const int l = __ffs(mask) - 1;
                rho = __fadd_rn(rho, __shfl_sync(0xffffffffu, wv, l));
                mask &= mask - 1u;
            }
        }
        if (lane == 0) {
            DensitySum d;
            d.rho = rho;
            d.listed = listed;
            density_finish(p, i, xi, vel, cx, cy, cz, distinct, d, rec, aux, bnd, nbr_count, L.host_dens,
                       L.defer_vel);
        }
    }
}


// Small models, where three lanes per particle still fit one wave of the GPU and one lane per
// particle would leave the SMs waiting on each thread's chain of candidate loads: the density pass
// with the 27-cell walk split over three lanes of one warp, lane r walking the rows of the z-plane
// dz = r - 1 (rows 3r..3r+2). Each lane sums its plane in visiting order and the particle's density
// is (plane 0 + plane 1) + plane 2, whatever the list capacity. The neighbour list is the planes'
// entries one after the other, the reference's visiting order as in k_density, so the force pass
// is the same in both modes. A plane whose shared list fills mid-walk keeps summing but its
// entries are not listed (the list length is then reported above the capacity, and the force
// pass walks the candidates again).
constexpr int kPlaneBlock = 96;  // 3 warps x 10 particles x 3 lanes (2 lanes of each warp idle)

template <bool kBatch>
__global__ void __launch_bounds__(kPlaneBlock)
    k_density_planes(StepLaunch L, const float4* __restrict__ pos, const float4* __restrict__ vel,
                     float4* __restrict__ rec, const uint32_t* __restrict__ scan,
                     float4* __restrict__ aux, float4* __restrict__ bnd,
                     uint32_t* __restrict__ nbr, uint32_t* __restrict__ nbr_count) {
    __shared__ uint32_t s_j[kListCap * kPlaneBlock];
    const uint32_t tid = threadIdx.x;
    const uint32_t lane = tid & 31u, pw = lane / 3u, pl = lane - 3u * pw;
    const uint32_t lead = lane - pl;
    const uint32_t i = (blockIdx.x * (kPlaneBlock / 32u) + (tid >> 5)) * 10u + pw;
    const bool active = lane < 30u && i < L.total;
    float rho = 0.0f;
    uint32_t n_pl = 0u;  // this plane's entries other than the particle itself
    bool lost = false;   // entries summed mid-walk and not kept for the list
    uint32_t s_end = tid;
    float4 xi = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (active) {
        const SceneParams& p = scene_params<kBatch>(L, i);
        xi = __ldg(pos + i);
        const uint32_t cx = cell_coord(xi.x, p.h), cy = cell_coord(xi.y, p.h),
                       cz = cell_coord(xi.z, p.h);
        const float s_inv_h = p.inv_h, h2 = p.h2;
        auto sum_list = [&]() {
#pragma unroll 2
            for (uint32_t o = tid; o < s_end; o += kPlaneBlock) {
                const uint32_t j = s_j[o];
                rho = __fadd_rn(rho, w_over_sigma_r2(in_range2(xi, __ldg(pos + j)), s_inv_h));
                n_pl += j != i ? 1u : 0u;
            }
        };
        for_each_candidate(p, scan, pos, xi, cx, cy, cz, [&](uint32_t j, const float4& xj) {
            const float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            s_j[s_end] = j;
            s_end += r2 <= h2 ? kPlaneBlock : 0u;
        }, [&]() {
            if (s_end > tid + kDrainAt * kPlaneBlock) {
                sum_list();
                lost = true;
                s_end = tid;
            }
        }, 3 * (int)pl, 3 * (int)pl + 3);
        sum_list();
    }
    // The three planes of a particle meet in its lead lane (lanes 30 and 31 exchange nothing
    // that is used).
    const uint32_t n0 = __shfl_sync(0xffffffffu, n_pl, lead);
    const uint32_t n1 = __shfl_sync(0xffffffffu, n_pl, lead + 1u);
    const uint32_t n2 = __shfl_sync(0xffffffffu, n_pl, lead + 2u);
    const float rho1 = __shfl_sync(0xffffffffu, rho, lead + 1u);
    const float rho2 = __shfl_sync(0xffffffffu, rho, lead + 2u);
    const uint32_t lost_bits = __ballot_sync(0xffffffffu, lost);
    if (!active) return;
    const SceneParams& p = scene_params<kBatch>(L, i);
    const bool any_lost = ((lost_bits >> lead) & 7u) != 0u;
    const uint32_t total = n0 + n1 + n2;
    if (!any_lost) {
        uint32_t k = (pl >= 1u ? n0 : 0u) + (pl >= 2u ? n1 : 0u);
        for (uint32_t o = tid; o < s_end; o += kPlaneBlock) {
            const uint32_t j = s_j[o];
            if (j == i) continue;
            if (k < p.nbr_cap) nbr[(size_t)k * L.total + i] = j;
            k++;
        }
    }
    if (pl != 0u) return;
    const uint32_t cx = cell_coord(xi.x, p.h), cy = cell_coord(xi.y, p.h), cz = cell_coord(xi.z, p.h);
    const uint32_t listed = any_lost ? max(total, p.nbr_cap + 1u) : total;
    nbr_count[i] = nbr_word(listed, cx, cy, cz, distinct_keys(p, cx, cy, cz));
    float bd, bgx, bgy, bgz;
    boundary_terms(p, xi.x, xi.y, xi.z, bd, bgx, bgy, bgz);
    rho = __fadd_rn(__fadd_rn(rho, rho1), rho2);
    rho = p.mass * p.cubic * rho + p.rho0 * bd;
    const float pr = p.stiffness * (powf(fmaxf(rho, p.rho0) / p.rho0, p.expoent) - 1.0f);
    const float pd = rho > 0.0f ? pr / (rho * rho) : 0.0f;
    const float mr = p.mass / fmaxf(rho, 1e-6f);
    const float pb = rho > 0.0f ? pr / (p.rho0 * p.rho0) : 0.0f;
    aux[i] = make_float4(pd, mr, rho, pb);
    if (L.host_dens) L.host_dens[i] = rho;
    rec[2 * (size_t)i] = make_float4(xi.x, xi.y, xi.z, pd);
    if (!L.defer_vel) {
        const float4 vi = __ldg(vel + i);
        rec[2 * (size_t)i + 1] = make_float4(vi.x, vi.y, vi.z, mr);
    }
    bnd[i] = make_float4(bgx, bgy, bgz, bd);
}

struct ForceAcc {
    float Px, Py, Pz, Vx, Vy, Vz;
};

// Pressure and viscosity contributions of one in-range neighbour (PressureAccel slang:234-249,
// ViscousAccel slang:301-318) with the constant factors taken out of the sums. With
// dW = grad_over_h * c(q) (c = -(1-q)^2 above q = 1/2, q (3q - 2) below, 0 outside the support or
// at r <= 1e-9) and u = c(q) / r, the reference's terms are
//   pressure:   mass * (pd_i + pd_j) * dW * x_ij / r  = (mass * grad_over_h) * [(pd_i + pd_j) u x_ij]
//   viscosity:  mr_j (v_ij . x_ij) dW x_ij / r / (r^2 + 0.01 h^2) = grad_over_h * [mr_j (v_ij . x_ij) u x_ij / (r^2 + eps)]
// and only the bracketed parts are summed here; k_force applies the factors once per particle.
// Every operation is an explicit round-to-nearest intrinsic, so no fusion is left to the
// compiler and every launch shape of the force pass gives bit-identical results.
__device__ __forceinline__ void force_term(const SceneParams& p, const float4& xi, const float4& vi,
                                           float pdi, const float4& xj, const float2& aj,
                                           const float4& vj, ForceAcc& f) {
    const float xx = __fsub_rn(xi.x, xj.x), xy = __fsub_rn(xi.y, xj.y), xz = __fsub_rn(xi.z, xj.z);
    const float r2 = __fmaf_rn(xz, xz, __fmaf_rn(xy, xy, __fmul_rn(xx, xx)));
    const float ir = rsqrtf(fmaxf(r2, 1e-30f));  // finite at r2 = 0, where u is 0 below
    const float r = __fmul_rn(r2, ir);
    const float q = __fmul_rn(r, p.inv_h);
    const float t = __fsub_rn(1.0f, q);
    const float c_out = -__fmul_rn(t, t);
    const float c_in = __fmul_rn(q, __fmaf_rn(3.0f, q, -2.0f));
    const float c = q > 0.5f ? c_out : c_in;
    const float u = (r > 1e-9f && q <= 1.0f) ? __fmul_rn(c, ir) : 0.0f;
    const float sp = __fmul_rn(__fadd_rn(pdi, aj.x), u);
    f.Px = __fmaf_rn(sp, xx, f.Px);
    f.Py = __fmaf_rn(sp, xy, f.Py);
    f.Pz = __fmaf_rn(sp, xz, f.Pz);
    const float dv = __fmaf_rn(__fsub_rn(vi.z, vj.z), xz,
                               __fmaf_rn(__fsub_rn(vi.y, vj.y), xy, __fmul_rn(__fsub_rn(vi.x, vj.x), xx)));
    const float iden = __fdividef(1.0f, __fadd_rn(r2, p.visc_eps));
    const float sv = __fmul_rn(__fmul_rn(__fmul_rn(aj.y, dv), u), iden);
    f.Vx = __fmaf_rn(sv, xx, f.Vx);
    f.Vy = __fmaf_rn(sv, xy, f.Vy);
    f.Vz = __fmaf_rn(sv, xz, f.Vz);
}

// A 32-byte force record in one 256-bit load (sm_100+; rec + 2j is 32-byte aligned because the
// buffer comes from cudaMalloc and each record is 32 bytes).
__device__ __forceinline__ void load_record(const float4* __restrict__ rec, uint32_t j, float4& a,
                                            float4& b) {
    const float4* q = rec + 2 * (size_t)j;
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(q));
}

// One neighbour's term from its force record: rec[2j] = (x, y, z, p/rho^2), rec[2j+1] =
// (vx, vy, vz, m/max(rho, 1e-6)), the same values as pos, vel and aux hold.
__device__ __forceinline__ void force_term_rec(const SceneParams& p, const float4& xi,
                                               const float4& vi, float pdi,
                                               const float4* __restrict__ rec, uint32_t j,
                                               ForceAcc& f) {
    float4 r0, r1;
    load_record(rec, j, r0, r1);
    force_term(p, xi, vi, pdi, r0, make_float2(r0.w, r1.w), r1, f);
}

// The rest of CalculatePressureAccel + CalculateViscousAccel + UpdatePositions for particle i
// once its sums are complete: the constant factors, the boundary term, gravity, the wall, and
// symplectic Euler.
__device__ __forceinline__ void force_finish(const SceneParams& p, uint32_t i, const float4& xi,
                                             const float4& vi, const float4& ai, ForceAcc f,
                                             const float4* __restrict__ bnd,
                                             float4* __restrict__ pos_out,
                                             float4* __restrict__ vel_out,
                                             float4* __restrict__ acc_out, float3& x_new,
                                             float3& v_new) {
    const float pdi = ai.x;
    // The factors force_term leaves out of the sums.
    const float cp = p.mass * p.grad_over_h, cv = p.visc_scale * p.grad_over_h;
    f.Px *= cp;
    f.Py *= cp;
    f.Pz *= cp;
    const float4 bi = __ldg(bnd + i);
    const float sb = (pdi + ai.w) * p.rho0;
    f.Px += sb * bi.x;
    f.Py += sb * bi.y;
    f.Pz += sb * bi.z;

    float ax = p.gx + -f.Px, ay = p.gy + -f.Py, az = p.gz + -f.Pz;
    ax += cv * f.Vx;
    ay += cv * f.Vy;
    az += cv * f.Vz;
    // WallAcceleration, wcsph_with_boundary_model.slang:336-347.
    const float dx = fminf(xi.x - p.lo[0], 0.0f) - fminf(p.hi[0] - xi.x, 0.0f);
    const float dyw = fminf(xi.y - p.lo[1], 0.0f) - fminf(p.hi[1] - xi.y, 0.0f);
    const float dzw = fminf(xi.z - p.lo[2], 0.0f) - fminf(p.hi[2] - xi.z, 0.0f);
    if (fabsf(dx) > 1e-9f || fabsf(dyw) > 1e-9f || fabsf(dzw) > 1e-9f) {
        ax += -p.wall_k * dx;
        ay += -p.wall_k * dyw;
        az += -p.wall_k * dzw;
    }
    if (acc_out) acc_out[i] = make_float4(ax, ay, az, 0.0f);
    const float nvx = vi.x + ax * p.dt, nvy = vi.y + ay * p.dt, nvz = vi.z + az * p.dt;
    v_new = make_float3(nvx, nvy, nvz);
    x_new = make_float3(xi.x + nvx * p.dt, xi.y + nvy * p.dt, xi.z + nvz * p.dt);
    vel_out[i] = make_float4(nvx, nvy, nvz, 0.0f);
    pos_out[i] = make_float4(x_new.x, x_new.y, x_new.z, xi.w);
}

// CalculatePressureAccel + CalculateViscousAccel + UpdatePositions
// (wcsph_with_boundary_model.slang:205-360), fused: both sums are accumulated separately in the
// reference's visiting order, then a = ((g - P) + V) + wall, v += a dt, x += v dt.
template <bool kBatch, int kNbrBlock, int kMinBlocks>
__global__ void __launch_bounds__(kNbrBlock, kMinBlocks)
    k_force(StepLaunch L, const float4* __restrict__ pos, const float4* __restrict__ vel,
            const float4* __restrict__ aux, const float4* __restrict__ rec,
            const float4* __restrict__ bnd,
            const uint32_t* __restrict__ scan, const uint32_t* __restrict__ nbr,
            const uint32_t* __restrict__ nbr_count, float4* __restrict__ pos_out,
            float4* __restrict__ vel_out, float4* __restrict__ acc_out,
            uint32_t* __restrict__ skin_stale, uint32_t* __restrict__ skin_ctl, HostOut ho) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // The density pass is done with the skin lists' flags: run each scene's build policy and clear
    // the flags for the next substep.
    if (skin_stale && blockIdx.x == 0) {
        for (uint32_t sc = threadIdx.x; sc < L.n_scenes; sc += blockDim.x) {
            uint32_t* c = skin_ctl + sc * kSkinCtl;
            const bool stale = skin_stale[sc] != 0u;
            uint32_t age = c[kCtlAge], wait = c[kCtlWait], since = c[kCtlSince];
            if (stale && c[kCtlFresh]) {  // the last build's lists just went stale: were they worth it?
                wait = age < kSkinMinLife || c[kCtlPoor] ? min(max(2u * wait, kSkinMinWait), kSkinMaxWait) : 0u;
                c[kCtlFresh] = 0u;
                since = 0u;
            }
            if (stale && c[kCtlAllow]) {  // the density pass rebuilt
                const uint32_t n = L.n_scenes > 1 ? L.scenes[sc].n : L.one.n;
                c[kCtlBuilds]++;
                c[kCtlFresh] = 1u;
                c[kCtlPoor] = 2u * c[kCtlUsable] < n ? 1u : 0u;
                c[kCtlUsable] = 0u;
                age = 0u;
            } else {
                age++;
                if (stale) since++;
            }
            skin_stale[sc] = 0u;
            c[kCtlAge] = age;
            c[kCtlWait] = wait;
            c[kCtlSince] = since;
            c[kCtlAllow] = !c[kCtlFresh] && since >= wait ? 1u : 0u;
        }
    }
    // The particle's new position and velocity and its density, for the host outputs.
    float3 x_new = make_float3(0.0f, 0.0f, 0.0f), v_new = x_new;
    float dens_i = 0.0f;
    if (i < L.total) {
        const SceneParams& p = scene_params<kBatch>(L, i);
        const float4 xi = __ldg(pos + i);
        const float4 vi = __ldg(vel + i);
        const float4 ai = __ldg(aux + i);
        const float pdi = ai.x;

        ForceAcc f{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        const uint32_t listed = nbr_count[i] & kNbrCountMask;
        if (listed <= p.nbr_cap) {
            // The density pass's list: the in-range neighbours in the reference's visiting order.
            uint32_t k = 0;
            const uint32_t* nl = nbr + i;  // slot k of particle i's list
            const size_t stride = L.total;
            // The next batch's indices load while the current batch is gathered and summed, so
            // each batch waits on one dependent load (the records) instead of two.
            uint32_t jn[4];
            if (listed >= 4u) {
#pragma unroll
                for (int u = 0; u < 4; u++) jn[u] = __ldg(nl + u * stride);
            }
#pragma unroll 1
            for (; k + 4u <= listed; k += 4u, nl += 4 * stride) {
                uint32_t j[4];
                float4 a[4], b[4];
#pragma unroll
                for (int u = 0; u < 4; u++) j[u] = jn[u];
                if (k + 8u <= listed) {
#pragma unroll
                    for (int u = 0; u < 4; u++) jn[u] = __ldg(nl + (4 + u) * stride);
                }
#pragma unroll
                for (int u = 0; u < 4; u++) load_record(rec, j[u], a[u], b[u]);
#pragma unroll
                for (int u = 0; u < 4; u++) force_term(p, xi, vi, pdi, a[u], make_float2(a[u].w, b[u].w), b[u], f);
            }
#pragma unroll 1
            for (; k < listed; k++, nl += stride) force_term_rec(p, xi, vi, pdi, rec, __ldg(nl), f);
        } else {
            // Overflowed list (very dense neighbourhood): walk the candidates again and add every
            // in-range one as it comes, in the same order. This path needs no shared memory, so
            // the pass keeps the whole on-chip memory as L1 for its record gathers.
            const uint32_t cx = cell_coord(xi.x, p.h), cy = cell_coord(xi.y, p.h),
                           cz = cell_coord(xi.z, p.h);
            for_each_candidate(p, scan, pos, xi, cx, cy, cz, [&](uint32_t j, const float4& xj) {
                const float xx = xi.x - xj.x, xy = xi.y - xj.y, xz = xi.z - xj.z;
                const float r2 = xx * xx + xy * xy + xz * xz;
                if (r2 <= p.h2 && j != i) force_term_rec(p, xi, vi, pdi, rec, j, f);
            }, [&]() {});
        }
        force_finish(p, i, xi, vi, ai, f, bnd, pos_out, vel_out, acc_out, x_new, v_new);
        dens_i = ai.z;
    }
    if (ho.pos3 || ho.vel3 || ho.dens) {
        // Host outputs (a single scene; the launch gives 7 floats of dynamic shared memory per
        // thread): the block's particles are consecutive slots, so each array's part is staged
        // and written out as contiguous words, whole lines over the host link.
        extern __shared__ float s_io[];
        const uint32_t t = threadIdx.x, base = blockIdx.x * (uint32_t)kNbrBlock;
        const uint32_t m = min((uint32_t)kNbrBlock, L.total - base);
        s_io[3 * t] = x_new.x;
        s_io[3 * t + 1] = x_new.y;
        s_io[3 * t + 2] = x_new.z;
        s_io[3 * kNbrBlock + 3 * t] = v_new.x;
        s_io[3 * kNbrBlock + 3 * t + 1] = v_new.y;
        s_io[3 * kNbrBlock + 3 * t + 2] = v_new.z;
        s_io[6 * kNbrBlock + t] = dens_i;
        __syncthreads();
        const size_t b3 = 3 * (size_t)base;
        for (uint32_t k = t; k < 3 * m; k += kNbrBlock) {
            if (ho.pos3) ho.pos3[b3 + k] = s_io[k];
            if (ho.vel3) ho.vel3[b3 + k] = s_io[3 * kNbrBlock + k];
        }
        if (ho.dens && t < m) ho.dens[base + t] = s_io[6 * kNbrBlock + t];
    }
}

// ---------------------------------------------------------------- incremental sort
// Particles move little per substep, so most keep the key they had in the previous substep, whose
// stably sorted keys `pkeys` line up with the current (reordered) particles. The particles whose
// key changed ("moved", in index order) are sorted stably by key and merged with the others by
// (key, index): exactly the stable sort of all (key, index) pairs. The unmoved particles' keys are
// pkeys[i], a subsequence of a sorted array, so they are already in order; this holds for any
// sorted pkeys (all moved when pkeys is the all-ones fill of a fresh model), so no step ever
// needs to know whether pkeys is current.

// Keys, moved flags and the moved particles' compaction, in two or three launches without a chain
// between tiles: the moved flags as a bitmask with one word per 32 particles, bits[w], and the
// number of moved particles before each word, pre[w] (pre[W] = total = *mcount, W = ceil(n / 32),
// pre = bits + W); (mkeys, midx)[rank] for the moved ones in index order; and the digit
// histograms of the moved keys. A tile is 256 threads x kDeltaItems particles (particle
// tile * kDeltaTile + item * 256 + thread, so every load is coalesced, and a warp's 32 particles
// of one item are one bitmask word: the tile's words are bits[32 tile, 32 tile + 32), in (item,
// warp) order).
//   k_keys_flags:    keys, moved flags, each tile's moved count (tile_cnt), histograms;
//   k_tile_scan:     one block: the tiles' exclusive prefixes in place, the total (only above
//                    kFoldTiles tiles; below, each compaction block sums its predecessors' counts);
//   k_moved_compact: per tile, each word's prefix and the moved particles' (key, index) pairs
//                    at their ranks (the key recomputed from the position: the same arithmetic).
// One launch would have to chain its tiles by a decoupled look-back, which resolves ~32 tiles per
// L2 round trip: ~22 us for the 1,024 tiles of a 1M-particle model, whatever the bytes.
constexpr int kDeltaItems = 4;
constexpr uint32_t kDeltaTile = 256u * kDeltaItems;

template <bool kBatch>
__device__ __forceinline__ uint32_t particle_key(const StepLaunch& L, uint32_t i, const float4& x) {
    const SceneParams& p = scene_params<kBatch>(L, i);
    return p.off + key_mod(hash_cell(cell_coord(x.x, p.h), cell_coord(x.y, p.h), cell_coord(x.z, p.h)),
                           p.mod_magic, p.n);
}

// kHostIn (a single scene's host round trip): the positions come from page-locked host memory,
// packed float3 in slot order (host3, its device address), and the kernel also stores them as the
// model's positions (pos_out, id = slot) and zeroes the densities, as the state upload does (with
// b_next, the build index under each slot's old id is stored under its new id first); the tile's
// 12 KB are read into shared memory with coalesced loads first.
template <bool kBatch, bool kHostIn>
__global__ void __launch_bounds__(256)
    k_keys_flags(StepLaunch L, const float4* __restrict__ pos, const uint32_t* __restrict__ pkeys,
                 uint32_t* __restrict__ bits, int passes, int digit_bits,
                 uint32_t* __restrict__ ghist, uint32_t* __restrict__ tile_cnt,
                 const float* __restrict__ host3, float4* __restrict__ pos_out,
                 float4* __restrict__ aux, const uint32_t* __restrict__ b_of_id,
                 uint32_t* __restrict__ b_next) {
    __shared__ uint32_t s_h[kMaxSortPasses * kMaxSortBins];
    __shared__ uint32_t s_n[8];
    __shared__ float s_p[kHostIn ? 3 * kDeltaTile : 1];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int bins = 1 << digit_bits;
    const uint32_t mask = (uint32_t)bins - 1u;
    for (int e = tid; e < passes * bins; e += 256) s_h[e] = 0u;
    const uint32_t t0 = blockIdx.x * kDeltaTile;
    if (kHostIn) {
        const uint32_t m3 = 3u * min(kDeltaTile, L.total - t0);
        const float* src = host3 + 3 * (size_t)t0;
        for (uint32_t k = (uint32_t)tid; k < m3; k += 256u) s_p[k] = src[k];
    }
    __syncthreads();
    const uint32_t base = t0 + (uint32_t)tid;
    const uint32_t W = (L.total + 31u) >> 5;
    // All of the thread's loads first (positions and previous keys), then the key arithmetic.
    float4 xs[kDeltaItems];
    uint32_t pks[kDeltaItems];
#pragma unroll
    for (int k = 0; k < kDeltaItems; k++) {
        const uint32_t i = base + (uint32_t)k * 256u;
        if (i < L.total) {
            if (kHostIn) {
                const uint32_t l = 3u * ((uint32_t)k * 256u + (uint32_t)tid);
                xs[k] = make_float4(s_p[l], s_p[l + 1u], s_p[l + 2u], __uint_as_float(i));
                if (b_next) {
                    const uint32_t old = __float_as_uint(pos_out[i].w);
                    b_next[i] = old < L.total ? b_of_id[old] : 0u;
                }
                pos_out[i] = xs[k];
                aux[i].z = 0.0f;
            } else {
                xs[k] = __ldg(pos + i);
            }
            pks[k] = __ldg(pkeys + i);
        }
    }
    uint32_t cnt = 0u;
#pragma unroll
    for (int k = 0; k < kDeltaItems; k++) {
        const uint32_t i = base + (uint32_t)k * 256u;
        bool moved = false;
        if (i < L.total) {
            const uint32_t key = particle_key<kBatch>(L, i, xs[k]);
            moved = key != pks[k];
            if (moved)
                for (int ps = 0; ps < passes; ps++)
                    atomicAdd(&s_h[ps * bins + ((key >> (ps * digit_bits)) & mask)], 1u);
        }
        const uint32_t ball = __ballot_sync(0xffffffffu, moved);
        const uint32_t word = (i - (uint32_t)lane) >> 5;
        if (lane == 0 && word < W) bits[word] = ball;
        cnt += (uint32_t)__popc(ball);
    }
    if (lane == 0) s_n[warp] = cnt;
    __syncthreads();
    if (tid == 0) {
        uint32_t t = 0u;
#pragma unroll
        for (int w = 0; w < 8; w++) t += s_n[w];
        tile_cnt[blockIdx.x] = t;
    }
    for (int e = tid; e < passes * bins; e += 256)
        if (s_h[e]) atomicAdd(&ghist[e], s_h[e]);
}

// Exclusive prefix sums of the tiles' moved counts, in place, by one block in chunks of 1,024
// tiles (one chunk up to 1M particles); the total goes to *mcount and pre[W].
__global__ void __launch_bounds__(1024)
    k_tile_scan(uint32_t tiles, uint32_t* __restrict__ tile_cnt, uint32_t* __restrict__ bits,
                uint32_t W, uint32_t* __restrict__ mcount) {
    __shared__ uint32_t s_w[32];
    __shared__ uint32_t s_carry;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) s_carry = 0u;
    __syncthreads();
    for (uint32_t b = 0; b < tiles; b += 1024u) {
        const uint32_t t = b + tid;
        const uint32_t v = t < tiles ? tile_cnt[t] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if ((int)lane >= o) x += y;
        }
        if (lane == 31u) s_w[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t y = s_w[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t z = __shfl_up_sync(0xffffffffu, y, o);
                if ((int)lane >= o) y += z;
            }
            s_w[lane] = y;
        }
        __syncthreads();
        const uint32_t incl = s_carry + (warp ? s_w[warp - 1] : 0u) + x;
        if (t < tiles) tile_cnt[t] = incl - v;
        __syncthreads();  // every thread has read s_carry and s_w
        if (tid == 1023u) s_carry = incl;
        __syncthreads();
    }
    if (tid == 0) {
        *mcount = s_carry;
        bits[2u * W] = s_carry;  // pre[W]
    }
}

// Up to this many tiles (4M particles) the compaction's blocks sum the earlier tiles' counts
// themselves (at most 16 loads per thread) and the scan kernel is not launched.
constexpr uint32_t kFoldTiles = 4096u;

// kFolded: tile_cnt holds the tiles' counts (k_tile_scan did not run): the block sums those of
// the tiles before its own, and the last tile writes the total. Otherwise tile_cnt holds the
// exclusive prefixes.
template <bool kBatch, bool kFolded>
__global__ void __launch_bounds__(256)
    k_moved_compact(StepLaunch L, const float4* __restrict__ pos, uint32_t* __restrict__ bits,
                    const uint32_t* __restrict__ tile_cnt, uint32_t* __restrict__ mkeys,
                    uint32_t* __restrict__ midx, uint32_t* __restrict__ mcount) {
    __shared__ uint32_t s_bits[32], s_off[32], s_sum[8];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t W = (L.total + 31u) >> 5;
    uint32_t excl;
    if (kFolded) {
        uint32_t part = 0u;
        for (uint32_t u = tid; u < blockIdx.x; u += 256u) part += tile_cnt[u];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if (lane == 0u) s_sum[warp] = part;
        __syncthreads();
        excl = 0u;
#pragma unroll
        for (int w = 0; w < 8; w++) excl += s_sum[w];
        if (tid == 0u && blockIdx.x == gridDim.x - 1u) {
            const uint32_t total = excl + tile_cnt[blockIdx.x];
            *mcount = total;
            bits[2u * W] = total;  // pre[W]
        }
    } else {
        excl = tile_cnt[blockIdx.x];
    }
    if (warp == 0) {
        const uint32_t w = blockIdx.x * 32u + lane;
        const uint32_t b = w < W ? bits[w] : 0u;
        const uint32_t c = (uint32_t)__popc(b);
        uint32_t x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if ((int)lane >= o) x += y;
        }
        const uint32_t off = excl + x - c;
        s_bits[lane] = b;
        s_off[lane] = off;
        if (w < W) bits[W + w] = off;
    }
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < kDeltaItems; k++) {
        const uint32_t i = blockIdx.x * kDeltaTile + (uint32_t)k * 256u + tid;
        const uint32_t b = s_bits[k * 8 + warp];
        if (i < L.total && ((b >> lane) & 1u)) {
            const uint32_t rank = s_off[k * 8 + warp] + (uint32_t)__popc(b & lt);
            mkeys[rank] = particle_key<kBatch>(L, i, __ldg(pos + i));
            midx[rank] = i;
        }
    }
}

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t* a, uint32_t n, uint32_t v) {
    uint32_t lo = 0u, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1u; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint32_t upper_bound_u32(const uint32_t* a, uint32_t n, uint32_t v) {
    uint32_t lo = 0u, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1u; else hi = mid;
    }
    return lo;
}

// Merge of the unmoved particles (keys pkeys[i], in index order) with the sorted moved ones
// (mk, mi) by (key, index). Thread t < n places unmoved particle t; thread n + r places the moved
// particle of sorted rank r. Every output position is computed independently.
// Moved particles with index < i (0 <= i <= n) from the bitmask and per-word prefix.
__device__ __forceinline__ uint32_t moved_before(const uint32_t* __restrict__ bits, uint32_t W,
                                                 uint32_t i) {
    const uint32_t w = i >> 5;
    if (w >= W) return bits[W + W];
    return bits[W + w] + __popc(bits[w] & ((1u << (i & 31u)) - 1u));
}

__global__ void __launch_bounds__(256)
    k_merge(uint32_t n, const uint32_t* __restrict__ pkeys, const uint32_t* __restrict__ bits,
            const uint32_t* __restrict__ mcount, const uint32_t* __restrict__ mk,
            const uint32_t* __restrict__ mi, uint32_t* __restrict__ out_keys,
            uint32_t* __restrict__ out_perm) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t m = min(*mcount, n);
    const uint32_t W = (n + 31u) >> 5;
    uint32_t key, idx, pos;
    if (t < n) {
        idx = (uint32_t)t;
        const uint32_t word = bits[idx >> 5];
        if ((word >> (idx & 31u)) & 1u) return;  // moved: placed by its sorted rank
        const uint32_t before = bits[W + (idx >> 5)] + __popc(word & ((1u << (idx & 31u)) - 1u));
        key = pkeys[idx];
        uint32_t lo = 0u, hi = m;  // moved particles ordered before (key, idx)
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            const uint32_t k2 = mk[mid];
            if (k2 < key || (k2 == key && mi[mid] < idx)) lo = mid + 1u; else hi = mid;
        }
        pos = (idx - before) + lo;
    } else if (t < (uint64_t)n + m) {
        const uint32_t r = (uint32_t)(t - n);
        key = mk[r];
        idx = mi[r];
        // Unmoved particles ordered before (key, idx): pkeys is sorted and unmoved j has key
        // pkeys[j], so they are the unmoved j below lower_bound(key) plus the unmoved j < idx in
        // the equal-key range [L, R).
        const uint32_t lb = lower_bound_u32(pkeys, n, key), ub = upper_bound_u32(pkeys, n, key);
        const uint32_t e = idx > lb ? min(idx, ub) : lb;
        const uint32_t mlb = moved_before(bits, W, lb);
        pos = r + (lb - mlb) + ((e - lb) - (moved_before(bits, W, e) - mlb));
    } else {
        return;
    }
    if (pos < n) {
        out_keys[pos] = key;
        out_perm[pos] = idx;
    }
}

constexpr int kSortBlock = 256;

template <int ITEMS>
cudaError_t launch_onesweep_t(uint32_t n, const SortConfig& sc, const SortScratch& scr, int pass,
                              const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                              uint32_t* vout, const uint32_t* n_dev, cudaStream_t s) {
    k_onesweep<kSortBlock, ITEMS><<<sc.tiles, kSortBlock, 0, s>>>(
        kin, vin, kout, vout, n, pass * sc.digit_bits, sc.bins, scr.ghist + pass * sc.bins,
        scr.counters + pass, scr.status + (size_t)pass * sc.tiles * sc.bins, scr.err, n_dev);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_lookback_selftest(bool published, uint32_t spin_limit, uint32_t* d_work,
                                     uint32_t* err, cudaStream_t s) {
    constexpr int bins = 32;
    uint32_t h[2 * bins];
    for (int b = 0; b < bins; b++) {
        h[b] = published ? (kFlagPrefix | (uint32_t)(b + 1)) : 0u;  // tile 0
        h[bins + b] = 0u;                                           // tile 1 (the waiter)
    }
    cudaError_t e = cudaMemcpyAsync(d_work, h, sizeof(h), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(s);  // h is a stack buffer
    if (e != cudaSuccess) return e;
    k_lookback_selftest<<<1, bins, 0, s>>>(d_work, bins, spin_limit, d_work + 2 * bins, err);
    return cudaGetLastError();
}


int key_bits_for(uint32_t max_key) {
    int bits = 1;
    while (bits < 32 && (((uint64_t)1 << bits) <= (uint64_t)max_key)) bits++;
    return bits;
}

SortConfig make_sort_config(uint32_t n, int digit_bits, int tile_items, int key_bits) {
    SortConfig c{};
    if (digit_bits < 4) digit_bits = 4;
    if (digit_bits > 8) digit_bits = 8;
    if (tile_items != 8 && tile_items != 12 && tile_items != 16) tile_items = 16;
    // Spatial-hash keys are < n.
    const int bits = key_bits > 0 ? (key_bits > 32 ? 32 : key_bits)
                                  : key_bits_for(n > 0 ? n - 1u : 0u);
    while ((bits + digit_bits - 1) / digit_bits > kMaxSortPasses) digit_bits++;  // <= 8 covers 32 bits
    c.digit_bits = digit_bits;
    c.passes = (bits + digit_bits - 1) / digit_bits;
    c.bins = 1 << digit_bits;
    c.tile = kSortBlock * tile_items;
    c.tiles = (uint32_t)(((uint64_t)n + c.tile - 1) / c.tile);
    if (c.tiles == 0) c.tiles = 1;
    c.delta_blocks = (uint32_t)(((uint64_t)n + kDeltaTile - 1u) / kDeltaTile);
    if (c.delta_blocks == 0) c.delta_blocks = 1;
    return c;
}

size_t sort_scratch_words(const SortConfig& c) {
    return (size_t)c.passes * c.bins + (size_t)c.passes + (size_t)c.passes * c.tiles * c.bins +
           1u + (size_t)c.delta_blocks;
}


cudaError_t launch_keys_delta(const StepLaunch& L, const float4* pos, const uint32_t* pkeys,
                              uint32_t* mkeys, uint32_t* midx, uint32_t* bits,
                              const SortConfig& sc, const SortScratch& scr, cudaStream_t s,
                              const float* host3, float4* pos_out, float4* aux,
                              const uint32_t* b_of_id, uint32_t* b_next) {
    if (L.total == 0) return cudaSuccess;
    const uint32_t tiles = sc.delta_blocks, W = (L.total + 31u) >> 5;
    if (L.n_scenes > 1)
        k_keys_flags<true, false><<<tiles, 256, 0, s>>>(L, pos, pkeys, bits, sc.passes, sc.digit_bits,
                                                        scr.ghist, scr.dstatus, nullptr, nullptr, nullptr,
                                                        nullptr, nullptr);
    else if (host3)
        k_keys_flags<false, true><<<tiles, 256, 0, s>>>(L, pos, pkeys, bits, sc.passes, sc.digit_bits,
                                                        scr.ghist, scr.dstatus, host3, pos_out, aux,
                                                        b_of_id, b_next);
    else
        k_keys_flags<false, false><<<tiles, 256, 0, s>>>(L, pos, pkeys, bits, sc.passes, sc.digit_bits,
                                                         scr.ghist, scr.dstatus, nullptr, nullptr, nullptr,
                                                         nullptr, nullptr);
    if (tiles <= kFoldTiles) {
        if (L.n_scenes > 1)
            k_moved_compact<true, true><<<tiles, 256, 0, s>>>(L, pos, bits, scr.dstatus, mkeys, midx, scr.mcount);
        else
            k_moved_compact<false, true><<<tiles, 256, 0, s>>>(L, pos, bits, scr.dstatus, mkeys, midx, scr.mcount);
        return cudaGetLastError();
    }
    k_tile_scan<<<1, 1024, 0, s>>>(tiles, scr.dstatus, bits, W, scr.mcount);
    if (L.n_scenes > 1)
        k_moved_compact<true, false><<<tiles, 256, 0, s>>>(L, pos, bits, scr.dstatus, mkeys, midx, scr.mcount);
    else
        k_moved_compact<false, false><<<tiles, 256, 0, s>>>(L, pos, bits, scr.dstatus, mkeys, midx, scr.mcount);
    return cudaGetLastError();
}

cudaError_t launch_merge(uint32_t n, const uint32_t* pkeys, const uint32_t* bits,
                         const uint32_t* mcount, const uint32_t* mk, const uint32_t* mi,
                         uint32_t* out_keys, uint32_t* out_perm, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint64_t threads = 2ull * n;
    k_merge<<<(unsigned)((threads + 255u) / 256u), 256, 0, s>>>(n, pkeys, bits, mcount, mk, mi,
                                                                 out_keys, out_perm);
    return cudaGetLastError();
}

cudaError_t launch_digit_hist(const uint32_t* keys, uint32_t n, const SortConfig& sc,
                              uint32_t* ghist, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    uint32_t blocks = (n + 255u) / 256u;
    if (blocks > 152u * 8u) blocks = 152u * 8u;
    k_digit_hist<<<blocks, 256, 0, s>>>(keys, n, sc.passes, sc.digit_bits, ghist);
    return cudaGetLastError();
}

cudaError_t launch_sort(uint32_t n, const SortConfig& sc, const SortScratch& scr, uint32_t* keys,
                        uint32_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                        uint32_t** sorted_keys, uint32_t** sorted_perm, cudaStream_t s,
                        bool vals_given, const uint32_t* n_dev) {
    const uint32_t* kin = keys;
    const uint32_t* vin = vals_given ? vals : nullptr;  // nullptr: pass 0 ranks (key, index)
    uint32_t* kout = keys_alt;
    uint32_t* vout = vals_alt;
    for (int pass = 0; pass < sc.passes; pass++) {
        cudaError_t e;
        const int items = sc.tile / kSortBlock;
        if (items == 8)
            e = launch_onesweep_t<8>(n, sc, scr, pass, kin, vin, kout, vout, n_dev, s);
        else if (items == 12)
            e = launch_onesweep_t<12>(n, sc, scr, pass, kin, vin, kout, vout, n_dev, s);
        else
            e = launch_onesweep_t<16>(n, sc, scr, pass, kin, vin, kout, vout, n_dev, s);
        if (e != cudaSuccess) return e;
        kin = kout;
        vin = vout;
        kout = (kout == keys_alt) ? keys : keys_alt;
        vout = (vout == vals_alt) ? vals : vals_alt;
    }
    *sorted_keys = const_cast<uint32_t*>(kin);
    *sorted_perm = const_cast<uint32_t*>(vin);
    return cudaSuccess;
}

namespace {
__global__ void __launch_bounds__(256)
    k_vel_records(uint32_t n, const uint32_t* __restrict__ perm, const float* __restrict__ vel3,
                  float4* __restrict__ vel_out, const float4* __restrict__ aux,
                  float4* __restrict__ rec) {
    const uint32_t i = blockIdx.x * 256u + threadIdx.x;
    if (i >= n) return;
    uint32_t src = perm[i];
    if (src >= n) src = i;  // only after a reported sort failure, as in the cell pass
    const float* v = vel3 + 3 * (size_t)src;
    const float vx = __ldg(v), vy = __ldg(v + 1), vz = __ldg(v + 2);
    vel_out[i] = make_float4(vx, vy, vz, 0.0f);
    rec[2 * (size_t)i + 1] = make_float4(vx, vy, vz, __ldg(aux + i).y);
}
}  // namespace

cudaError_t launch_vel_records(uint32_t n, const uint32_t* perm, const float* vel3,
                               float4* vel_out, const float4* aux, float4* rec, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_vel_records<<<(n + 255u) / 256u, 256, 0, s>>>(n, perm, vel3, vel_out, aux, rec);
    return cudaGetLastError();
}

cudaError_t launch_cells_reorder(const StepLaunch& L, uint32_t n, const uint32_t* skeys, const uint32_t* perm,
                                 uint32_t* cell_scan, const float4* pos_in, const float4* vel_in,
                                 float4* pos_out, float4* vel_out, uint32_t* zero,
                                 uint32_t zero_words, uint32_t* pkeys_out, uint32_t* guess,
                                 const SkinLists& sk, const KernelConfig& kc, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    switch (kc.cell_block) {
        case 128:
            k_cells_reorder<128><<<(n + 128u) / 128u, 128, 0, s>>>(L, n, skeys, perm, cell_scan, pos_in,
                                                                 vel_in, pos_out, vel_out, zero, zero_words, pkeys_out, guess, sk.b_of_id, sk.xcur, sk.x_build, sk.stale, sk.ctl);
            break;
        case 512:
            k_cells_reorder<512><<<(n + 512u) / 512u, 512, 0, s>>>(L, n, skeys, perm, cell_scan, pos_in,
                                                                 vel_in, pos_out, vel_out, zero, zero_words, pkeys_out, guess, sk.b_of_id, sk.xcur, sk.x_build, sk.stale, sk.ctl);
            break;
        default:
            k_cells_reorder<256><<<(n + 256u) / 256u, 256, 0, s>>>(L, n, skeys, perm, cell_scan, pos_in,
                                                                 vel_in, pos_out, vel_out, zero, zero_words, pkeys_out, guess, sk.b_of_id, sk.xcur, sk.x_build, sk.stale, sk.ctl);
    }
    return cudaGetLastError();
}

// SMs of the current device (0 if unknown), cached per device.
static int sm_count() {
    static std::atomic<int> sms[16];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16) return 0;
    int n = sms[dev].load(std::memory_order_relaxed);
    if (n == 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
        sms[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

// One resident wave of the walk kernel: its blocks take runs of slots until none is left, so
// more blocks would only start after the work is gone. Residency per SM is asked of the
// occupancy calculator once per instantiation.
template <bool kBatch, int B, int M, bool kStaging>
void launch_walk(const StepLaunch& L, const float4* pos, const float4* vel, float4* rec,
                 const uint32_t* cell_scan, float4* aux, float4* bnd, uint32_t* nbr,
                 uint32_t* nbr_count, const SkinLists& sk, uint32_t* sched, cudaStream_t s) {
    static std::atomic<int> per_sm{0};
    int r = per_sm.load(std::memory_order_relaxed);
    if (r == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_density<kBatch, B, M, kStaging>, B, 0) ==
                cudaSuccess && r > 0)
            per_sm.store(r, std::memory_order_relaxed);
        else
            r = M;
    }
    const int sms = sm_count();
    const uint32_t all_blocks = (L.total + B - 1) / B;
    const uint32_t blocks = sms > 0 ? min(all_blocks, (uint32_t)sms * (uint32_t)r) : all_blocks;
    k_density<kBatch, B, M, kStaging><<<blocks, B, 0, s>>>(L, pos, vel, rec, cell_scan, aux, bnd, nbr,
                                                           nbr_count, sk, sched);
}

template <int B, int M>
void density_shape(const StepLaunch& L, const float4* pos, const float4* vel, float4* rec,
                   const uint32_t* cell_scan, float4* aux, float4* bnd, uint32_t* nbr,
                   uint32_t* nbr_count, const SkinLists& sk, uint32_t* sched, bool staging,
                   cudaStream_t s) {
    if (sk.list) {
        // Skin lists: the list pass first; the walk passes then take the queue it leaves.
        const uint32_t lb = (L.total + kListBlock - 1) / kListBlock;
        if (L.n_scenes > 1) {
            k_density_list<true><<<lb, kListBlock, 0, s>>>(L, pos, vel, rec, aux, bnd, nbr, nbr_count, sk);
        } else {
            cudaMemsetAsync(sk.wcount, 0, sizeof(uint32_t), s);
            k_density_list<false><<<lb, kListBlock, 0, s>>>(L, pos, vel, rec, aux, bnd, nbr, nbr_count, sk);
            const int sms = sm_count();
            const uint32_t wb = (uint32_t)(sms > 0 ? sms : 148) * 8u;  // 32 warps per SM
            k_density_walkers<<<wb, kWalkerWarps * 32, 0, s>>>(L, pos, vel, rec, cell_scan, aux, bnd,
                                                               nbr, nbr_count, sk);
        }
    }
    if (L.n_scenes > 1) {
        if (staging)
            launch_walk<true, B, M, true>(L, pos, vel, rec, cell_scan, aux, bnd, nbr, nbr_count, sk, sched, s);
        else
            launch_walk<true, B, M, false>(L, pos, vel, rec, cell_scan, aux, bnd, nbr, nbr_count, sk, sched, s);
    } else {
        if (staging)
            launch_walk<false, B, M, true>(L, pos, vel, rec, cell_scan, aux, bnd, nbr, nbr_count, sk, sched, s);
        else
            launch_walk<false, B, M, false>(L, pos, vel, rec, cell_scan, aux, bnd, nbr, nbr_count, sk, sched, s);
    }
}

template <int B, int M>
void force_shape(const StepLaunch& L, const float4* pos, const float4* vel, const float4* aux,
                 const float4* rec, const float4* bnd, const uint32_t* cell_scan, const uint32_t* nbr,
                 const uint32_t* nbr_count, float4* pos_out, float4* vel_out, float4* acc_out,
                 const SkinLists& sk, cudaStream_t s, const HostOut& ho) {
    const uint32_t blocks = (L.total + B - 1) / B;
    if (L.n_scenes > 1)
        k_force<true, B, M><<<blocks, B, 0, s>>>(L, pos, vel, aux, rec, bnd, cell_scan, nbr, nbr_count,
                                                 pos_out, vel_out, acc_out, sk.stale, sk.ctl, HostOut{});
    else  // shared memory only for host outputs: without them the whole on-chip memory stays L1
        k_force<false, B, M><<<blocks, B, ho.any() ? 7 * B * sizeof(float) : 0, s>>>(
            L, pos, vel, aux, rec, bnd, cell_scan, nbr, nbr_count, pos_out, vel_out, acc_out,
            sk.stale, sk.ctl, ho);
}

bool planes_mode(uint32_t total) {
    const int n = sm_count();
    return n > 0 && (uint64_t)total * 3u <= (uint64_t)n * 768u;
}

cudaError_t launch_density(const StepLaunch& L, const float4* pos, const float4* vel, float4* rec,
                           const uint32_t* cell_scan, float4* aux, float4* bnd, uint32_t* nbr,
                           uint32_t* nbr_count, const SkinLists& sk, uint32_t* walk_sched,
                           const KernelConfig& kc, cudaStream_t s) {
    if (L.total == 0) return cudaSuccess;
    if (planes_mode(L.total)) {
        const uint32_t blocks = (L.total + 29u) / 30u;
        if (L.n_scenes > 1)
            k_density_planes<true><<<blocks, kPlaneBlock, 0, s>>>(L, pos, vel, rec, cell_scan, aux, bnd,
                                                                  nbr, nbr_count);
        else
            k_density_planes<false><<<blocks, kPlaneBlock, 0, s>>>(L, pos, vel, rec, cell_scan, aux, bnd,
                                                                   nbr, nbr_count);
        return cudaGetLastError();
    }
    const bool st = kc.walk_staging != 0;
    switch (kc.nbr_shape) {
        case kNbr128x8: density_shape<128, 8>(L, pos, vel, rec, cell_scan, aux, bnd, nbr, nbr_count, sk, walk_sched, st, s); break;
        case kNbr96x8: density_shape<96, 8>(L, pos, vel, rec, cell_scan, aux, bnd, nbr, nbr_count, sk, walk_sched, st, s); break;
        case kNbr64x12: density_shape<64, 12>(L, pos, vel, rec, cell_scan, aux, bnd, nbr, nbr_count, sk, walk_sched, st, s); break;
        default: density_shape<128, 6>(L, pos, vel, rec, cell_scan, aux, bnd, nbr, nbr_count, sk, walk_sched, st, s);
    }
    return cudaGetLastError();
}

cudaError_t launch_force(const StepLaunch& L, const float4* pos, const float4* vel,
                         const float4* aux, const float4* rec, const float4* bnd, const uint32_t* cell_scan,
                         const uint32_t* nbr, const uint32_t* nbr_count, float4* pos_out,
                         float4* vel_out, float4* acc_out, const SkinLists& sk,
                         const KernelConfig& kc, cudaStream_t s, const HostOut& ho) {
    if (L.total == 0) return cudaSuccess;
    switch (kc.force_shape) {
        case kNbr128x8:
            force_shape<128, 8>(L, pos, vel, aux, rec, bnd, cell_scan, nbr, nbr_count, pos_out, vel_out, acc_out, sk, s, ho);
            break;
        case kNbr96x8:
            force_shape<96, 8>(L, pos, vel, aux, rec, bnd, cell_scan, nbr, nbr_count, pos_out, vel_out, acc_out, sk, s, ho);
            break;
        case kNbr64x12:
            force_shape<64, 12>(L, pos, vel, aux, rec, bnd, cell_scan, nbr, nbr_count, pos_out, vel_out, acc_out, sk, s, ho);
            break;
        default:
            force_shape<128, 6>(L, pos, vel, aux, rec, bnd, cell_scan, nbr, nbr_count, pos_out, vel_out, acc_out, sk, s, ho);
    }
    return cudaGetLastError();
}

cudaError_t launch_offsets(uint32_t n, uint32_t off, const uint32_t* cell_scan, uint32_t* offsets,
                           cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_offsets<<<(n + 255u) / 256u, 256, 0, s>>>(n, off, cell_scan, offsets);
    return cudaGetLastError();
}

}  // namespace vfs
