// The oracle: a CPU restatement of VkFluidSim's WCSPH-with-boundary substep.
//
// TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs
// load this library, and only as the reference results / the timed CPU baseline. The product path
// (vkfluidsim_gb300) never links, loads or calls it.
//
// PARITY UNPINNED: the reference publishes no golden vectors or known-answer tests for this path,
// and its Slang/Vulkan compute shaders cannot be compiled or run without slangc and a Vulkan
// stack. Every function below is a restatement written from the reference sources it cites; the
// only reference data it is checked against are the Gauss-Legendre table
// (src/util/gaussian_quadrature.cpp:8-2292, extracted to tests/golden by a committed script) and
// the two scene JSON fixtures (assets/scenes/*.json).
//
// Semantics where the reference is non-deterministic or undefined (each one has a test):
//   1. The counting sort is executed sequentially in ascending index, i.e. it is STABLE
//      (assets/shaders/simulation/spatial_hash/sort.slang:33-45 scatters with an atomic cursor).
//   2. Duplicate neighbour keys are walked as often as they occur among the 27 neighbour cells
//      (wcsph_with_boundary_model.slang:166-190 does not de-duplicate).
//   3. The shader's extra 1/h in the kernel gradient is kept (kernels_3d.slang:78-81 divides the
//      host scale 48/(pi h^4) from src/models/model.cpp:232 by h once more).
//   4. Grid sampling clamps the cell index to [0, n-2] and extrapolates linearly outside
//      (wcsph_with_boundary_model.slang:51-66 reads out of bounds there).
//   5. The boundary pass is guarded by id < N (wcsph_with_boundary_model.slang:102-106 is not).
//   6. Float->int cell conversion saturates and maps NaN to 0 (the reference leaves it undefined).
//
// Arithmetic is FP32 like the shaders; the same code instantiated with double is the FP64 twin
// used to state the FP32 error. Build with -ffp-contract=off so results do not depend on the
// host ISA's fused multiply-add.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// Flattened parameter blocks: SimulationParameters (src/simulation.h:10-13),
// SPHModel::Parameters (src/models/model.h:14-21) and WCSPHWithBoundaryModel::Parameters
// (src/models/wcsph_with_boundary_model.h:26-33).
typedef struct vfs_oracle_params {
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
} vfs_oracle_params;
}

namespace {

constexpr uint32_t kHashK1 = 15823u;      // spatial_hash_3d.slang:12
constexpr uint32_t kHashK2 = 9737333u;    // spatial_hash_3d.slang:13
constexpr uint32_t kHashK3 = 440817757u;  // spatial_hash_3d.slang:14
constexpr uint32_t kBlock = 50u;          // spatial_hash_3d.slang:21

// offsets_3d order, spatial_hash_3d.slang:3-10: x fastest, then y, then z.
inline void neighbour_offset(int i, int& dx, int& dy, int& dz) {
    dx = i % 3 - 1;
    dy = (i / 3) % 3 - 1;
    dz = i / 9 - 1;
}

// HashCell3D, spatial_hash_3d.slang:20-28 (uint arithmetic with wrap-around).
inline uint32_t hash_cell(int32_t cx, int32_t cy, int32_t cz) {
    const uint32_t ux = (uint32_t)cx + kBlock / 2;
    const uint32_t uy = (uint32_t)cy + kBlock / 2;
    const uint32_t uz = (uint32_t)cz + kBlock / 2;
    const uint32_t lx = ux % kBlock, ly = uy % kBlock, lz = uz % kBlock;
    const uint32_t bx = ux / kBlock, by = uy / kBlock, bz = uz / kBlock;
    const uint32_t block_hash = bx * kHashK1 + by * kHashK2 + bz * kHashK3;
    return lx + kBlock * (ly + kBlock * lz) + block_hash;
}

// float -> int with saturation and NaN -> 0 (semantics 6).
template <typename T>
inline int32_t sat_to_int(T f) {
    if (!(f == f)) return 0;
    if (f >= (T)2147483648.0) return std::numeric_limits<int32_t>::max();
    if (f < (T)-2147483648.0) return std::numeric_limits<int32_t>::min();
    return (int32_t)f;
}

// GetCell3D, spatial_hash_3d.slang:16-18: floor(position / radius) with true division.
template <typename T>
inline int32_t cell_coord(T x, T h) {
    return sat_to_int<T>(std::floor(x / h));
}

template <typename T>
struct V3 {
    T x, y, z;
};
template <typename T>
inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T>
inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T>
inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename T>
inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename T>
inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <typename T>
inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

template <typename T>
inline T tpow(T a, T b) { return std::pow(a, b); }
template <>
inline float tpow<float>(float a, float b) { return powf(a, b); }

// Boundary object, WCSPHWithBoundaryModel::BoundaryObjectInfo (wcsph_with_boundary_model.h:16-24);
// matrices are glm column-major: element (row r, col c) at [c*4 + r].
struct Object {
    float transform[16];
    float rotation[16];
    float box_size[3];
    float box_pos[3];
    uint32_t res[3];
    std::vector<float> sdf;
    std::vector<float> vm;
};

template <typename T>
struct Coeffs {
    T h, h2, cubic, grad_cubic_over_h, mass, rho0, k, gamma, nu, wall_k, dt;
    V3<T> g;
    V3<T> bb_lo, bb_hi;
};

template <typename T>
Coeffs<T> make_coeffs(const vfs_oracle_params& p);

// FP32: the host computes the kernel scales in float through std::pow (src/models/model.cpp:225-234);
// the shader computes the particle volume as 0.8 * pow(h, 3) / 8 in float
// (wcsph_with_boundary_model.slang:39-41) and dt = time_scale * fixed_dt / iterations
// (src/models/wcsph_with_boundary_model.cpp:84-89).
template <>
Coeffs<float> make_coeffs<float>(const vfs_oracle_params& p) {
    Coeffs<float> c{};
    const float r = p.smooth_radius;
    const float pi_f = 3.14159265358979323846f;  // glm::pi<float>()
    c.h = r;
    c.h2 = r * r;
    c.cubic = 8.0f / (pi_f * (float)std::pow(r, 3));
    const float grad_scale = 48.0f / (pi_f * (float)std::pow(r, 4));
    c.grad_cubic_over_h = grad_scale / r;  // kernels_3d.slang:80-81
    c.mass = p.target_density * (0.8f * powf(r, 3.0f) / 8.0f);
    c.rho0 = p.target_density;
    c.k = p.stiffness;
    c.gamma = p.expoent;
    c.nu = p.viscosity_strenght;
    c.wall_k = p.wall_stiffness;
    c.dt = p.time_scale * p.fixed_dt / (float)p.iterations;
    c.g = {p.gravity[0], p.gravity[1], p.gravity[2]};
    c.bb_lo = {p.bbox_pos[0], p.bbox_pos[1], p.bbox_pos[2]};
    c.bb_hi = {p.bbox_pos[0] + p.bbox_size[0], p.bbox_pos[1] + p.bbox_size[1],
               p.bbox_pos[2] + p.bbox_size[2]};
    return c;
}

// FP64 twin: the same formulas in double from the float parameters.
template <>
Coeffs<double> make_coeffs<double>(const vfs_oracle_params& p) {
    Coeffs<double> c{};
    const double r = p.smooth_radius;
    c.h = r;
    c.h2 = r * r;
    c.cubic = 8.0 / (M_PI * r * r * r);
    c.grad_cubic_over_h = 48.0 / (M_PI * r * r * r * r) / r;
    c.mass = (double)p.target_density * (0.8 * r * r * r / 8.0);
    c.rho0 = p.target_density;
    c.k = p.stiffness;
    c.gamma = p.expoent;
    c.nu = p.viscosity_strenght;
    c.wall_k = p.wall_stiffness;
    c.dt = (double)p.time_scale * (double)p.fixed_dt / (double)p.iterations;
    c.g = {(double)p.gravity[0], (double)p.gravity[1], (double)p.gravity[2]};
    c.bb_lo = {(double)p.bbox_pos[0], (double)p.bbox_pos[1], (double)p.bbox_pos[2]};
    c.bb_hi = {(double)p.bbox_pos[0] + (double)p.bbox_size[0],
               (double)p.bbox_pos[1] + (double)p.bbox_size[1],
               (double)p.bbox_pos[2] + (double)p.bbox_size[2]};
    return c;
}

// CubicSpline, kernels_3d.slang:62-76.
template <typename T>
inline T cubic_spline(T dst, const Coeffs<T>& c) {
    const T q = dst / c.h;
    const T sigma = c.cubic;
    if (q <= (T)1) {
        if (q > (T)0.5) {
            return sigma * (T)2 * tpow<T>((T)1 - q, (T)3);
        } else {
            const T q2 = q * q;
            const T q3 = q2 * q;
            return sigma * ((T)6 * q3 - (T)6 * q2 + (T)1);
        }
    }
    return (T)0;
}

// GradCubicSpline, kernels_3d.slang:78-91 (scale already divided by h once more).
template <typename T>
inline T grad_cubic_spline(T dst, const Coeffs<T>& c) {
    const T q = dst / c.h;
    const T sigma = c.grad_cubic_over_h;
    if ((dst > (T)1e-9f) && (q <= (T)1)) {
        if (q > (T)0.5) {
            return -sigma * tpow<T>((T)1 - q, (T)2);
        } else {
            return sigma * q * ((T)3 * q - (T)2);
        }
    }
    return (T)0;
}

// PressureFromDensityEOS, wcsph_with_boundary_model.slang:199-203.
template <typename T>
inline T eos(T rho, const Coeffs<T>& c) {
    rho = std::max(rho, c.rho0);
    return c.k * (tpow<T>(rho / c.rho0, c.gamma) - (T)1);
}

// ToUVW, wcsph_with_boundary_model.slang:43-45.
template <typename T>
inline V3<T> to_uvw(const Object& o, V3<T> p) {
    return {(p.x - (T)o.box_pos[0]) / (T)o.box_size[0], (p.y - (T)o.box_pos[1]) / (T)o.box_size[1],
            (p.z - (T)o.box_pos[2]) / (T)o.box_size[2]};
}

// One axis of SampleGrid's cell lookup with the clamp of semantics 4.
template <typename T>
inline void grid_axis(uint32_t n, T u, uint32_t& cell, T& chi) {
    const T x = ((T)n - (T)1) * u;
    T f = std::floor(x);
    const T hi = (T)(n - 2);
    if (!(f >= (T)0)) f = (T)0;  // also maps NaN to cell 0
    if (f > hi) f = hi;
    cell = (uint32_t)f;
    chi = (T)2 * (x - f) - (T)1;
}

// SampleGrid, wcsph_with_boundary_model.slang:51-66 (trilinear in chi-space, divided by 8).
template <typename T>
inline T sample_grid(const std::vector<float>& grid, const uint32_t* n, V3<T> uvw) {
    uint32_t cx, cy, cz;
    T chx, chy, chz;
    grid_axis<T>(n[0], uvw.x, cx, chx);
    grid_axis<T>(n[1], uvw.y, cy, chy);
    grid_axis<T>(n[2], uvw.z, cz, chz);
    static const uint32_t off[8][3] = {{0, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 1, 1},
                                       {1, 0, 0}, {1, 1, 0}, {1, 0, 1}, {1, 1, 1}};
    T val = (T)0;
    for (int i = 0; i < 8; i++) {
        const T fx = (T)1 + ((T)2 * (T)off[i][0] - (T)1) * chx;
        const T fy = (T)1 + ((T)2 * (T)off[i][1] - (T)1) * chy;
        const T fz = (T)1 + ((T)2 * (T)off[i][2] - (T)1) * chz;
        const size_t idx = (size_t)(cx + off[i][0]) + (size_t)n[0] * (cy + off[i][1]) +
                           (size_t)n[0] * n[1] * (cz + off[i][2]);  // GetIndex3D, :47-49
        val += (T)grid[idx] * (fx * fy * fz);
    }
    return val / (T)8;
}

// GradientVector, wcsph_with_boundary_model.slang:68-85.
template <typename T>
inline V3<T> gradient_vector(const Object& o, V3<T> x, T h) {
    const T eps = (T)0.1f * h;
    const V3<T> dx{eps, 0, 0}, dy{0, eps, 0}, dz{0, 0, eps};
    const T v1x = sample_grid<T>(o.sdf, o.res, to_uvw<T>(o, x + dx));
    const T v0x = sample_grid<T>(o.sdf, o.res, to_uvw<T>(o, x - dx));
    const T v1y = sample_grid<T>(o.sdf, o.res, to_uvw<T>(o, x + dy));
    const T v0y = sample_grid<T>(o.sdf, o.res, to_uvw<T>(o, x - dy));
    const T v1z = sample_grid<T>(o.sdf, o.res, to_uvw<T>(o, x + dz));
    const T v0z = sample_grid<T>(o.sdf, o.res, to_uvw<T>(o, x - dz));
    const T den = (T)2 * eps;
    return {(v1x - v0x) / den, (v1y - v0y) / den, (v1z - v0z) / den};
}

// mul(M, float4(v, w)).xyz with M glm column-major; sums in row order ((m0 x + m1 y) + m2 z) + m3 w.
template <typename T>
inline V3<T> mat_apply(const float* M, V3<T> v, T w) {
    V3<T> r;
    r.x = (T)M[0] * v.x + (T)M[4] * v.y + (T)M[8] * v.z + (T)M[12] * w;
    r.y = (T)M[1] * v.x + (T)M[5] * v.y + (T)M[9] * v.z + (T)M[13] * w;
    r.z = (T)M[2] * v.x + (T)M[6] * v.y + (T)M[10] * v.z + (T)M[14] * w;
    return r;
}

template <typename T>
class Model {
public:
    Model(const vfs_oracle_params& p, uint32_t n) : prm(p), n(n) {
        pos.resize(n);
        vel.resize(n);
        dens.assign(n, (T)0);
        acc.resize(n);
        bdens.assign(n, (T)0);
        bgrad.resize(n);
        ids.resize(n);
        keys.assign(n, 0);
        perm.resize(n);
        offsets.assign(n, n);
        for (uint32_t i = 0; i < n; i++) {
            perm[i] = i;
            ids[i] = i;
            pos[i] = {0, 0, 0};
            vel[i] = {0, 0, 0};
            acc[i] = {0, 0, 0};
            bgrad[i] = {0, 0, 0};
        }
    }

    vfs_oracle_params prm;
    uint32_t n;
    std::vector<Object> objects;
    std::vector<V3<T>> pos, vel, acc, bgrad;
    std::vector<T> dens, bdens;
    std::vector<uint32_t> ids, keys, perm, offsets;

    void substeps(int count) {
        const Coeffs<T> c = make_coeffs<T>(prm);
        for (int s = 0; s < count; s++) substep(c);
    }

private:
    // One iteration of WCSPHWithBoundaryModel::Step's loop
    // (src/models/wcsph_with_boundary_model.cpp:93-116).
    void substep(const Coeffs<T>& c) {
        if (n == 0) return;
        external_accel(c);
        spatial_hash(c);
        reorder();
        boundary_volume(c);
        densities(c);
        pressure_accel(c);
        viscous_accel(c);
        update_positions(c);
    }

    // ExternalAccel, wcsph_with_boundary_model.slang:87-100.
    void external_accel(const Coeffs<T>& c) {
        for (uint32_t i = 0; i < n; i++) acc[i] = c.g;
    }

    // SPHModel::RunSpatialHash (src/models/model.cpp:210-223) -> SpatialHash::Run
    // (src/compute/spatial_hash.cpp:52-63): key pass, counting sort, offsets.
    void spatial_hash(const Coeffs<T>& c) {
        // UpdateSpatialHash, update_spatial_hash.slang:18-28.
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n; i++) {
            const int32_t cx = cell_coord<T>(pos[i].x, c.h);
            const int32_t cy = cell_coord<T>(pos[i].y, c.h);
            const int32_t cz = cell_coord<T>(pos[i].z, c.h);
            keys[i] = hash_cell(cx, cy, cz) % n;  // KeyFromHash, spatial_hash_3d.slang:30-32
        }
        // GPUCountSort::Run (src/compute/sort.cpp:107-143): ClearCounts, CalculateCounts,
        // exclusive scan (scan.slang:27-83), ScatterOutputs run in ascending id (stable).
        std::vector<uint32_t> counts(n, 0), sorted_keys(n), items(n);
        for (uint32_t i = 0; i < n; i++) counts[keys[i]]++;
        uint32_t run = 0;
        for (uint32_t k = 0; k < n; k++) {
            const uint32_t cnt = counts[k];
            counts[k] = run;
            run += cnt;
        }
        for (uint32_t i = 0; i < n; i++) {
            const uint32_t dst = counts[keys[i]]++;
            items[dst] = i;
            sorted_keys[dst] = keys[i];
        }
        keys.swap(sorted_keys);  // CopyBack, sort.slang:47-55
        perm.swap(items);
        // InitOffsets / CalculateOffsets, spatial_offsets.slang:10-31.
        std::fill(offsets.begin(), offsets.end(), n);
        for (uint32_t i = 0; i < n; i++) {
            const uint32_t prev = i == 0 ? n : keys[i - 1];
            if (keys[i] != prev) offsets[keys[i]] = i;
        }
    }

    // BufferReorder::Reorder + Copyback (src/compute/sort.cpp:206-227, reorder.slang:11-19) for
    // positions and velocities; ids travel with them (extension: the reference has no ids).
    void reorder() {
        std::vector<V3<T>> p2(n), v2(n);
        std::vector<uint32_t> id2(n);
        for (uint32_t i = 0; i < n; i++) {
            p2[i] = pos[perm[i]];
            v2[i] = vel[perm[i]];
            id2[i] = ids[perm[i]];
        }
        pos.swap(p2);
        vel.swap(v2);
        ids.swap(id2);
    }

    // CalculateBoundaryVolume, wcsph_with_boundary_model.slang:102-151.
    void boundary_volume(const Coeffs<T>& c) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n; i++) {
            T bd = (T)0;
            V3<T> bg{0, 0, 0};
            const V3<T> p = pos[i];
            for (const Object& o : objects) {
                const V3<T> local = mat_apply<T>(o.transform, p, (T)1);
                const T radius = c.h;
                const T lx = local.x, ly = local.y, lz = local.z;
                const bool outside = (lx < (T)o.box_pos[0]) || (ly < (T)o.box_pos[1]) ||
                                     (lz < (T)o.box_pos[2]) ||
                                     (lx > (T)o.box_pos[0] + (T)o.box_size[0]) ||
                                     (ly > (T)o.box_pos[1] + (T)o.box_size[1]) ||
                                     (lz > (T)o.box_pos[2] + (T)o.box_size[2]);
                if (outside) continue;
                const V3<T> uvw = to_uvw<T>(o, local);
                const T dist = sample_grid<T>(o.sdf, o.res, uvw);
                if (!(dist >= (T)0 && dist < radius)) continue;
                const T volume = sample_grid<T>(o.vm, o.res, uvw);
                if (!(volume > (T)0)) continue;
                V3<T> normal = gradient_vector<T>(o, local, c.h);
                const T modn = std::sqrt(dot(normal, normal));
                if (!(modn > (T)1e-9f)) continue;
                normal = mat_apply<T>(o.rotation, normal, (T)1);
                normal = normal / modn;
                const T d = std::max(dist + (T)0.125f * radius, (T)0.5f * radius);
                const V3<T> x_boundary = p - d * normal;
                const V3<T> xij = p - x_boundary;
                const T xij_mod = std::sqrt(dot(xij, xij));
                const V3<T> xij_norm = xij_mod > (T)0 ? xij / xij_mod : V3<T>{0, 0, 0};
                bd += volume * cubic_spline<T>(xij_mod, c);
                bg = bg + (volume * grad_cubic_spline<T>(xij_mod, c)) * xij_norm;
            }
            bdens[i] = bd;
            bgrad[i] = bg;
        }
    }

    // The 27-key bucket walk shared by the three neighbour passes (slang:166-190, 217-251,
    // 284-320): visit every sorted index j in the bucket of each neighbour key, in offsets_3d
    // order and in sorted order inside a bucket, duplicates included.
    template <typename F>
    inline void for_each_candidate(uint32_t i, const Coeffs<T>& c, F&& f) const {
        const int32_t cx = cell_coord<T>(pos[i].x, c.h);
        const int32_t cy = cell_coord<T>(pos[i].y, c.h);
        const int32_t cz = cell_coord<T>(pos[i].z, c.h);
        for (int o = 0; o < 27; o++) {
            int dx, dy, dz;
            neighbour_offset(o, dx, dy, dz);
            const uint32_t key = hash_cell((int32_t)((uint32_t)cx + (uint32_t)dx),
                                           (int32_t)((uint32_t)cy + (uint32_t)dy),
                                           (int32_t)((uint32_t)cz + (uint32_t)dz)) %
                                 n;
            uint32_t cur = offsets[key];
            while (cur < n) {
                const uint32_t j = cur;
                cur++;
                if (keys[j] != key) break;
                f(j);
            }
        }
    }

    // CalculateDensities, wcsph_with_boundary_model.slang:153-197.
    void densities(const Coeffs<T>& c) {
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t ii = 0; ii < (int64_t)n; ii++) {
            const uint32_t i = (uint32_t)ii;
            const V3<T> p = pos[i];
            T density = (T)0;
            for_each_candidate(i, c, [&](uint32_t j) {
                const V3<T> off = pos[j] - p;
                const T r2 = dot(off, off);
                if (r2 > c.h2) return;
                const T dst = std::sqrt(r2);
                density += c.mass * cubic_spline<T>(dst, c);
            });
            density += c.rho0 * bdens[i];
            dens[i] = density;
        }
    }

    // PressureAccel / CalculatePressureAccel, wcsph_with_boundary_model.slang:205-271.
    void pressure_accel(const Coeffs<T>& c) {
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t ii = 0; ii < (int64_t)n; ii++) {
            const uint32_t i = (uint32_t)ii;
            V3<T> force{0, 0, 0};
            const T di = dens[i];
            const T pi = eos<T>(di, c);
            const T pdi = di > (T)0 ? pi / (di * di) : (T)0;
            const V3<T> xi = pos[i];
            for_each_candidate(i, c, [&](uint32_t j) {
                if (j == i) return;
                const V3<T> xij = xi - pos[j];
                const T r2 = dot(xij, xij);
                if (r2 > c.h2) return;
                const T dj = dens[j];
                const T pj = eos<T>(dj, c);
                const T r = std::sqrt(r2);
                const V3<T> xn = r > (T)0 ? xij / r : V3<T>{0, 1, 0};
                const T pdj = dj > (T)0 ? pj / (dj * dj) : (T)0;
                force = force + ((c.mass * (pdi + pdj)) * grad_cubic_spline<T>(r, c)) * xn;
            });
            const T pdb = di > (T)0 ? pi / (c.rho0 * c.rho0) : (T)0;
            force = force + ((pdi + pdb) * c.rho0) * bgrad[i];
            acc[i] = acc[i] + (T)-1 * force;
        }
    }

    // ViscousAccel / CalculateViscousAccel, wcsph_with_boundary_model.slang:273-334.
    void viscous_accel(const Coeffs<T>& c) {
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t ii = 0; ii < (int64_t)n; ii++) {
            const uint32_t i = (uint32_t)ii;
            V3<T> force{0, 0, 0};
            const V3<T> xi = pos[i];
            const V3<T> vi = vel[i];
            for_each_candidate(i, c, [&](uint32_t j) {
                if (j == i) return;
                const V3<T> xij = xi - pos[j];
                const T r2 = dot(xij, xij);
                if (r2 > c.h2) return;
                const T r = std::sqrt(r2);
                const V3<T> xn = r > (T)0 ? xij / r : V3<T>{0, 1, 0};
                const V3<T> vij = vi - vel[j];
                const T rhoj = std::max(dens[j], (T)1e-6f);
                const V3<T> grad_w = xn * grad_cubic_spline<T>(r, c);
                const T s = (c.mass / rhoj) * dot(vij, xij);
                force = force + (s * grad_w) / (r2 + (T)0.01f * c.h2);
            });
            const T scale = (T)2 * ((T)3 + (T)2) * c.nu;
            acc[i] = acc[i] + scale * force;
        }
    }

    // WallAcceleration + UpdatePositions, wcsph_with_boundary_model.slang:336-360.
    void update_positions(const Coeffs<T>& c) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n; i++) {
            const V3<T> p = pos[i];
            const V3<T> d1{std::min(p.x - c.bb_lo.x, (T)0), std::min(p.y - c.bb_lo.y, (T)0),
                           std::min(p.z - c.bb_lo.z, (T)0)};
            const V3<T> d2{std::min(c.bb_hi.x - p.x, (T)0), std::min(c.bb_hi.y - p.y, (T)0),
                           std::min(c.bb_hi.z - p.z, (T)0)};
            const V3<T> diff = d1 - d2;
            const T tiny = (T)1e-9f;
            if (std::fabs(diff.x) > tiny || std::fabs(diff.y) > tiny || std::fabs(diff.z) > tiny) {
                acc[i] = acc[i] + (-c.wall_k) * diff;
            }
            vel[i] = vel[i] + acc[i] * c.dt;
            pos[i] = pos[i] + vel[i] * c.dt;
        }
    }
};

struct Handle {
    int fp64;
    std::unique_ptr<Model<float>> m32;
    std::unique_ptr<Model<double>> m64;
};

// ---- Volume maps from analytic SDFs (src/util/volume_map.cpp:9-54, discretization.cpp:16-57,
// mesh_sdf.cpp:28-44, gaussian_quadrature.cpp:2293-2334) ----

// Gauss-Legendre nodes and weights on [-1, 1] by Newton iteration on P_n (own computation of
// the published rule; checked against the reference's table in tests/golden).
void gauss_legendre(int n, double* x, double* w) {
    for (int i = 0; i < n; i++) {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
        double dp = 0.0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; k++) {
                const double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = pk;
            }
            if (n == 1) p0 = 1.0;
            dp = n * (z * p1 - p0) / (z * z - 1.0);
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
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[i] = -z;  // ascending order
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

// Analytic SDFs in object-local coordinates (negative inside the solid).
//   kind 0: sphere, params[0] = radius
//   kind 1: solid box, params[0..2] = half extents
//   kind 2: container (inverted box): positive inside the box, params[0..2] = half extents
double analytic_sdf(int kind, const double* prm, double x, double y, double z) {
    if (kind == 0) return std::sqrt(x * x + y * y + z * z) - prm[0];
    const double qx = std::fabs(x) - prm[0], qy = std::fabs(y) - prm[1], qz = std::fabs(z) - prm[2];
    const double ox = std::max(qx, 0.0), oy = std::max(qy, 0.0), oz = std::max(qz, 0.0);
    const double box = std::sqrt(ox * ox + oy * oy + oz * oz) + std::min(std::max(qx, std::max(qy, qz)), 0.0);
    return kind == 1 ? box : -box;
}

void shape_aabb(int kind, const double* prm, float lo[3], float hi[3]) {
    for (int a = 0; a < 3; a++) {
        const double e = kind == 0 ? prm[0] : prm[a];
        lo[a] = (float)-e;
        hi[a] = (float)e;
    }
}

// CubicSplineKernel::W in double (src/util/kernel.cpp:10-38).
struct KernelD {
    double radius, factor, w_zero;
    explicit KernelD(double r) : radius(r), factor(8.0 / (M_PI * r * r * r)) { w_zero = W(0.0); }
    double W(double r) const {
        const double q = r / radius;
        if (q <= 1.0) {
            if (q <= 0.5) {
                const double q2 = q * q, q3 = q2 * q;
                return factor * (6.0 * q3 - 6.0 * q2 + 1.0);
            }
            return factor * (2.0 * std::pow(1.0 - q, 3.0));
        }
        return 0.0;
    }
};

// A triangle mesh with the reference's pseudonormals (MeshPseudonormals::Build,
// src/util/mesh_pseudonormals.cpp:11-88: face normals; vertex normals weighted by acos(|cos|) of
// the corner angle; edge normals the normalised sum of the faces on the edge) and the
// closest-point query of DistancePointToTriangle (src/util/geometry.cpp, Eberly's region method).
struct OracleMesh {
    struct V {
        double x, y, z;
    };
    std::vector<V> p;
    std::vector<uint32_t> t;
    std::vector<V> fn, vn, en;  // en: 3 per triangle (edges 01, 12, 02)
    float lo[3], hi[3];

    static V sub(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
    static double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

    bool build(const float* v, uint32_t nv, const uint32_t* tri, uint32_t nt) {
        if (nv < 3 || nt < 1) return false;
        for (uint32_t k = 0; k < 3 * nt; k++)
            if (tri[k] >= nv) return false;
        p.resize(nv);
        for (uint32_t k = 0; k < nv; k++) p[k] = {v[3 * k], v[3 * k + 1], v[3 * k + 2]};
        t.assign(tri, tri + 3 * (size_t)nt);
        for (int a = 0; a < 3; a++) {
            lo[a] = INFINITY;
            hi[a] = -INFINITY;
        }
        for (uint32_t k = 0; k < 3 * nt; k++) {
            const float q[3] = {v[3 * t[k]], v[3 * t[k] + 1], v[3 * t[k] + 2]};
            for (int a = 0; a < 3; a++) {
                lo[a] = std::min(lo[a], q[a]);
                hi[a] = std::max(hi[a], q[a]);
            }
        }
        // Float math like the reference's glm::vec3 pseudonormals.
        struct F {
            float x, y, z;
        };
        auto fs = [](F a, F b) { return F{a.x - b.x, a.y - b.y, a.z - b.z}; };
        auto fd = [](F a, F b) { return a.x * b.x + a.y * b.y + a.z * b.z; };
        auto fnorm = [&](F a) {
            const float l = std::sqrt(fd(a, a));
            return F{a.x / l, a.y / l, a.z / l};
        };
        auto P = [&](uint32_t i) { return F{v[3 * i], v[3 * i + 1], v[3 * i + 2]}; };
        std::vector<F> vacc(nv, F{0, 0, 0});
        std::map<uint64_t, F> edges;
        std::vector<F> fnf(nt);
        auto key = [&](uint32_t a, uint32_t b) { return (uint64_t)std::max(a, b) + (uint64_t)std::min(a, b) * nv; };
        for (uint32_t i = 0; i < nt; i++) {
            const uint32_t ia = t[3 * i], ib = t[3 * i + 1], ic = t[3 * i + 2];
            const F a = P(ia), b = P(ib), c = P(ic);
            const F e1 = fs(b, a), e2 = fs(c, a);
            const F cr = {e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
            if (!(fd(cr, cr) > 0.0f)) return false;
            const F n = fnorm(cr);
            fnf[i] = n;
            const float a0 = std::acos(std::fabs(fd(fnorm(fs(b, a)), fnorm(fs(c, a)))));
            const float a1 = std::acos(std::fabs(fd(fnorm(fs(a, b)), fnorm(fs(c, b)))));
            const float a2 = std::acos(std::fabs(fd(fnorm(fs(b, c)), fnorm(fs(a, c)))));
            for (auto pr : {std::make_pair(ia, a0), std::make_pair(ib, a1), std::make_pair(ic, a2)}) {
                F& q = vacc[pr.first];
                q = F{q.x + pr.second * n.x, q.y + pr.second * n.y, q.z + pr.second * n.z};
            }
            for (auto e : {std::make_pair(ia, ib), std::make_pair(ib, ic), std::make_pair(ia, ic)}) {
                F& q = edges[key(e.first, e.second)];
                q = F{q.x + n.x, q.y + n.y, q.z + n.z};
            }
        }
        fn.resize(nt);
        en.resize(3 * (size_t)nt);
        vn.assign(nv, V{0, 0, 0});
        for (uint32_t k = 0; k < nv; k++)
            if (fd(vacc[k], vacc[k]) > 0.0f) {
                const F n = fnorm(vacc[k]);
                vn[k] = {n.x, n.y, n.z};
            }
        for (uint32_t i = 0; i < nt; i++) {
            fn[i] = {fnf[i].x, fnf[i].y, fnf[i].z};
            const uint32_t ia = t[3 * i], ib = t[3 * i + 1], ic = t[3 * i + 2];
            const uint64_t ks[3] = {key(ia, ib), key(ib, ic), key(ia, ic)};
            for (int e = 0; e < 3; e++) {
                const F s = edges[ks[e]];
                const F n = fd(s, s) > 0.0f ? fnorm(s) : fnf[i];
                en[3 * i + e] = {n.x, n.y, n.z};
            }
        }
        return true;
    }

    // Squared distance and closest entity (0-2 vertices, 3 E01, 4 E12, 5 E02, 6 face).
    static double closest(V pt, V v0, V v1, V v2, double& s, double& u, int& ent) {
        const V e0 = sub(v1, v0), e1 = sub(v2, v0), d = sub(v0, pt);
        const double a00 = dot(e0, e0), a01 = dot(e0, e1), a11 = dot(e1, e1);
        const double b0 = dot(d, e0), b1 = dot(d, e1);
        const double det = std::max(a00 * a11 - a01 * a01, 0.0);
        s = a01 * b1 - a11 * b0;
        u = a01 * b0 - a00 * b1;
        auto edge_s0 = [&]() {  // s = 0: t in [0, 1]
            s = 0;
            if (b1 >= 0) { u = 0; ent = 0; }
            else if (-b1 >= a11) { u = 1; ent = 2; }
            else { u = -b1 / a11; ent = 5; }
        };
        auto edge_t0 = [&]() {  // t = 0: s in [0, 1]
            u = 0;
            if (b0 >= 0) { s = 0; ent = 0; }
            else if (-b0 >= a00) { s = 1; ent = 1; }
            else { s = -b0 / a00; ent = 3; }
        };
        if (s + u <= det) {
            if (s < 0) {
                if (u < 0) {
                    if (b0 < 0) {
                        u = 0;
                        if (-b0 >= a00) { s = 1; ent = 1; }
                        else { s = -b0 / a00; ent = 3; }
                    } else {
                        edge_s0();
                    }
                } else {
                    edge_s0();
                }
            } else if (u < 0) {
                edge_t0();
            } else {
                s /= det;
                u /= det;
                ent = 6;
            }
        } else if (s < 0) {
            const double t0 = a01 + b0, t1 = a11 + b1;
            if (t1 > t0) {
                const double num = t1 - t0, den = a00 - 2 * a01 + a11;
                if (num >= den) { s = 1; u = 0; ent = 1; }
                else { s = num / den; u = 1 - s; ent = 4; }
            } else {
                s = 0;
                if (t1 <= 0) { u = 1; ent = 2; }
                else if (b1 >= 0) { u = 0; ent = 0; }
                else { u = -b1 / a11; ent = 5; }
            }
        } else if (u < 0) {
            const double t0 = a01 + b1, t1 = a00 + b0;
            if (t1 > t0) {
                const double num = t1 - t0, den = a00 - 2 * a01 + a11;
                if (num >= den) { u = 1; s = 0; ent = 2; }
                else { u = num / den; s = 1 - u; ent = 4; }
            } else {
                u = 0;
                if (t1 <= 0) { s = 1; ent = 1; }
                else if (b0 >= 0) { s = 0; ent = 0; }
                else { s = -b0 / a00; ent = 3; }
            }
        } else {
            const double num = a11 + b1 - a01 - b0;
            if (num <= 0) { s = 0; u = 1; ent = 2; }
            else {
                const double den = a00 - 2 * a01 + a11;
                if (num >= den) { s = 1; u = 0; ent = 1; }
                else { s = num / den; u = 1 - s; ent = 4; }
            }
        }
        const V q = {v0.x + s * e0.x + u * e1.x - pt.x, v0.y + s * e0.y + u * e1.y - pt.y,
                     v0.z + s * e0.z + u * e1.z - pt.z};
        return dot(q, q);
    }

    double signed_distance(float x, float y, float z) const {
        const V pt = {x, y, z};
        double best = INFINITY, bs = 0, bu = 0;
        size_t bt = 0;
        int be = 6;
        for (size_t i = 0; i < t.size() / 3; i++) {
            double s, u;
            int ent;
            const double d2 = closest(pt, p[t[3 * i]], p[t[3 * i + 1]], p[t[3 * i + 2]], s, u, ent);
            if (d2 < best) {
                best = d2;
                bt = i;
                be = ent;
                bs = s;
                bu = u;
            }
        }
        const V a = p[t[3 * bt]], b = p[t[3 * bt + 1]], c = p[t[3 * bt + 2]];
        const V cp = {a.x + bs * (b.x - a.x) + bu * (c.x - a.x), a.y + bs * (b.y - a.y) + bu * (c.y - a.y),
                      a.z + bs * (b.z - a.z) + bu * (c.z - a.z)};
        V n;
        if (be <= 2) n = vn[t[3 * bt + be]];
        else if (be <= 5) n = en[3 * bt + (be - 3)];
        else n = fn[bt];
        const double d = std::sqrt(best);
        return dot(sub(pt, cp), n) >= 0 ? d : -d;
    }
};


template <typename T>
void set_state_t(Model<T>* m, const float* pos, const float* vel, const uint32_t* ids) {
    for (uint32_t i = 0; i < m->n; i++) {
        m->pos[i] = {(T)pos[3 * i], (T)pos[3 * i + 1], (T)pos[3 * i + 2]};
        m->vel[i] = {(T)vel[3 * i], (T)vel[3 * i + 1], (T)vel[3 * i + 2]};
        m->ids[i] = ids ? ids[i] : i;
    }
}

template <typename T>
void get_state_t(Model<T>* m, float* pos, float* vel, float* dens, uint32_t* ids) {
    for (uint32_t i = 0; i < m->n; i++) {
        if (pos) {
            pos[3 * i] = (float)m->pos[i].x;
            pos[3 * i + 1] = (float)m->pos[i].y;
            pos[3 * i + 2] = (float)m->pos[i].z;
        }
        if (vel) {
            vel[3 * i] = (float)m->vel[i].x;
            vel[3 * i + 1] = (float)m->vel[i].y;
            vel[3 * i + 2] = (float)m->vel[i].z;
        }
        if (dens) dens[i] = (float)m->dens[i];
        if (ids) ids[i] = m->ids[i];
    }
}

template <typename T>
void get_fields_t(Model<T>* m, float* acc, float* bdens, float* bgrad) {
    for (uint32_t i = 0; i < m->n; i++) {
        if (acc) {
            acc[3 * i] = (float)m->acc[i].x;
            acc[3 * i + 1] = (float)m->acc[i].y;
            acc[3 * i + 2] = (float)m->acc[i].z;
        }
        if (bdens) bdens[i] = (float)m->bdens[i];
        if (bgrad) {
            bgrad[3 * i] = (float)m->bgrad[i].x;
            bgrad[3 * i + 1] = (float)m->bgrad[i].y;
            bgrad[3 * i + 2] = (float)m->bgrad[i].z;
        }
    }
}

}  // namespace

// Grid box, SDF grid and volume map of a shape given by its local bounds and signed-distance
// function, following MeshSDF::Build (src/util/mesh_sdf.cpp:28-44, tolerance 0, margin passed in:
// the scene uses 8h, src/scenes/generic_scene.cpp:88-124), LinearLagrangeDiscreteGrid::Init
// (src/util/discretization.cpp:16-32) and GenerateVolumeMap (src/util/volume_map.cpp:9-54) with
// a 16-point Gauss-Legendre rule per axis (gaussian_quadrature.cpp:2293-2334). The float
// roundings of the reference (node and quadrature points passed as glm::vec3, the grid step
// computed in float) are kept.
template <typename Sdf>
int volume_map_of(const Sdf& sdf_fn, const float lo[3], const float hi[3], float support_radius,
                  const uint32_t* res, float margin, int quad_n, float* box_size_out,
                  float* box_pos_out, float* sdf_out, float* vm_out) {
    if (res[0] < 2 || res[1] < 2 || res[2] < 2) return -1;
    if (quad_n < 2) quad_n = 2;
    if (quad_n > 64) quad_n = 64;
    float bpos[3], bsize[3];
    for (int a = 0; a < 3; a++) {
        const float size = hi[a] - lo[a];
        bsize[a] = size + 2.0f * margin;
        bpos[a] = lo[a] - margin;
        box_size_out[a] = bsize[a];
        box_pos_out[a] = bpos[a];
    }
    float dmin[3], dmax[3];
    double step[3];
    for (int a = 0; a < 3; a++) {
        dmin[a] = bpos[a];
        dmax[a] = bpos[a] + bsize[a];
        step[a] = (double)((dmax[a] - dmin[a]) / (float)(res[a] - 1u));
    }
    std::vector<double> gx(quad_n), gw(quad_n);
    gauss_legendre(quad_n, gx.data(), gw.data());
    const float sr = support_radius;
    const KernelD kern((double)sr);
    // Integration domain [-h, h]^3: c0 = 0.5 (max - min), c1 = 0.5 (max + min) (both float
    // vectors converted to double).
    const double c0 = 0.5 * (double)(sr - (-sr));
    const double c1 = 0.5 * (double)(sr + (-sr));
    const int64_t total = (int64_t)res[0] * res[1] * res[2];
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t lin = 0; lin < total; lin++) {
        const uint32_t i = (uint32_t)(lin % res[0]);
        const uint32_t j = (uint32_t)((lin / res[0]) % res[1]);
        const uint32_t k = (uint32_t)(lin / ((int64_t)res[0] * res[1]));
        const double ex = step[0] * (double)i + (double)dmin[0];
        const double ey = step[1] * (double)j + (double)dmin[1];
        const double ez = step[2] * (double)k + (double)dmin[2];
        const float fx = (float)ex, fy = (float)ey, fz = (float)ez;  // func(const glm::vec3&)
        const double node_sdf = sdf_fn(fx, fy, fz);
        sdf_out[lin] = (float)node_sdf;
        double value = 0.0;
        if (!(node_sdf > 2.0 * (double)sr)) {
            double integral = 0.0;
            for (int a = 0; a < quad_n; a++) {
                const double wa = gw[a];
                for (int b = 0; b < quad_n; b++) {
                    const double wab = wa * gw[b];
                    for (int cidx = 0; cidx < quad_n; cidx++) {
                        const double wabc = wab * gw[cidx];
                        const float xi_x = (float)(c0 * gx[a] + c1);
                        const float xi_y = (float)(c0 * gx[b] + c1);
                        const float xi_z = (float)(c0 * gx[cidx] + c1);
                        double f = 0.0;
                        const float len2 = xi_x * xi_x + xi_y * xi_y + xi_z * xi_z;
                        if (!(len2 > sr * sr)) {
                            const float px = fx + xi_x, py = fy + xi_y, pz = fz + xi_z;
                            const double di = sdf_fn(px, py, pz);
                            if (di <= 0.0)
                                f = 1.0;
                            else if (di < (double)sr)
                                f = kern.W(di) / kern.w_zero;
                        }
                        integral += wabc * f;
                    }
                }
            }
            integral *= c0 * c0 * c0;
            value = 0.8 * integral;
        }
        vm_out[lin] = (float)value;
    }
    return 0;
}

extern "C" {

void* vfs_oracle_create(const vfs_oracle_params* p, uint32_t n, int fp64) {
    Handle* h = new Handle();
    h->fp64 = fp64;
    if (fp64)
        h->m64.reset(new Model<double>(*p, n));
    else
        h->m32.reset(new Model<float>(*p, n));
    return h;
}

void vfs_oracle_destroy(void* hp) { delete (Handle*)hp; }

void vfs_oracle_set_params(void* hp, const vfs_oracle_params* p) {
    Handle* h = (Handle*)hp;
    if (h->fp64)
        h->m64->prm = *p;
    else
        h->m32->prm = *p;
}

int vfs_oracle_add_object(void* hp, const float* transform, const float* rotation,
                          const float* box_size, const float* box_pos, const uint32_t* res,
                          const float* sdf, const float* vm) {
    Handle* h = (Handle*)hp;
    if (res[0] < 2 || res[1] < 2 || res[2] < 2) return -1;
    Object o;
    std::memcpy(o.transform, transform, sizeof(o.transform));
    std::memcpy(o.rotation, rotation, sizeof(o.rotation));
    std::memcpy(o.box_size, box_size, sizeof(o.box_size));
    std::memcpy(o.box_pos, box_pos, sizeof(o.box_pos));
    std::memcpy(o.res, res, sizeof(o.res));
    const size_t cnt = (size_t)res[0] * res[1] * res[2];
    o.sdf.assign(sdf, sdf + cnt);
    o.vm.assign(vm, vm + cnt);
    if (h->fp64)
        h->m64->objects.push_back(std::move(o));
    else
        h->m32->objects.push_back(std::move(o));
    return 0;
}

void vfs_oracle_set_state(void* hp, const float* pos, const float* vel, const uint32_t* ids) {
    Handle* h = (Handle*)hp;
    if (h->fp64)
        set_state_t(h->m64.get(), pos, vel, ids);
    else
        set_state_t(h->m32.get(), pos, vel, ids);
}

void vfs_oracle_set_state_f64(void* hp, const double* pos, const double* vel, const uint32_t* ids) {
    Handle* h = (Handle*)hp;
    Model<double>* m = h->m64.get();
    if (!m) return;
    for (uint32_t i = 0; i < m->n; i++) {
        m->pos[i] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        m->vel[i] = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
        m->ids[i] = ids ? ids[i] : i;
    }
}

void vfs_oracle_substeps(void* hp, int count) {
    Handle* h = (Handle*)hp;
    if (h->fp64)
        h->m64->substeps(count);
    else
        h->m32->substeps(count);
}

// Simulation::Step -> GenericScene::Step -> WCSPHWithBoundaryModel::Step: `iterations` substeps.
void vfs_oracle_step(void* hp) {
    Handle* h = (Handle*)hp;
    const int it = h->fp64 ? h->m64->prm.iterations : h->m32->prm.iterations;
    vfs_oracle_substeps(hp, it);
}

void vfs_oracle_get_state(void* hp, float* pos, float* vel, float* dens, uint32_t* ids) {
    Handle* h = (Handle*)hp;
    if (h->fp64)
        get_state_t(h->m64.get(), pos, vel, dens, ids);
    else
        get_state_t(h->m32.get(), pos, vel, dens, ids);
}

void vfs_oracle_get_state_f64(void* hp, double* pos, double* vel, double* dens, uint32_t* ids) {
    Handle* h = (Handle*)hp;
    Model<double>* m = h->m64.get();
    if (!m) return;
    for (uint32_t i = 0; i < m->n; i++) {
        if (pos) {
            pos[3 * i] = m->pos[i].x;
            pos[3 * i + 1] = m->pos[i].y;
            pos[3 * i + 2] = m->pos[i].z;
        }
        if (vel) {
            vel[3 * i] = m->vel[i].x;
            vel[3 * i + 1] = m->vel[i].y;
            vel[3 * i + 2] = m->vel[i].z;
        }
        if (dens) dens[i] = m->dens[i];
        if (ids) ids[i] = m->ids[i];
    }
}

// Neighbour arrays of the last substep: sorted keys, sorted_indices (permutation) and
// spatial_offsets (cell start, N when the key is empty).
void vfs_oracle_get_neighbors(void* hp, uint32_t* keys, uint32_t* perm, uint32_t* offsets) {
    Handle* h = (Handle*)hp;
    const std::vector<uint32_t>* k = h->fp64 ? &h->m64->keys : &h->m32->keys;
    const std::vector<uint32_t>* p = h->fp64 ? &h->m64->perm : &h->m32->perm;
    const std::vector<uint32_t>* o = h->fp64 ? &h->m64->offsets : &h->m32->offsets;
    if (keys) std::memcpy(keys, k->data(), k->size() * 4);
    if (perm) std::memcpy(perm, p->data(), p->size() * 4);
    if (offsets) std::memcpy(offsets, o->data(), o->size() * 4);
}

// Per-particle fields of the last substep in sorted order: total acceleration, boundary density
// Psi_b and boundary gradient.
void vfs_oracle_get_fields(void* hp, float* acc, float* bdens, float* bgrad) {
    Handle* h = (Handle*)hp;
    if (h->fp64)
        get_fields_t(h->m64.get(), acc, bdens, bgrad);
    else
        get_fields_t(h->m32.get(), acc, bdens, bgrad);
}

void vfs_oracle_set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

int vfs_oracle_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

uint32_t vfs_oracle_hash_cell(int32_t x, int32_t y, int32_t z) { return hash_cell(x, y, z); }

int32_t vfs_oracle_cell_coord(float x, float h) { return cell_coord<float>(x, h); }

void vfs_oracle_gauss_legendre(int n, double* x, double* w) { gauss_legendre(n, x, w); }

// Grid box, SDF grid and volume map of an analytic shape (volume_map_of above).
int vfs_oracle_volume_map(int kind, const double* shape_params, float support_radius,
                          const uint32_t* res, float margin, int quad_n, float* box_size_out,
                          float* box_pos_out, float* sdf_out, float* vm_out) {
    float lo[3], hi[3];
    shape_aabb(kind, shape_params, lo, hi);
    auto fn = [&](float x, float y, float z) { return analytic_sdf(kind, shape_params, x, y, z); };
    return volume_map_of(fn, lo, hi, support_radius, res, margin, quad_n, box_size_out,
                         box_pos_out, sdf_out, vm_out);
}

// Signed distances of points to a triangle mesh (brute force over the triangles), restating
// SignedDistanceToMesh (src/util/geometry.cpp:267-328) with the pseudonormals of
// MeshPseudonormals::Build (src/util/mesh_pseudonormals.cpp:11-88). Returns -1 for a mesh with a
// degenerate triangle or an out-of-range index.
int vfs_oracle_mesh_distance(const float* vertices, uint32_t n_vertices, const uint32_t* triangles,
                             uint32_t n_triangles, const float* points, uint32_t n_points,
                             double* out) {
    OracleMesh mesh;
    if (!mesh.build(vertices, n_vertices, triangles, n_triangles)) return -1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n_points; i++)
        out[i] = mesh.signed_distance(points[3 * i], points[3 * i + 1], points[3 * i + 2]);
    return 0;
}

// Grid box, SDF grid and volume map of a triangle mesh (GenericScene::AddBoundaryObject,
// src/scenes/generic_scene.cpp:89-124), all in double like the reference.
int vfs_oracle_mesh_volume_map(const float* vertices, uint32_t n_vertices,
                               const uint32_t* triangles, uint32_t n_triangles,
                               float support_radius, const uint32_t* res, float margin,
                               int quad_n, float* box_size_out, float* box_pos_out,
                               float* sdf_out, float* vm_out) {
    OracleMesh mesh;
    if (!mesh.build(vertices, n_vertices, triangles, n_triangles)) return -1;
    auto fn = [&](float x, float y, float z) { return mesh.signed_distance(x, y, z); };
    return volume_map_of(fn, mesh.lo, mesh.hi, support_radius, res, margin, quad_n, box_size_out,
                         box_pos_out, sdf_out, vm_out);
}

}  // extern "C"
