// Density field on a grid and the density raymarch, with no graphics API.
//
//   k_density_grid  the SPH density rho(x) = sum_j m W(|x - x_j|) (CubicSpline,
//                   kernels_3d.slang:62-76) of the current particles at the nodes of a regular
//                   grid: one thread per particle adds its kernel to every node within h
//                   (float atomics, so the summation order, and the last bits, vary run to run).
//   k_raymarch      assets/shaders/draw/raymarch.slang as DensityRaymarchDrawPipeline::Draw
//                   (src/pipelines/raymarch_pipeline.cpp:62-115) uses it: the field's bounding box
//                   is drawn with culling off and a LESS_OR_EQUAL depth test, so every pixel whose
//                   ray meets the box starts at the nearest face it sees (the entry face from
//                   outside, the exit face from inside); from there it steps `step` world units at
//                   a time, at most n_steps times while inside the box, adding
//                   step * colormap(d * color_scale) * d * emission (colormap = the IDL "Mac style"
//                   map with alpha 1; reference values 0.05, 1000, 5, 200). The fragment colour is
//                   clamped to [0, 1] (the reference's B8G8R8A8_UNORM draw image) and alpha-blended
//                   over the image: rgb = src.rgb src.a + dst.rgb (1 - src.a),
//                   a = src.a + dst.a (1 - src.a) (GraphicsPipelineBuilder::SetBlendingAlphaBlend,
//                   src/gfx/vk_util.cpp:343-356). The 8-bit quantisation of that image is not applied.
//
// The field is sampled like the reference's Sampler3D: normalised coordinates
// uvw = 0.5 (p - centre) / half + 0.5, texel centres at (i + 0.5) / n, trilinear weights in full
// float precision (hardware filtering uses fixed-point weights), and wrap-around addressing (the
// zero-initialised VkSamplerCreateInfo of model_render_scene.cpp:191-198 selects REPEAT).
// Matrices are column-major 4x4 (glm layout); pixel (x, y) is sampled at its centre, row 0 at
// NDC y = -1 (Vulkan's framebuffer convention), as in the particle renderer.
#include <cmath>
#include <string>

#include "vfs_internal.h"
#include "vfs_model.h"

namespace vfs {
namespace {

struct GridSpec {
    float lo[3], step[3], inv_step[3];
    int res[3];
    float h, h2, inv_h, m_sigma;  // m_sigma = mass * 8 / (pi h^3)
};

// Nodes along one axis that may lie within h of coordinate x (the distance test decides).
__device__ __forceinline__ void node_range(const GridSpec& G, int a, float x, int& i0, int& i1) {
    if (G.res[a] == 1) {
        i0 = i1 = 0;
        return;
    }
    const float lo = (x - G.h - G.lo[a]) * G.inv_step[a];
    const float hi = (x + G.h - G.lo[a]) * G.inv_step[a];
    i0 = max(0, (int)ceilf(fmaxf(lo - 1e-4f, -1.0f)));
    i1 = min(G.res[a] - 1, (int)floorf(fminf(hi + 1e-4f, (float)G.res[a])));
}

__global__ void __launch_bounds__(256)
    k_density_grid(GridSpec G, uint32_t n, const float4* __restrict__ pos, float* __restrict__ grid) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const float4 x = __ldg(pos + j);
    int ix0, ix1, iy0, iy1, iz0, iz1;
    node_range(G, 0, x.x, ix0, ix1);
    node_range(G, 1, x.y, iy0, iy1);
    node_range(G, 2, x.z, iz0, iz1);
    for (int k = iz0; k <= iz1; k++) {
        const float dz = fmaf((float)k, G.step[2], G.lo[2]) - x.z;
        for (int jy = iy0; jy <= iy1; jy++) {
            const float dy = fmaf((float)jy, G.step[1], G.lo[1]) - x.y;
            const float dyz = dy * dy + dz * dz;
            if (dyz > G.h2) continue;
            float* row = grid + ((size_t)k * G.res[1] + jy) * G.res[0];
            for (int i = ix0; i <= ix1; i++) {
                const float dx = fmaf((float)i, G.step[0], G.lo[0]) - x.x;
                const float r2 = dx * dx + dyz;
                if (r2 > G.h2) continue;
                const float q = sqrtf(r2) * G.inv_h;
                float w;
                if (q <= 0.5f) {
                    const float q2 = q * q;
                    w = 6.0f * q2 * q - 6.0f * q2 + 1.0f;
                } else {
                    const float t = 1.0f - q;
                    w = 2.0f * t * t * t;
                }
                atomicAdd(row + i, G.m_sigma * w);
            }
        }
    }
}

// IDL "Mac style" colour map with alpha 1 (colormap.slang), as the particle renderer uses it.
__device__ float3 mac_style_rgb(float x) {
    x = fminf(fmaxf(x, 0.0f), 1.0f);
    float h = __fadd_rn(__fmul_rn(-7.44992704834645E-01f, x), 7.47986634976377E-01f);
    const float i2 = fmodf(fmodf(__fmul_rn(x, 256.0f), 2.0f) + 2.0f, 2.0f);
    const float v = (i2 >= 0.0f && i2 < 1.0f) ? 1.0f : 254.0f / 255.0f;
    float r = v, g = v, b = v;
    h = __fmul_rn(h, 6.0f);
    const int i = (int)h;
    const float f = __fsub_rn(h, (float)i);
    // s = 1: 1 - s f and 1 - s (1 - f), rounded as written.
    const float f1 = __fsub_rn(1.0f, f);
    const float f2 = __fsub_rn(1.0f, f1);
    if (i == 1) {
        r = __fmul_rn(r, f1);
        b = 0.0f;
    } else if (i == 2) {
        r = 0.0f;
        b = __fmul_rn(b, f2);
    } else if (i == 3) {
        r = 0.0f;
        g = __fmul_rn(g, f1);
    } else if (i == 4) {
        r = __fmul_rn(r, f2);
        g = 0.0f;
    } else if (i == 5) {
        g = 0.0f;
        b = __fmul_rn(b, f1);
    } else {
        g = __fmul_rn(g, f2);
        b = 0.0f;
    }
    return make_float3(r, g, b);
}

struct RayParams {
    float inv_vp[16];  // (proj * view)^-1, column-major
    float cam[3];      // camera position (view^-1 applied to the origin)
    float lo[3], hi[3], center[3], half[3];
    int width, height;
    int nx, ny, nz;
    float step, color_scale, emission;
    int n_steps;
};

__device__ __forceinline__ float3 unproject(const float* m, float x, float y, float z) {
    const float X = m[0] * x + m[4] * y + m[8] * z + m[12];
    const float Y = m[1] * x + m[5] * y + m[9] * z + m[13];
    const float Z = m[2] * x + m[6] * y + m[10] * z + m[14];
    const float W = m[3] * x + m[7] * y + m[11] * z + m[15];
    return make_float3(X / W, Y / W, Z / W);
}

// Index of texel i along an axis of n texels under wrap-around addressing.
__device__ __forceinline__ int wrap(int i, int n) {
    const int r = i % n;
    return r < 0 ? r + n : r;
}

// Trilinear sample at normalised coordinate u (texel centres at (i + 0.5) / n).
__device__ float sample_field(const RayParams& P, const float* __restrict__ f, float u, float v,
                              float w) {
    const float tu = __fsub_rn(__fmul_rn(u, (float)P.nx), 0.5f);
    const float tv = __fsub_rn(__fmul_rn(v, (float)P.ny), 0.5f);
    const float tw = __fsub_rn(__fmul_rn(w, (float)P.nz), 0.5f);
    const float fu = floorf(tu), fv = floorf(tv), fw = floorf(tw);
    const float au = __fsub_rn(tu, fu), av = __fsub_rn(tv, fv), aw = __fsub_rn(tw, fw);
    const int i0 = wrap((int)fu, P.nx), i1 = wrap((int)fu + 1, P.nx);
    const int j0 = wrap((int)fv, P.ny), j1 = wrap((int)fv + 1, P.ny);
    const int k0 = wrap((int)fw, P.nz), k1 = wrap((int)fw + 1, P.nz);
    auto at = [&](int i, int j, int k) { return __ldg(f + ((size_t)k * P.ny + j) * P.nx + i); };
    auto lerp = [](float a, float b, float t) { return __fmaf_rn(t, __fsub_rn(b, a), a); };
    const float c00 = lerp(at(i0, j0, k0), at(i1, j0, k0), au);
    const float c10 = lerp(at(i0, j1, k0), at(i1, j1, k0), au);
    const float c01 = lerp(at(i0, j0, k1), at(i1, j0, k1), au);
    const float c11 = lerp(at(i0, j1, k1), at(i1, j1, k1), au);
    return lerp(lerp(c00, c10, av), lerp(c01, c11, av), aw);
}


__global__ void __launch_bounds__(128)
    k_raymarch(RayParams P, const float* __restrict__ field, float4* __restrict__ img) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y;
    if (px >= P.width) return;
    const float nx = __fsub_rn(__fdiv_rn(2.0f * (float)px + 1.0f, (float)P.width), 1.0f);
    const float ny = __fsub_rn(__fdiv_rn(2.0f * (float)py + 1.0f, (float)P.height), 1.0f);
    const float3 a = unproject(P.inv_vp, nx, ny, 0.0f), b = unproject(P.inv_vp, nx, ny, 1.0f);
    float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    const float il = 1.0f / sqrtf(dx * dx + dy * dy + dz * dz);
    dx *= il;
    dy *= il;
    dz *= il;
    // Slab test of the ray cam + t d against the box.
    float t0 = -INFINITY, t1 = INFINITY;
    const float o[3] = {P.cam[0], P.cam[1], P.cam[2]}, d[3] = {dx, dy, dz};
    for (int k = 0; k < 3; k++) {
        if (d[k] != 0.0f) {
            const float ta = (P.lo[k] - o[k]) / d[k], tb = (P.hi[k] - o[k]) / d[k];
            t0 = fmaxf(t0, fminf(ta, tb));
            t1 = fminf(t1, fmaxf(ta, tb));
        } else if (o[k] < P.lo[k] || o[k] > P.hi[k]) {
            t1 = -INFINITY;
        }
    }
    if (!(t1 >= fmaxf(t0, 0.0f))) return;  // no face of the box under this pixel
    const float tf = t0 > 0.0f ? t0 : t1;   // the face the depth test keeps
    // The face point (the rasterised fragment's world position).
    float x = fmaf(tf, dx, o[0]), y = fmaf(tf, dy, o[1]), z = fmaf(tf, dz, o[2]);
    float lr = 0.0f, lg = 0.0f, lb = 0.0f, la = 0.0f;
    const float sdx = __fmul_rn(dx, P.step), sdy = __fmul_rn(dy, P.step), sdz = __fmul_rn(dz, P.step);
    for (int s = 0; s < P.n_steps; s++) {
        // IsInsideAABB and DensityAtPosition on p / field_size (here relative to the box centre).
        float ax = __fdiv_rn(__fsub_rn(x, P.center[0]), P.half[0]);
        float ay = __fdiv_rn(__fsub_rn(y, P.center[1]), P.half[1]);
        float az = __fdiv_rn(__fsub_rn(z, P.center[2]), P.half[2]);
        if (s == 0) {  // the face point itself, on the box up to rounding
            ax = fminf(fmaxf(ax, -1.0f), 1.0f);
            ay = fminf(fmaxf(ay, -1.0f), 1.0f);
            az = fminf(fmaxf(az, -1.0f), 1.0f);
        }
        if (!(ax >= -1.0f && ax <= 1.0f && ay >= -1.0f && ay <= 1.0f && az >= -1.0f && az <= 1.0f))
            break;
        const float dval = sample_field(P, field, __fmul_rn(0.5f, __fadd_rn(ax, 1.0f)),
                                        __fmul_rn(0.5f, __fadd_rn(ay, 1.0f)),
                                        __fmul_rn(0.5f, __fadd_rn(az, 1.0f)));
        const float3 c = mac_style_rgb(__fmul_rn(dval, P.color_scale));
        // light += step * (colormap(d * 5) * d * 200), channel by channel (alpha: 1 * d * 200).
        lr = __fadd_rn(lr, __fmul_rn(P.step, __fmul_rn(__fmul_rn(c.x, dval), P.emission)));
        lg = __fadd_rn(lg, __fmul_rn(P.step, __fmul_rn(__fmul_rn(c.y, dval), P.emission)));
        lb = __fadd_rn(lb, __fmul_rn(P.step, __fmul_rn(__fmul_rn(c.z, dval), P.emission)));
        la = __fadd_rn(la, __fmul_rn(P.step, __fmul_rn(dval, P.emission)));
        x = __fadd_rn(x, sdx);
        y = __fadd_rn(y, sdy);
        z = __fadd_rn(z, sdz);
    }
    const float sr = fminf(fmaxf(lr, 0.0f), 1.0f), sg = fminf(fmaxf(lg, 0.0f), 1.0f);
    const float sb = fminf(fmaxf(lb, 0.0f), 1.0f), sa = fminf(fmaxf(la, 0.0f), 1.0f);
    float4* q = img + (size_t)py * P.width + px;
    const float4 dst = *q;
    const float ia = __fsub_rn(1.0f, sa);
    *q = make_float4(__fmaf_rn(dst.x, ia, __fmul_rn(sr, sa)), __fmaf_rn(dst.y, ia, __fmul_rn(sg, sa)),
                     __fmaf_rn(dst.z, ia, __fmul_rn(sb, sa)), __fmaf_rn(dst.w, ia, sa));
}

// Inverse of a column-major 4x4 matrix by Gauss-Jordan elimination with partial pivoting, in
// double; false when singular.
bool invert4(const double* m, double* out) {
    double a[4][8];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            a[r][c] = m[4 * c + r];
            a[r][4 + c] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; c++) {
        int piv = c;
        for (int r = c + 1; r < 4; r++)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (a[piv][c] == 0.0) return false;
        if (piv != c)
            for (int k = 0; k < 8; k++) std::swap(a[c][k], a[piv][k]);
        const double inv = 1.0 / a[c][c];
        for (int k = 0; k < 8; k++) a[c][k] *= inv;
        for (int r = 0; r < 4; r++) {
            if (r == c) continue;
            const double f = a[r][c];
            if (f == 0.0) continue;
            for (int k = 0; k < 8; k++) a[r][k] -= f * a[c][k];
        }
    }
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) out[4 * c + r] = a[r][4 + c];
    return true;
}

// Column-major product a * b.
void mul4x4(const double* a, const double* b, double* out) {
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            double s = 0.0;
            for (int k = 0; k < 4; k++) s += a[4 * k + r] * b[4 * c + k];
            out[4 * c + r] = s;
        }
}

// Per-particle node boxes larger than this (a grid far finer than h) are rejected.
constexpr double kMaxNodesPerParticle = double(1 << 21);

}  // namespace

int density_grid(Model& m, uint32_t scene, const float* lo, const float* hi, const int32_t* res,
                 float* grid_out) {
    if (!lo || !hi || !res || !grid_out) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (scene >= m.scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    const SceneHost& sh = m.scenes[scene];
    const SceneParams& sp = sh.params;
    GridSpec G;
    size_t nodes = 1;
    double box = 1.0;
    for (int a = 0; a < 3; a++) {
        if (res[a] < 1 || res[a] > 4096) return fail(VFS_ERR_INVALID_ARGUMENT, "grid resolution must be in [1, 4096]");
        if (!(hi[a] >= lo[a])) return fail(VFS_ERR_INVALID_ARGUMENT, "grid box needs hi >= lo");
        if (res[a] > 1 && !(hi[a] > lo[a])) return fail(VFS_ERR_INVALID_ARGUMENT, "grid box is flat along a resolved axis");
        G.lo[a] = lo[a];
        G.res[a] = res[a];
        G.step[a] = res[a] > 1 ? (hi[a] - lo[a]) / (float)(res[a] - 1) : 0.0f;
        G.inv_step[a] = res[a] > 1 ? 1.0f / G.step[a] : 0.0f;
        nodes *= (size_t)res[a];
        box *= res[a] > 1 ? std::min<double>(res[a], 2.0 * sp.h / G.step[a] + 2.0) : 1.0;
    }
    if (box > kMaxNodesPerParticle) return fail(VFS_ERR_INVALID_ARGUMENT, "grid too fine for the smoothing radius");
    G.h = sp.h;
    G.h2 = sp.h2;
    G.inv_h = sp.inv_h;
    G.m_sigma = sp.mass * sp.cubic;
    float* dst = static_cast<float*>(device_alias(grid_out));
    float* tmp = nullptr;
    int rc = VFS_OK;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == VFS_OK) rc = fail(VFS_ERR_CUDA, std::string("density grid: ") + cudaGetErrorString(e));
        return rc == VFS_OK;
    };
    // Host-memory outputs are accumulated on the device and copied once (no atomics over the
    // host link).
    cudaPointerAttributes attr{};
    const bool on_device = dst && cudaPointerGetAttributes(&attr, grid_out) == cudaSuccess &&
                           attr.type == cudaMemoryTypeDevice;
    cudaGetLastError();
    if (!on_device) {
        if (!ok(cudaMallocAsync(&tmp, nodes * 4, m.stream))) return rc;
        dst = tmp;
    }
    if (ok(cudaMemsetAsync(dst, 0, nodes * 4, m.stream)) && sh.n) {
        k_density_grid<<<(sh.n + 255) / 256, 256, 0, m.stream>>>(G, sh.n, m.pos[m.cur] + sh.off, dst);
        ok(cudaGetLastError());
    }
    if (rc == VFS_OK && tmp) ok(cudaMemcpyAsync(grid_out, tmp, nodes * 4, cudaMemcpyDefault, m.stream));
    if (tmp) cudaFreeAsync(tmp, m.stream);
    if (rc) return rc;
    return m.check_device();
}

}  // namespace vfs

namespace vfs {

int render_density_raymarch(const float* field, const int32_t* res, const float* center,
                            const float* half_extent, const float* view, const float* proj,
                            int width, int height, float step, int n_steps, float color_scale,
                            float emission, float* rgba) {
    if (!field || !res || !center || !half_extent || !view || !proj || !rgba)
        return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (width < 1 || height < 1 || width > 16384 || height > 16384)
        return fail(VFS_ERR_INVALID_ARGUMENT, "image size must be in [1, 16384]^2");
    if (!(step > 0.0f) || n_steps < 0 || n_steps > (1 << 24))
        return fail(VFS_ERR_INVALID_ARGUMENT, "step must be > 0 and n_steps in [0, 2^24]");
    RayParams P;
    size_t cells = 1;
    for (int a = 0; a < 3; a++) {
        if (res[a] < 1 || res[a] > 4096) return fail(VFS_ERR_INVALID_ARGUMENT, "field resolution must be in [1, 4096]");
        if (!(half_extent[a] > 0.0f)) return fail(VFS_ERR_INVALID_ARGUMENT, "half_extent must be > 0");
        cells *= (size_t)res[a];
        P.center[a] = center[a];
        P.half[a] = half_extent[a];
        P.lo[a] = center[a] - half_extent[a];
        P.hi[a] = center[a] + half_extent[a];
    }
    double v[16], pj[16], vp[16], ivp[16], iv[16];
    for (int k = 0; k < 16; k++) {
        v[k] = view[k];
        pj[k] = proj[k];
    }
    mul4x4(pj, v, vp);
    if (!invert4(vp, ivp) || !invert4(v, iv)) return fail(VFS_ERR_INVALID_ARGUMENT, "singular view or projection matrix");
    for (int k = 0; k < 16; k++) P.inv_vp[k] = (float)ivp[k];
    for (int a = 0; a < 3; a++) P.cam[a] = (float)(iv[12 + a] / iv[15]);
    P.width = width;
    P.height = height;
    P.nx = res[0];
    P.ny = res[1];
    P.nz = res[2];
    P.step = step;
    P.n_steps = n_steps;
    P.color_scale = color_scale;
    P.emission = emission;
    // Inputs and the image are used in place when the device can reach them (device or
    // page-locked memory), else staged.
    cudaStream_t s = cudaStreamPerThread;
    const size_t pixels = (size_t)width * height;
    const float* d_field = static_cast<const float*>(device_alias(field));
    float* d_img = static_cast<float*>(device_alias(rgba));
    float *f_tmp = nullptr, *i_tmp = nullptr;
    int rc = VFS_OK;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == VFS_OK) rc = fail(VFS_ERR_CUDA, std::string("raymarch: ") + cudaGetErrorString(e));
        return rc == VFS_OK;
    };
    if (!d_field && ok(cudaMallocAsync(&f_tmp, cells * 4, s)) &&
        ok(cudaMemcpyAsync(f_tmp, field, cells * 4, cudaMemcpyHostToDevice, s)))
        d_field = f_tmp;
    if (rc == VFS_OK && !d_img && ok(cudaMallocAsync(&i_tmp, pixels * 16, s)) &&
        ok(cudaMemcpyAsync(i_tmp, rgba, pixels * 16, cudaMemcpyHostToDevice, s)))
        d_img = i_tmp;
    if (rc == VFS_OK) {
        k_raymarch<<<dim3((width + 127) / 128, height), 128, 0, s>>>(P, d_field, reinterpret_cast<float4*>(d_img));
        ok(cudaGetLastError());
    }
    if (rc == VFS_OK && i_tmp) ok(cudaMemcpyAsync(rgba, i_tmp, pixels * 16, cudaMemcpyDeviceToHost, s));
    if (f_tmp) cudaFreeAsync(f_tmp, s);
    if (i_tmp) cudaFreeAsync(i_tmp, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    if (rc == VFS_OK && e != cudaSuccess) rc = fail(VFS_ERR_CUDA, std::string("raymarch: ") + cudaGetErrorString(e));
    return rc;
}

}  // namespace vfs

using vfs::fail;

extern "C" {

int vfs_model_density_grid(vfs_model* h, const float* lo, const float* hi, const int32_t* res,
                           float* grid) {
    vfs::Model* m = vfs_model_impl(h);
    if (!m) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL model");
    return vfs::density_grid(*m, 0, lo, hi, res, grid);
}

int vfs_batch_density_grid(vfs_batch* h, int32_t scene, const float* lo, const float* hi,
                           const int32_t* res, float* grid) {
    vfs::Model* m = vfs_batch_impl(h);
    if (!m || scene < 0) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL batch or negative scene");
    return vfs::density_grid(*m, (uint32_t)scene, lo, hi, res, grid);
}

int vfs_render_density_raymarch(const float* field, const int32_t* res, const float* center,
                                const float* half_extent, const float* view, const float* proj,
                                int32_t width, int32_t height, float step, int32_t n_steps,
                                float color_scale, float emission, float* rgba) {
    return vfs::render_density_raymarch(field, res, center, half_extent, view, proj, width, height,
                                        step, n_steps, color_scale, emission, rgba);
}

}  // extern "C"
