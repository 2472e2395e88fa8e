// Headless particle rendering into a device image: the reference's sphere-impostor particle pass
// (assets/shaders/draw/particles_3d.slang, drawn by src/gui/scene_renderer.cpp:101-109 with the
// quad of src/gui/common.cpp:24-39) re-expressed as two CUDA kernels, with no graphics API.
//
//   1. splat: one thread per particle projects its screen-facing quad (side `quad_side` in view
//      units, offset in clip space as the vertex shader does), and for every covered pixel whose
//      quad coordinates fall inside the unit disc writes (depth, particle) with a 64-bit atomicMin
//      into a visibility buffer. The depth is that of the impostor's sphere point,
//      view + depth_radius * n, like the fragment shader's SV_Depth, and the comparison is the
//      pipeline's LESS_OR_EQUAL (equal depths: the later-drawn, higher-index particle wins).
//   2. resolve: one thread per pixel recomputes the winner's normal and shades it: colour from
//      the IDL "Mac style" colour map of |v| / v_max (assets/shaders/draw/colormap.slang) times
//      the diffuse term max(0, n . normalize(0, 1, 1)), alpha 1, background (0, 0, 0, 1).
//
// Matrices are column-major 4x4 (element (row r, column c) at m[4c + r]), as glm stores them.
// Pixel (x, y) covers NDC x in [2x/W - 1, 2(x+1)/W - 1] and y likewise with row 0 at NDC y = -1
// (Vulkan's framebuffer convention); fragments with depth outside [0, 1] are clipped, and a particle
// whose quad covers more than 2^20 pixels is skipped.

#include <cuda_runtime.h>

#include <string>

#include "vfs_cuda.h"
#include "vfs_internal.h"
#include "vfs_model.h"

namespace vfs {

namespace {

// A particle whose quad covers more pixels than this (it sits practically at the camera) is not
// drawn, which bounds every splat thread's work.
constexpr long long kMaxSplatPixels = 1ll << 20;

struct RenderParams {
    float mv[16], pj[16];
    int width, height;
    float half_side;     // quad half side (view units)
    float depth_radius;  // sphere radius used for the impostor depth
    float v_max;
    float light[3];
};

__device__ __forceinline__ float4 mul4(const float* m, float x, float y, float z, float w) {
    return make_float4(m[0] * x + m[4] * y + m[8] * z + m[12] * w,
                       m[1] * x + m[5] * y + m[9] * z + m[13] * w,
                       m[2] * x + m[6] * y + m[10] * z + m[14] * w,
                       m[3] * x + m[7] * y + m[11] * z + m[15] * w);
}

// Order-preserving map of a float to an unsigned key.
__device__ __forceinline__ uint32_t depth_key(float d) {
    const uint32_t b = __float_as_uint(d);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// IDL "Mac style" colour map (the colormap-shaders formulation used by colormap.slang).
__device__ float3 mac_style(float x) {
    x = fminf(fmaxf(x, 0.0f), 1.0f);
    float h = -7.44992704834645E-01f * x + 7.47986634976377E-01f;
    const float s = 1.0f;
    const float i2 = fmodf(fmodf(x * 256.0f, 2.0f) + 2.0f, 2.0f);
    const float v = (i2 >= 0.0f && i2 < 1.0f) ? 1.0f : 254.0f / 255.0f;
    float r = v, g = v, b = v;
    h *= 6.0f;
    const int i = (int)h;
    const float f = h - (float)i;
    if (i == 1) {
        r *= 1.0f - s * f;
        b *= 1.0f - s;
    } else if (i == 2) {
        r *= 1.0f - s;
        b *= 1.0f - s * (1.0f - f);
    } else if (i == 3) {
        r *= 1.0f - s;
        g *= 1.0f - s * f;
    } else if (i == 4) {
        r *= 1.0f - s * (1.0f - f);
        g *= 1.0f - s;
    } else if (i == 5) {
        g *= 1.0f - s;
        b *= 1.0f - s * f;
    } else {
        g *= 1.0f - s * (1.0f - f);
        b *= 1.0f - s;
    }
    return make_float3(r, g, b);
}

// The quad of particle p in NDC: lower-left and upper-right corners (after each corner's own
// perspective divide), and its view-space centre. False when the particle is behind the camera.
struct Quad {
    float x0, y0, x1, y1;
    float3 view;
};

__device__ bool particle_quad(const RenderParams& R, float3 p, Quad& q) {
    const float4 v = mul4(R.mv, p.x, p.y, p.z, 1.0f);
    const float4 c = mul4(R.pj, v.x, v.y, v.z, v.w);
    const float hs = R.half_side;
    // Clip position of a corner: P (MV p) + P (corner, 1) (particles_3d.slang vertex_main).
    const float4 ll = mul4(R.pj, -hs, -hs, 0.0f, 1.0f);
    const float4 ur = mul4(R.pj, hs, hs, 0.0f, 1.0f);
    const float wl = c.w + ll.w, wu = c.w + ur.w;
    if (!(wl > 0.0f) || !(wu > 0.0f)) return false;
    q.x0 = (c.x + ll.x) / wl;
    q.y0 = (c.y + ll.y) / wl;
    q.x1 = (c.x + ur.x) / wu;
    q.y1 = (c.y + ur.y) / wu;
    q.view = make_float3(v.x, v.y, v.z);
    return q.x1 != q.x0 && q.y1 != q.y0;
}

// Disc normal at pixel (px, py) of a quad; false outside the unit disc (the fragment's discard).
__device__ __forceinline__ bool disc_normal(const RenderParams& R, const Quad& q, int px, int py,
                                            float3& n) {
    const float nx = (2.0f * (px + 0.5f)) / R.width - 1.0f;
    const float ny = (2.0f * (py + 0.5f)) / R.height - 1.0f;
    const float u = (nx - q.x0) / (q.x1 - q.x0), w = (ny - q.y0) / (q.y1 - q.y0);
    n.x = u * 2.0f - 1.0f;
    n.y = w * 2.0f - 1.0f;
    const float r2 = n.x * n.x + n.y * n.y;
    if (r2 > 1.0f) return false;
    n.z = sqrtf(1.0f - r2);
    return true;
}

__device__ __forceinline__ float impostor_depth(const RenderParams& R, const Quad& q, float3 n) {
    const float4 c = mul4(R.pj, q.view.x + R.depth_radius * n.x, q.view.y + R.depth_radius * n.y,
                          q.view.z + R.depth_radius * n.z, 1.0f);
    return c.z / c.w;
}

__global__ void k_splat(RenderParams R, uint32_t n, const float4* __restrict__ pos,
                        unsigned long long* __restrict__ vis) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    Quad q;
    if (!particle_quad(R, make_float3(p.x, p.y, p.z), q)) return;
    const float lox = fminf(q.x0, q.x1), hix = fmaxf(q.x0, q.x1);
    const float loy = fminf(q.y0, q.y1), hiy = fmaxf(q.y0, q.y1);
    // Pixels whose centres may fall inside the quad, clamped to the image.
    const float fx0 = (lox + 1.0f) * 0.5f * R.width - 0.5f, fx1 = (hix + 1.0f) * 0.5f * R.width - 0.5f;
    const float fy0 = (loy + 1.0f) * 0.5f * R.height - 0.5f, fy1 = (hiy + 1.0f) * 0.5f * R.height - 0.5f;
    if (!(fx1 >= 0.0f) || !(fy1 >= 0.0f) || !(fx0 <= R.width - 1.0f) || !(fy0 <= R.height - 1.0f)) return;
    const int x0 = max(0, (int)ceilf(fx0)), x1 = min(R.width - 1, (int)floorf(fx1));
    const int y0 = max(0, (int)ceilf(fy0)), y1 = min(R.height - 1, (int)floorf(fy1));
    if ((long long)(x1 - x0 + 1) * (long long)(y1 - y0 + 1) > kMaxSplatPixels) return;
    const unsigned long long low = 0xFFFFFFFFull - i;  // equal depths: the higher index wins
    for (int py = y0; py <= y1; py++)
        for (int px = x0; px <= x1; px++) {
            float3 nrm;
            if (!disc_normal(R, q, px, py, nrm)) continue;
            const float d = impostor_depth(R, q, nrm);
            if (!(d >= 0.0f && d <= 1.0f)) continue;
            const unsigned long long key = ((unsigned long long)depth_key(d) << 32) | low;
            atomicMin(vis + (size_t)py * R.width + px, key);
        }
}

__global__ void k_resolve(RenderParams R, uint32_t n, const float4* __restrict__ pos,
                          const float4* __restrict__ vel, const unsigned long long* __restrict__ vis,
                          uchar4* __restrict__ rgba, float* __restrict__ depth) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x;
    const int py = blockIdx.y;
    if (px >= R.width) return;
    const size_t pix = (size_t)py * R.width + px;
    const unsigned long long key = vis[pix];
    uchar4 out = make_uchar4(0, 0, 0, 255);
    float dep = 1.0f;
    if (key != ~0ull) {
        const uint32_t i = 0xFFFFFFFFu - (uint32_t)(key & 0xFFFFFFFFull);
        if (i < n) {
            const float4 p = pos[i];
            Quad q;
            float3 nrm;
            if (particle_quad(R, make_float3(p.x, p.y, p.z), q) && disc_normal(R, q, px, py, nrm)) {
                const float4 v = vel[i];
                const float speed = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
                const float3 c = mac_style(fminf(fmaxf(speed / R.v_max, 0.0f), 1.0f));
                const float diff = fmaxf(0.0f, nrm.x * R.light[0] + nrm.y * R.light[1] + nrm.z * R.light[2]);
                auto u8 = [](float x) {
                    return (unsigned char)__float2int_rn(fminf(fmaxf(x, 0.0f), 1.0f) * 255.0f);
                };
                out = make_uchar4(u8(c.x * diff), u8(c.y * diff), u8(c.z * diff), 255);
                dep = impostor_depth(R, q, nrm);
            }
        }
    }
    rgba[pix] = out;
    if (depth) depth[pix] = dep;
}

}  // namespace

int render_particles(Model& m, uint32_t scene, const float* model_view, const float* proj,
                     int width, int height, float quad_side, float depth_radius, float v_max,
                     uint8_t* rgba_host, float* depth_host) {
    if (!model_view || !proj || !rgba_host) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL argument");
    if (width < 1 || height < 1 || width > 16384 || height > 16384)
        return fail(VFS_ERR_INVALID_ARGUMENT, "image size must be in [1, 16384]^2");
    if (!(quad_side > 0.0f) || !(depth_radius >= 0.0f) || !(v_max > 0.0f))
        return fail(VFS_ERR_INVALID_ARGUMENT, "quad_side and v_max must be > 0, depth_radius >= 0");
    if (scene >= m.scenes.size()) return fail(VFS_ERR_INVALID_ARGUMENT, "scene index out of range");
    const SceneHost& sh = m.scenes[scene];
    RenderParams R;
    for (int k = 0; k < 16; k++) {
        R.mv[k] = model_view[k];
        R.pj[k] = proj[k];
    }
    R.width = width;
    R.height = height;
    R.half_side = 0.5f * quad_side;
    R.depth_radius = depth_radius;
    R.v_max = v_max;
    const float inv = 1.0f / sqrtf(2.0f);
    R.light[0] = 0.0f;
    R.light[1] = inv;
    R.light[2] = inv;
    const size_t pixels = (size_t)width * height;
    unsigned long long* vis = nullptr;
    uchar4* img = nullptr;
    float* dep = nullptr;
    int rc = VFS_OK;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == VFS_OK) rc = fail(VFS_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
        return rc == VFS_OK;
    };
    if (ok(cudaMallocAsync(&vis, pixels * 8, m.stream)) && ok(cudaMallocAsync(&img, pixels * 4, m.stream)) &&
        (!depth_host || ok(cudaMallocAsync(&dep, pixels * 4, m.stream))) &&
        ok(cudaMemsetAsync(vis, 0xFF, pixels * 8, m.stream))) {
        if (sh.n) {
            k_splat<<<(sh.n + 255) / 256, 256, 0, m.stream>>>(R, sh.n, m.pos[m.cur] + sh.off, vis);
            ok(cudaGetLastError());
        }
        if (rc == VFS_OK) {
            k_resolve<<<dim3((width + 127) / 128, height), 128, 0, m.stream>>>(
                R, sh.n, m.pos[m.cur] + sh.off, m.vel[m.cur] + sh.off, vis, img, dep);
            ok(cudaGetLastError());
        }
        if (rc == VFS_OK) ok(cudaMemcpyAsync(rgba_host, img, pixels * 4, cudaMemcpyDeviceToHost, m.stream));
        if (rc == VFS_OK && depth_host)
            ok(cudaMemcpyAsync(depth_host, dep, pixels * 4, cudaMemcpyDeviceToHost, m.stream));
    }
    if (vis) cudaFreeAsync(vis, m.stream);
    if (img) cudaFreeAsync(img, m.stream);
    if (dep) cudaFreeAsync(dep, m.stream);
    if (rc) return rc;
    return m.check_device();
}

}  // namespace vfs

using vfs::fail;

extern "C" {

int vfs_model_render_particles(vfs_model* h, const float* model_view, const float* proj,
                               int32_t width, int32_t height, float quad_side, float depth_radius,
                               float v_max, uint8_t* rgba, float* depth) {
    vfs::Model* m = vfs_model_impl(h);
    if (!m) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL model");
    return vfs::render_particles(*m, 0, model_view, proj, width, height, quad_side, depth_radius,
                                 v_max, rgba, depth);
}

int vfs_batch_render_particles(vfs_batch* h, int32_t scene, const float* model_view,
                               const float* proj, int32_t width, int32_t height, float quad_side,
                               float depth_radius, float v_max, uint8_t* rgba, float* depth) {
    vfs::Model* m = vfs_batch_impl(h);
    if (!m || scene < 0) return fail(VFS_ERR_INVALID_ARGUMENT, "NULL batch or negative scene");
    return vfs::render_particles(*m, (uint32_t)scene, model_view, proj, width, height, quad_side,
                                 depth_radius, v_max, rgba, depth);
}

}  // extern "C"
