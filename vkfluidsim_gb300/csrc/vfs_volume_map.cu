// GPU generation of the SDF grid and volume map of an analytic boundary shape.
//
// Replaces the single-threaded double-precision setup loop of the reference
// (GenerateVolumeMap, src/util/volume_map.cpp:9-54, over LinearLagrangeDiscreteGrid::Init,
// src/util/discretization.cpp:16-32, with GaussLegendreQuadrature3D,
// src/util/gaussian_quadrature.cpp:2293-2334). One thread per grid node; the node's value is
//   0.8 * integral over [-h, h]^3 of gamma(sdf(x + xi)) with gamma = 1 inside the solid,
//   W(d)/W(0) for 0 < d < h, 0 otherwise, and |xi| > h contributing 0,
// skipped (0) when sdf(x) > 2h. The reference's float roundings are kept: node and quadrature
// points are rounded to float (they pass through glm::vec3 parameters), x + xi is a float sum,
// and the grid step is computed in float. Node distances (the SDF grid and the 2h test) are
// evaluated in double with round-to-nearest intrinsics, bit-identical to an unfused double
// restatement. The integrand is continuous in the distance (gamma -> 1 as d -> 0+, -> 0 as
// d -> h), so at quadrature points it is evaluated in float and only accumulated in double: the
// map then differs from an all-double evaluation by rounding only (~1e-7 relative), at FP32
// instead of FP64 throughput.
#include <cuda_runtime.h>
#include <stdint.h>

#include "vfs_mesh.h"
#include "vfs_volume_map.h"

namespace vfs {
namespace {

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

// Analytic SDFs in object-local coordinates, negative inside the solid.
__device__ __forceinline__ double shape_sdf(int shape, const double* prm, double x, double y,
                                            double z) {
    if (shape == 0) return ds(__dsqrt_rn(da(da(dm(x, x), dm(y, y)), dm(z, z))), prm[0]);
    const double qx = ds(fabs(x), prm[0]), qy = ds(fabs(y), prm[1]), qz = ds(fabs(z), prm[2]);
    const double ox = fmax(qx, 0.0), oy = fmax(qy, 0.0), oz = fmax(qz, 0.0);
    const double box = da(__dsqrt_rn(da(da(dm(ox, ox), dm(oy, oy)), dm(oz, oz))),
                          fmin(fmax(qx, fmax(qy, qz)), 0.0));
    return shape == 1 ? box : -box;
}

// ---------------------------------------------------------------- triangle meshes

enum : int { kEntV0 = 0, kEntV1, kEntV2, kEntE01, kEntE12, kEntE02, kEntF };

template <typename T>
struct Vec3T {
    T x, y, z;
};
template <typename T>
__device__ __forceinline__ Vec3T<T> vsub(Vec3T<T> a, Vec3T<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T>
__device__ __forceinline__ T vdot(Vec3T<T> a, Vec3T<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Closest point of triangle (v0, v1, v2) to p by the region classification of Eberly ("Distance
// Between Point and Triangle in 3D", Geometric Tools), the method the reference's
// DistancePointToTriangle follows: minimise |v0 + s e0 + t e1 - p|^2 over s, t >= 0, s + t <= 1.
// Returns the squared distance; (s, t) and the closest entity (vertex, edge or face) by reference.
template <typename T>
__device__ T point_triangle(Vec3T<T> p, Vec3T<T> v0, Vec3T<T> v1, Vec3T<T> v2, T& s, T& t, int& ent) {
    const Vec3T<T> e0 = vsub(v1, v0), e1 = vsub(v2, v0), d = vsub(v0, p);
    const T a00 = vdot(e0, e0), a01 = vdot(e0, e1), a11 = vdot(e1, e1);
    const T b0 = vdot(d, e0), b1 = vdot(d, e1), c = vdot(d, d);
    const T det = fmax(a00 * a11 - a01 * a01, T(0));
    s = a01 * b1 - a11 * b0;
    t = a01 * b0 - a00 * b1;
    if (s + t <= det) {
        if (s < T(0)) {
            if (t < T(0)) {  // region 4: nearest to v0 along e0 or e1
                if (b0 < T(0)) {
                    t = T(0);
                    if (-b0 >= a00) { s = T(1); ent = kEntV1; }
                    else { s = -b0 / a00; ent = kEntE01; }
                } else {
                    s = T(0);
                    if (b1 >= T(0)) { t = T(0); ent = kEntV0; }
                    else if (-b1 >= a11) { t = T(1); ent = kEntV2; }
                    else { t = -b1 / a11; ent = kEntE02; }
                }
            } else {  // region 3: edge s = 0
                s = T(0);
                if (b1 >= T(0)) { t = T(0); ent = kEntV0; }
                else if (-b1 >= a11) { t = T(1); ent = kEntV2; }
                else { t = -b1 / a11; ent = kEntE02; }
            }
        } else if (t < T(0)) {  // region 5: edge t = 0
            t = T(0);
            if (b0 >= T(0)) { s = T(0); ent = kEntV0; }
            else if (-b0 >= a00) { s = T(1); ent = kEntV1; }
            else { s = -b0 / a00; ent = kEntE01; }
        } else {  // region 0: inside the face
            const T inv = T(1) / det;
            s *= inv;
            t *= inv;
            ent = kEntF;
        }
    } else {
        if (s < T(0)) {  // region 2
            const T tmp0 = a01 + b0, tmp1 = a11 + b1;
            if (tmp1 > tmp0) {
                const T num = tmp1 - tmp0, den = a00 - T(2) * a01 + a11;
                if (num >= den) { s = T(1); t = T(0); ent = kEntV1; }
                else { s = num / den; t = T(1) - s; ent = kEntE12; }
            } else {
                s = T(0);
                if (tmp1 <= T(0)) { t = T(1); ent = kEntV2; }
                else if (b1 >= T(0)) { t = T(0); ent = kEntV0; }
                else { t = -b1 / a11; ent = kEntE02; }
            }
        } else if (t < T(0)) {  // region 6
            const T tmp0 = a01 + b1, tmp1 = a00 + b0;
            if (tmp1 > tmp0) {
                const T num = tmp1 - tmp0, den = a00 - T(2) * a01 + a11;
                if (num >= den) { t = T(1); s = T(0); ent = kEntV2; }
                else { t = num / den; s = T(1) - t; ent = kEntE12; }
            } else {
                t = T(0);
                if (tmp1 <= T(0)) { s = T(1); ent = kEntV1; }
                else if (b0 >= T(0)) { s = T(0); ent = kEntV0; }
                else { s = -b0 / a00; ent = kEntE01; }
            }
        } else {  // region 1: edge s + t = 1
            const T num = a11 + b1 - a01 - b0;
            if (num <= T(0)) { s = T(0); t = T(1); ent = kEntV2; }
            else {
                const T den = a00 - T(2) * a01 + a11;
                if (num >= den) { s = T(1); t = T(0); ent = kEntV1; }
                else { s = num / den; t = T(1) - s; ent = kEntE12; }
            }
        }
    }
    const Vec3T<T> q = {v0.x + s * e0.x + t * e1.x - p.x, v0.y + s * e0.y + t * e1.y - p.y,
                        v0.z + s * e0.z + t * e1.z - p.z};
    return vdot(q, q);
}

// Signed distance from p to the mesh (SignedDistanceToMesh): nearest triangle through the BVH
// (nearer child first, boxes farther than the best distance skipped), sign of (p - closest) .
// pseudonormal of the closest entity. T = double for grid nodes, float for quadrature points.
template <typename T>
__device__ double mesh_signed_distance(const MeshDev& M, float px, float py, float pz) {
    const Vec3T<T> p = {(T)px, (T)py, (T)pz};
    T best = T(INFINITY);
    int best_tri = -1, best_ent = kEntF;
    T best_s = T(0), best_t = T(0);
    int stack[64];
    int sp = 0;
    stack[sp++] = 0;
    auto box_d2 = [&](const BvhNode& nd) {
        T d2 = T(0);
        const T q[3] = {p.x, p.y, p.z};
        for (int k = 0; k < 3; k++) {
            const T lo = (T)nd.lo[k], hi = (T)nd.hi[k];
            const T e = q[k] < lo ? lo - q[k] : (q[k] > hi ? q[k] - hi : T(0));
            d2 += e * e;
        }
        return d2;
    };
    while (sp > 0) {
        const BvhNode nd = M.nodes[stack[--sp]];
        if (box_d2(nd) > best) continue;
        if (nd.count > 0) {
            for (int k = 0; k < nd.count; k++) {
                const int ti = nd.first + k;
                const uint4 tr = M.tri[ti];
                const float4 a = M.pos[tr.x], b = M.pos[tr.y], c = M.pos[tr.z];
                T s, t;
                int ent;
                const T d2 = point_triangle<T>(p, {(T)a.x, (T)a.y, (T)a.z}, {(T)b.x, (T)b.y, (T)b.z},
                                               {(T)c.x, (T)c.y, (T)c.z}, s, t, ent);
                if (d2 < best) {
                    best = d2;
                    best_tri = ti;
                    best_ent = ent;
                    best_s = s;
                    best_t = t;
                }
            }
        } else if (sp + 2 <= 64) {
            const BvhNode l = M.nodes[nd.first], r = M.nodes[nd.first + 1];
            const T dl = box_d2(l), dr = box_d2(r);
            if (dl <= dr) {
                stack[sp++] = nd.first + 1;
                stack[sp++] = nd.first;
            } else {
                stack[sp++] = nd.first;
                stack[sp++] = nd.first + 1;
            }
        }
    }
    if (best_tri < 0) return (double)INFINITY;
    const uint4 tr = M.tri[best_tri];
    float4 n;
    switch (best_ent) {
        case kEntV0: n = M.vertex_normal[tr.x]; break;
        case kEntV1: n = M.vertex_normal[tr.y]; break;
        case kEntV2: n = M.vertex_normal[tr.z]; break;
        case kEntE01: n = M.edge_normal[3 * best_tri]; break;
        case kEntE12: n = M.edge_normal[3 * best_tri + 1]; break;
        case kEntE02: n = M.edge_normal[3 * best_tri + 2]; break;
        default: n = M.tri_normal[best_tri];
    }
    const float4 a = M.pos[tr.x], b = M.pos[tr.y], c = M.pos[tr.z];
    const T cx = (T)a.x + best_s * ((T)b.x - (T)a.x) + best_t * ((T)c.x - (T)a.x);
    const T cy = (T)a.y + best_s * ((T)b.y - (T)a.y) + best_t * ((T)c.y - (T)a.y);
    const T cz = (T)a.z + best_s * ((T)b.z - (T)a.z) + best_t * ((T)c.z - (T)a.z);
    const T u = (p.x - cx) * (T)n.x + (p.y - cy) * (T)n.y + (p.z - cz) * (T)n.z;
    const double d = sqrt((double)best);
    return u >= T(0) ? d : -d;
}

struct MeshSdf {
    MeshDev m;
    __device__ double node(float x, float y, float z) const { return mesh_signed_distance<double>(m, x, y, z); }
    // Quadrature points: the integrand is continuous in the distance (1 at d = 0+, 0 at d = h),
    // so the float query changes the integral only by rounding.
    __device__ float point(float x, float y, float z) const { return (float)mesh_signed_distance<float>(m, x, y, z); }
};

__global__ void k_mesh_distance(MeshDev M, const float* __restrict__ pts, uint32_t n,
                                double* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = mesh_signed_distance<double>(M, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
}

// The analytic SDFs in float, for quadrature points.
__device__ __forceinline__ float shape_sdf_f(int shape, const float* prm, float x, float y, float z) {
    if (shape == 0) return sqrtf(x * x + y * y + z * z) - prm[0];
    const float qx = fabsf(x) - prm[0], qy = fabsf(y) - prm[1], qz = fabsf(z) - prm[2];
    const float ox = fmaxf(qx, 0.0f), oy = fmaxf(qy, 0.0f), oz = fmaxf(qz, 0.0f);
    const float box = sqrtf(ox * ox + oy * oy + oz * oz) + fminf(fmaxf(qx, fmaxf(qy, qz)), 0.0f);
    return shape == 1 ? box : -box;
}

struct AnalyticSdf {
    int shape;
    double prm[3];
    float prmf[3];
    __device__ double node(float x, float y, float z) const { return shape_sdf(shape, prm, x, y, z); }
    __device__ float point(float x, float y, float z) const { return shape_sdf_f(shape, prmf, x, y, z); }
};

template <typename Sdf>
__global__ void __launch_bounds__(128) k_volume_map(VolumeMapParams P, Sdf sdf, float* __restrict__ sdf_out,
                                                    float* __restrict__ vm_out) {
    const uint64_t total = (uint64_t)P.res[0] * P.res[1] * P.res[2];
    const uint64_t lin = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (lin >= total) return;
    const uint32_t i = (uint32_t)(lin % P.res[0]);
    const uint32_t j = (uint32_t)((lin / P.res[0]) % P.res[1]);
    const uint32_t k = (uint32_t)(lin / ((uint64_t)P.res[0] * P.res[1]));
    const float fx = __double2float_rn(da(dm(P.step[0], (double)i), (double)P.dmin[0]));
    const float fy = __double2float_rn(da(dm(P.step[1], (double)j), (double)P.dmin[1]));
    const float fz = __double2float_rn(da(dm(P.step[2], (double)k), (double)P.dmin[2]));
    const double node_sdf = sdf.node(fx, fy, fz);
    sdf_out[lin] = __double2float_rn(node_sdf);
    double value = 0.0;
    const float sr = P.h;
    // sdf is 1-Lipschitz, so below -h (with a margin for the float rounding of x + xi) every
    // quadrature point is inside the solid and the node takes the precomputed full-ball value.
    const double deep = -((double)sr + 4e-6 * (1.0 + fabs((double)fx) + fabs((double)fy) +
                                               fabs((double)fz)));
    if (node_sdf < deep) {
        value = P.full_ball;
    } else if (!(node_sdf > 2.0 * (double)sr)) {
        // Integrand gamma(d) = 1 inside, W(d)/W(0) for 0 < d < h, else 0: continuous in d, so it is
        // evaluated in float (FP32 throughput) and accumulated with the weights in double.
        const float sr2 = __fmul_rn(sr, sr);
        const float inv_sr = 1.0f / sr;
        double integral = 0.0;
        for (int a = 0; a < P.qn; a++) {
            const double wa = P.gw[a];
            const float xa = P.gxf[a];
            for (int b = 0; b < P.qn; b++) {
                const double wab = dm(wa, P.gw[b]);
                const float xb = P.gxf[b];
                const float xab2 = __fadd_rn(__fmul_rn(xa, xa), __fmul_rn(xb, xb));
                const float px = __fadd_rn(fx, xa), py = __fadd_rn(fy, xb);
                for (int c = 0; c < P.qn; c++) {
                    const float xc = P.gxf[c];
                    float f = 0.0f;
                    const float len2 = __fadd_rn(xab2, __fmul_rn(xc, xc));
                    if (!(len2 > sr2)) {
                        const float di = sdf.point(px, py, __fadd_rn(fz, xc));
                        if (di <= 0.0f) {
                            f = 1.0f;
                        } else if (di < sr) {
                            const float q = di * inv_sr;
                            const float t = 1.0f - q;
                            f = q <= 0.5f ? 6.0f * q * q * q - 6.0f * q * q + 1.0f : 2.0f * t * t * t;
                        }
                    }
                    integral = fma(dm(wab, P.gw[c]), (double)f, integral);
                }
            }
        }
        integral = dm(integral, dm(dm(P.c0, P.c0), P.c0));
        value = dm(0.8, integral);
    }
    vm_out[lin] = __double2float_rn(value);
}

}  // namespace

double volume_map_full_ball(const VolumeMapParams& p) {
    const float sr = p.h;
    const float sr2 = sr * sr;
    double integral = 0.0;
    for (int a = 0; a < p.qn; a++) {
        const double wa = p.gw[a];
        const float xa = (float)(p.c0 * p.gx[a] + p.c1);
        for (int b = 0; b < p.qn; b++) {
            const double wab = wa * p.gw[b];
            const float xb = (float)(p.c0 * p.gx[b] + p.c1);
            const float xab2 = xa * xa + xb * xb;
            for (int c = 0; c < p.qn; c++) {
                const double wabc = wab * p.gw[c];
                const float xc = (float)(p.c0 * p.gx[c] + p.c1);
                const float len2 = xab2 + xc * xc;
                integral = integral + wabc * (!(len2 > sr2) ? 1.0 : 0.0);
            }
        }
    }
    integral = integral * ((p.c0 * p.c0) * p.c0);
    return 0.8 * integral;
}

cudaError_t launch_volume_map(const VolumeMapParams& p, float* sdf, float* vm, cudaStream_t s) {
    const uint64_t total = (uint64_t)p.res[0] * p.res[1] * p.res[2];
    if (total == 0) return cudaSuccess;
    const uint64_t blocks = (total + 127) / 128;
    AnalyticSdf a{p.shape, {p.prm[0], p.prm[1], p.prm[2]},
                  {(float)p.prm[0], (float)p.prm[1], (float)p.prm[2]}};
    k_volume_map<<<(unsigned)blocks, 128, 0, s>>>(p, a, sdf, vm);
    return cudaGetLastError();
}

cudaError_t launch_mesh_volume_map(const VolumeMapParams& p, const MeshDev& mesh, float* sdf,
                                   float* vm, cudaStream_t s) {
    const uint64_t total = (uint64_t)p.res[0] * p.res[1] * p.res[2];
    if (total == 0) return cudaSuccess;
    const uint64_t blocks = (total + 127) / 128;
    MeshSdf m{mesh};
    k_volume_map<<<(unsigned)blocks, 128, 0, s>>>(p, m, sdf, vm);
    return cudaGetLastError();
}

cudaError_t launch_mesh_distance(const MeshDev& mesh, const float* points, uint32_t n,
                                 double* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_mesh_distance<<<(n + 127) / 128, 128, 0, s>>>(mesh, points, n, out);
    return cudaGetLastError();
}

}  // namespace vfs
