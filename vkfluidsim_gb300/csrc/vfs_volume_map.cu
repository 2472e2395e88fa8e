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
// and the grid step is computed in float. Products and sums use round-to-nearest intrinsics so
// no fused multiply-add changes a threshold decision.
#include <cuda_runtime.h>
#include <stdint.h>

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

// CubicSplineKernel::W in double (src/util/kernel.cpp:22-38).
__device__ __forceinline__ double kernel_w(double r, double radius, double factor) {
    const double q = r / radius;
    if (q <= 1.0) {
        if (q <= 0.5) {
            const double q2 = dm(q, q), q3 = dm(q2, q);
            return dm(factor, da(ds(dm(6.0, q3), dm(6.0, q2)), 1.0));
        }
        return dm(factor, dm(2.0, pow(ds(1.0, q), 3.0)));
    }
    return 0.0;
}

__global__ void __launch_bounds__(128) k_volume_map(VolumeMapParams P, float* __restrict__ sdf_out,
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
    const double node_sdf = shape_sdf(P.shape, P.prm, fx, fy, fz);
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
        const double w_zero = kernel_w(0.0, (double)sr, P.w_factor);
        const float sr2 = __fmul_rn(sr, sr);
        double integral = 0.0;
        for (int a = 0; a < P.qn; a++) {
            const double wa = P.gw[a];
            const float xa = __double2float_rn(da(dm(P.c0, P.gx[a]), P.c1));
            for (int b = 0; b < P.qn; b++) {
                const double wab = dm(wa, P.gw[b]);
                const float xb = __double2float_rn(da(dm(P.c0, P.gx[b]), P.c1));
                const float xab2 = __fadd_rn(__fmul_rn(xa, xa), __fmul_rn(xb, xb));
                for (int c = 0; c < P.qn; c++) {
                    const double wabc = dm(wab, P.gw[c]);
                    const float xc = __double2float_rn(da(dm(P.c0, P.gx[c]), P.c1));
                    double f = 0.0;
                    const float len2 = __fadd_rn(xab2, __fmul_rn(xc, xc));
                    if (!(len2 > sr2)) {
                        const float px = __fadd_rn(fx, xa), py = __fadd_rn(fy, xb),
                                    pz = __fadd_rn(fz, xc);
                        const double di = shape_sdf(P.shape, P.prm, px, py, pz);
                        if (di <= 0.0)
                            f = 1.0;
                        else if (di < (double)sr)
                            f = kernel_w(di, (double)sr, P.w_factor) / w_zero;
                    }
                    integral = da(integral, dm(wabc, f));
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
    k_volume_map<<<(unsigned)blocks, 128, 0, s>>>(p, sdf, vm);
    return cudaGetLastError();
}

}  // namespace vfs
