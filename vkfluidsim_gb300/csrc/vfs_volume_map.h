// GPU SDF + volume-map generation for analytic boundary shapes and triangle meshes.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vfs {

constexpr int kMaxQuadrature = 32;

struct VolumeMapParams {
    int shape;          // 0 sphere, 1 solid box, 2 container
    double prm[3];      // radius or half extents
    float h;            // support radius
    uint32_t res[3];
    float dmin[3];      // grid origin (float, like the reference's AABB)
    double step[3];     // grid step, computed in float then widened
    int qn;             // Gauss-Legendre points per axis
    double gx[kMaxQuadrature], gw[kMaxQuadrature];
    float gxf[kMaxQuadrature];  // quadrature coordinates c0 * gx + c1 rounded to float (the points' offsets)
    double c0, c1;      // integration-domain half width and centre
    double w_factor;    // 8 / (pi h^3) in double
    double full_ball;   // the integral when every quadrature point lies inside the solid
};

// Quadrature sum of a node whose whole h-ball lies inside the solid (integrand 1 wherever
// |xi| <= h), accumulated in the kernel's order so it equals the per-node sum bit for bit.
double volume_map_full_ball(const VolumeMapParams& p);

cudaError_t launch_volume_map(const VolumeMapParams& p, float* sdf, float* vm, cudaStream_t s);

struct MeshDev;
// The same grids for a triangle mesh (p.shape unused): node SDF values from the mesh's exact
// signed distance in double, quadrature points in float.
cudaError_t launch_mesh_volume_map(const VolumeMapParams& p, const MeshDev& mesh, float* sdf,
                                   float* vm, cudaStream_t s);
// Signed distances of n points (3 floats each, device) to the mesh, in double.
cudaError_t launch_mesh_distance(const MeshDev& mesh, const float* points, uint32_t n,
                                 double* out, cudaStream_t s);

}  // namespace vfs
