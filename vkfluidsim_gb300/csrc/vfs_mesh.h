// Triangle-mesh boundary objects: OBJ parsing, angle-weighted pseudonormals and a bounding volume
// hierarchy on the host (the reference's LoadObjMesh, MeshPseudonormals and MeshBVH,
// src/util/mesh_loader.cpp, src/util/mesh_pseudonormals.cpp:11-88, src/util/mesh_bvh.cpp), and the
// signed-distance query the SDF grid and volume map of a mesh object are built from
// (SignedDistanceToMesh, src/util/geometry.cpp:267-328).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace vfs {

struct BvhNode {
    float lo[3], hi[3];
    int32_t first;  // leaf: first triangle; inner: left child (the right child is first + 1)
    int32_t count;  // leaf: triangle count (> 0); inner: 0
};

struct MeshHost {
    std::vector<float> pos;            // 3 per vertex
    std::vector<uint32_t> tri;         // 3 vertex indices per triangle (BVH order)
    std::vector<float> tri_normal;     // 3 per triangle
    std::vector<float> edge_normal;    // 9 per triangle: edges (0,1), (1,2), (0,2)
    std::vector<float> vertex_normal;  // 3 per vertex
    std::vector<BvhNode> nodes;        // nodes[0] is the root
    float lo[3], hi[3];                // bounds of the triangles
};

// Device view of a mesh (arrays of MeshHost uploaded as float4 / uint4 rows).
struct MeshDev {
    const float4* pos;
    const uint4* tri;
    const float4* tri_normal;
    const float4* edge_normal;  // 3 per triangle
    const float4* vertex_normal;
    const BvhNode* nodes;
};

// Parses the last object of an OBJ file (polygons triangulated as fans, vertex positions only);
// false with a message on failure.
bool load_obj(const std::string& path, std::vector<float>& pos, std::vector<uint32_t>& tri,
              std::string& err);

// Pseudonormals and BVH of a triangle soup; false with a message if it is degenerate.
bool build_mesh(const std::vector<float>& pos, const std::vector<uint32_t>& tri, MeshHost& out,
                std::string& err);

}  // namespace vfs
