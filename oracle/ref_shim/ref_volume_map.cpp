// Host driver of the reference's own CPU volume-map code (test infrastructure): a triangle mesh
// through MeshSDF::Init/Build (src/util/mesh_sdf.cpp:15-44) with tolerance 0 and margin 8h, then
// GenerateVolumeMap (src/util/volume_map.cpp:9-54), both grids rounded to float as
// GenericScene::AddBoundaryObject uploads them (src/scenes/generic_scene.cpp:96-118). The
// reference's util/*.cpp are compiled beside this file against glm_shim.hpp and the gfx
// stand-ins by oracle/ref_build.py.
#include <cstdint>
#include <vector>

#include "gfx/mesh.h"
#include "util/mesh_sdf.h"
#include "util/volume_map.h"

extern "C" int vfs_ref_mesh_volume_map(const float* vertices, uint32_t n_vertices,
                                       const uint32_t* triangles, uint32_t n_triangles, float h,
                                       const uint32_t res[3], float box_size[3], float box_pos[3],
                                       float* sdf_out, float* vm_out) {
    if (!vertices || !triangles || !res || n_vertices == 0 || n_triangles == 0) return 1;
    gfx::CPUMesh mesh;
    mesh.vertices.resize(n_vertices);
    for (uint32_t v = 0; v < n_vertices; v++) {
        mesh.vertices[v].pos = glm::vec3(vertices[3 * v], vertices[3 * v + 1], vertices[3 * v + 2]);
        mesh.vertices[v].uv = glm::vec2(0.0f, 0.0f);
        mesh.vertices[v].normal = glm::vec3(0.0f, 0.0f, 0.0f);
    }
    mesh.indices.assign(triangles, triangles + 3 * (size_t)n_triangles);
    mesh.position_indices = mesh.indices;  // the vertices are unique positions already
    vfs::MeshSDF sdf;
    sdf.Init(mesh, glm::uvec3(res[0], res[1], res[2]), 0.0, 8.0 * h);
    sdf.Build();
    vfs::LinearLagrangeDiscreteGrid volume_map;
    vfs::GenerateVolumeMap(sdf, h, volume_map);
    const gfx::BoundingBox box = sdf.GetBox();
    box_size[0] = box.size.x;
    box_size[1] = box.size.y;
    box_size[2] = box.size.z;
    box_pos[0] = box.pos.x;
    box_pos[1] = box.pos.y;
    box_pos[2] = box.pos.z;
    const std::vector<double>& g = sdf.GetSDF();
    const std::vector<double>& m = volume_map.GetGrid();
    for (size_t k = 0; k < g.size(); k++) sdf_out[k] = (float)g[k];
    for (size_t k = 0; k < m.size(); k++) vm_out[k] = (float)m[k];
    return 0;
}
