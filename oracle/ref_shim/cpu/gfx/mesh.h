// Stand-in for the reference's gfx/mesh.h (Vulkan buffers omitted): the CPU mesh types its
// volume-map code reads, with the reference's field names (src/gfx/mesh.h:13-36): BoundingBox
// {size, pos}, Vertex {pos, uv, normal}, CPUMesh {name, vertices, indices, position_indices}.
#pragma once

#include "gfx/common.h"

namespace gfx {

struct BoundingBox {
    glm::vec3 size{0.0f};
    glm::vec3 pos{0.0f};
};

struct Vertex {
    glm::vec3 pos;
    glm::vec2 uv;
    glm::vec3 normal;
};

struct CPUMesh {
    std::string name;
    std::vector<Vertex> vertices;
    std::vector<u32> indices;
    std::vector<u32> position_indices;
};

}  // namespace gfx
