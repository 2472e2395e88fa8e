// Drives the C++ adapter include/vfs_gb300_model.hpp the way the reference's code would: parameter
// blocks with the reference's field names (stand-ins for vfs::SimulationParameters,
// vfs::SPHModel::Parameters, vfs::WCSPHWithBoundaryModel::Parameters and glm::vec3), a jittered
// lattice set with SetParticleState, one Step, then CopyDataBuffers and the spatial hash's
// buffers written to a binary file for the test to compare with the oracle; then a second model
// takes the same lattice through StepHost (the same round trip in one call) and its positions,
// velocities and densities are appended.
// Usage: adapter_check <output file>. Exit codes: 0 done, 3 the library reported an error (no
// CUDA device, for instance), 2 bad usage.
#include <cstdio>
#include <exception>
#include <vector>

#include "vfs_gb300_model.hpp"

namespace ref {
struct vec3 {
    float x, y, z;
};
struct BoundingBox {
    vec3 size;
    vec3 pos;
};
struct SimulationParameters {
    vec3 gravity;
    float smooth_radius;
};
struct SPHParameters {
    float time_scale;
    int iterations;
    int n_particles;
    float fixed_dt;
    float target_density;
    BoundingBox bounding_box;
};
struct WCSPHParameters {
    float wall_stiffness;
    float stiffness;
    float expoent;
    float viscosity_strenght;
};
}  // namespace ref

int main(int argc, char** argv) {
    if (argc != 2) return 2;
    const uint32_t dims[3] = {8, 8, 8};
    const float origin[3] = {0.0f, 0.0f, 0.0f};
    const uint32_t n = dims[0] * dims[1] * dims[2];
    std::vector<ref::vec3> pos(n), vel(n, ref::vec3{0.0f, 0.0f, 0.0f});
    if (vfs_generate_lattice(dims, origin, 0.02f, 0.1f, 0, &pos[0].x) != VFS_OK) return 3;
    std::vector<ref::vec3> pos2 = pos, vel2 = vel;
    const ref::SimulationParameters g{{0.0f, 0.0f, -9.81f}, 0.04f};
    const ref::SPHParameters p{1.0f, 1, (int)n, 2e-4f, 1000.0f, {{0.4f, 0.4f, 0.4f}, {0.0f, 0.0f, 0.0f}}};
    const ref::WCSPHParameters w{1e4f, 50.0f, 7.0f, 0.01f};
    try {
        vfs_gb300::GB300WCSPHModel<ref::SimulationParameters, ref::SPHParameters, ref::WCSPHParameters>
            model(g, p, w);
        model.SetParticleState(pos, vel);
        model.Step();
        model.Synchronize();
        std::vector<float> dens;
        std::vector<uint32_t> keys, perm, offs;
        model.CopyDataBuffers(pos, vel, dens);
        model.GetNeighborArrays(keys, perm, offs);
        FILE* f = std::fopen(argv[1], "wb");
        if (!f) return 2;
        std::fwrite(&n, 4, 1, f);
        std::fwrite(pos.data(), 12, n, f);
        std::fwrite(vel.data(), 12, n, f);
        std::fwrite(dens.data(), 4, n, f);
        std::fwrite(keys.data(), 4, n, f);
        std::fwrite(perm.data(), 4, n, f);
        std::fwrite(offs.data(), 4, n, f);
        vfs_gb300::GB300WCSPHModel<ref::SimulationParameters, ref::SPHParameters, ref::WCSPHParameters>
            model2(g, p, w);
        std::vector<float> dens2;
        model2.StepHost(pos2, vel2, dens2);
        std::fwrite(pos2.data(), 12, n, f);
        std::fwrite(vel2.data(), 12, n, f);
        std::fwrite(dens2.data(), 4, n, f);
        std::fclose(f);
    } catch (const std::exception& e) {
        std::printf("%s\n", e.what());
        return 3;
    }
    return 0;
}
