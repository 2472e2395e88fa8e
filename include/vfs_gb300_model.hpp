// GB300WCSPHModel: a C++ drop-in for VkFluidSim's WCSPHWithBoundaryModel over the C ABI of
// vfs_cuda.h, header-only. It keeps the shape of the reference's SPHModel interface
// (src/models/model.h:58-84): construction from the parameter blocks (the model's constructor +
// Init, src/models/wcsph_with_boundary_model.cpp:25-79), Step (wcsph_with_boundary_model.cpp:81-117),
// SetParticleState (model.h:77-81), CopyDataBuffers as host arrays (model.h:84, the render
// hand-off), GetParameters / parameter edits, boundary objects as GenericScene packs them
// (src/scenes/generic_scene.cpp:125-145), and the spatial hash's buffers (keys, sorted indices,
// offsets). Vulkan command buffers and device addresses are replaced by the library's own
// stream and device buffers.
//
// It is a template over the reference's parameter types (vfs::SimulationParameters,
// vfs::SPHModel::Parameters, vfs::WCSPHWithBoundaryModel::Parameters), which it reads field by
// field, and over the 3-vector type of the host arrays (glm::vec3: three packed floats), so it
// compiles inside the reference's tree without depending on its headers. Errors of the library
// (its int status codes) are thrown as std::runtime_error with vfs_last_error()'s message, as the
// reference reports failures by exceptions (nlohmann JSON) or aborts (VK_CHECK).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "vfs_cuda.h"

namespace vfs_gb300 {

inline void check(int rc) {
    if (rc != VFS_OK) throw std::runtime_error(std::string("vfs: ") + vfs_last_error());
}

template <class SimParams, class SPHParams, class WCSPHParams>
class GB300WCSPHModel {
public:
    GB300WCSPHModel(const SimParams& g, const SPHParams& p, const WCSPHParams& w) {
        const vfs_sim_params sim = to_c(g);
        const vfs_sph_params sph = to_c(p);
        const vfs_wcsph_params wc = to_c(w);
        check(vfs_model_create(&sim, &sph, &wc, &m_));
    }
    ~GB300WCSPHModel() {
        if (m_) vfs_model_destroy(m_);
    }
    GB300WCSPHModel(const GB300WCSPHModel&) = delete;
    GB300WCSPHModel& operator=(const GB300WCSPHModel&) = delete;

    // One Simulation::Step: `iterations` substeps; returns without waiting for the GPU.
    void Step() { check(vfs_model_step(m_)); }
    void Synchronize() { check(vfs_model_synchronize(m_)); }

    template <class Vec3>
    void SetParticleState(const std::vector<Vec3>& pos, const std::vector<Vec3>& vel,
                          uint32_t offset = 0) {
        static_assert(sizeof(Vec3) == 3 * sizeof(float), "three packed floats");
        if (pos.size() != vel.size()) throw std::invalid_argument("pos and vel differ in size");
        check(vfs_model_set_particle_state(m_, reinterpret_cast<const float*>(pos.data()),
                                           reinterpret_cast<const float*>(vel.data()), offset,
                                           (int64_t)pos.size()));
    }

    // The render hand-off of CopyDataBuffers, into host arrays (resized to the particle count).
    template <class Vec3>
    void CopyDataBuffers(std::vector<Vec3>& pos, std::vector<Vec3>& vel, std::vector<float>& dens) {
        static_assert(sizeof(Vec3) == 3 * sizeof(float), "three packed floats");
        const uint32_t n = NumParticles();
        pos.resize(n);
        vel.resize(n);
        dens.resize(n);
        check(vfs_model_copy_data_buffers(m_, reinterpret_cast<float*>(pos.data()),
                                          reinterpret_cast<float*>(vel.data()), dens.data(),
                                          nullptr));
    }

    // SetParticleState of every particle from pos / vel, `substeps` substeps, then the
    // CopyDataBuffers hand-off into the same arrays, with one wait (vfs_model_step_host). With
    // page-locked storage behind the vectors' data the last substep's passes write the outputs.
    template <class Vec3>
    void StepHost(std::vector<Vec3>& pos, std::vector<Vec3>& vel, std::vector<float>& dens,
                  int32_t substeps = 1) {
        static_assert(sizeof(Vec3) == 3 * sizeof(float), "three packed floats");
        const uint32_t n = NumParticles();
        if (pos.size() != n || vel.size() != n)
            throw std::invalid_argument("pos and vel must hold every particle");
        dens.resize(n);
        float* p = reinterpret_cast<float*>(pos.data());
        float* v = reinterpret_cast<float*>(vel.data());
        check(vfs_model_step_host(m_, p, v, substeps, p, v, dens.data()));
    }

    // SpatialHash's buffers after the last substep: keys, sorted indices, offsets.
    void GetNeighborArrays(std::vector<uint32_t>& keys, std::vector<uint32_t>& sorted_indices,
                           std::vector<uint32_t>& offsets) {
        const uint32_t n = NumParticles();
        keys.resize(n);
        sorted_indices.resize(n);
        offsets.resize(n);
        check(vfs_model_get_neighbor_arrays(m_, keys.data(), sorted_indices.data(), offsets.data()));
    }

    // A boundary object as GenericScene::CreateBoundaryObjectBuffer packs it: the inverse of the
    // object's transform and its rotation as column-major 4x4 floats, the SDF grid's box and
    // resolution, and the SDF and volume-map grids (copied).
    void AddBoundaryObject(const float transform[16], const float rotation[16],
                           const float box_size[3], const float box_pos[3],
                           const uint32_t resolution[3], const float* sdf, const float* volume_map) {
        vfs_boundary_object o{};
        for (int k = 0; k < 16; k++) {
            o.transform[k] = transform[k];
            o.rotation[k] = rotation[k];
        }
        for (int k = 0; k < 3; k++) {
            o.box_size[k] = box_size[k];
            o.box_pos[k] = box_pos[k];
            o.resolution[k] = resolution[k];
        }
        o.sdf_grid = sdf;
        o.volume_map_grid = volume_map;
        check(vfs_model_add_boundary_object(m_, &o));
    }

    // The parameter edits of DrawDebugUI and Simulation::SetGlobalParameters.
    void SetParameters(const SimParams& g, const SPHParams& p, const WCSPHParams& w) {
        const vfs_sim_params sim = to_c(g);
        const vfs_sph_params sph = to_c(p);
        const vfs_wcsph_params wc = to_c(w);
        check(vfs_model_set_parameters(m_, &sim, &sph, &wc));
    }

    uint32_t NumParticles() const { return vfs_model_num_particles(m_); }
    vfs_model* Handle() const { return m_; }

private:
    static vfs_sim_params to_c(const SimParams& g) {
        return vfs_sim_params{{g.gravity.x, g.gravity.y, g.gravity.z}, g.smooth_radius};
    }
    static vfs_sph_params to_c(const SPHParams& p) {
        return vfs_sph_params{p.time_scale,
                              (int32_t)p.iterations,
                              (int32_t)p.n_particles,
                              p.fixed_dt,
                              p.target_density,
                              {p.bounding_box.size.x, p.bounding_box.size.y, p.bounding_box.size.z},
                              {p.bounding_box.pos.x, p.bounding_box.pos.y, p.bounding_box.pos.z}};
    }
    static vfs_wcsph_params to_c(const WCSPHParams& w) {
        return vfs_wcsph_params{w.wall_stiffness, w.stiffness, w.expoent, w.viscosity_strenght};
    }

    vfs_model* m_ = nullptr;
};

}  // namespace vfs_gb300
