// cuda_nbody_sim.hpp -- C++ adapter with the reference simulator's shape.
//
// Mirrors src/Sim/INBodySim.hpp:11-28 and src/Sim/INBodySim.cpp:7-39 on top
// of the C-ABI in nbody_gb300.h: Init keeps a non-owning pointer to the
// caller's particle vector and uploads it; Update(dt) runs one kick-drift
// step on the GPU and writes Position, Velocity and Forces back into the
// caller's records, exactly where the reference's Update leaves them.  The
// render hand-off and the octree export stand in for RenderDebug's D3D draws.
// Errors from the C-ABI surface as std::runtime_error on the C++ side.
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "nbody_gb300.h"

namespace nbgb {

enum class ENBodySim {
    BruteForceCPU = NB_SIM_BRUTE_FORCE,      // same GPU direct sum for both brute-force kinds
    BruteForceGPU = NB_SIM_BRUTE_FORCE_GPU,
    BarnesHut = NB_SIM_BARNES_HUT,
    NumSims = 3
};

using Particle = nb_particle;

class INBodySim {
  public:
    virtual ~INBodySim() = default;
    virtual void Init(std::vector<Particle>& particles) = 0;
    virtual void Update(float dt) = 0;
    virtual void RenderDebug() {}
};

class CudaNBodySim : public INBodySim {
  public:
    explicit CudaNBodySim(ENBodySim kind, const nb_params* params = nullptr) {
        nb_params p;
        if (params) p = *params;
        else nb_default_params(&p);
        p.kind = static_cast<int>(kind);
        const int rc = nb_create(&p, &sim_);
        if (rc != NB_OK) throw std::runtime_error("nb_create failed (" + std::to_string(rc) + ")");
    }
    ~CudaNBodySim() override {
        if (sim_) nb_destroy(sim_);
    }
    CudaNBodySim(const CudaNBodySim&) = delete;
    CudaNBodySim& operator=(const CudaNBodySim&) = delete;

    // INBodySim::Init: the vector must outlive the simulator; call Init again
    // after resizing it (as the reference requires).
    void Init(std::vector<Particle>& particles) override {
        particles_ = &particles;
        check(nb_init_particles(sim_, particles.data(), particles.size()), "nb_init_particles");
    }

    // INBodySim::Update: one step, then the caller's records are updated.
    void Update(float dt) override { UpdateMany(dt, 1); }

    // nsteps steps on the GPU, one write-back at the end.
    void UpdateMany(float dt, int nsteps) {
        if (!particles_) throw std::runtime_error("Update before Init");
        check(nb_step(sim_, dt, nsteps), "nb_step");
        check(nb_write_back(sim_, particles_->data(), particles_->size()), "nb_write_back");
    }

    // Headless render hand-off: LWParticle-like vertices of the current state.
    std::vector<nb_render_vertex> RenderVertices(float scale = 1.0f) {
        std::vector<nb_render_vertex> v(particles_ ? particles_->size() : 0);
        std::vector<float> colour(4 * v.size());
        for (size_t i = 0; i < v.size(); ++i)
            for (int k = 0; k < 4; ++k) colour[4 * i + k] = (*particles_)[i].colour[k];
        check(nb_render_vertices(sim_, colour.data(), scale, v.data(), v.size()), "nb_render_vertices");
        return v;
    }

    // Device vertex buffer (LWParticle layout) that every following Update
    // fills in the kick-drift's epilogue, coloured from the records; valid
    // until the next Init.
    void* AttachRenderBuffer(float scale = 1.0f) {
        if (!particles_) throw std::runtime_error("AttachRenderBuffer before Init");
        std::vector<float> colour(4 * particles_->size());
        for (size_t i = 0; i < particles_->size(); ++i)
            for (int k = 0; k < 4; ++k) colour[4 * i + k] = (*particles_)[i].colour[k];
        void* dev = nullptr;
        check(nb_render_attach(sim_, colour.data(), scale, &dev), "nb_render_attach");
        return dev;
    }

    // Octree of the current positions (Barnes-Hut), for debug drawing.
    std::vector<nb_tree_node> TreeNodes() {
        size_t n = 0;
        check(nb_tree_size(sim_, &n), "nb_tree_size");
        std::vector<nb_tree_node> nodes(n);
        check(nb_tree_nodes(sim_, nodes.data(), n), "nb_tree_nodes");
        return nodes;
    }

    nb_sim* handle() { return sim_; }

  private:
    void check(int rc, const char* what) {
        if (rc != NB_OK) throw std::runtime_error(std::string(what) + ": " + nb_last_error(sim_));
    }
    nb_sim* sim_ = nullptr;
    std::vector<Particle>* particles_ = nullptr;
};

// CreateNBodySim (src/Sim/INBodySim.cpp:7-27); no graphics context is needed.
inline std::unique_ptr<INBodySim> CreateNBodySim(ENBodySim type, const nb_params* params = nullptr) {
    return std::unique_ptr<INBodySim>(new CudaNBodySim(type, params));
}

// NBodySimGetName (src/Sim/INBodySim.cpp:29-39).
inline std::string NBodySimGetName(ENBodySim type) { return nb_sim_name(static_cast<int>(type)); }

}  // namespace nbgb
