// mps_system.hpp -- C++ layer over mps_c.h with the names of the reference's step API.
//
// moonsh5009/MPS_CUDA drives its step through mps::System (src/MPS_System/MPSSystem.h:24-76) with
// an SPH model made of an SPHObject, an SPHMaterial (src/MPS_Object/MPSSPHMaterial.h:9-45) and a
// SpatialHash, a boundary ObstacleModel sampled from a mesh, and PhysicsParam
// (src/MPS_Object/MPSUniformDef.h:19-25).  mps::System here owns one library handle and the
// reference-shaped models over it (mps_reference.hpp: SPHModel, ObstacleModel, GBArchiver), so that
// the reference's OnUpdate body runs against it with its call sequence unchanged
// (m_pSPHModel, m_pBoundaryModel, m_pGBArchiver, m_frame, b_runSim), and adds:
//   - scene set-up that the reference hard-codes in Initalize / *TestScene, passed in instead
//     (SetPhysics, SetMaterial, SetFluid, SetBoundary, SampleBoundaryMesh);
//   - OnUpdate as one graph-launched frame (mps_step), the fast path;
//   - GetFluid / GetField to read the state back (the reference reads GL-mapped buffers).
// Errors throw mps::Error (the reference reports nothing).
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "mps_c.h"
#include "mps_reference.hpp"

namespace mps {

// The step of mps::System on one GPU.
class System {
public:
    System() {
        mps_default_config(&m_config);
        m_pGBArchiver = std::make_unique<GBArchiver>();
        m_pGBArchiver->m_physicsParam = m_physics;
    }
    virtual ~System() {
        m_pSPHModel.reset();
        m_pBoundaryModel.reset();
        if (m_h) {
            detail::Forget(m_h);
            mps_destroy(m_h);
        }
    }
    System(const System&) = delete;
    System& operator=(const System&) = delete;

    void SetDevice(int device) { m_device = device; }
    mps_config& Config() { return m_config; }   // before Initalize
    void SetPhysics(const PhysicsParam& p) {
        m_physics = p;
        m_pGBArchiver->m_physicsParam = p;
        if (m_h) {
            const mps_physics c = ToC(p);
            Check(mps_set_physics(m_h, &c));
        }
    }
    void SetMaterial(const SPHMaterial& m) {
        m_material = m;
        if (m_pSPHModel) static_cast<SPHMaterial*>(m_pSPHModel->GetMaterial())->GetParam() = m.GetParam();
        if (m_h) {
            const mps_material c = ToC(m.GetParam());
            Check(mps_set_material(m_h, &c));
        }
    }
    // Creates the simulation and its models (the part of System::Initalize that is not rendering):
    // an SPHModel (SPHObject, SPHMaterial, SpatialHash) and an ObstacleModel (MeshObject,
    // BoundaryParticleObject, MeshMaterial, SpatialHash), bound to one library handle.
    void Initalize() {
        if (m_h) return;
        const mps_material mat = ToC(m_material.GetParam());
        const mps_physics phys = ToC(m_physics);
        Check(mps_create(&mat, &phys, &m_config, m_device, &m_h));
        auto sph = std::make_unique<SPHObject>();
        sph->Bind(m_h);
        auto sphMat = std::make_unique<SPHMaterial>(m_material);
        m_pSPHModel = std::make_unique<SPHModel>(std::move(sph), std::move(sphMat), std::make_unique<SpatialHash>());
        auto bp = std::make_unique<BoundaryParticleObject>();
        bp->Bind(m_h);
        m_pBoundaryModel = std::make_unique<ObstacleModel>(std::make_unique<MeshObject>(), std::move(bp),
                                                           std::make_unique<MeshMaterial>(),
                                                           std::make_unique<SpatialHash>());
    }
    // Boundary particles: positions (x, y, z) and particle radii; volumes computed on the device.
    void SetBoundary(const std::vector<double>& pos3, const std::vector<double>& radius) {
        Initalize();
        Check(mps_set_boundary(m_h, int64_t(radius.size()), pos3.data(), radius.data(), nullptr));
    }
    // Boundary particles sampled on a triangle mesh (MeshObject::LoadMesh + ParticleSampling).
    size_t SampleBoundaryMesh(const std::string& obj_path, const Vec3d& center, const Vec3d& size, double mesh_radius) {
        int64_t nv = 0, nf = 0;
        Check(mps_mesh_load_obj(obj_path.c_str(), center.data(), size.data(), &nv, &nf, nullptr, nullptr));
        std::vector<double> v(size_t(nv) * 3);
        std::vector<uint32_t> f(size_t(nf) * 3);
        Check(mps_mesh_load_obj(obj_path.c_str(), center.data(), size.data(), &nv, &nf, v.data(), f.data()));
        const int64_t n = mps_mesh_sample(v.data(), nv, f.data(), nf, mesh_radius, nullptr, nullptr);
        if (n < 0) Check(int(n));
        std::vector<float> p4(size_t(n) * 4);
        const int64_t n2 = mps_mesh_sample(v.data(), nv, f.data(), nf, mesh_radius, p4.data(), nullptr);
        if (n2 != n) Check(n2 < 0 ? int(n2) : MPS_E_STATE);
        std::vector<double> pos3(static_cast<size_t>(n) * 3), rad(static_cast<size_t>(n));
        for (size_t i = 0; i < size_t(n); ++i) {
            for (int k = 0; k < 3; ++k) pos3[3 * i + size_t(k)] = p4[4 * i + size_t(k)];
            rad[i] = p4[4 * i + 3];
        }
        SetBoundary(pos3, rad);
        auto* mesh = m_pBoundaryModel->GetTarget<MeshObject>();
        mesh->m_vertices = v;
        mesh->m_faces = f;
        return size_t(n);
    }
    // Fluid particles as the reference stores them (xyz position / velocity, mass and radius, FP64).
    void SetFluid(const std::vector<double>& pos3, const std::vector<double>& vel3, const std::vector<double>& mass,
                  const std::vector<double>& radius) {
        Initalize();
        Check(mps_set_fluid(m_h, int64_t(mass.size()), pos3.data(), vel3.data(), mass.data(), radius.data(), nullptr));
    }
    // Native FP32 layout: pos4 = (x, y, z, particle radius), vel4 = (vx, vy, vz, mass).
    void SetFluid(const std::vector<float>& pos4, const std::vector<float>& vel4) {
        Initalize();
        Check(mps_set_fluid_f32(m_h, int64_t(pos4.size() / 4), pos4.data(), vel4.data(), 0, nullptr));
    }

    void SetRunning(bool run) { b_runSim = run; }
    bool IsRunning() const { return b_runSim; }
    // One frame of MPSSystem.cpp:191-291 (nothing while paused).
    void OnUpdate(void* stream = nullptr) {
        if (!b_runSim) return;
        Check(mps_step(m_h, 1, stream));
        m_frame++;
    }
    uint64_t GetFrame() const { return m_frame; }

    void GetFluid(std::vector<float>& pos4, std::vector<float>& vel4) const {
        const int64_t n = mps_field_size(m_h, "ids");
        pos4.resize(size_t(n) * 4);
        vel4.resize(size_t(n) * 4);
        Check(mps_get_fluid_f32(m_h, pos4.data(), vel4.data(), 0, nullptr));
    }
    // A floating-point per-particle field in particle-ID order ("density", "pressure", "color", ...).
    std::vector<float> GetField(const std::string& name) const {
        if (name == "ids" || name == "nbr_count" || name == "cell_key")
            throw Error(MPS_E_INVALID, "integer field " + name + ": use mps_get_field");
        const int64_t n = mps_field_size(m_h, name.c_str());
        if (n < 0) throw Error(MPS_E_INVALID, "unknown field " + name);
        std::vector<float> out(static_cast<size_t>(n));
        Check(mps_get_field(m_h, name.c_str(), out.data(), 1));
        return out;
    }
    mps_stats GetStats() const {
        mps_stats s;
        Check(mps_get_stats(m_h, &s, nullptr));
        return s;
    }
    mps_handle* Handle() const { return m_h; }
    // One sub-phase of the frame (MPS_PHASE_SORT ... MPS_PHASE_ADVECT, in order); the last one
    // completes the frame.
    void Phase(int32_t phase, void* stream = nullptr) {
        Check(mps_phase(m_h, phase, stream));
        if (phase == MPS_PHASE_ADVECT) m_frame++;
    }

protected:
    // the reference's members that its OnUpdate body reads (MPSSystem.h:60-72)
    std::unique_ptr<SPHModel> m_pSPHModel;
    std::unique_ptr<ObstacleModel> m_pBoundaryModel;
    std::unique_ptr<GBArchiver> m_pGBArchiver;
    bool b_runSim = true;
    uint64_t m_frame = 0;

private:
    mps_handle* m_h = nullptr;
    int m_device = 0;
    mps_config m_config{};
    PhysicsParam m_physics{};
    SPHMaterial m_material{};
};

}  // namespace mps
