// mps_system.hpp -- C++ layer over mps_c.h with the names of the reference's step API.
//
// moonsh5009/MPS_CUDA drives its step through mps::System (src/MPS_System/MPSSystem.h:24-76) with
// an SPH model made of an SPHObject, an SPHMaterial (src/MPS_Object/MPSSPHMaterial.h:9-45) and a
// SpatialHash, a boundary ObstacleModel sampled from a mesh, and PhysicsParam
// (src/MPS_Object/MPSUniformDef.h:19-25).  This header keeps those names, fields and setter
// semantics so that a caller of the reference moves over with few edits:
//   - mps::PhysicsParam {dt, gravity, min, max} and mps::SPHMaterialParam (same fields);
//   - mps::SPHMaterial: the constructor's defaults and SetParam / SetRadius / SetViscosity /
//     SetXSPH / SetSurfaceTension / SetColor (MPSSPHMaterial.cpp:4-44);
//   - mps::System: SetDevice, OnUpdate (one frame of MPSSystem.cpp:191-291, skipped while the
//     simulation is paused as b_runSim does), the frame counter; the scene set-up that the
//     reference hard-codes in Initalize / *TestScene is passed in (SetPhysics, SetMaterial,
//     SetFluid, SetBoundary, SampleBoundaryMesh);
//   - mps::kernel::*: the frame's phases under the names of the functions OnUpdate calls.
// Differences: errors throw mps::Error (the reference reports nothing); state lives in the
// library and is read back with GetFluid / GetField instead of GL-mapped buffers.
#pragma once

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "mps_c.h"

namespace mps {

using REAL = double;
using REAL3 = std::array<REAL, 3>;

class Error : public std::runtime_error {
public:
    Error(int code, const std::string& what) : std::runtime_error(what), m_code(code) {}
    int code() const { return m_code; }

private:
    int m_code;
};

inline void Check(int code) {
    if (code != MPS_OK) {
        const char* m = mps_last_error();
        throw Error(code, m ? m : "mps error");
    }
}

// PhysicsParam (MPSUniformDef.h:19-25).
struct PhysicsParam {
    REAL dt = 0.005;
    REAL3 gravity{0.0, -9.8, 0.0};
    REAL3 min{-5.0, -5.0, -5.0};
    REAL3 max{5.0, 5.0, 5.0};
};

// SPHMaterialParam (MPSSPHMaterial.h:9-21).
struct SPHMaterialParam {
    REAL radius;
    REAL mass;
    REAL density;
    REAL volume;
    REAL viscosity;
    REAL XSPH;
    REAL surfaceTension;
    std::array<float, 4> color;
};

// SPHMaterial (MPSSPHMaterial.cpp): radius is the support radius h (the reference calls
// SetRadius(4 r)); V = h^3 / 48 * 3.141592 and m = density * V as the reference computes them.
class SPHMaterial {
public:
    SPHMaterial() {
        SetParam(0.01, 1.0);
        SetViscosity(0.025);
        SetXSPH(0.1);
        SetSurfaceTension(100.0);
        SetColor({0.3f, 0.8f, 0.2f, 1.0f});
    }
    void SetParam(REAL radius, REAL density) {
        m_param.radius = radius;
        m_param.volume = radius * radius * radius / 48.0 * 3.141592;
        m_param.density = density;
        m_param.mass = density * m_param.volume;
    }
    void SetRadius(REAL radius) { SetParam(radius, GetDensity()); }
    void SetViscosity(REAL viscosity) { m_param.viscosity = viscosity; }
    void SetXSPH(REAL XSPH) { m_param.XSPH = XSPH; }
    void SetSurfaceTension(REAL surfaceTension) { m_param.surfaceTension = surfaceTension; }
    void SetColor(const std::array<float, 4>& color) { m_param.color = color; }

    REAL GetRadius() const { return m_param.radius; }
    REAL GetMass() const { return m_param.mass; }
    REAL GetDensity() const { return m_param.density; }
    REAL GetVolume() const { return m_param.volume; }
    REAL GetViscosity() const { return m_param.viscosity; }
    REAL GetXSPH() const { return m_param.XSPH; }
    REAL GetSurfaceTension() const { return m_param.surfaceTension; }
    const std::array<float, 4>& GetColor() const { return m_param.color; }
    const SPHMaterialParam& GetParam() const { return m_param; }
    // A material with explicit mass and volume (physical units, V = spacing^3).
    void SetPhysical(REAL radius, REAL density, REAL volume) {
        m_param.radius = radius;
        m_param.density = density;
        m_param.volume = volume;
        m_param.mass = density * volume;
    }

private:
    SPHMaterialParam m_param{};
};

inline mps_material ToC(const SPHMaterialParam& m) {
    mps_material c{};
    c.radius = m.radius;
    c.mass = m.mass;
    c.density = m.density;
    c.volume = m.volume;
    c.viscosity = m.viscosity;
    c.xsph = m.XSPH;
    c.surface_tension = m.surfaceTension;
    return c;
}

inline mps_physics ToC(const PhysicsParam& p) {
    mps_physics c{};
    c.dt = p.dt;
    for (int k = 0; k < 3; ++k) {
        c.gravity[k] = p.gravity[size_t(k)];
        c.min[k] = p.min[size_t(k)];
        c.max[k] = p.max[size_t(k)];
    }
    return c;
}

// The step of mps::System on one GPU.
class System {
public:
    System() { mps_default_config(&m_config); }
    ~System() {
        if (m_h) mps_destroy(m_h);
    }
    System(const System&) = delete;
    System& operator=(const System&) = delete;

    void SetDevice(int device) { m_device = device; }
    mps_config& Config() { return m_config; }   // before Initalize
    void SetPhysics(const PhysicsParam& p) {
        m_physics = p;
        if (m_h) {
            const mps_physics c = ToC(p);
            Check(mps_set_physics(m_h, &c));
        }
    }
    void SetMaterial(const SPHMaterial& m) {
        m_material = m;
        if (m_h) {
            const mps_material c = ToC(m.GetParam());
            Check(mps_set_material(m_h, &c));
        }
    }
    // Creates the simulation (the part of System::Initalize that is not rendering).
    void Initalize() {
        if (m_h) return;
        const mps_material mat = ToC(m_material.GetParam());
        const mps_physics phys = ToC(m_physics);
        Check(mps_create(&mat, &phys, &m_config, m_device, &m_h));
    }
    // Boundary particles: positions (x, y, z) and particle radii; volumes computed on the device.
    void SetBoundary(const std::vector<REAL>& pos3, const std::vector<REAL>& radius) {
        Initalize();
        Check(mps_set_boundary(m_h, int64_t(radius.size()), pos3.data(), radius.data(), nullptr));
    }
    // Boundary particles sampled on a triangle mesh (MeshObject::LoadMesh + ParticleSampling).
    size_t SampleBoundaryMesh(const std::string& obj_path, const REAL3& center, const REAL3& size, REAL mesh_radius) {
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
        std::vector<REAL> pos3(static_cast<size_t>(n) * 3), rad(static_cast<size_t>(n));
        for (size_t i = 0; i < size_t(n); ++i) {
            for (int k = 0; k < 3; ++k) pos3[3 * i + size_t(k)] = p4[4 * i + size_t(k)];
            rad[i] = p4[4 * i + 3];
        }
        SetBoundary(pos3, rad);
        return size_t(n);
    }
    // Fluid particles as the reference stores them (REAL3 pos / vel, REAL mass and radius).
    void SetFluid(const std::vector<REAL>& pos3, const std::vector<REAL>& vel3, const std::vector<REAL>& mass,
                  const std::vector<REAL>& radius) {
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

private:
    mps_handle* m_h = nullptr;
    int m_device = 0;
    mps_config m_config{};
    PhysicsParam m_physics{};
    SPHMaterial m_material{};
    bool b_runSim = true;
    uint64_t m_frame = 0;
};

// The frame's phases under the names of the reference's functions that OnUpdate calls
// (MPSSystem.cpp:220-278), so that its call sequence can be kept.  Each runs on all of the
// System's particles; several reference calls map to one phase, as noted.
namespace kernel {
// SpatialHash::UpdateHash + ZSort (MPSSpatialHash.cu:53-140): cell keys, sort, reorder.
inline void UpdateHash(System& sys, void* stream = nullptr) { sys.Phase(MPS_PHASE_SORT, stream); }
// SpatialHash::BuildNeighorhood, fluid-fluid and fluid-boundary (MPSSpatialHash.cu:142-218).
inline void BuildNeighorhood(System& sys, void* stream = nullptr) { sys.Phase(MPS_PHASE_NEIGHBORS, stream); }
namespace SPH {
// ComputeBoundaryParticleVolumeSub/Final (MPSSPHBaseUtil.cu:9-53); a no-op unless the config
// asks for the reference's accumulating volume (the static boundary's volume is set once).
inline void ComputeBoundaryParticleVolume(System& sys, void* stream = nullptr) { sys.Phase(MPS_PHASE_BVOLUME, stream); }
// ComputeDensitySub/Final + DensityColorTest + ComputeDFSPHFactorSub/Final, then ResetForce /
// ApplyGravity / UpdateVelocity (MPSSystem.cpp:240-255): one fused pass.
inline void ComputeDensityAndDFSPHFactor(System& sys, void* stream = nullptr) {
    sys.Phase(MPS_PHASE_DENSITY_ALPHA, stream);
}
// ComputeDFSPHDivergenceFree (MPSSPHDFSPHUtil.h:80-87).
inline void ComputeDFSPHDivergenceFree(System& sys, void* stream = nullptr) { sys.Phase(MPS_PHASE_DF, stream); }
// ApplyImplicitViscosityNSurfaceTension (MPSSPHNonPressureUtil.h:61-65).
inline void ApplyImplicitViscosityNSurfaceTension(System& sys, void* stream = nullptr) {
    sys.Phase(MPS_PHASE_VISCST, stream);
}
// ComputeDFSPHConstantDensity (MPSSPHDFSPHUtil.h:72-79).
inline void ComputeDFSPHConstantDensity(System& sys, void* stream = nullptr) { sys.Phase(MPS_PHASE_CD, stream); }
}  // namespace SPH
namespace Advect {
// BoundaryCollision + UpdatePosition (MPSAdvectUtil.h:17-19); completes the frame.
inline void BoundaryCollisionAndUpdatePosition(System& sys, void* stream = nullptr) {
    sys.Phase(MPS_PHASE_ADVECT, stream);
}
}  // namespace Advect
}  // namespace kernel

}  // namespace mps
