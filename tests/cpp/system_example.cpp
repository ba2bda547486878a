// The small dam break (10^3 fluid particles, r = 0.01, spacing 0.02, walls of a 0.5 m box) driven
// through the C++ layer the way mps::System drives the reference's step; writes the final fluid
// state (pos4 then vel4, float32, particle-ID order) to argv[1]; argv[3] = "phases" runs each frame
// through the reference's step functions (mps_reference.hpp) in mps::System::OnUpdate's call
// sequence instead of the graph-launched OnUpdate.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <sstream>
#include <string>
#include <vector>

#include "mps_system.hpp"

// The body of the reference's mps::System::OnUpdate (src/MPS_System/MPSSystem.cpp:191-291), kept
// statement for statement on purpose: this program checks that the reference's call sequence
// compiles and runs against the drop-in API and gives the same frames as the library's own step.
class ReferenceSystem : public mps::System {
public:
    void OnUpdateReference() {
        if (!b_runSim) return;
        {
            cudaDeviceSynchronize();
            std::stringstream ss;
            ss << "Frame " << m_frame;
            MTimer::Start(ss.str());
        }
        auto pBoundaryParticleObject = static_cast<mps::BoundaryParticleObject*>(m_pBoundaryModel->GetSubObject());
        auto pBoundaryParticleMaterial = static_cast<mps::MeshMaterial*>(m_pBoundaryModel->GetMaterial());
        auto pBoundaryParticleHash = static_cast<mps::SpatialHash*>(
            m_pBoundaryModel->GetTree(static_cast<uint32_t>(mps::ObstacleTreeIdx::SpatialHash)));
        auto pSPHObject = m_pSPHModel->GetTarget<mps::SPHObject>();
        auto pSPHMaterial = static_cast<mps::SPHMaterial*>(m_pSPHModel->GetMaterial());
        auto pSPHHash = static_cast<mps::SpatialHash*>(m_pSPHModel->GetTree());

        const auto pBoundaryParticleRes = pBoundaryParticleObject->GetDeviceResource<mps::BoundaryParticleResource>();
        const auto pBoundaryParticleParam = pBoundaryParticleRes->GetBoundaryParticleParam().lock();
        if (!pBoundaryParticleParam) return;
        const auto pSPHRes = pSPHObject->GetDeviceResource<mps::SPHResource>();
        const auto pSPHParam = pSPHRes->GetSPHParam().lock();
        if (!pSPHParam) return;
        const auto& physParam = m_pGBArchiver->m_physicsParam;

        if ((m_frame % 50u) == 1u) {
            pBoundaryParticleHash->ZSort(*pBoundaryParticleParam);
            pSPHHash->ZSort(*pSPHParam);
        }
        pBoundaryParticleHash->UpdateHash(*pBoundaryParticleParam);
        pSPHHash->UpdateHash(*pSPHParam);

        pBoundaryParticleHash->BuildNeighorhood(*pBoundaryParticleParam);
        pSPHHash->BuildNeighorhood(*pSPHParam);
        pSPHHash->BuildNeighorhood(*pSPHParam, *pBoundaryParticleParam, pBoundaryParticleHash);

        const auto neiBP2BP = pBoundaryParticleHash->GetNeighborhood(*pBoundaryParticleParam).value_or(mps::NeiParam{nullptr, nullptr});
        const auto neiSPH2SPH = pSPHHash->GetNeighborhood(*pSPHParam).value_or(mps::NeiParam{nullptr, nullptr});
        const auto neiSPH2BP = pSPHHash->GetNeighborhood(*pBoundaryParticleParam).value_or(mps::NeiParam{nullptr, nullptr});

        mps::kernel::SPH::ComputeBoundaryParticleVolumeSub(*pBoundaryParticleParam, neiBP2BP);
        mps::kernel::SPH::ComputeBoundaryParticleVolumeFinal(*pBoundaryParticleParam);

        mps::kernel::Advect::ResetREAL(pSPHParam->pDensity, pSPHParam->size);
        mps::kernel::SPH::ComputeDensitySub(pSPHMaterial->GetParam(), *pSPHParam, neiSPH2SPH);
        mps::kernel::SPH::ComputeDensitySub(*pSPHParam, neiSPH2BP, *pBoundaryParticleParam);
        mps::kernel::SPH::ComputeDensityFinal(pSPHMaterial->GetParam(), *pSPHParam);

        mps::kernel::SPH::DensityColorTest(pSPHMaterial->GetParam(), *pSPHParam);

        mps::kernel::Advect::ResetREAL(pSPHParam->pFactorDFSPH, pSPHParam->size);
        mps::kernel::Advect::ResetREAL(reinterpret_cast<REAL*>(pSPHParam->pTempVec3), pSPHParam->size * 3);
        mps::kernel::SPH::ComputeDFSPHFactorSub(pSPHMaterial->GetParam(), *pSPHParam, neiSPH2SPH);
        mps::kernel::SPH::ComputeDFSPHFactorSub(*pSPHParam, neiSPH2BP, *pBoundaryParticleParam);
        mps::kernel::SPH::ComputeDFSPHFactorFinal(*pSPHParam);

        mps::kernel::Advect::ResetForce(*pSPHParam);
        mps::kernel::Advect::ApplyGravity(physParam, *pSPHParam);
        mps::kernel::Advect::UpdateVelocity(physParam, *pSPHParam);

        mps::kernel::SPH::ComputeDFSPHDivergenceFree(physParam, pSPHMaterial->GetParam(), *pSPHParam,
                                                     pBoundaryParticleMaterial->GetParam(), *pBoundaryParticleParam,
                                                     neiSPH2SPH, neiSPH2BP);
        mps::kernel::SPH::ApplyImplicitViscosityNSurfaceTension(physParam, pSPHMaterial->GetParam(), *pSPHParam,
                                                                neiSPH2SPH);
        mps::kernel::SPH::ComputeDFSPHConstantDensity(physParam, pSPHMaterial->GetParam(), *pSPHParam,
                                                      pBoundaryParticleMaterial->GetParam(), *pBoundaryParticleParam,
                                                      neiSPH2SPH, neiSPH2BP);

        mps::kernel::Advect::BoundaryCollision(physParam, *pSPHParam);
        mps::kernel::Advect::UpdatePosition(physParam, *pSPHParam);
        {
            cudaDeviceSynchronize();
            std::stringstream ss;
            ss << "Frame " << m_frame;
            MTimer::End(ss.str());
            OutputDebugStringA("\n");
        }
        m_frame++;
    }
};

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s out.bin frames\n", argv[0]);
        return 2;
    }
    const int frames = std::atoi(argv[2]);
    try {
        const double spacing = 0.02, r = 0.01;
        mps::SPHMaterial mat;
        mat.SetPhysical(4 * r, 1000.0, spacing * spacing * spacing);
        mat.SetViscosity(0.01);
        mat.SetXSPH(0.1);
        mat.SetSurfaceTension(0.05);
        mps::PhysicsParam phys;
        phys.dt = 1.0e-3;
        phys.gravity = {0.0, -9.81, 0.0};
        phys.min = {0.0, 0.0, 0.0};
        phys.max = {0.5, 0.5, 0.5};

        ReferenceSystem sys;
        sys.SetDevice(0);
        mps_config& cfg = sys.Config();
        cfg.kernel = MPS_KERNEL_CUBIC_SPLINE;
        cfg.df_tol = 1.0e-3;
        cfg.cd_tol = 1.0e-3;
        cfg.df_min_iter = 1;
        cfg.cd_min_iter = 2;
        cfg.max_iter = 100;
        sys.SetPhysics(phys);
        sys.SetMaterial(mat);
        sys.Initalize();

        const double lo[3] = {0.0, 0.0, 0.0}, hi[3] = {0.5, 0.5, 0.5};
        const int64_t nb = mps_gen_box_walls(lo, hi, spacing, r, 0, nullptr);
        std::vector<float> b4(size_t(nb) * 4);
        mps_gen_box_walls(lo, hi, spacing, r, 0, b4.data());
        std::vector<double> bpos(static_cast<size_t>(nb) * 3), brad(static_cast<size_t>(nb));
        for (size_t i = 0; i < size_t(nb); ++i) {
            for (int k = 0; k < 3; ++k) bpos[3 * i + size_t(k)] = b4[4 * i + size_t(k)];
            brad[i] = b4[4 * i + 3];
        }
        sys.SetBoundary(bpos, brad);

        const int n = 10 * 10 * 10;
        std::vector<float> p4(size_t(n) * 4), v4(size_t(n) * 4);
        mps::Check(mps_gen_block(10, 10, 10, lo, spacing, r, mat.GetMass(), 0.002, 0, p4.data(), v4.data()));
        sys.SetFluid(p4, v4);

        const bool phases = argc > 3 && std::string(argv[3]) == "phases";
        for (int f = 0; f < frames; ++f) {
            if (!phases) {
                sys.OnUpdate();
                continue;
            }
            sys.OnUpdateReference();
        }
        sys.SetRunning(false);
        sys.OnUpdate();   // paused: no step
        std::vector<float> pos, vel;
        sys.GetFluid(pos, vel);
        const mps_stats st = sys.GetStats();
        std::printf("frames %llu steps %lld cd_iters %d\n", (unsigned long long)sys.GetFrame(), (long long)st.steps,
                    st.cd_iters);
        FILE* fp = std::fopen(argv[1], "wb");
        if (!fp) return 3;
        std::fwrite(pos.data(), sizeof(float), pos.size(), fp);
        std::fwrite(vel.data(), sizeof(float), vel.size(), fp);
        std::fclose(fp);
    } catch (const mps::Error& e) {
        std::fprintf(stderr, "mps error %d: %s\n", e.code(), e.what());
        return 1;
    }
    return 0;
}
