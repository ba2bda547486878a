// Headless driver of the reference's own CUDA step -- TEST INFRASTRUCTURE ONLY.
//
// Links against the reference's compiled sources (oracle/build_ref.sh builds them from the
// reference tree into oracle/_ref/) and replays mps::System::OnUpdate
// (src/MPS_System/MPSSystem.cpp:220-278) on device buffers that it owns instead of OpenGL
// buffers.  Used to pin the FP64 oracle (golden vectors) and as the reference arm of bench.py.
// Differences from the shipped app, all outside the step: no window, no renderer, buffers from
// cudaMalloc instead of GL interop, the frame timer's debug strings go to mps_ref_debug_sink
// (which records the solver loop counts) instead of the Windows debugger.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <thrust/device_vector.h>

#include "MPS_Object/MPSSPHParam.h"
#include "MPS_Object/MPSBoundaryParticleParam.h"
#include "MPS_Object/MPSSpatialHash.h"
#include "MPS_Object/MPSSPHMaterial.h"
#include "MPS_Object/MPSMeshMaterial.h"
#include "MPS_Object/MPSUniformDef.h"
#include "MPS_Computer/MPSAdvectUtil.h"
#include "MPS_Computer/MPSSPHUtil.h"
#include "MPS_Object/MPSMeshObject.cuh"
#include "MPS_Computer/MPSParticleSamplingUtil.cuh"
#include <thrust/scan.h>
#include <thrust/sort.h>
#include <thrust/transform.h>
#include <algorithm>

#define REF_API extern "C" __attribute__((visibility("default")))

namespace {
int g_loops[3] = {0, 0, 0};  // DF, CG, CD loop counters of the last step

bool parse_loop(const char* msg, const char* key, int* out) {
    const char* k = std::strstr(msg, key);
    if (!k) return false;
    const char* l = std::strstr(k, "Loop");
    if (!l) return false;
    const char* c = std::strchr(l, ':');
    if (!c) return false;
    *out = std::atoi(c + 1);
    return true;
}

template <class T>
T* dalloc(size_t n) {
    T* p = nullptr;
    cudaMalloc(&p, (n ? n : 1) * sizeof(T));
    cudaMemset(p, 0, (n ? n : 1) * sizeof(T));
    return p;
}
}  // namespace

extern "C" void mps_ref_debug_sink(const char* msg) {
    parse_loop(msg, "ComputeDFSPHDivergenceFree", &g_loops[0]);
    parse_loop(msg, "ApplyImplicitViscosityNSurfaceTension", &g_loops[1]);
    parse_loop(msg, "ComputeDFSPHConstantDensity", &g_loops[2]);
}

struct RefSim {
    mps::PhysicsParam phys{};
    mps::SPHMaterialParam mat{};
    mps::MeshMaterialParam bmat{};
    mps::SPHParam sph{};
    mps::BoundaryParticleParam bp{};
    mps::SpatialHash hash_sph, hash_bp;
    unsigned frame = 0;
    std::vector<void*> owned;
    template <class T>
    T* own(size_t n) {
        T* p = dalloc<T>(n);
        owned.push_back(p);
        return p;
    }
    ~RefSim() {
        for (void* p : owned) cudaFree(p);
    }
};

// sphmat: radius, mass, density, volume, viscosity, xsph, surface tension
// phys: dt, gravity[3], min[3], max[3]
REF_API void* ref_create(long long n, const double* pos, const double* vel, const double* mass, const double* radius,
                         long long nb, const double* bpos, const double* bradius, const double* sphmat,
                         const double* phys, double hash_cell, const unsigned* hash_size) {
    auto* s = new RefSim();
    s->phys.dt = phys[0];
    s->phys.gravity = REAL3{phys[1], phys[2], phys[3]};
    s->phys.min = REAL3{phys[4], phys[5], phys[6]};
    s->phys.max = REAL3{phys[7], phys[8], phys[9]};
    s->mat.radius = sphmat[0];
    s->mat.mass = sphmat[1];
    s->mat.density = sphmat[2];
    s->mat.volume = sphmat[3];
    s->mat.viscosity = sphmat[4];
    s->mat.XSPH = sphmat[5];
    s->mat.surfaceTension = sphmat[6];
    s->mat.color = glm::fvec4{0.3f, 0.8f, 0.2f, 1.0f};
    s->bmat.radius = sphmat[0];
    s->bmat.density = 1.0;
    s->bmat.mass = 0.0;

    auto& f = s->sph;
    f.size = size_t(n);
    f.phaseID = 2;
    f.pColor = s->own<glm::fvec4>(n);
    f.pPosition = s->own<REAL3>(n);
    f.pMass = s->own<REAL>(n);
    f.pVelocity = s->own<REAL3>(n);
    f.pForce = s->own<REAL3>(n);
    f.pRadius = s->own<REAL>(n);
    f.pDensity = s->own<REAL>(n);
    f.pPressure = s->own<REAL>(n);
    f.pFactorDFSPH = s->own<REAL>(n);
    f.pFactorST = s->own<REAL>(n);
    f.pFactorSTB = s->own<REAL>(n);
    f.pTempReal = s->own<REAL>(n);
    f.pTempVec3 = s->own<REAL3>(n);
    f.pTempMat3 = s->own<REAL3x3>(n);
    f.pPreviousVel = s->own<REAL3>(n);
    f.pPredictVel = s->own<REAL3>(n);
    cudaMemcpy(f.pPosition, pos, size_t(n) * sizeof(REAL3), cudaMemcpyHostToDevice);
    cudaMemcpy(f.pVelocity, vel, size_t(n) * sizeof(REAL3), cudaMemcpyHostToDevice);
    cudaMemcpy(f.pMass, mass, size_t(n) * sizeof(REAL), cudaMemcpyHostToDevice);
    cudaMemcpy(f.pRadius, radius, size_t(n) * sizeof(REAL), cudaMemcpyHostToDevice);

    auto& b = s->bp;
    b.size = size_t(nb);
    b.phaseID = 1;
    b.pColor = s->own<glm::fvec4>(nb);
    b.pPosition = s->own<REAL3>(nb);
    b.pMass = s->own<REAL>(nb);
    b.pVelocity = s->own<REAL3>(nb);
    b.pForce = s->own<REAL3>(nb);
    b.pRadius = s->own<REAL>(nb);
    b.pFaceID = s->own<uint32_t>(nb);
    b.pBCC = s->own<REAL2>(nb);
    b.pVolume = s->own<REAL>(nb);
    b.pPreviousVel = s->own<REAL3>(nb);
    b.pPredictVel = s->own<REAL3>(nb);
    if (nb) {
        cudaMemcpy(b.pPosition, bpos, size_t(nb) * sizeof(REAL3), cudaMemcpyHostToDevice);
        cudaMemcpy(b.pRadius, bradius, size_t(nb) * sizeof(REAL), cudaMemcpyHostToDevice);
    }
    // SetObjectSize / SetCeilSize / SetHashSize as System::Initalize does (MPSSystem.cpp:70-72, :625-627)
    const glm::uvec3 hs{hash_size[0], hash_size[1], hash_size[2]};
    s->hash_sph.SetObjectSize(size_t(n));
    s->hash_sph.SetCeilSize(hash_cell);
    s->hash_sph.SetHashSize(hs);
    s->hash_bp.SetObjectSize(size_t(nb));
    s->hash_bp.SetCeilSize(hash_cell);
    s->hash_bp.SetHashSize(hs);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        delete s;
        return nullptr;
    }
    return s;
}

REF_API void ref_destroy(void* h) { delete static_cast<RefSim*>(h); }
REF_API void ref_set_frame(void* h, int frame) { static_cast<RefSim*>(h)->frame = unsigned(frame); }
REF_API void ref_loops(int* out3) { for (int k = 0; k < 3; ++k) out3[k] = g_loops[k]; }

// Phase ids match oracle/mps_oracle.h.
REF_API int ref_phase(void* hp, int phase) {
    auto* s = static_cast<RefSim*>(hp);
    auto& sph = s->sph;
    auto& bp = s->bp;
    const auto nei = [&](const mps::SpatialHash& h, const mps::ParticleParam& p) {
        return h.GetNeighborhood(p).value_or(mps::NeiParam{nullptr, nullptr});
    };
    switch (phase) {
        case 0:  // MPSSystem.cpp:220-224
            if ((s->frame % 50u) == 1u) {
                s->hash_bp.ZSort(bp);
                s->hash_sph.ZSort(sph);
            }
            break;
        case 1:  // :226-231
            s->hash_bp.UpdateHash(bp);
            s->hash_sph.UpdateHash(sph);
            s->hash_bp.BuildNeighorhood(bp);
            s->hash_sph.BuildNeighorhood(sph);
            s->hash_sph.BuildNeighorhood(sph, bp, &s->hash_bp);
            break;
        case 2:  // :237-238
            mps::kernel::SPH::ComputeBoundaryParticleVolumeSub(bp, nei(s->hash_bp, bp));
            mps::kernel::SPH::ComputeBoundaryParticleVolumeFinal(bp);
            break;
        case 3:  // :240-245
            mps::kernel::Advect::ResetREAL(sph.pDensity, sph.size);
            mps::kernel::SPH::ComputeDensitySub(s->mat, sph, nei(s->hash_sph, sph));
            mps::kernel::SPH::ComputeDensitySub(sph, nei(s->hash_sph, bp), bp);
            mps::kernel::SPH::ComputeDensityFinal(s->mat, sph);
            mps::kernel::SPH::DensityColorTest(s->mat, sph);
            break;
        case 4:  // :247-251
            mps::kernel::Advect::ResetREAL(sph.pFactorDFSPH, sph.size);
            mps::kernel::Advect::ResetREAL(reinterpret_cast<REAL*>(sph.pTempVec3), sph.size * 3);
            mps::kernel::SPH::ComputeDFSPHFactorSub(s->mat, sph, nei(s->hash_sph, sph));
            mps::kernel::SPH::ComputeDFSPHFactorSub(sph, nei(s->hash_sph, bp), bp);
            mps::kernel::SPH::ComputeDFSPHFactorFinal(sph);
            break;
        case 5:  // :253-255
            mps::kernel::Advect::ResetForce(sph);
            mps::kernel::Advect::ApplyGravity(s->phys, sph);
            mps::kernel::Advect::UpdateVelocity(s->phys, sph);
            break;
        case 6:  // :257-264
            mps::kernel::SPH::ComputeDFSPHDivergenceFree(s->phys, s->mat, sph, s->bmat, bp, nei(s->hash_sph, sph),
                                                         nei(s->hash_sph, bp));
            break;
        case 7:  // :266
            mps::kernel::SPH::ApplyImplicitViscosityNSurfaceTension(s->phys, s->mat, sph, nei(s->hash_sph, sph));
            break;
        case 8:  // :268-275
            mps::kernel::SPH::ComputeDFSPHConstantDensity(s->phys, s->mat, sph, s->bmat, bp, nei(s->hash_sph, sph),
                                                          nei(s->hash_sph, bp));
            break;
        case 9:  // :277-278, frame++
            mps::kernel::Advect::BoundaryCollision(s->phys, sph);
            mps::kernel::Advect::UpdatePosition(s->phys, sph);
            s->frame++;
            break;
        default:
            return -1;
    }
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : -2;
}

// One OnUpdate per step, with the reference's frame-start and frame-end device syncs.
REF_API int ref_step(void* hp, int nsteps) {
    for (int k = 0; k < nsteps; ++k) {
        cudaDeviceSynchronize();
        for (int ph = 0; ph <= 9; ++ph) {
            const int r = ref_phase(hp, ph);
            if (r) return r;
        }
        if (cudaDeviceSynchronize() != cudaSuccess) return -2;
    }
    return 0;
}

// Copies a named array to host memory; returns element count (doubles, floats or u32) or -1.
REF_API long long ref_get(void* hp, const char* name, void* out) {
    auto* s = static_cast<RefSim*>(hp);
    const std::string k(name);
    const size_t n = s->sph.size, nb = s->bp.size;
    auto cp = [&](const void* src, size_t bytes, long long count) {
        if (out) cudaMemcpy(out, src, bytes, cudaMemcpyDeviceToHost);
        return count;
    };
    if (k == "pos") return cp(s->sph.pPosition, n * sizeof(REAL3), (long long)(3 * n));
    if (k == "vel") return cp(s->sph.pVelocity, n * sizeof(REAL3), (long long)(3 * n));
    if (k == "mass") return cp(s->sph.pMass, n * sizeof(REAL), (long long)n);
    if (k == "radius") return cp(s->sph.pRadius, n * sizeof(REAL), (long long)n);
    if (k == "density") return cp(s->sph.pDensity, n * sizeof(REAL), (long long)n);
    if (k == "alpha") return cp(s->sph.pFactorDFSPH, n * sizeof(REAL), (long long)n);
    if (k == "pressure") return cp(s->sph.pPressure, n * sizeof(REAL), (long long)n);
    if (k == "stfac") return cp(s->sph.pFactorST, n * sizeof(REAL), (long long)n);
    if (k == "color") return cp(s->sph.pColor, n * sizeof(glm::fvec4), (long long)(4 * n));
    if (k == "bpos") return cp(s->bp.pPosition, nb * sizeof(REAL3), (long long)(3 * nb));
    if (k == "bvol") return cp(s->bp.pVolume, nb * sizeof(REAL), (long long)nb);
    if (k.rfind("nei_", 0) == 0) {
        const bool ff = k.find("ff") != std::string::npos, fb = k.find("fb") != std::string::npos;
        const mps::SpatialHash& h = (ff || fb) ? s->hash_sph : s->hash_bp;
        const mps::ParticleParam& key = ff ? static_cast<const mps::ParticleParam&>(s->sph)
                                           : static_cast<const mps::ParticleParam&>(s->bp);
        const auto np = h.GetNeighborhood(key);
        if (!np) return -1;
        const size_t rows = (ff || fb) ? n : nb;
        std::vector<uint32_t> idx(rows + 1);
        cudaMemcpy(idx.data(), np->pIdx, (rows + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        if (k.size() > 7 && k.compare(k.size() - 4, 4, "_idx") == 0) {
            if (out) std::memcpy(out, idx.data(), idx.size() * sizeof(uint32_t));
            return (long long)idx.size();
        }
        if (out) cudaMemcpy(out, np->pID, idx[rows] * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        return (long long)idx[rows];
    }
    return -1;
}

// The reference's mesh path on given vertices/faces: adjacency and R-triangle ownership as
// MeshObject::buildAdjacency does (MPSMeshObject.cu:172-214), then ParticleSampling
// (MPSParticleSamplingUtil.cu:42-133).  Writes up to cap positions (x, y, z) and returns the
// sample count (or -1 on a CUDA error).
REF_API long long ref_sample_mesh(const double* verts, long long nv, const unsigned* faces, long long nf,
                                  double mesh_radius, double* out_pos3, long long cap) {
    thrust::device_vector<glm::uvec3> d_face(reinterpret_cast<const glm::uvec3*>(faces),
                                             reinterpret_cast<const glm::uvec3*>(faces) + nf);
    thrust::device_vector<REAL3> d_pos(reinterpret_cast<const REAL3*>(verts), reinterpret_cast<const REAL3*>(verts) + nv);
    const unsigned nb = 256u;
    const unsigned grid = unsigned((nf + nb - 1) / nb);
    thrust::device_vector<uint32_t> nbFacesID(size_t(nv) + 1, 0u);
    ComputeNbFacesSize_kernel<<<grid, nb>>>(thrust::raw_pointer_cast(d_face.data()), size_t(nf),
                                            thrust::raw_pointer_cast(nbFacesID.data()));
    thrust::exclusive_scan(nbFacesID.begin(), nbFacesID.end(), nbFacesID.begin());
    thrust::device_vector<uint32_t> nbFacesIdx = nbFacesID;
    const uint32_t total = nbFacesID.back();
    thrust::device_vector<uint2> vertexID(total);
    thrust::device_vector<uint32_t> nbFaces(total);
    ComputeNbFaces_kernel<<<grid, nb>>>(thrust::raw_pointer_cast(d_face.data()), size_t(nf),
                                        thrust::raw_pointer_cast(vertexID.data()),
                                        thrust::raw_pointer_cast(nbFacesID.data()));
    thrust::sort(vertexID.begin(), vertexID.end(), mcuda::util::SortUint2CMP());
    thrust::transform(vertexID.begin(), vertexID.end(), nbFaces.begin(), mcuda::util::TransformUint2CMP());
    thrust::device_vector<uint32_t> rTri(nf, 0u);
    RTriangleBuild_kernel<<<grid, nb>>>(thrust::raw_pointer_cast(d_face.data()), size_t(nf),
                                        thrust::raw_pointer_cast(nbFaces.data()),
                                        thrust::raw_pointer_cast(nbFacesIdx.data()),
                                        thrust::raw_pointer_cast(rTri.data()));
    mps::MeshMaterialParam mat{};
    mat.radius = mesh_radius;
    mat.frontColor = glm::fvec4{0.0f, 0.0f, 0.0f, 1.0f};
    thrust::device_vector<uint32_t> sampSize(nf, 0u), shortEdge(nf, 0u), prevIdx(size_t(nf) + 1, 0u),
        currIdx(size_t(nf) + 1, 0u);
    thrust::device_vector<bool> isGen(nf, false), applied(1, false);
    ComputeSamplingNum_kernel<<<grid, nb>>>(mat, thrust::raw_pointer_cast(d_face.data()),
                                            thrust::raw_pointer_cast(d_pos.data()), thrust::raw_pointer_cast(rTri.data()),
                                            thrust::raw_pointer_cast(sampSize.data()),
                                            thrust::raw_pointer_cast(shortEdge.data()), size_t(nf),
                                            thrust::raw_pointer_cast(prevIdx.data()),
                                            thrust::raw_pointer_cast(currIdx.data()),
                                            thrust::raw_pointer_cast(isGen.data()),
                                            thrust::raw_pointer_cast(applied.data()));
    thrust::exclusive_scan(prevIdx.begin(), prevIdx.end(), prevIdx.begin());
    thrust::exclusive_scan(currIdx.begin(), currIdx.end(), currIdx.begin());
    const uint32_t count = currIdx.back();
    thrust::device_vector<uint32_t> faceID(count);
    thrust::device_vector<REAL2> bcc(count);
    thrust::device_vector<REAL3> pos(count);
    thrust::device_vector<REAL> rad(count);
    thrust::device_vector<glm::fvec4> col(count);
    GenerateBoundaryParticle_kernel<<<grid, nb>>>(
        mat, thrust::raw_pointer_cast(d_face.data()), thrust::raw_pointer_cast(d_pos.data()),
        thrust::raw_pointer_cast(rTri.data()), thrust::raw_pointer_cast(shortEdge.data()), size_t(nf),
        thrust::raw_pointer_cast(faceID.data()), thrust::raw_pointer_cast(bcc.data()), thrust::raw_pointer_cast(pos.data()),
        thrust::raw_pointer_cast(rad.data()), thrust::raw_pointer_cast(col.data()), nullptr, nullptr, nullptr, nullptr,
        nullptr, thrust::raw_pointer_cast(prevIdx.data()), thrust::raw_pointer_cast(currIdx.data()),
        thrust::raw_pointer_cast(isGen.data()));
    if (cudaDeviceSynchronize() != cudaSuccess) return -1;
    if (out_pos3 && count > 0)
        cudaMemcpy(out_pos3, thrust::raw_pointer_cast(pos.data()), size_t(std::min<long long>(count, cap)) * sizeof(REAL3),
                   cudaMemcpyDeviceToHost);
    return (long long)count;
}

REF_API int ref_put(void* hp, const char* name, const double* in, long long count) {
    auto* s = static_cast<RefSim*>(hp);
    const std::string k(name);
    const size_t n = s->sph.size, nb = s->bp.size;
    if (k == "vel" && count == (long long)(3 * n)) return cudaMemcpy(s->sph.pVelocity, in, count * 8, cudaMemcpyHostToDevice) ? -2 : 0;
    if (k == "bvol" && count == (long long)nb) return cudaMemcpy(s->bp.pVolume, in, count * 8, cudaMemcpyHostToDevice) ? -2 : 0;
    return -1;
}
