// Boundary particles sampled on triangle meshes (scene set-up, not the per-frame step).
//
// Restates, in code of its own, the reference's mesh path:
//  - MeshObject::LoadMesh (src/MPS_Object/MPSMeshObject.cu:58-103): OBJ "v"/"f" records, the
//    mesh's bounding box fitted per axis to a target box (TranslateMesh_kernel, MPSMeshObject.cuh:28-39);
//  - R-triangle ownership (RTriangleBuild_kernel, MPSMeshObject.cuh:41-100): a face owns vertex i
//    when it is the smallest face id around that vertex, and edge (i, i+1) when no other face with a
//    smaller id shares it, so shared vertices and edges are sampled once;
//  - ParticleSampling (src/MPS_Computer/MPSParticleSamplingUtil.cu:42-133, .cuh:10-246): per face,
//    owned vertices, owned edges at spacing d = radius / 2, then scanlines parallel to the shortest
//    edge, each line holding ceil((l - 1.01 d) / d) evenly spaced interior points.
// The per-face counting and generation run on the GPU in FP64 (the reference's precision for this
// set-up step), one thread per face; the count of a face bounds what its generation may write.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "mps_c.h"

namespace {

struct V3 { double x, y, z; };
__host__ __device__ inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ inline V3 mul(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline double len(V3 a) { return sqrt(dot(a, a)); }
__host__ __device__ inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

// Interior points of a segment of length l at spacing about d (GetLineSamplingNum, .cuh:12-17).
__device__ inline unsigned line_points(double l, double d) {
    const double x = (l - d * 1.01) / d;
    if (x <= 0.0) return 0u;
    return unsigned(ceilf(float(x)));
}

struct Emit {
    float4* out;       // may be null (count only)
    unsigned* face_id;
    unsigned at, end;  // next slot, end of this face's slots
    float radius;
    unsigned face;
    __device__ void put(V3 p) {
        if (at < end && out) {
            out[at] = make_float4(float(p.x), float(p.y), float(p.z), radius);
            if (face_id) face_id[at] = face;
        }
        at++;
    }
};

// Interior points of segment a -> b (GenerateLineParticle, .cuh:36-64; the spacing argument is
// single precision there, and so it is here).
__device__ void emit_line(V3 a, V3 b, float d, Emit& e) {
    b = sub(b, a);
    const double l = len(b);
    const unsigned num = line_points(l, d);
    if (num == 0u) return;
    d = float(l / double(num + 1u));
    b = mul(b, double(d) / l);
    for (unsigned k = 0; k < num; ++k) {
        a = add(a, b);
        e.put(a);
    }
}

// Counts (out == null) or writes the samples of face f: the corners and edges the face owns
// (bits 0-2 and 3-5 of rtri[f]), then a sweep of lines parallel to the face's shortest edge,
// stepping both ends along the two other edges.  The steps are the reference's
// (MPSParticleSamplingUtil.cuh:69-240), so that a mesh gives the same boundary particles: the
// parity test of mps_mesh_sample compares count and points with the reference's own sampler.
__device__ unsigned sample_face(const double* V, const unsigned* F, const unsigned* rtri, unsigned f, double R,
                                float4* out, unsigned* face_id, unsigned at, unsigned end) {
    V3 corner[3];
    for (int k = 0; k < 3; ++k) {
        const unsigned v = F[3 * f + k];
        corner[k] = V3{V[3 * v], V[3 * v + 1], V[3 * v + 2]};
    }
    V3 edge[3] = {sub(corner[1], corner[0]), sub(corner[2], corner[1]), sub(corner[0], corner[2])};
    const double elen[3] = {len(edge[0]), len(edge[1]), len(edge[2])};
    unsigned shortest = 0u;
    if (elen[shortest] > elen[1]) shortest = 1u;
    if (elen[shortest] > elen[2]) shortest = 2u;
    const double spacing = (R + R) * 0.25;
    const unsigned owned = rtri[f];
    Emit e{out, face_id, at, end, float(R * 0.25), f};
    for (unsigned c = 0; c < 3u; ++c) {
        if ((owned >> c) & 1u) e.put(corner[c]);
        if ((owned >> (c + 3u)) & 1u) {
            if (out) emit_line(corner[c], corner[(c + 1u) % 3u], float(spacing), e);
            else e.at += line_points(elen[c], spacing);
        }
    }
    // sweep: end A walks edge `ea` from its start, end B walks the reversed edge `eb` from the
    // shortest edge's start (both edges meet the shortest one's far corner)
    const unsigned ea = (shortest + 1u) % 3u, eb = (shortest + 2u) % 3u;
    V3 endA = corner[ea], endB = corner[shortest];
    const V3 normal_in_plane = cross(edge[shortest], cross(edge[shortest], edge[eb]));
    const V3 across = mul(normal_in_plane, 1.0 / sqrt(dot(normal_in_plane, normal_in_plane)));
    const V3 stepB = mul(edge[eb], -1.0);
    const double height = dot(across, edge[ea]);
    const unsigned rows = line_points(height, spacing);
    if (rows > 0u) {
        const double frac = (height / double(rows + 1u)) / height;
        for (unsigned r = 0; r < rows; ++r) {
            endA = add(endA, mul(edge[ea], frac));
            endB = add(endB, mul(stepB, frac));
            if (out) emit_line(endA, endB, float(spacing), e);
            else e.at += line_points(len(sub(endA, endB)), spacing);
        }
    }
    return e.at - at;
}

__global__ void k_mesh_count(const double* V, const unsigned* F, const unsigned* rtri, unsigned nf, double R,
                             unsigned* counts) {
    const unsigned f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    counts[f] = sample_face(V, F, rtri, f, R, nullptr, nullptr, 0u, 0u);
}

__global__ void k_mesh_generate(const double* V, const unsigned* F, const unsigned* rtri, unsigned nf, double R,
                                const unsigned* offsets, float4* out, unsigned* face_id) {
    const unsigned f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    sample_face(V, F, rtri, f, R, out, face_id, offsets[f], offsets[f + 1]);
}

// Ownership flags per face: bit i vertex i, bit 3+i edge (i, i+1).
std::vector<unsigned> ownership(const std::vector<unsigned>& F, size_t nv) {
    const size_t nf = F.size() / 3;
    std::vector<std::vector<unsigned>> around(nv);
    for (size_t f = 0; f < nf; ++f)
        for (int k = 0; k < 3; ++k) around[F[3 * f + k]].push_back(unsigned(f));  // ascending face ids
    std::vector<unsigned> info(nf, 0u);
    for (size_t f = 0; f < nf; ++f) {
        unsigned flags = 0u;
        for (unsigned i = 0; i < 3u; ++i) {
            const auto& a = around[F[3 * f + i]];
            const auto& b = around[F[3 * f + (i + 1u) % 3u]];
            if (a.front() == unsigned(f)) flags |= 1u << i;
            unsigned other = 0xffffffffu;
            for (unsigned t : a) {
                if (t == unsigned(f)) continue;
                if (std::find(b.begin(), b.end(), t) != b.end()) { other = t; break; }
            }
            if (unsigned(f) < other) flags |= 1u << (i + 3u);
        }
        info[f] = flags;
    }
    return info;
}

}  // namespace

extern "C" {

int mps_mesh_load_obj(const char* path, const double center[3], const double size[3], int64_t* nverts,
                      int64_t* nfaces, double* verts3, uint32_t* faces3) {
    if (!path || !nverts || !nfaces) return MPS_E_INVALID;
    std::ifstream in(path);
    if (!in) return MPS_E_INVALID;
    std::vector<double> V;
    std::vector<uint32_t> F;
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        std::string head;
        if (!(ss >> head)) continue;
        if (head == "v") {
            double x, y, z;
            if (ss >> x >> y >> z) { V.push_back(x); V.push_back(y); V.push_back(z); }
        } else if (head == "f") {
            std::vector<uint32_t> idx;
            std::string tok;
            while (ss >> tok) {
                const long v = std::strtol(tok.c_str(), nullptr, 10);  // "a", "a/b", "a/b/c"
                if (v <= 0) return MPS_E_INVALID;
                idx.push_back(uint32_t(v - 1));
            }
            for (size_t k = 1; k + 1 < idx.size(); ++k) {  // fan polygons into triangles
                F.push_back(idx[0]); F.push_back(idx[k]); F.push_back(idx[k + 1]);
            }
        }
    }
    const size_t nv = V.size() / 3;
    if (nv == 0 || F.empty()) return MPS_E_INVALID;
    for (uint32_t i : F)
        if (i >= nv) return MPS_E_INVALID;
    if (center && size) {
        double lo[3] = {V[0], V[1], V[2]}, hi[3] = {V[0], V[1], V[2]};
        for (size_t v = 0; v < nv; ++v)
            for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], V[3 * v + a]); hi[a] = std::max(hi[a], V[3 * v + a]); }
        for (size_t v = 0; v < nv; ++v)
            for (int a = 0; a < 3; ++a) {
                const double oc = (lo[a] + hi[a]) * 0.5, os = hi[a] - lo[a];
                const double sc = os > 1.0e-10 ? size[a] / os : 0.0;
                V[3 * v + a] = (V[3 * v + a] - oc) * sc + center[a];
            }
    }
    *nverts = int64_t(nv);
    *nfaces = int64_t(F.size() / 3);
    if (verts3) std::memcpy(verts3, V.data(), V.size() * sizeof(double));
    if (faces3) std::memcpy(faces3, F.data(), F.size() * sizeof(uint32_t));
    return MPS_OK;
}

int64_t mps_mesh_sample(const double* verts3, int64_t nv, const uint32_t* faces3, int64_t nf, double mesh_radius,
                        float* pos4, uint32_t* face_id) {
    if (!verts3 || !faces3 || nv <= 0 || nf <= 0 || !(mesh_radius > 0.0)) return MPS_E_INVALID;
    std::vector<unsigned> F(faces3, faces3 + 3 * nf);
    for (unsigned i : F)
        if (int64_t(i) >= nv) return MPS_E_INVALID;
    const std::vector<unsigned> info = ownership(F, size_t(nv));
    double* dV = nullptr;
    unsigned *dF = nullptr, *dI = nullptr, *dC = nullptr, *dFace = nullptr;
    float4* dOut = nullptr;
    int64_t total = 0;
    cudaError_t e = cudaSuccess;
    auto check = [&](cudaError_t r) { if (r != cudaSuccess && e == cudaSuccess) e = r; return e == cudaSuccess; };
    const unsigned n = unsigned(nf);
    if (check(cudaMalloc(&dV, size_t(nv) * 3 * sizeof(double))) && check(cudaMalloc(&dF, F.size() * sizeof(unsigned))) &&
        check(cudaMalloc(&dI, info.size() * sizeof(unsigned))) && check(cudaMalloc(&dC, (size_t(n) + 1) * sizeof(unsigned))) &&
        check(cudaMemcpy(dV, verts3, size_t(nv) * 3 * sizeof(double), cudaMemcpyHostToDevice)) &&
        check(cudaMemcpy(dF, F.data(), F.size() * sizeof(unsigned), cudaMemcpyHostToDevice)) &&
        check(cudaMemcpy(dI, info.data(), info.size() * sizeof(unsigned), cudaMemcpyHostToDevice))) {
        k_mesh_count<<<(n + 127) / 128, 128>>>(dV, dF, dI, n, mesh_radius, dC);
        std::vector<unsigned> counts(size_t(n) + 1, 0u);
        if (check(cudaGetLastError()) && check(cudaMemcpy(counts.data(), dC, size_t(n) * sizeof(unsigned), cudaMemcpyDeviceToHost))) {
            std::vector<unsigned> off(size_t(n) + 1, 0u);
            for (unsigned f = 0; f < n; ++f) off[f + 1] = off[f] + counts[f];
            total = off[n];
            if (pos4 && total > 0 && check(cudaMemcpy(dC, off.data(), off.size() * sizeof(unsigned), cudaMemcpyHostToDevice)) &&
                check(cudaMalloc(&dOut, size_t(total) * sizeof(float4))) &&
                (!face_id || check(cudaMalloc(&dFace, size_t(total) * sizeof(unsigned))))) {
                k_mesh_generate<<<(n + 127) / 128, 128>>>(dV, dF, dI, n, mesh_radius, dC, dOut, dFace);
                if (check(cudaGetLastError()) && check(cudaMemcpy(pos4, dOut, size_t(total) * sizeof(float4), cudaMemcpyDeviceToHost)) && face_id)
                    check(cudaMemcpy(face_id, dFace, size_t(total) * sizeof(unsigned), cudaMemcpyDeviceToHost));
            }
        }
    }
    cudaFree(dV); cudaFree(dF); cudaFree(dI); cudaFree(dC); cudaFree(dOut); cudaFree(dFace);
    if (e != cudaSuccess) return MPS_E_CUDA;
    return total;
}

}  // extern "C"
