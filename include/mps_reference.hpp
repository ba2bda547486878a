// mps_reference.hpp -- the reference's step API over libmps_gb300.so (C ABI: mps_c.h).
//
// moonsh5009/MPS_CUDA steps its fluid in mps::System::OnUpdate (src/MPS_System/MPSSystem.cpp:
// 191-291) through free functions of mps::kernel::SPH / mps::kernel::Advect that take non-owning
// `*Param` views of the particle objects, and the neighbour search class mps::SpatialHash.  This
// header keeps those names, signatures and call semantics so that OnUpdate's body compiles and runs
// against this library with its call sequence unchanged:
//   - views: ObjectParam / ParticleParam / SPHParam / BoundaryParticleParam (MPSObjectParam.h:8-18,
//     MPSParticleParam.h:7-10, MPSSPHParam.h:7-20, MPSBoundaryParticleParam.h:7-15), NeiParam and
//     SpatialHashParam (MPSSpatialHash.h:14-18, MPSSpatialHashParam.h:8-18);
//   - objects and their device resources: Object::GetDeviceResource<T>() (MPSObject.h:26-34),
//     SPHObject, BoundaryParticleObject, SPHResource::GetSPHParam(),
//     BoundaryParticleResource::GetBoundaryParticleParam();
//   - models: Model::GetTarget<T>() / GetSubObject() / GetMaterial() / GetTree() (MPSModel.h:8-98),
//     SPHModel, ObstacleModel with ObstacleTreeIdx (MPSSPHModel.h, MPSObstacleModel.h);
//   - materials: SPHMaterial / MeshMaterial with the reference's defaults and setters
//     (MPSSPHMaterial.cpp:4-44, MPSMeshMaterial.cpp:4-20); PhysicsParam (MPSUniformDef.h:19-25) in
//     a GBArchiver (MPSGBArchiver.h:16-35);
//   - mps::SpatialHash::{SetObjectSize, SetCeilSize, SetHashSize, UpdateHash, ZSort,
//     BuildNeighorhood, GetNeighborhood} (MPSSpatialHash.h:20-48);
//   - mps::kernel::SPH::{ComputeBoundaryParticleVolumeSub/Final, ComputeDensitySub/Final,
//     DensityColorTest, ComputeDFSPHFactorSub/Final, ComputeDFSPHDivergenceFree,
//     ComputeDFSPHConstantDensity, ApplyImplicitViscosityNSurfaceTension,
//     ComputeSurfaceTensionFactor} and mps::kernel::Advect::{ResetREAL, ResetForce, ApplyGravity,
//     UpdateVelocity, UpdatePosition, BoundaryCollision}.
//
// What differs, by design of the GB300 step:
//   - REAL, the element type of the device views, is float: the library computes in FP32 (the
//     reference's float branch of MPSDef.h:5-22).  Host parameters (PhysicsParam, materials) stay
//     FP64 as in the reference's build.
//   - The views name the library's arrays in its layout: structure of arrays in the per-step cell
//     order ("slots", padded), positions as float4 (x, y, z, support radius h = 4 r), velocities
//     as float4 (vx, vy, vz, mass).  Fields with no array of their own are null: pMass and
//     pRadius (in pVelocity[i].w and pPosition[i].w), pForce (forces are applied where they are
//     computed), pFactorST, pTempMat3, pPreviousVel, pPredictVel, pFaceID, pBCC.  pTempVec3 names
//     four floats of scratch a slot.  Positions and velocities move to the other of two buffers at
//     every cell sort (UpdateHash): views taken before it name the previous order.
//   - The fluid is re-sorted by cell in every UpdateHash, so ZSort is a no-op; the boundary is
//     static, sorted once when it is set, and its volumes are computed then (the reference's
//     accumulating volume is reproduced when mps_config.volume_accumulate is set).
//   - Neighbour lists: BuildNeighorhood of the fluid builds the fluid-fluid and fluid-boundary
//     lists in one pass (the second BuildNeighorhood call finds them current); NeiParam names them
//     (pID = the interleaved lists, pIdx = the per-slot counts, see mps_device_views).
//   - The Sub functions name the neighbour sets of the sum; the Final function runs one pass over
//     them (the reference accumulates partial sums into the arrays with atomics).  ApplyGravity
//     names gravity for the next UpdateVelocity.  The solver drivers run their loops on the device.
//   - One fluid object and one boundary object per library handle: the overloads that take a
//     second fluid object (refSPHMaterial, refSPH) throw mps::Error.  The inner steps of the solver
//     drivers (ComputeDensityDeltaSub, ComputeDFSPH*Sub, ApplyDFSPHSub/Final, the CG's Ap and b
//     functions) are not exposed one by one: the drivers' loops run on the device.
//   - Errors throw mps::Error (the reference reports nothing; its CUDA_CHECK is a no-op in Release).
//   - Work goes to the stream set with mps::kernel::SetStream (default: the legacy default stream,
//     as in the reference).
#pragma once

#include <array>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <optional>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "mps_c.h"

namespace mps {

// ------------------------------------------------------------------ types
using REAL = float;
struct REAL2 { float x, y; };
struct REAL3 { float x, y, z; };
struct REAL4 { float x, y, z, w; };
struct REAL3x3 { float m[3][3]; };
using Vec3d = std::array<double, 3>;
using Color4 = std::array<float, 4>;

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
    double dt = 0.005;
    Vec3d gravity{0.0, -9.8, 0.0};
    Vec3d min{-5.0, -5.0, -5.0};
    Vec3d max{5.0, 5.0, 5.0};
};

// SPHMaterialParam (MPSSPHMaterial.h:9-21) and MeshMaterialParam (MPSMeshMaterial.h:9-20).
struct SPHMaterialParam {
    double radius;
    double mass;
    double density;
    double volume;
    double viscosity;
    double XSPH;
    double surfaceTension;
    Color4 color;
};
struct MeshMaterialParam {
    double radius;
    double mass;
    double density;
    double viscosity;
    double surfaceTension;
    Color4 frontColor;
    Color4 backColor;
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

// ------------------------------------------------------------------ materials (MPSMaterial.h)
class Material {
public:
    virtual ~Material() = default;
};
template <class T>
class VirtualMaterial : public Material {
public:
    T& GetParam() { return m_param; }
    const T& GetParam() const { return m_param; }

private:
    T m_param{};
};

// SPHMaterial (MPSSPHMaterial.cpp): radius is the support radius h (the reference calls
// SetRadius(4 r)); V = h^3 / 48 * 3.141592 and m = density * V as the reference computes them.
class SPHMaterial : public VirtualMaterial<SPHMaterialParam> {
public:
    SPHMaterial() {
        SetParam(0.01, 1.0);
        SetViscosity(0.025);
        SetXSPH(0.1);
        SetSurfaceTension(100.0);
        SetColor({0.3f, 0.8f, 0.2f, 1.0f});
    }
    void SetParam(double radius, double density) {
        GetParam().radius = radius;
        GetParam().volume = radius * radius * radius / 48.0 * 3.141592;
        GetParam().density = density;
        GetParam().mass = density * GetParam().volume;
    }
    void SetRadius(double radius) { SetParam(radius, GetDensity()); }
    void SetViscosity(double viscosity) { GetParam().viscosity = viscosity; }
    void SetXSPH(double XSPH) { GetParam().XSPH = XSPH; }
    void SetSurfaceTension(double surfaceTension) { GetParam().surfaceTension = surfaceTension; }
    void SetColor(const Color4& color) { GetParam().color = color; }
    // A material with explicit mass and volume (physical units, V = spacing^3); no counterpart in
    // the reference, whose volume always follows SetRadius.
    void SetPhysical(double radius, double density, double volume) {
        GetParam().radius = radius;
        GetParam().density = density;
        GetParam().volume = volume;
        GetParam().mass = density * volume;
    }
    double GetRadius() const { return GetParam().radius; }
    double GetMass() const { return GetParam().mass; }
    double GetDensity() const { return GetParam().density; }
    double GetVolume() const { return GetParam().volume; }
    double GetViscosity() const { return GetParam().viscosity; }
    double GetXSPH() const { return GetParam().XSPH; }
    double GetSurfaceTension() const { return GetParam().surfaceTension; }
    const Color4& GetColor() const { return GetParam().color; }
};

// MeshMaterial (MPSMeshMaterial.cpp:4-20): the boundary's material.  The step reads nothing from
// it (boundary particles act through their Akinci volumes); it is kept for the drivers' signatures.
class MeshMaterial : public VirtualMaterial<MeshMaterialParam> {
public:
    MeshMaterial() {
        SetParam(0.1, 1.0);
        GetParam().viscosity = 0.0;
        GetParam().surfaceTension = 0.0;
        GetParam().frontColor = {0.0f, 0.0f, 0.0f, 1.0f};
        GetParam().backColor = {0.0f, 0.0f, 0.0f, 1.0f};
    }
    void SetParam(double radius, double density) {
        GetParam().radius = radius;
        const double volume = radius * radius * radius / 48.0 * 3.141592;
        GetParam().density = density;
        GetParam().mass = density * volume;
    }
};

// ------------------------------------------------------------------ views
enum class ObjectKind : int32_t { Fluid = 0, Boundary = 1 };

struct ObjectParam {
    size_t size;
    size_t phaseID;
    REAL4* pColor;       // colour per slot (the reference's GL colour buffer, headless)
    REAL4* pPosition;    // (x, y, z, h) per slot
    REAL* pMass;         // null: the mass is pVelocity[i].w
    REAL4* pVelocity;    // (vx, vy, vz, m) per slot
    REAL3* pForce;       // null: forces are applied where they are computed
    mps_handle* handle;  // the library state the view belongs to (no counterpart in the reference)
    ObjectKind kind;
};
struct ParticleParam : public ObjectParam {
    REAL* pRadius;       // null: the support radius is pPosition[i].w
};
struct SPHParam : public ParticleParam {
    REAL* pDensity;
    REAL* pPressure;     // stiffness kappa of the last solver iteration
    REAL* pFactorDFSPH;  // alpha
    REAL* pFactorST;
    REAL* pFactorSTB;
    REAL* pTempReal;     // density change rate of the last pressure iteration
    REAL3* pTempVec3;    // four floats of scratch a slot
    REAL3x3* pTempMat3;
    REAL3* pPreviousVel;
    REAL3* pPredictVel;
};
struct BoundaryParticleParam : public ParticleParam {
    uint32_t* pFaceID;
    REAL2* pBCC;
    REAL* pVolume;
    REAL3* pPreviousVel;
    REAL3* pPredictVel;
};
// A neighbour set: pID = interleaved lists (k-th neighbour of slot i at pID[k * stride + i]),
// pIdx = per-slot counts (fluid | boundary << 16); {nullptr, nullptr} names no set.
struct NeiParam {
    const uint32_t* pID;
    const uint32_t* pIdx;
    int32_t set = 0;      // MPS_PART_FLUID or MPS_PART_BOUNDARY
    int64_t stride = 0;
};
struct SpatialHashParam {
    size_t objSize;
    REAL ceilSize;
    std::array<uint32_t, 3> hashSize;
    uint32_t* pKey;      // null: the cell keys are 64-bit and internal to the library
    uint32_t* pID;
    uint32_t* pStartIdx;
    uint32_t* pEndIdx;
};

// ------------------------------------------------------------------ resources and objects
class ObjectResource {
public:
    ObjectResource(mps_handle* h, ObjectKind kind) : m_handle(h), m_kind(kind) {}
    virtual ~ObjectResource() = default;
    std::weak_ptr<ObjectParam> GetObjectParam() const { return m_pParam; }
    virtual void SetParam() {
        if (!m_pParam) m_pParam = std::make_shared<ObjectParam>();
        Fill(*m_pParam);
    }

protected:
    void Fill(ObjectParam& p) {
        if (!m_handle) throw Error(MPS_E_STATE, "object not bound to a simulation");
        mps_device_views v;
        Check(mps_get_device_views(m_handle, &v));
        const bool fluid = m_kind == ObjectKind::Fluid;
        p.size = size_t(fluid ? v.n : v.nb);
        p.phaseID = fluid ? 0 : 1;
        p.pColor = fluid ? reinterpret_cast<REAL4*>(v.color4) : nullptr;
        p.pPosition = reinterpret_cast<REAL4*>(fluid ? v.pos4 : v.bpos4);
        p.pMass = nullptr;
        p.pVelocity = fluid ? reinterpret_cast<REAL4*>(v.vel4) : nullptr;
        p.pForce = nullptr;
        p.handle = m_handle;
        p.kind = m_kind;
        m_views = v;
    }
    std::shared_ptr<ObjectParam> m_pParam;
    mps_handle* m_handle;
    ObjectKind m_kind;
    mps_device_views m_views{};
};
class ParticleResource : public ObjectResource {
public:
    using ObjectResource::ObjectResource;
    std::weak_ptr<ParticleParam> GetParticleParam() const { return std::static_pointer_cast<ParticleParam>(m_pParam); }
    void SetParam() override {
        if (!m_pParam) m_pParam = std::make_shared<ParticleParam>();
        FillParticle(*std::static_pointer_cast<ParticleParam>(m_pParam));
    }

protected:
    void FillParticle(ParticleParam& p) {
        Fill(p);
        p.pRadius = nullptr;
    }
};
class SPHResource : public ParticleResource {
public:
    explicit SPHResource(mps_handle* h) : ParticleResource(h, ObjectKind::Fluid) {}
    std::weak_ptr<SPHParam> GetSPHParam() const { return std::static_pointer_cast<SPHParam>(m_pParam); }
    void SetParam() override {
        if (!m_pParam) m_pParam = std::make_shared<SPHParam>();
        auto& p = *std::static_pointer_cast<SPHParam>(m_pParam);
        FillParticle(p);
        p.pDensity = m_views.density;
        p.pPressure = m_views.pressure;
        p.pFactorDFSPH = m_views.alpha;
        p.pFactorST = nullptr;
        p.pFactorSTB = nullptr;
        p.pTempReal = m_views.delta;
        p.pTempVec3 = reinterpret_cast<REAL3*>(m_views.scratch4);
        p.pTempMat3 = nullptr;
        p.pPreviousVel = nullptr;
        p.pPredictVel = nullptr;
    }
};
class BoundaryParticleResource : public ParticleResource {
public:
    explicit BoundaryParticleResource(mps_handle* h) : ParticleResource(h, ObjectKind::Boundary) {}
    std::weak_ptr<BoundaryParticleParam> GetBoundaryParticleParam() const {
        return std::static_pointer_cast<BoundaryParticleParam>(m_pParam);
    }
    void SetParam() override {
        if (!m_pParam) m_pParam = std::make_shared<BoundaryParticleParam>();
        auto& p = *std::static_pointer_cast<BoundaryParticleParam>(m_pParam);
        FillParticle(p);
        p.pFaceID = nullptr;
        p.pBCC = nullptr;
        p.pVolume = m_views.bvol;
        p.pPreviousVel = nullptr;
        p.pPredictVel = nullptr;
    }
};

// Object (MPSObject.h:9-47): here a view of one particle set of a library handle; the arrays
// belong to the handle.  GetDeviceResource<T>() returns a resource whose views are current at
// the time of the call.
class Object {
public:
    virtual ~Object() = default;
    void Bind(mps_handle* h) { m_handle = h; }
    mps_handle* Handle() const { return m_handle; }
    size_t GetSize() const {
        if (!m_handle) return 0;
        mps_device_views v;
        Check(mps_get_device_views(m_handle, &v));
        return size_t(Kind() == ObjectKind::Fluid ? v.n : v.nb);
    }
    template <class T>
    std::shared_ptr<const T> GetDeviceResource() {
        std::shared_ptr<T> r = std::static_pointer_cast<T>(GenerateDeviceResource());
        if (!r) return nullptr;
        r->SetParam();
        return std::const_pointer_cast<const T>(r);
    }

protected:
    virtual ObjectKind Kind() const = 0;
    virtual std::shared_ptr<ObjectResource> GenerateDeviceResource() = 0;
    mps_handle* m_handle = nullptr;
};
class ParticleObject : public Object {};
class SPHObject : public ParticleObject {
protected:
    ObjectKind Kind() const override { return ObjectKind::Fluid; }
    std::shared_ptr<ObjectResource> GenerateDeviceResource() override { return std::make_shared<SPHResource>(m_handle); }
};
class BoundaryParticleObject : public ParticleObject {
protected:
    ObjectKind Kind() const override { return ObjectKind::Boundary; }
    std::shared_ptr<ObjectResource> GenerateDeviceResource() override {
        return std::make_shared<BoundaryParticleResource>(m_handle);
    }
};
// MeshObject: the obstacle's triangle mesh in host memory (vertices xyz, faces as vertex
// triples), the source of its boundary particles (System::SampleBoundaryMesh).
class MeshObject : public Object {
public:
    std::vector<double> m_vertices;
    std::vector<uint32_t> m_faces;

protected:
    ObjectKind Kind() const override { return ObjectKind::Boundary; }
    std::shared_ptr<ObjectResource> GenerateDeviceResource() override { return nullptr; }
};

// ------------------------------------------------------------------ trees (MPSTree.h)
class Tree {
public:
    virtual ~Tree() = default;
};
template <class T>
class VirtualTree : public Tree {
public:
    T& GetParam() { return m_param; }
    const T& GetParam() const { return m_param; }

private:
    T m_param{};
};

namespace kernel {
// Stream of the drop-in API's work (per host thread; default: the legacy default stream).
inline void*& CurrentStream() {
    thread_local void* s = nullptr;
    return s;
}
inline void SetStream(void* stream) { CurrentStream() = stream; }
inline void* GetStream() { return CurrentStream(); }
}  // namespace kernel

// SpatialHash (MPSSpatialHash.h:20-57).  The fluid's hash sorts the fluid by cell (64-bit keys,
// radix sort, reorder into slots) and builds its neighbour lists; the boundary's hash has nothing
// to do per step (the boundary is sorted once when it is set).
class SpatialHash : public VirtualTree<SpatialHashParam> {
public:
    void SetObjectSize(size_t size) { GetParam().objSize = size; }
    // The library sizes its grid from the collision box and the largest support radius; the
    // reference's cell size and 64^3 wrapped table size are recorded only.
    void SetCeilSize(REAL size) { GetParam().ceilSize = size; }
    void SetHashSize(const std::array<uint32_t, 3>& size) { GetParam().hashSize = size; }
    uint32_t GetObjectSize() const { return uint32_t(GetParam().objSize); }
    REAL GetCeilSize() const { return GetParam().ceilSize; }
    const std::array<uint32_t, 3>& GetHashSize() const { return GetParam().hashSize; }

    void UpdateHash(const ParticleParam& p) {
        if (p.kind != ObjectKind::Fluid) return;
        Check(mps_phase(p.handle, MPS_PHASE_SORT, kernel::GetStream()));
        m_listsCurrent = false;
    }
    // The reference re-sorts by Morton code every 50 frames; here the fluid is re-sorted by cell
    // in every UpdateHash.
    void ZSort(ParticleParam&) {}
    void ZSort(SPHParam&) {}
    void ZSort(BoundaryParticleParam&) {}
    void BuildNeighorhood(const ParticleParam& p) {
        if (p.kind == ObjectKind::Fluid) BuildLists(p.handle);
    }
    void BuildNeighorhood(const ParticleParam& p, const ParticleParam& ref, const SpatialHash*) {
        if (p.kind == ObjectKind::Fluid && ref.kind == ObjectKind::Boundary) BuildLists(p.handle);
    }
    std::optional<NeiParam> GetNeighborhood(const ParticleParam& p) const {
        if (!m_handle || !m_listsCurrent) return std::nullopt;
        mps_device_views v;
        Check(mps_get_device_views(m_handle, &v));
        if (p.kind == ObjectKind::Fluid) return NeiParam{v.nbr_fluid, v.nbr_count, MPS_PART_FLUID, v.nbr_stride};
        return NeiParam{v.nbr_boundary, v.nbr_count, MPS_PART_BOUNDARY, v.nbr_stride};
    }

private:
    void BuildLists(mps_handle* h) {
        m_handle = h;
        if (m_listsCurrent) return;
        Check(mps_phase(h, MPS_PHASE_NEIGHBORS, kernel::GetStream()));
        m_listsCurrent = true;
    }
    mps_handle* m_handle = nullptr;
    bool m_listsCurrent = false;
};

// ------------------------------------------------------------------ models (MPSModel.h)
class Model {
public:
    explicit Model(std::unique_ptr<Object>&& main) : m_pMainObject(std::move(main)) {}
    virtual ~Model() = default;
    template <class T>
    T* GetTarget() const { return static_cast<T*>(m_pMainObject.get()); }
    virtual Object* GetSubObject() const = 0;
    virtual Material* GetMaterial() const = 0;
    virtual Tree* GetTree() const = 0;
    virtual Object* GetSubObject(uint32_t idx) const = 0;
    virtual Material* GetMaterial(uint32_t idx) const = 0;
    virtual Tree* GetTree(uint32_t idx) const = 0;

protected:
    std::unique_ptr<Object> m_pMainObject;
};
template <uint32_t NS, uint32_t NM, uint32_t NT>
class VirtualModel : public Model {
public:
    using Model::Model;
    Object* GetSubObject() const override { return NS ? m_aSubObject[0].get() : nullptr; }
    Material* GetMaterial() const override { return NM ? m_aMaterial[0].get() : nullptr; }
    Tree* GetTree() const override { return NT ? m_aTree[0].get() : nullptr; }
    Object* GetSubObject(uint32_t idx) const override { return idx < NS ? m_aSubObject[idx].get() : nullptr; }
    Material* GetMaterial(uint32_t idx) const override { return idx < NM ? m_aMaterial[idx].get() : nullptr; }
    Tree* GetTree(uint32_t idx) const override { return idx < NT ? m_aTree[idx].get() : nullptr; }

protected:
    std::array<std::unique_ptr<Object>, NS ? NS : 1> m_aSubObject;
    std::array<std::unique_ptr<Material>, NM ? NM : 1> m_aMaterial;
    std::array<std::unique_ptr<Tree>, NT ? NT : 1> m_aTree;
};
class SPHModel : public VirtualModel<0u, 1u, 1u> {
public:
    SPHModel(std::unique_ptr<SPHObject>&& object, std::unique_ptr<SPHMaterial>&& material,
             std::unique_ptr<SpatialHash>&& tree)
        : VirtualModel<0u, 1u, 1u>(std::move(object)) {
        m_aMaterial[0] = std::move(material);
        m_aTree[0] = std::move(tree);
    }
};
enum class ObstacleSubObjectIdx : uint32_t { BoundaryParticle, Size };
enum class ObstacleTreeIdx : uint32_t { SpatialHash, Size };
class ObstacleModel : public VirtualModel<uint32_t(ObstacleSubObjectIdx::Size), 1u, uint32_t(ObstacleTreeIdx::Size)> {
    using Super = VirtualModel<uint32_t(ObstacleSubObjectIdx::Size), 1u, uint32_t(ObstacleTreeIdx::Size)>;

public:
    ObstacleModel(std::unique_ptr<MeshObject>&& mesh, std::unique_ptr<BoundaryParticleObject>&& particles,
                  std::unique_ptr<MeshMaterial>&& material, std::unique_ptr<SpatialHash>&& hash)
        : Super(std::move(mesh)) {
        m_aSubObject[uint32_t(ObstacleSubObjectIdx::BoundaryParticle)] = std::move(particles);
        m_aMaterial[0] = std::move(material);
        m_aTree[uint32_t(ObstacleTreeIdx::SpatialHash)] = std::move(hash);
    }
};

// GBArchiver (MPSGBArchiver.h:16-35): here only its PhysicsParam (camera and light buffers are
// rendering state).
struct GBArchiver {
    PhysicsParam m_physicsParam;
};

// ------------------------------------------------------------------ step functions
namespace detail {
// The library keeps the physics and material it was given; a driver called with different
// values (the caller edited its PhysicsParam or material) passes them on first.
struct Sent {
    mps_physics phys{};
    mps_material mat{};
    bool has_phys = false, has_mat = false;
};
inline std::unordered_map<const mps_handle*, Sent>& SentTable() {
    static std::unordered_map<const mps_handle*, Sent> t;
    return t;
}
inline std::mutex& SentMutex() {
    static std::mutex m;
    return m;
}
inline void Forget(const mps_handle* h) {
    std::lock_guard<std::mutex> lk(SentMutex());
    SentTable().erase(h);
}
inline void SyncPhysics(mps_handle* h, const PhysicsParam& p) {
    const mps_physics c = ToC(p);
    std::lock_guard<std::mutex> lk(SentMutex());
    Sent& s = SentTable()[h];
    if (s.has_phys && std::memcmp(&s.phys, &c, sizeof(c)) == 0) return;
    Check(mps_set_physics(h, &c));
    s.phys = c;
    s.has_phys = true;
}
inline void SyncMaterial(mps_handle* h, const SPHMaterialParam& m) {
    const mps_material c = ToC(m);
    std::lock_guard<std::mutex> lk(SentMutex());
    Sent& s = SentTable()[h];
    if (s.has_mat && std::memcmp(&s.mat, &c, sizeof(c)) == 0) return;
    Check(mps_set_material(h, &c));
    s.mat = c;
    s.has_mat = true;
}
inline void NoSecondFluid() {
    throw Error(MPS_E_INVALID, "one fluid object per simulation: sums against a second fluid object are not supported");
}
inline void Op(const ObjectParam& o, int32_t op, int32_t parts = 0) {
    Check(mps_op(o.handle, op, parts, kernel::GetStream()));
}
inline void Phase(const ObjectParam& o, int32_t phase) { Check(mps_phase(o.handle, phase, kernel::GetStream())); }
}  // namespace detail

namespace kernel {
namespace SPH {
// MPSSPHBaseUtil.h:9-38
inline void ComputeBoundaryParticleVolumeSub(const BoundaryParticleParam& bp, const NeiParam&) {
    detail::Phase(bp, MPS_PHASE_BVOLUME);   // accumulating form only; otherwise set with the boundary
}
inline void ComputeBoundaryParticleVolumeSub(const BoundaryParticleParam& bp, const NeiParam& nei,
                                             const BoundaryParticleParam&) {
    ComputeBoundaryParticleVolumeSub(bp, nei);
}
inline void ComputeBoundaryParticleVolumeFinal(const BoundaryParticleParam&) {}
inline void ComputeDensitySub(const SPHMaterialParam& mat, const SPHParam& sph, const NeiParam&) {
    detail::SyncMaterial(sph.handle, mat);
    detail::Op(sph, MPS_OP_DENSITY_SUB, MPS_PART_FLUID);
}
inline void ComputeDensitySub(const SPHParam&, const NeiParam&, const SPHMaterialParam&, const SPHParam&) {
    detail::NoSecondFluid();
}
inline void ComputeDensitySub(const SPHParam& sph, const NeiParam&, const BoundaryParticleParam&) {
    detail::Op(sph, MPS_OP_DENSITY_SUB, MPS_PART_BOUNDARY);
}
inline void ComputeDensityFinal(const SPHMaterialParam& mat, const SPHParam& sph) {
    detail::SyncMaterial(sph.handle, mat);
    detail::Op(sph, MPS_OP_DENSITY_FINAL);
}
inline void DensityColorTest(const SPHMaterialParam& mat, const SPHParam& sph) {
    detail::SyncMaterial(sph.handle, mat);
    detail::Op(sph, MPS_OP_COLOR);
}
// MPSSPHDFSPHUtil.h:10-25, 72-87
inline void ComputeDFSPHFactorSub(const SPHMaterialParam& mat, const SPHParam& sph, const NeiParam&) {
    detail::SyncMaterial(sph.handle, mat);
    detail::Op(sph, MPS_OP_FACTOR_SUB, MPS_PART_FLUID);
}
inline void ComputeDFSPHFactorSub(const SPHParam&, const NeiParam&, const SPHMaterialParam&, const SPHParam&) {
    detail::NoSecondFluid();
}
inline void ComputeDFSPHFactorSub(const SPHParam& sph, const NeiParam&, const BoundaryParticleParam&) {
    detail::Op(sph, MPS_OP_FACTOR_SUB, MPS_PART_BOUNDARY);
}
inline void ComputeDFSPHFactorFinal(const SPHParam& sph) { detail::Op(sph, MPS_OP_FACTOR_FINAL); }
inline void ComputeDFSPHDivergenceFree(const PhysicsParam& phys, const SPHMaterialParam& mat, const SPHParam& sph,
                                       const MeshMaterialParam&, const BoundaryParticleParam&, const NeiParam&,
                                       const NeiParam&) {
    detail::SyncPhysics(sph.handle, phys);
    detail::SyncMaterial(sph.handle, mat);
    detail::Phase(sph, MPS_PHASE_DF);
}
inline void ComputeDFSPHConstantDensity(const PhysicsParam& phys, const SPHMaterialParam& mat, const SPHParam& sph,
                                        const MeshMaterialParam&, const BoundaryParticleParam&, const NeiParam&,
                                        const NeiParam&) {
    detail::SyncPhysics(sph.handle, phys);
    detail::SyncMaterial(sph.handle, mat);
    detail::Phase(sph, MPS_PHASE_CD);
}
// MPSSPHNonPressureUtil.h:34-37, 61-65
inline void ComputeSurfaceTensionFactor(const SPHMaterialParam& mat, const SPHParam& sph, const NeiParam&) {
    detail::SyncMaterial(sph.handle, mat);
    detail::Op(sph, MPS_OP_ST_FACTOR);
}
inline void ApplyImplicitViscosityNSurfaceTension(const PhysicsParam& phys, const SPHMaterialParam& mat,
                                                  const SPHParam& sph, const NeiParam&) {
    detail::SyncPhysics(sph.handle, phys);
    detail::SyncMaterial(sph.handle, mat);
    detail::Phase(sph, MPS_PHASE_VISCST);
}
}  // namespace SPH

namespace Advect {
// MPSAdvectUtil.h:12-20.  The boundary is static: the functions do nothing for its views.
inline void ResetREAL(REAL* ptr, size_t size) {
    Check(mps_device_zero(ptr, int64_t(size * sizeof(REAL)), GetStream()));
}
inline void ResetForce(const ObjectParam&) {}
inline void ApplyGravity(const PhysicsParam& phys, const ObjectParam& obj) {
    if (obj.kind != ObjectKind::Fluid) return;
    detail::SyncPhysics(obj.handle, phys);
    detail::Op(obj, MPS_OP_GRAVITY);
}
inline void UpdateVelocity(const PhysicsParam& phys, const ObjectParam& obj) {
    if (obj.kind != ObjectKind::Fluid) return;
    detail::SyncPhysics(obj.handle, phys);
    detail::Op(obj, MPS_OP_UPDATE_VELOCITY);
}
inline void UpdatePosition(const PhysicsParam& phys, const ObjectParam& obj) {
    if (obj.kind != ObjectKind::Fluid) return;
    detail::SyncPhysics(obj.handle, phys);
    detail::Op(obj, MPS_OP_POSITION);
}
inline void BoundaryCollision(const PhysicsParam& phys, const ObjectParam& obj) {
    if (obj.kind != ObjectKind::Fluid) return;
    detail::SyncPhysics(obj.handle, phys);
    detail::Op(obj, MPS_OP_COLLISION);
}
}  // namespace Advect
}  // namespace kernel

// ------------------------------------------------------------------ host instrumentation
// The reference times its frames with MTimer (src/MCUDA_Lib/MTimer.h) and prints through
// OutputDebugStringA.  Here the printing goes to a sink (default: none; mps::SetDebugOutput(stderr)
// to see it), and MTimer keys are owned strings (the reference keys by string_view).
inline std::FILE*& DebugOutput() {
    static std::FILE* f = nullptr;
    return f;
}
inline void SetDebugOutput(std::FILE* f) { DebugOutput() = f; }

}  // namespace mps

// The reference declares its element types at global scope (MPSDef.h:5-22); so does this header,
// with the library's FP32 (define MPS_NO_GLOBAL_REAL to keep them inside namespace mps).
#ifndef MPS_NO_GLOBAL_REAL
using REAL = mps::REAL;
using REAL2 = mps::REAL2;
using REAL3 = mps::REAL3;
using REAL4 = mps::REAL4;
using REAL3x3 = mps::REAL3x3;
#endif

#ifndef MPS_NO_HOST_INSTRUMENTATION
#ifndef _WIN32
inline void OutputDebugStringA(const char* s) {
    if (mps::DebugOutput() && s) std::fputs(s, mps::DebugOutput());
}
#endif
class MTimer {
public:
    static void Start(const std::string& key) {
        std::lock_guard<std::mutex> lk(Mutex());
        Table()[key] = std::chrono::system_clock::now();
    }
    static void End(const std::string& key) {
        std::chrono::system_clock::time_point t0;
        {
            std::lock_guard<std::mutex> lk(Mutex());
            auto it = Table().find(key);
            if (it == Table().end()) return;
            t0 = it->second;
            Table().erase(it);
        }
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::system_clock::now() - t0).count();
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s : %f ms\n", key.c_str(), ms);
        OutputDebugStringA(buf);
    }

private:
    static std::unordered_map<std::string, std::chrono::system_clock::time_point>& Table() {
        static std::unordered_map<std::string, std::chrono::system_clock::time_point> t;
        return t;
    }
    static std::mutex& Mutex() {
        static std::mutex m;
        return m;
    }
};
#endif
