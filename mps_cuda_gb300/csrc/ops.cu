// Function-granular entry points of the step: the C-ABI building blocks of the C++ drop-in API
// (include/mps_reference.hpp), which keeps the reference's step functions -- the free functions of
// mps::kernel::SPH / mps::kernel::Advect (src/MPS_Computer/MPSSPHBaseUtil.h:9-38,
// MPSSPHDFSPHUtil.h:9-87, MPSSPHNonPressureUtil.h:29-65, MPSAdvectUtil.h:12-20) -- callable one by
// one in mps::System::OnUpdate's order (src/MPS_System/MPSSystem.cpp:220-278).
//
// The step fuses several of those functions into one kernel (density + colour + alpha + gravity;
// collision + position); here each runs alone with the same arithmetic, so that a frame driven
// call by call gives the same bits as mps_step.  The reference's Sub/Final pairs accumulate
// partial sums into arrays with atomics; here the Sub calls name the neighbour sets (fluid,
// boundary) and the Final call runs the one pass that sums them.
#include <cstring>

#include "handle.cuh"
#include "mps_c.h"
#include "mps_internal.cuh"

using namespace mpsg;

namespace {
struct DeviceGuard {
    int prev = 0;
    explicit DeviceGuard(int dev) { cudaGetDevice(&prev); cudaSetDevice(dev); }
    ~DeviceGuard() { cudaSetDevice(prev); }
};
constexpr int W_DENSITY = 1, W_COLOR = 2, W_ALPHA = 4, W_GRAVITY = 8;   // launch_density_part
}  // namespace

extern "C" {

int mps_op(mps_handle* h, int32_t op, int32_t parts, void* stream) {
    const int r = host::check_ready(h);
    if (r) return r;
    if (h->batched) return host::fail(MPS_E_STATE, "mps_op drives single-scene handles");
    if ((op == MPS_OP_DENSITY_SUB || op == MPS_OP_FACTOR_SUB) &&
        (parts <= 0 || (parts & ~(MPS_PART_FLUID | MPS_PART_BOUNDARY)) != 0))
        return host::fail(MPS_E_INVALID, "parts must name the fluid and/or boundary neighbours");
    DeviceGuard g(h->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const Params p = host::make_params(h);
    const Dev d = host::make_dev(h, h->cur);
    const int bs = host::block_size(h);
    switch (op) {
        case MPS_OP_DENSITY_SUB: h->pending_density |= parts; return MPS_OK;
        case MPS_OP_DENSITY_FINAL:
            if (!h->pending_density) return host::fail(MPS_E_STATE, "ComputeDensityFinal without ComputeDensitySub");
            launch_density_part(d, p, bs, W_DENSITY, h->pending_density, s);
            h->pending_density = 0;
            break;
        case MPS_OP_COLOR: launch_density_part(d, p, bs, W_COLOR, 0, s); break;
        case MPS_OP_FACTOR_SUB: h->pending_alpha |= parts; return MPS_OK;
        case MPS_OP_FACTOR_FINAL:
            if (!h->pending_alpha) return host::fail(MPS_E_STATE, "ComputeDFSPHFactorFinal without ComputeDFSPHFactorSub");
            launch_density_part(d, p, bs, W_ALPHA, h->pending_alpha, s);
            h->pending_alpha = 0;
            break;
        case MPS_OP_GRAVITY: h->pending_gravity = true; return MPS_OK;
        case MPS_OP_UPDATE_VELOCITY:
            // v += dt F / m with F the gravity named since the last update (the step's only force
            // outside the solvers, which update velocities themselves)
            if (h->pending_gravity) launch_density_part(d, p, bs, W_GRAVITY, 0, s);
            h->pending_gravity = false;
            break;
        case MPS_OP_COLLISION: launch_advect_part(d, p, 1, s); break;
        case MPS_OP_POSITION:
            launch_advect_part(d, p, 2, s);
            h->steps++;
            break;
        case MPS_OP_ST_FACTOR: launch_st_factor(d, p, bs, s); break;
        default: return host::fail(MPS_E_INVALID, "unknown op");
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return host::fail(MPS_E_CUDA, std::string("op launch: ") + cudaGetErrorString(e));
    return MPS_OK;
}

int mps_get_device_views(mps_handle* h, mps_device_views* out) {
    const int r = host::check_ready(h);
    if (r) return r;
    if (!out) return host::fail(MPS_E_INVALID, "null views");
    std::memset(out, 0, sizeof(*out));
    const int c = h->cur;
    out->n = h->n;
    out->nb = h->nb;
    out->slots = h->slots;
    out->pos4 = reinterpret_cast<float*>(h->pos[c]);
    out->vel4 = reinterpret_cast<float*>(h->vel[c]);
    out->ids = h->ids[c];
    out->density = h->rho;
    out->pressure = h->kappa;
    out->alpha = h->alpha;
    out->delta = h->delta;
    out->color4 = reinterpret_cast<float*>(h->color);
    out->scratch4 = reinterpret_cast<float*>(h->cg_ap);
    out->bpos4 = reinterpret_cast<float*>(h->bpos);
    out->bvol = h->bvol;
    out->nbr_fluid = h->nbr_f;
    out->nbr_boundary = h->nbr_b;
    out->nbr_count = h->cnt;
    out->nbr_stride = h->slots;
    out->cap_fluid = h->cfg.max_fluid_neighbors;
    out->cap_boundary = h->cfg.max_boundary_neighbors;
    out->volume_accumulate = h->cfg.volume_accumulate;
    return MPS_OK;
}

int mps_device_zero(void* dev_ptr, int64_t bytes, void* stream) {
    if (bytes < 0 || (bytes > 0 && !dev_ptr)) return host::fail(MPS_E_INVALID, "bad zero range");
    if (bytes == 0) return MPS_OK;
    const cudaError_t e = cudaMemsetAsync(dev_ptr, 0, size_t(bytes), static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return host::fail(MPS_E_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    return MPS_OK;
}

}  // extern "C"
