// The simulation handle behind the C ABI (include/mps_c.h) and the host-side helpers that the
// translation units other than api.cu (the adjoint) use to drive a step.
#pragma once
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "mps_c.h"
#include "mps_internal.cuh"

namespace mpsg {
struct AdjointStore;
}

struct mps_handle {
    int device = 0;
    mps_material mat{};
    mps_physics phys{};
    mps_config cfg{};
    bool batched = false;
    int nscenes = 1;
    std::vector<double> boxes;           // 6 per scene (batched); single scene uses phys
    std::vector<int64_t> fluid_off, bnd_off;
    std::vector<mpsg::Scene> scenes;
    int64_t n = 0, nb = 0;
    int slots = 0;
    unsigned long long total_cells = 0;
    int key_bits = 0;
    bool have_fluid = false;
    bool have_boundary = false;
    bool bvol_given = false;
    bool layout_ready = false;
    int cur = 0;                         // state buffer holding the current order
    int64_t steps = 0;
    // drop-in API (ops.cu): neighbour sets named by the *Sub calls since the last *Final, and
    // gravity named by ApplyGravity since the last UpdateVelocity
    int pending_density = 0, pending_alpha = 0;
    bool pending_gravity = false;

    // device memory
    float4* pos[2] = {nullptr, nullptr};
    float4* vel[2] = {nullptr, nullptr};
    unsigned* ids[2] = {nullptr, nullptr};
    unsigned long long* slot_key = nullptr;
    uint2* ftable = nullptr;
    uint2* btable = nullptr;
    mpsg::Scene* d_scenes = nullptr;
    int* chunk_scene = nullptr;
    unsigned* nbr_f = nullptr;
    unsigned* nbr_b = nullptr;
    unsigned* cnt = nullptr;
    float *rho = nullptr, *rdev = nullptr, *alpha = nullptr, *kappa = nullptr, *delta = nullptr;
    float4* xk = nullptr;
    float2* aux = nullptr;
    float4* color = nullptr;
    float4 *cg_x = nullptr, *cg_r = nullptr, *cg_p = nullptr, *cg_ap = nullptr, *cg_b = nullptr, *cg_s = nullptr;
    float2* cg_coef = nullptr;
    float4* bpos = nullptr;
    float* bvol = nullptr;
    float* bvol_lo = nullptr;           // low part of the boundary volume as a float-float pair
    double* partial = nullptr;
    unsigned long long* acc = nullptr;
    unsigned short* nbr_t = nullptr;
    unsigned int* tile_j = nullptr;
    int* tile_n = nullptr;
    mpsg::SceneSolve* solve = nullptr;
    mpsg::StepCounters* ctr = nullptr;
    int* scene_iters = nullptr;
    double* scene_err = nullptr;
    unsigned long long *keys = nullptr, *keys_tmp = nullptr;
    unsigned *vals = nullptr, *vals_tmp = nullptr;
    unsigned* sort_counts = nullptr;
    float4 *stage_pos = nullptr, *stage_vel = nullptr;   // ID-order staging for I/O
    int* h_nactive = nullptr;                            // pinned
    mpsg::AdjointStore* adj = nullptr;                   // adjoint checkpoints and tape (adjoint.cu)

    std::vector<uint32_t> bperm;        // sorted boundary index -> user boundary index
    std::vector<float4> bpos_user;      // boundary positions as given (x,y,z,h) in user order
    std::vector<float> bvol_user, bvol_user_lo;

    cudaStream_t cap_stream = nullptr;
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;  // (cur, nsteps) -> exec
    std::vector<cudaGraph_t> graph_defs;

    ~mps_handle() { release(); if (cap_stream) { cudaStreamDestroy(cap_stream); cap_stream = nullptr; } }
    void drop_graphs();
    void release();   // frees every device buffer and forgets the layout
};

namespace mpsg {
namespace host {
int fail(int code, const std::string& msg);
Params make_params(const mps_handle* h);
Dev make_dev(const mps_handle* h, int sorted_buf);
int block_size(const mps_handle* h);
int run_phase(mps_handle* h, int phase, cudaStream_t s);
int step_n(mps_handle* h, int nsteps, cudaStream_t s);    // mps_step without argument checks
int check_ready(mps_handle* h);
void adjoint_release(mps_handle* h);                      // frees h->adj (adjoint.cu)
}  // namespace host
}  // namespace mpsg
