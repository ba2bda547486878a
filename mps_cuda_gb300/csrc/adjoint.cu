// Reverse-mode gradient of a DFSPH rollout (the adjoint form of the step).  The reference has no
// differentiation; this file adds it on top of the same step kernels (sph.cu), which it re-runs
// with recording hooks.
//
// Differentiated step (fixed iteration counts K, Jacobi viscosity/surface-tension solve):
//   rho_i   = rho0 (V W_ii + V sum_j W_ij + sum_b Vb W_ib)                     (density)
//   alpha_i = 1 / (|V sum_j G_ij x_ij + sum_b Vb G_ib x_ib|^2 + sum_j |V G_ij x_ij|^2)
//   v      += dt g
//   K x DF:  delta_i = V sum_j G_ij x_ij.(u_i - u_j) + sum_b Vb G_ib x_ib.u_i,
//            kappa_i = max(0, min(dt delta_i, rho_i/rho0 + dt delta_i - 0.8)) alpha_i / dt^2,
//            u_i    += -dt [0.5 V sum_j (kappa_i + kappa_j) G_ij x_ij + 0.5 kappa_i sum_b Vb G_ib x_ib]
//   viscosity + surface tension + XSPH: coefficients c_ij, cv_ij, b_i from (x, v, rho, st factor)
//            (k_cg_b), then K block-Jacobi sweeps q += D^-1 (b + f x0 - (A_0 + f I) q) from
//            q = x0 = v, D = each particle's 3x3 diagonal block
//   K x CD:  as DF with kappa_i = max(0, rho_i/rho0 + dt delta_i - 1) alpha_i / dt^2
//   collision (per axis: v, -0.4 v or 0) and x += dt v.
// Neighbour sets are piecewise constant in x (no derivative).  Every pair term's reverse is
// evaluated in gather form: particle i adds the derivatives of the terms it owns (pairs (i, j) of
// its list) and of the terms its neighbours own (pairs (j, i), found through the reverse index
// rev[k][i] = position of i in j's list), so each cotangent is written by one thread and the
// result is deterministic.  The Jacobi solve reverses exactly as K transposed sweeps
// y = D^-1 qbar, qbar -= (A_0 + f I)^T y (D symmetric).  A pair whose reverse entry is missing
// (asymmetric lists, only after a capacity overflow) is skipped and the call reports it.
//
// Memory: checkpoints of the slot-order state every `every` steps and the tapes of one segment:
// per step, K + 1 velocity fields per pressure solve, K + 1 Jacobi iterates, stiffness and branch
// codes, and the step's neighbour lists / solve coefficients / densities the reverse reads; plus
// per-pair cotangents of the solve's coefficients.  The reverse sweep records a segment once from
// its checkpoint (eager, bit-identical to the graph step) and then reverses its steps.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "handle.cuh"
#include "mps_c.h"
#include "mps_internal.cuh"

namespace mpsg {

struct AdjointStore {
    int nsteps = 0, every = 0;       // the recorded forward
    int K = 0, ncp_cap = 0, every_cap = 0;   // capacities of the buffers
    int slots = 0, cap = 0, nscenes = 0;
    int64_t n = 0;
    size_t bytes = 0;
    bool ready = false;              // a forward was recorded
    // checkpoints (slot order of the buffer that was current) and the final state
    float4 *cp_pos = nullptr, *cp_vel = nullptr;
    unsigned* cp_ids = nullptr;
    std::vector<int> cp_cur;
    float4 *fin_pos = nullptr, *fin_vel = nullptr;
    unsigned* fin_ids = nullptr;
    int fin_cur = 0;
    int64_t fin_steps = 0;
    // the tapes of the steps of one segment (every_cap slots, each field laid out slot after slot):
    // velocities before each pressure iteration and after the solve, Jacobi iterates, positions,
    // stiffness and branch codes, collision codes, and the step's neighbour lists, solve
    // coefficients, Jacobi blocks, densities and alphas that the reverse kernels read
    float4 *t_udf = nullptr, *t_ucd = nullptr, *t_q = nullptr, *t_x = nullptr;
    float *t_kdf = nullptr, *t_kcd = nullptr;
    unsigned char *t_cdf = nullptr, *t_ccd = nullptr, *t_adv = nullptr;
    unsigned *t_nbrf = nullptr, *t_nbrb = nullptr, *t_cnt = nullptr, *t_ids = nullptr;
    float2 *t_coef = nullptr, *t_aux = nullptr;
    float4 *t_jd = nullptr, *t_jd2 = nullptr;
    float *t_rho = nullptr, *t_alpha = nullptr;
    int capb = 0;
    // cotangents
    float4 *gx = nullptr, *gv = nullptr, *gx_id = nullptr, *gv_id = nullptr;
    float4 *qbar0 = nullptr, *qbar1 = nullptr, *bbar = nullptr, *gg = nullptr;
    float4 *Dbar = nullptr, *Dbar2 = nullptr;   // symmetric 3x3 cotangent of the Jacobi block: (xx, yy, zz, xy), (xz, yz)
    float4 *y0 = nullptr, *y1 = nullptr;        // D^-1 qbar of a reverse sweep's input / output
    float *grho = nullptr, *galpha = nullptr, *gsf = nullptr;
    double *gsig = nullptr, *gmu = nullptr;   // per-slot parameter cotangents (FP64)
    float4* pa = nullptr;            // per slot (dt gv where the mass is positive, kappa): pass A's neighbour data
    float4* pb = nullptr;            // per slot (u, delta cotangent): pass B's neighbour data
    float2* pc = nullptr;            // per pair (cbar, cvbar), interleaved like nbr_f
    float4* px = nullptr;            // per pair explicit x_ij cotangent
    unsigned char* rev = nullptr;    // per pair: position of i in the neighbour's list
    double* gparam = nullptr;        // 2 per scene
    int* flag = nullptr;             // bit0: asymmetric neighbour lists
    StepCounters* ctr_save = nullptr;

    void free_all() {
        void* ptrs[] = {cp_pos, cp_vel, cp_ids, fin_pos, fin_vel, fin_ids, t_udf, t_ucd, t_q, t_x, t_kdf, t_kcd,
                        t_cdf, t_ccd, t_adv, t_nbrf, t_nbrb, t_cnt, t_ids, t_coef, t_aux, t_jd, t_jd2, t_rho,
                        t_alpha, gx, gv, gx_id, gv_id, qbar0, qbar1, bbar,
                        Dbar, Dbar2, y0, y1, gg, grho, galpha, gsf, gsig, gmu, pa, pb, pc, px, rev, gparam, flag,
                        ctr_save};
        for (void* q : ptrs)
            if (q) cudaFree(q);
        *this = AdjointStore{};
    }
};

namespace {

constexpr int kAB = 128;   // threads per block of the adjoint kernels (divides the slot padding)

__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3& operator+=(float3& a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
__device__ __forceinline__ float3& operator-=(float3& a, float3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// symmetric 3x3 stored as (xx, yy, zz, xy) + (xz, yz)
__device__ __forceinline__ float3 sym_mul(float4 m, float4 m2, float3 v) {
    return make_float3(m.x * v.x + m.w * v.y + m2.x * v.z, m.w * v.x + m.y * v.y + m2.y * v.z,
                       m2.x * v.x + m2.y * v.y + m.z * v.z);
}

// Kernel values and radial derivatives at distance r: W, dW/dr, G (grad W = G x), dG/dr.
// Same piecewise forms as kW / kG (MPSSPHKernel.cuh:28-65), differentiated per piece.
struct KD {
    float W, dW, G, dG;
};
__device__ __forceinline__ KD kern_d(float r, float invh, int cubic) {
    KD k{0.0f, 0.0f, 0.0f, 0.0f};
    const float q = r * invh;
    if (q >= 1.0f) return k;
    const float ih2 = invh * invh, ih4 = ih2 * ih2;
    if (cubic) {
        if (q > 0.5f) {
            const float t = 1.0f - q;
            const float ir = 1.0f / r;
            k.W = 2.0f * KC::cw * t * t * t * ih2 * invh;
            k.dW = -6.0f * KC::cw * t * t * ih4;
            k.G = -KC::cg * t * t * ih4 * ir;
            k.dG = KC::cg * ih4 * t * ir * (2.0f * invh + t * ir);
        } else {
            k.W = KC::cw * ih2 * invh * ((6.0f * q - 6.0f) * q * q + 1.0f);
            k.dW = KC::cw * ih4 * (18.0f * q * q - 12.0f * q);
            k.G = (q < 1.0e-20f) ? 0.0f : KC::cg * ih4 * invh * (3.0f * q - 2.0f);
            k.dG = (q < 1.0e-20f) ? 0.0f : 3.0f * KC::cg * ih4 * ih2;
        }
        return k;
    }
    const float s = 1.0f - q * q;
    k.W = KC::w * s * s * s * ih2 * invh;
    k.dW = -6.0f * KC::w * q * s * s * ih4;
    if (q >= 1.0e-20f) {
        const float t = 1.0f - q;
        const float ir = 1.0f / r;
        k.G = -KC::g * t * t * ih4 * ir;
        k.dG = KC::g * ih4 * t * ir * (2.0f * invh + t * ir);
    }
    return k;
}
// Surface-tension kernels (MPSSPHKernel.cuh:67-84): STW, dSTW/dr, STG, dSTG/dr.
__device__ __forceinline__ KD kern_st(float r, float invh) {
    KD k{0.0f, 0.0f, 0.0f, 0.0f};
    const float q = r * invh;
    if (q >= 1.0f) return k;
    const float ih2 = invh * invh, ih4 = ih2 * ih2;
    const float qq = fmaxf(q, 0.5f);
    const float tt = 1.0f - qq;
    k.W = KC::stw * tt * tt * tt * ih2 * invh;
    if (q > 0.5f) {
        const float t = 1.0f - q;
        const float ir = 1.0f / r;
        k.dW = -3.0f * KC::stw * t * t * ih4;
        k.G = -KC::stg * t * t * ih4 * ir;
        k.dG = KC::stg * ih4 * t * ir * (2.0f * invh + t * ir);
    }
    return k;
}

// Like visit_batched, with the streamed value also passed to the gather (the reverse index of a
// pair selects where the neighbour's coefficient is read).
template <int B, class S, class T, class Stream, class Gather, class Use>
__device__ __forceinline__ void visit2(const unsigned* __restrict__ list, size_t stride, int i, int n, Stream stream,
                                       Gather gather, Use use) {
    int k = 0;
    for (; k + B <= n; k += B) {
        unsigned jj[B];
        S ss[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            jj[u] = list[size_t(k + u) * stride + size_t(i)];
            ss[u] = stream(k + u);
        }
        T v[B];
#pragma unroll
        for (int u = 0; u < B; ++u) v[u] = gather(jj[u], ss[u], k + u);
#pragma unroll
        for (int u = 0; u < B; ++u) use(v[u], ss[u], k + u);
    }
    for (; k < n; ++k) {
        const S sk = stream(k);
        use(gather(list[size_t(k) * stride + size_t(i)], sk, k), sk, k);
    }
}
constexpr int kAdjBatch = 2;
struct AG { float4 x, a; };                      // pass A: position, (dt gv masked by the mass, stiffness)
struct BG { float4 x, u; };                      // pass B: position, velocity (w: delta cotangent)
struct JS { float2 c; unsigned rv; };            // Jacobi reverse, streamed: own coefficient, reverse index
struct JG { float4 x, y, q; float2 cji; };

__device__ __forceinline__ bool slot_live(const Dev& d, int i, int& s) {
    s = d.chunk_scene[i / kChunk];
    const Scene& sc = d.scenes[s];
    return i < sc.slot_begin + sc.n;
}

// ------------------------------------------------------------------ bookkeeping kernels
__global__ void k_adj_rev(Dev d, Params p, unsigned char* rev, int* flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    if (!slot_live(d, i, s)) return;
    const size_t S = size_t(p.slots);
    const int nf = int(d.cnt[i] & 0xffffu);
    for (int k = 0; k < nf; ++k) {
        const unsigned j = d.nbr_f[size_t(k) * S + size_t(i)];
        const int nj = int(d.cnt[j] & 0xffffu);
        int r = 255;
        for (int t = 0; t < nj; ++t)
            if (d.nbr_f[size_t(t) * S + j] == unsigned(i)) { r = t; break; }
        if (r == 255) atomicOr(flag, 1);
        rev[size_t(k) * S + size_t(i)] = (unsigned char)r;
    }
}

// ID order -> slot order of the current layout, and per-step accumulators reset.
__global__ void k_adj_gather(Dev d, Params p, const float4* gx_id, const float4* gv_id, float4* gx, float4* gv,
                             float* grho, float* galpha) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    grho[i] = 0.0f;
    galpha[i] = 0.0f;
    if (!slot_live(d, i, s)) {
        gx[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        gv[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const unsigned id = d.ids[i];
    gx[i] = gx_id[id];
    gv[i] = gv_id[id];
}

__global__ void k_adj_scatter(Dev d, Params p, const float4* gx, const float4* gv, float4* gx_id, float4* gv_id) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    if (!slot_live(d, i, s)) return;
    const unsigned id = d.ids[i];
    float4 a = gx[i], b = gv[i];
    a.w = 0.0f;
    b.w = 0.0f;
    gx_id[id] = a;
    gv_id[id] = b;
}

// ------------------------------------------------------------------ collision + position
// x' = x + dt v_c, v_c = s v per axis (s = 1, -0.4 or 0 by the recorded branch).
__global__ void k_adj_advect(Dev d, Params p, const unsigned char* code, float4* gx, float4* gv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    if (!slot_live(d, i, s)) return;
    const float4 X = gx[i];
    float4 V = gv[i];
    const unsigned c = code[i];
    auto sc = [](unsigned b) { return b == 0u ? 1.0f : (b == 1u ? -0.4f : 0.0f); };
    V.x = sc(c & 3u) * (V.x + p.dt * X.x);
    V.y = sc((c >> 2) & 3u) * (V.y + p.dt * X.y);
    V.z = sc((c >> 4) & 3u) * (V.z + p.dt * X.z);
    gv[i] = V;
}

// ------------------------------------------------------------------ pressure iteration
// First half of one DF/CD iteration's reverse: abar = dt ubar' (massive particles), the
// stiffness cotangent kbar_i, its chain through the clamp / min branch into delta, rho, alpha,
// and the x cotangent of the pressure-force terms.
// What the reverse of pass A gathers from each neighbour, in one 16-byte record: dt gv (zero for a
// particle without mass, which pass B leaves unchanged) and the iteration's stiffness.
__global__ void __launch_bounds__(kAB) k_adj_pack_a(Dev d, Params p, const float4* gv, const float* kap, float4* pa) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    if (!slot_live(d, i, s)) return;
    const float4 g = gv[i];
    const bool m = d.vel[i].w > 1.0e-10f;
    pa[i] = make_float4(m ? p.dt * g.x : 0.0f, m ? p.dt * g.y : 0.0f, m ? p.dt * g.z : 0.0f, kap[i]);
}

__global__ void __launch_bounds__(kAB) k_adj_pA(Dev d, Params p, const float4* X, const float* kap,
                                                 const unsigned char* code, const float4* gv, const float4* pa,
                                                 const float4* U, float4* pb, float* grho, float* galpha, float4* gx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    if (!slot_live(d, i, s)) return;
    const size_t S = size_t(p.slots);
    const float4 xi = X[i];
    const float invhi = 1.0f / xi.w;
    const float ki = kap[i];
    const float4 gvi = gv[i];
    const float4 vi = d.vel[i];   // mass in w (unchanged through the step)
    const float3 ai = vi.w > 1.0e-10f ? p.dt * f3(gvi) : make_float3(0.f, 0.f, 0.f);
    const unsigned c = d.cnt[i];
    const int nf = int(c & 0xffffu), nb = int(c >> 16);
    float kbar = 0.0f;
    float3 xa = make_float3(0.f, 0.f, 0.f);
    visit2<kAdjBatch, NoStream, AG>(d.nbr_f, S, i, nf, [&](int) { return NoStream{}; },
                                    [&](unsigned j, NoStream, int) { return AG{X[j], pa[j]}; },
                                    [&](const AG& t, NoStream, int) {
        const float4 xj = t.x;
        const float kj = t.a.w;
        const float3 aj = f3(t.a);
        const float3 e = make_float3(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        const float r = sqrtf(dot3(e, e));
        const KD Ki = kern_d(r, invhi, p.cubic);
        const KD Kj = xj.w == xi.w ? Ki : kern_d(r, 1.0f / xj.w, p.cubic);
        const float aie = dot3(ai, e), aje = dot3(aj, e);
        kbar += -0.5f * p.V * (Ki.G * aie - Kj.G * aje);
        const float ir = r > 0.0f ? 1.0f / r : 0.0f;
        const float3 ti = Ki.G * ai + (Ki.dG * ir * aie) * e;
        const float3 tj = Kj.G * aj + (Kj.dG * ir * aje) * e;
        xa += (-0.5f * p.V * (ki + kj)) * (ti - tj);
    });
    for (int k = 0; k < nb; ++k) {
        const unsigned b = d.nbr_b[size_t(k) * S + size_t(i)];
        const float4 xb = d.bpos[b];
        const float vb = d.bvol[b];
        const float3 e = make_float3(xi.x - xb.x, xi.y - xb.y, xi.z - xb.z);
        const float r = sqrtf(dot3(e, e));
        const KD K = kern_d(r, invhi, p.cubic);
        const float aie = dot3(ai, e);
        kbar += -0.5f * vb * K.G * aie;
        const float ir = r > 0.0f ? 1.0f / r : 0.0f;
        xa += (-0.5f * ki * vb) * (K.G * ai + (K.dG * ir * aie) * e);
    }
    float4 g = gx[i];
    g.x += xa.x; g.y += xa.y; g.z += xa.z;
    gx[i] = g;
    const unsigned char cd = code[i];
    float gd = 0.0f;
    if (cd != 0) {
        const float al = d.alpha[i];
        const float kb = kbar * al * (p.inv_dt * p.inv_dt);
        if (al > 0.0f) galpha[i] += kbar * ki / al;
        gd = kb * p.dt;
        if (cd == 2) grho[i] += kb * p.inv_rho0;
    }
    const float4 u = U[i];
    pb[i] = make_float4(u.x, u.y, u.z, gd);   // pass B's reverse gathers velocity and delta cotangent together
}

// Second half: the delta terms' cotangents into u^k and x.
__global__ void __launch_bounds__(kAB) k_adj_pB(Dev d, Params p, const float4* X, const float4* pb, float4* gv,
                                                 float4* gx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    if (!slot_live(d, i, s)) return;
    const size_t S = size_t(p.slots);
    const float4 xi = X[i];
    const float invhi = 1.0f / xi.w;
    const float4 ub = pb[i];
    const float3 ui = f3(ub);
    const float di = ub.w;
    const unsigned c = d.cnt[i];
    const int nf = int(c & 0xffffu), nb = int(c >> 16);
    float3 au = make_float3(0.f, 0.f, 0.f), xa = make_float3(0.f, 0.f, 0.f);
    visit2<kAdjBatch, NoStream, BG>(d.nbr_f, S, i, nf, [&](int) { return NoStream{}; },
                                    [&](unsigned j, NoStream, int) { return BG{X[j], pb[j]}; },
                                    [&](const BG& t, NoStream, int) {
        const float4 xj = t.x;
        const float dj = t.u.w;
        const float3 uij = ui - f3(t.u);
        const float3 e = make_float3(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        const float r = sqrtf(dot3(e, e));
        const KD Ki = kern_d(r, invhi, p.cubic);
        const KD Kj = xj.w == xi.w ? Ki : kern_d(r, 1.0f / xj.w, p.cubic);
        au += (p.V * (di * Ki.G + dj * Kj.G)) * e;
        const float ir = r > 0.0f ? 1.0f / r : 0.0f;
        const float eu = dot3(e, uij);
        xa += (p.V * di) * (Ki.G * uij + (Ki.dG * ir * eu) * e);
        xa += (p.V * dj) * (Kj.G * uij + (Kj.dG * ir * eu) * e);
    });
    for (int k = 0; k < nb; ++k) {
        const unsigned b = d.nbr_b[size_t(k) * S + size_t(i)];
        const float4 xb = d.bpos[b];
        const float vb = d.bvol[b];
        const float3 e = make_float3(xi.x - xb.x, xi.y - xb.y, xi.z - xb.z);
        const float r = sqrtf(dot3(e, e));
        const KD K = kern_d(r, invhi, p.cubic);
        au += (di * vb * K.G) * e;
        const float ir = r > 0.0f ? 1.0f / r : 0.0f;
        xa += (di * vb) * (K.G * ui + (K.dG * ir * dot3(e, ui)) * e);
    }
    float4 v = gv[i];
    v.x += au.x; v.y += au.y; v.z += au.z;
    gv[i] = v;
    float4 g = gx[i];
    g.x += xa.x; g.y += xa.y; g.z += xa.z;
    gx[i] = g;
}

// ------------------------------------------------------------------ Jacobi solve reverse
// One transposed sweep: y = qbar / D, qbar' = qbar - (A_0 + f I)^T y, plus the sweep's share of
// the cotangents of b, D and of each pair's coefficients (c, cv) and explicit x_ij.
// y = D^-1 qbar for every live slot: the first reverse sweep's input (later sweeps write the
// next sweep's y themselves, so that a sweep gathers a neighbour's y instead of its qbar and
// 3x3 block).
__global__ void __launch_bounds__(kAB) k_adj_y(Dev d, Params p, const float4* qbar, float4* y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    if (!slot_live(d, i, s)) return;
    const float3 v = sym_mul(d.jac_d[i], d.jac_d2[i], f3(qbar[i]));
    y[i] = make_float4(v.x, v.y, v.z, 0.0f);
}

__global__ void __launch_bounds__(kAB) k_adj_jacobi(Dev d, Params p, const float4* X, const unsigned char* rev,
                                                     const float4* qk, const float4* qk1, const float4* qbar,
                                                     float4* qbar_out, const float4* yin, float4* yout, float4* bbar,
                                                     float4* Dbar, float4* Dbar2, float2* pc, float4* px) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    if (!slot_live(d, i, s)) return;
    const size_t S = size_t(p.slots);
    const float4 xi = X[i];
    const float4 qb = qbar[i];
    const float3 y = f3(yin[i]);   // D_i^-1 qbar_i (yin: every slot's, written by the previous sweep)
    const float3 qi = f3(qk[i]);
    const int nf = int(d.cnt[i] & 0xffffu);
    float3 aty = (1.0f + p.cg_factor) * y;
    visit2<kAdjBatch, JS, JG>(d.nbr_f, S, i, nf,
        [&](int k) { const size_t at = size_t(k) * S + size_t(i); return JS{d.cg_coef[at], unsigned(rev[at])}; },
        [&](unsigned j, const JS& st, int) {
            return JG{X[j], yin[j], qk[j],
                      st.rv != 255u ? d.cg_coef[size_t(st.rv) * S + j] : make_float2(0.f, 0.f)};
        },
        [&](const JG& t, const JS& st, int k) {
        const size_t at = size_t(k) * S + size_t(i);
        const float2 cij = st.c;
        const float4 xj = t.x;
        const float3 e = make_float3(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        const float ye = dot3(y, e);
        aty += p.dt * (cij.x * y - (cij.y * ye) * e);
        if (st.rv != 255u) {
            const float2 cji = t.cji;
            const float3 yj = f3(t.y);
            const float yje = dot3(yj, e);
            aty -= p.dt * (cji.x * yj - (cji.y * yje) * e);
        }
        const float3 pp = qi - f3(t.q);
        const float pe = dot3(pp, e);
        float2 a = pc[at];
        a.x += -p.dt * dot3(y, pp);
        a.y += p.dt * pe * ye;
        pc[at] = a;
        float4 b = px[at];
        const float3 tt = (p.dt * cij.y) * (pe * y + ye * pp);
        b.x += tt.x; b.y += tt.y; b.z += tt.z;
        px[at] = b;
    });
    const float3 qn = make_float3(qb.x - aty.x, qb.y - aty.y, qb.z - aty.z);
    qbar_out[i] = make_float4(qn.x, qn.y, qn.z, 0.0f);
    const float3 yn = sym_mul(d.jac_d[i], d.jac_d2[i], qn);   // the next sweep's y_i
    yout[i] = make_float4(yn.x, yn.y, yn.z, 0.0f);
    float4 bb = bbar[i];
    bb.x += y.x; bb.y += y.y; bb.z += y.z;
    bbar[i] = bb;
    // Dbar -= sym(y dq^T), dq = q^{k+1} - q^k = D^-1 r
    const float3 dq = f3(qk1[i]) - qi;
    float4 db = Dbar[i];
    db.x -= y.x * dq.x; db.y -= y.y * dq.y; db.z -= y.z * dq.z;
    db.w -= 0.5f * (y.x * dq.y + y.y * dq.x);
    Dbar[i] = db;
    float4 db2 = Dbar2[i];
    db2.x -= 0.5f * (y.x * dq.z + y.z * dq.x);
    db2.y -= 0.5f * (y.y * dq.z + y.z * dq.y);
    Dbar2[i] = db2;
}

// Inputs of one pair term of the solve set-up (k_cg_b), owner o, neighbour n.
struct PairIn {
    float3 e;          // x_o - x_n
    float3 vo, vn;     // pre-solve velocities
    float ro, rn;      // densities
    float so, sn;      // surface-tension factors
    float mo, mn;      // masses
    float ho;          // support radius of the owner
};
struct PairBar {
    float C, Cv;       // cotangents of c_on and cv_on
    float3 Bb;         // cotangent of b_o (the pair's share of b is st_scale_o * (-c e))
    float3 X;          // explicit cotangent of x_o - x_n
};
struct PairGrad {
    float3 e, vo, vn;
    float ro, rn, so, sn;
    double sig, mu;    // parameter cotangents: small totals of cancelling terms, kept in FP64
};

// Reverse of the pair term: c = mbar g_on, b share = -st_scale c e,
// c_on = st_scale c + xsph/dt m_n/rho_n W, cv_on = 10 rho0 mu / rho_o mbar / rho_n G / ((d^2 + 0.01 h^2)(d + eps))
// with g_on = (STW + dt (STG e.v_on - (s_o + s_n) invD STW / 2)) invD, invD = 2 / (rho_o + rho_n)
// (MPSSPHNonPressureUtil.cuh:510-515,567-633; the forward is k_cg_b).
__device__ PairGrad pair_reverse(const Params& p, const PairIn& in, const PairBar& bar) {
    PairGrad g{};
    const float r2 = dot3(in.e, in.e);
    const float r = sqrtf(r2);
    const float invh = 1.0f / in.ho;
    const float invD = 2.0f / (in.ro + in.rn);
    const KD st = kern_st(r, invh);
    const KD kd = kern_d(r, invh, p.cubic);
    const float3 vij = in.vo - in.vn;
    const float ev = dot3(in.e, vij);
    const float vdot = st.G * ev;
    const float S = in.so + in.sn;
    const float E = st.W + p.dt * (vdot - S * invD * 0.5f * st.W);
    const float gg = E * invD;
    const float mbar = 0.5f * (in.mo + in.mn);
    const float c = mbar * gg;
    const float st_scale = p.dt * p.sigma / in.mo;
    const float xs = p.xsph * p.inv_dt;
    const float den = r2 + 0.01f * in.ho * in.ho;
    const float rr = r + kFltEps;
    const float vs0 = 10.0f * p.rho0 / in.ro * mbar / in.rn;   // cv / (mu G / (den rr))
    const float cv = p.visc * vs0 * kd.G / (den * rr);

    float rbar = 0.0f;
    float3 ebar = bar.X;
    // cv
    g.mu = double(bar.Cv) * double(vs0) * double(kd.G) / (double(den) * double(rr));
    g.ro = -bar.Cv * cv / in.ro;
    g.rn = -bar.Cv * cv / in.rn;
    rbar += bar.Cv * p.visc * vs0 * (kd.dG / (den * rr) - kd.G * 2.0f * r / (den * den * rr) - kd.G / (den * rr * rr));
    // c_on
    float cbar = bar.C * st_scale;
    const double dtm = double(p.dt) / double(in.mo);
    g.sig = double(bar.C) * dtm * double(c);
    g.rn += -bar.C * xs * in.mn * kd.W / (in.rn * in.rn);
    rbar += bar.C * xs * (in.mn / in.rn) * kd.dW;
    // b share: st_scale * (-c e)
    const float3 Bt = st_scale * bar.Bb;
    cbar += -dot3(Bt, in.e);
    ebar -= c * Bt;
    g.sig -= dtm * double(c) * (double(bar.Bb.x) * in.e.x + double(bar.Bb.y) * in.e.y + double(bar.Bb.z) * in.e.z);
    // c = mbar g; g = E invD
    const float gbar = cbar * mbar;
    const float Ebar = gbar * invD;
    float invDbar = gbar * E;
    const float stwbar = Ebar * (1.0f - 0.5f * p.dt * S * invD);
    const float vdotbar = Ebar * p.dt;
    const float Sbar = -Ebar * 0.5f * p.dt * invD * st.W;
    invDbar += -Ebar * 0.5f * p.dt * S * st.W;
    g.so = Sbar;
    g.sn = Sbar;
    const float rhob = -invDbar * invD * invD * 0.5f;
    g.ro += rhob;
    g.rn += rhob;
    const float stgbar = vdotbar * ev;
    const float evbar = vdotbar * st.G;
    ebar += evbar * vij;
    g.vo = evbar * in.e;
    g.vn = (-evbar) * in.e;
    rbar += stwbar * st.dW + stgbar * st.dG;
    if (r > 0.0f) ebar += (rbar / r) * in.e;
    g.e = ebar;
    return g;
}

// The solve set-up's reverse: every pair term's cotangents (from the sweeps, the diagonal D and b)
// into x, the pre-solve velocity, rho, the ST factor and the per-particle sigma / mu shares.
__global__ void __launch_bounds__(kAB) k_adj_visc_coef(Dev d, Params p, const float4* X, const float4* V0,
                                                        const unsigned char* rev, const float4* qbar0,
                                                        const float4* bbar, const float4* Dbar, const float4* Dbar2,
                                                        const float2* pc, const float4* px, float4* gv, float4* gx,
                                                        float* grho, float* gsf, double* gsig, double* gmu) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    if (!slot_live(d, i, s)) return;
    const size_t S = size_t(p.slots);
    const float4 xi = X[i];
    const float4 vi4 = V0[i];
    const float2 ai = d.aux[i];
    const float4 bbi = bbar[i];
    const bool keep_i = d.jac_d2[i].z == 0.0f;   // a replaced block does not depend on the coefficients
    const float4 Dbi = keep_i ? Dbar[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 Dbi2 = keep_i ? Dbar2[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int nf = int(d.cnt[i] & 0xffffu);
    float3 gvi = f3(qbar0[i]) + (1.0f + p.cg_factor) * f3(bbi);
    float3 gxi = make_float3(0.f, 0.f, 0.f);
    float grhoi = 0.0f, gsfi = 0.0f;
    double sig = 0.0, mu = 0.0;
    const float tri = Dbi.x + Dbi.y + Dbi.z;
    for (int k = 0; k < nf; ++k) {
        const size_t at = size_t(k) * S + size_t(i);
        const unsigned j = d.nbr_f[at];
        const float4 xj = X[j];
        const float4 vj4 = V0[j];
        const float2 aj = d.aux[j];
        const float3 e = make_float3(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        // D = (1 + f + dt sum c) I - dt sum cv x x^T: c gets dt tr(Dbar), cv gets -dt x^T Dbar x, x gets
        // -2 dt cv Dbar x
        const float3 Dbe = sym_mul(Dbi, Dbi2, e);
        // term owned by i
        {
            const float2 cf = d.cg_coef[at];
            const float2 a = pc[at];
            const float4 xb = px[at];
            PairIn in{e, f3(vi4), f3(vj4), ai.x, aj.x, ai.y, aj.y, vi4.w, vj4.w, xi.w};
            PairBar bar;
            bar.C = a.x + p.dt * tri;
            bar.Cv = a.y - p.dt * dot3(e, Dbe);
            bar.Bb = f3(bbi);
            bar.X = f3(xb) + (-2.0f * p.dt * cf.y) * Dbe;
            const PairGrad g = pair_reverse(p, in, bar);
            gxi += g.e;
            gvi += g.vo;
            grhoi += g.ro;
            gsfi += g.so;
            sig += g.sig;
            mu += g.mu;
        }
        // term owned by j (i is its neighbour)
        const unsigned rv = rev[at];
        if (rv != 255u) {
            const size_t bt = size_t(rv) * S + j;
            const float2 cf = d.cg_coef[bt];
            const float2 a = pc[bt];
            const float4 xb = px[bt];
            const bool keep_j = d.jac_d2[j].z == 0.0f;
            const float4 Dbj = keep_j ? Dbar[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 Dbj2 = keep_j ? Dbar2[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float3 ej = (-1.0f) * e;
            const float3 Dbje = sym_mul(Dbj, Dbj2, ej);
            PairIn in{ej, f3(vj4), f3(vi4), aj.x, ai.x, aj.y, ai.y, vj4.w, vi4.w, xj.w};
            PairBar bar;
            bar.C = a.x + p.dt * (Dbj.x + Dbj.y + Dbj.z);
            bar.Cv = a.y - p.dt * dot3(ej, Dbje);
            bar.Bb = f3(bbar[j]);
            bar.X = f3(xb) + (-2.0f * p.dt * cf.y) * Dbje;
            const PairGrad g = pair_reverse(p, in, bar);
            gxi -= g.e;
            gvi += g.vn;
            grhoi += g.rn;
            gsfi += g.sn;
        }
    }
    float4 v = gv[i];
    v.x = gvi.x; v.y = gvi.y; v.z = gvi.z;
    gv[i] = v;
    float4 gg = gx[i];
    gg.x += gxi.x; gg.y += gxi.y; gg.z += gxi.z;
    gx[i] = gg;
    grho[i] += grhoi;
    gsf[i] = gsfi;
    gsig[i] += sig;
    gmu[i] += mu;
}

// Surface-tension factor reverse: s_i = sum_j m_j G_ij x_ij.(v_i - v_j) (k_st_factor).
__global__ void __launch_bounds__(kAB) k_adj_stfac(Dev d, Params p, const float4* X, const float4* V0,
                                                    const float* gsf, float4* gv, float4* gx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    if (!slot_live(d, i, s)) return;
    const size_t S = size_t(p.slots);
    const float4 xi = X[i];
    const float invhi = 1.0f / xi.w;
    const float4 vi = V0[i];
    const float si = gsf[i];
    const int nf = int(d.cnt[i] & 0xffffu);
    float3 av = make_float3(0.f, 0.f, 0.f), xa = make_float3(0.f, 0.f, 0.f);
    for (int k = 0; k < nf; ++k) {
        const unsigned j = d.nbr_f[size_t(k) * S + size_t(i)];
        const float4 xj = X[j];
        const float4 vj = V0[j];
        const float sj = gsf[j];
        const float3 e = make_float3(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        const float r = sqrtf(dot3(e, e));
        const KD Ki = kern_d(r, invhi, p.cubic);
        const KD Kj = xj.w == xi.w ? Ki : kern_d(r, 1.0f / xj.w, p.cubic);
        const float3 vij = f3(vi) - f3(vj);
        const float wi = si * vj.w, wj = sj * vi.w;
        av += (wi * Ki.G + wj * Kj.G) * e;
        const float ir = r > 0.0f ? 1.0f / r : 0.0f;
        const float ev = dot3(e, vij);
        xa += wi * (Ki.G * vij + (Ki.dG * ir * ev) * e);
        xa += wj * (Kj.G * vij + (Kj.dG * ir * ev) * e);
    }
    float4 v = gv[i];
    v.x += av.x; v.y += av.y; v.z += av.z;
    gv[i] = v;
    float4 g = gx[i];
    g.x += xa.x; g.y += xa.y; g.z += xa.z;
    gx[i] = g;
}

// ------------------------------------------------------------------ density + alpha reverse
// gg_i = (gbar_i, sbar_i) from alphabar: alpha = 1 / f, f = s + |g|^2.
__global__ void __launch_bounds__(kAB) k_adj_dens_a(Dev d, Params p, const float4* X, const float* galpha,
                                                     float4* gg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    if (!slot_live(d, i, s)) return;
    const size_t S = size_t(p.slots);
    const float4 xi = X[i];
    const float invhi = 1.0f / xi.w;
    const unsigned c = d.cnt[i];
    const int nf = int(c & 0xffffu), nb = int(c >> 16);
    float3 gs = make_float3(0.f, 0.f, 0.f);
    for (int k = 0; k < nf; ++k) {
        const float4 xj = X[d.nbr_f[size_t(k) * S + size_t(i)]];
        const float3 e = make_float3(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        gs += (p.V * kern_d(sqrtf(dot3(e, e)), invhi, p.cubic).G) * e;
    }
    for (int k = 0; k < nb; ++k) {
        const unsigned b = d.nbr_b[size_t(k) * S + size_t(i)];
        const float4 xb = d.bpos[b];
        const float3 e = make_float3(xi.x - xb.x, xi.y - xb.y, xi.z - xb.z);
        gs += (d.bvol[b] * kern_d(sqrtf(dot3(e, e)), invhi, p.cubic).G) * e;
    }
    const float al = d.alpha[i];
    const float fbar = al > 0.0f ? -al * al * galpha[i] : 0.0f;
    gg[i] = make_float4(2.0f * fbar * gs.x, 2.0f * fbar * gs.y, 2.0f * fbar * gs.z, fbar);
}

__global__ void __launch_bounds__(kAB) k_adj_dens_b(Dev d, Params p, const float4* X, const float* grho,
                                                     const float4* gg, float4* gx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    int s;
    if (!slot_live(d, i, s)) return;
    const size_t S = size_t(p.slots);
    const float4 xi = X[i];
    const float invhi = 1.0f / xi.w;
    const float rbi = grho[i] * p.rho0;
    const float4 ggi = gg[i];
    const float3 gbi = f3(ggi);
    const unsigned c = d.cnt[i];
    const int nf = int(c & 0xffffu), nb = int(c >> 16);
    float3 xa = make_float3(0.f, 0.f, 0.f);
    for (int k = 0; k < nf; ++k) {
        const unsigned j = d.nbr_f[size_t(k) * S + size_t(i)];
        const float4 xj = X[j];
        const float rbj = grho[j] * p.rho0;
        const float4 ggj = gg[j];
        const float3 gbj = f3(ggj);
        const float3 e = make_float3(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        const float r = sqrtf(dot3(e, e));
        const KD Ki = kern_d(r, invhi, p.cubic);
        const KD Kj = xj.w == xi.w ? Ki : kern_d(r, 1.0f / xj.w, p.cubic);
        const float ir = r > 0.0f ? 1.0f / r : 0.0f;
        // rho terms (radial), the s terms (|V G x|^2 = V^2 G^2 r^2, radial)
        float rad = p.V * (rbi * Ki.dW + rbj * Kj.dW) * ir;
        rad += p.V * p.V * 2.0f * (ggi.w * Ki.G * (r * Ki.dG + Ki.G) + ggj.w * Kj.G * (r * Kj.dG + Kj.G));
        xa += rad * e;
        // gradient-sum terms (vector)
        xa += p.V * (Ki.G * gbi + (Ki.dG * ir * dot3(gbi, e)) * e);
        xa -= p.V * (Kj.G * gbj + (Kj.dG * ir * dot3(gbj, e)) * e);
    }
    for (int k = 0; k < nb; ++k) {
        const unsigned b = d.nbr_b[size_t(k) * S + size_t(i)];
        const float4 xb = d.bpos[b];
        const float vb = d.bvol[b];
        const float3 e = make_float3(xi.x - xb.x, xi.y - xb.y, xi.z - xb.z);
        const float r = sqrtf(dot3(e, e));
        const KD K = kern_d(r, invhi, p.cubic);
        const float ir = r > 0.0f ? 1.0f / r : 0.0f;
        xa += (vb * rbi * K.dW * ir) * e;
        xa += vb * (K.G * gbi + (K.dG * ir * dot3(gbi, e)) * e);
    }
    float4 g = gx[i];
    g.x += xa.x; g.y += xa.y; g.z += xa.z;
    gx[i] = g;
}

// Per-scene sums of the sigma / mu shares (one block per scene, fixed order: deterministic).
__global__ void k_adj_param_reduce(Dev d, Params p, const double* gsig, const double* gmu, double* gparam) {
    __shared__ double sa[256], sb[256];
    const int s = blockIdx.x;
    const Scene& sc = d.scenes[s];
    double a = 0.0, b = 0.0;
    for (int i = sc.slot_begin + threadIdx.x; i < sc.slot_begin + sc.n; i += blockDim.x) {
        a += gsig[i];
        b += gmu[i];
    }
    sa[threadIdx.x] = a;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (int(threadIdx.x) < w) {
            sa[threadIdx.x] += sa[threadIdx.x + w];
            sb[threadIdx.x] += sb[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        gparam[2 * s] += sb[0];       // d/d viscosity
        gparam[2 * s + 1] += sa[0];   // d/d surface tension
    }
}

// ------------------------------------------------------------------ host side
using host::fail;

#define ADJ_TRY(expr)                                                                           \
    do {                                                                                        \
        cudaError_t e_ = (expr);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return fail(e_ == cudaErrorMemoryAllocation ? MPS_E_NOMEM : MPS_E_CUDA,             \
                        std::string(#expr) + ": " + cudaGetErrorString(e_));                    \
    } while (0)

struct Guard {
    int prev = 0;
    explicit Guard(int dev) { cudaGetDevice(&prev); cudaSetDevice(dev); }
    ~Guard() { cudaSetDevice(prev); }
};

int nb_of(int n) { return (n + kAB - 1) / kAB; }

size_t store_bytes(const mps_handle* h, int nsteps, int every) {
    const size_t S = size_t(h->slots), cap = size_t(h->cfg.max_fluid_neighbors), K = size_t(h->cfg.fixed_iters);
    const size_t capb = size_t(h->cfg.max_boundary_neighbors), E = size_t(every);
    const size_t ncp = size_t((nsteps + every - 1) / every);
    const size_t state = S * (2 * sizeof(float4) + sizeof(unsigned));
    size_t b = (ncp + 1) * state;
    size_t step = (3 * (K + 1) + 1) * S * sizeof(float4);               // tapes u (DF, CD), q, x
    step += 2 * K * S * (sizeof(float) + 1) + S;                         // stiffness, codes, collision codes
    step += (cap + capb + 2) * S * sizeof(unsigned) + cap * S * sizeof(float2);   // lists, counts, ids, coefficients
    step += S * (sizeof(float2) + 2 * sizeof(float4) + 2 * sizeof(float));      // aux, Jacobi blocks, rho, alpha
    b += E * step;
    b += 14 * S * sizeof(float4) + 3 * S * sizeof(float) + 2 * S * sizeof(double);   // cotangents
    b += cap * S * (sizeof(float2) + sizeof(float4) + 1);   // per-pair cotangents + reverse index
    b += size_t(h->nscenes) * 2 * sizeof(double) + 64;
    return b;
}

template <class T>
cudaError_t alloc(T** p, size_t count, size_t& total) {
    total += count * sizeof(T);
    return cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T));
}

int ensure_store(mps_handle* h, int nsteps, int every) {
    if (!h->adj) h->adj = new AdjointStore();
    AdjointStore& A = *h->adj;
    const int K = h->cfg.fixed_iters;
    const int ncp = (nsteps + every - 1) / every;
    if (A.slots == h->slots && A.K == K && A.ncp_cap >= ncp && A.every_cap >= every &&
        A.cap == h->cfg.max_fluid_neighbors && A.nscenes == h->nscenes && A.cp_pos)
        return MPS_OK;
    A.free_all();
    A.slots = h->slots;
    A.K = K;
    A.ncp_cap = ncp;
    A.every_cap = every;
    A.cap = h->cfg.max_fluid_neighbors;
    A.capb = h->cfg.max_boundary_neighbors;
    A.nscenes = h->nscenes;
    A.n = h->n;
    const size_t S = size_t(h->slots), cap = size_t(A.cap), capb = size_t(A.capb), E = size_t(every);
    size_t& t = A.bytes;
    ADJ_TRY(alloc(&A.cp_pos, S * ncp, t));
    ADJ_TRY(alloc(&A.cp_vel, S * ncp, t));
    ADJ_TRY(alloc(&A.cp_ids, S * ncp, t));
    ADJ_TRY(alloc(&A.fin_pos, S, t));
    ADJ_TRY(alloc(&A.fin_vel, S, t));
    ADJ_TRY(alloc(&A.fin_ids, S, t));
    ADJ_TRY(alloc(&A.t_udf, E * S * (K + 1), t));
    ADJ_TRY(alloc(&A.t_ucd, E * S * (K + 1), t));
    ADJ_TRY(alloc(&A.t_q, E * S * (K + 1), t));
    ADJ_TRY(alloc(&A.t_x, E * S, t));
    ADJ_TRY(alloc(&A.t_kdf, E * S * K, t));
    ADJ_TRY(alloc(&A.t_kcd, E * S * K, t));
    ADJ_TRY(alloc(&A.t_cdf, E * S * K, t));
    ADJ_TRY(alloc(&A.t_ccd, E * S * K, t));
    ADJ_TRY(alloc(&A.t_adv, E * S, t));
    ADJ_TRY(alloc(&A.t_nbrf, E * S * cap, t));
    ADJ_TRY(alloc(&A.t_nbrb, E * S * capb, t));
    ADJ_TRY(alloc(&A.t_cnt, E * S, t));
    ADJ_TRY(alloc(&A.t_ids, E * S, t));
    ADJ_TRY(alloc(&A.t_coef, E * S * cap, t));
    ADJ_TRY(alloc(&A.t_aux, E * S, t));
    ADJ_TRY(alloc(&A.t_jd, E * S, t));
    ADJ_TRY(alloc(&A.t_jd2, E * S, t));
    ADJ_TRY(alloc(&A.t_rho, E * S, t));
    ADJ_TRY(alloc(&A.t_alpha, E * S, t));
    float4** f4[] = {&A.gx, &A.gv, &A.qbar0, &A.qbar1, &A.bbar, &A.Dbar, &A.Dbar2, &A.gg, &A.y0, &A.y1, &A.pa, &A.pb};
    for (float4** q : f4) ADJ_TRY(alloc(q, S, t));
    ADJ_TRY(alloc(&A.gx_id, size_t(std::max<int64_t>(h->n, 1)), t));
    ADJ_TRY(alloc(&A.gv_id, size_t(std::max<int64_t>(h->n, 1)), t));
    float** f1[] = {&A.grho, &A.galpha, &A.gsf};
    for (float** q : f1) ADJ_TRY(alloc(q, S, t));
    ADJ_TRY(alloc(&A.gsig, S, t));
    ADJ_TRY(alloc(&A.gmu, S, t));
    ADJ_TRY(alloc(&A.pc, S * cap, t));
    ADJ_TRY(alloc(&A.px, S * cap, t));
    ADJ_TRY(alloc(&A.rev, S * cap, t));
    ADJ_TRY(alloc(&A.gparam, 2 * size_t(h->nscenes), t));
    ADJ_TRY(alloc(&A.flag, 1, t));
    ADJ_TRY(alloc(&A.ctr_save, 1, t));
    A.cp_cur.assign(size_t(ncp), 0);
    // zero what the kernels read before writing (padding slots of the cotangents)
    for (float4** q : f4) ADJ_TRY(cudaMemset(*q, 0, S * sizeof(float4)));
    for (float** q : f1) ADJ_TRY(cudaMemset(*q, 0, S * sizeof(float)));
    ADJ_TRY(cudaMemset(A.gsig, 0, S * sizeof(double)));
    ADJ_TRY(cudaMemset(A.gmu, 0, S * sizeof(double)));
    return MPS_OK;
}

cudaError_t copy_state(mps_handle* h, int buf, float4* pos, float4* vel, unsigned* ids, bool save, cudaStream_t s) {
    const size_t S = size_t(h->slots);
    const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
    cudaError_t e;
    if (save) {
        if ((e = cudaMemcpyAsync(pos, h->pos[buf], S * sizeof(float4), k, s))) return e;
        if ((e = cudaMemcpyAsync(vel, h->vel[buf], S * sizeof(float4), k, s))) return e;
        return cudaMemcpyAsync(ids, h->ids[buf], S * sizeof(unsigned), k, s);
    }
    if ((e = cudaMemcpyAsync(h->pos[buf], pos, S * sizeof(float4), k, s))) return e;
    if ((e = cudaMemcpyAsync(h->vel[buf], vel, S * sizeof(float4), k, s))) return e;
    return cudaMemcpyAsync(h->ids[buf], ids, S * sizeof(unsigned), k, s);
}

// The tape of step k of the current segment.
struct Slot {
    float4 *udf, *ucd, *q, *x;
    float *kdf, *kcd;
    unsigned char *cdf, *ccd, *adv;
    unsigned *nbrf, *nbrb, *cnt, *ids;
    float2 *coef, *aux;
    float4 *jd, *jd2;
    float *rho, *alpha;
};
Slot slot_of(const AdjointStore& A, int k) {
    const size_t S = size_t(A.slots), K = size_t(A.K), kk = size_t(k);
    Slot t;
    t.udf = A.t_udf + kk * S * (K + 1);
    t.ucd = A.t_ucd + kk * S * (K + 1);
    t.q = A.t_q + kk * S * (K + 1);
    t.x = A.t_x + kk * S;
    t.kdf = A.t_kdf + kk * S * K;
    t.kcd = A.t_kcd + kk * S * K;
    t.cdf = A.t_cdf + kk * S * K;
    t.ccd = A.t_ccd + kk * S * K;
    t.adv = A.t_adv + kk * S;
    t.nbrf = A.t_nbrf + kk * S * size_t(A.cap);
    t.nbrb = A.t_nbrb + kk * S * size_t(A.capb);
    t.cnt = A.t_cnt + kk * S;
    t.ids = A.t_ids + kk * S;
    t.coef = A.t_coef + kk * S * size_t(A.cap);
    t.aux = A.t_aux + kk * S;
    t.jd = A.t_jd + kk * S;
    t.jd2 = A.t_jd2 + kk * S;
    t.rho = A.t_rho + kk * S;
    t.alpha = A.t_alpha + kk * S;
    return t;
}

// One pressure solve recorded: u^k before each iteration, kappa^k and the branch codes.
int taped_pressure(mps_handle* h, int mode, float4* tu, float* tk, unsigned char* tc, cudaStream_t s) {
    const Params p = host::make_params(h);
    Dev d = host::make_dev(h, h->cur);
    const int bs = host::block_size(h);
    const size_t S = size_t(h->slots);
    const int K = h->cfg.fixed_iters;
    launch_solver_init(d, p, s);
    for (int k = 0; k < K; ++k) {
        ADJ_TRY(cudaMemcpyAsync(tu + size_t(k) * S, h->vel[h->cur], S * sizeof(float4), cudaMemcpyDeviceToDevice, s));
        d.tape_code = tc + size_t(k) * S;
        launch_pressure_A(d, p, mode, bs, 0ull, 0, s);
        ADJ_TRY(cudaMemcpyAsync(tk + size_t(k) * S, h->kappa, S * sizeof(float), cudaMemcpyDeviceToDevice, s));
        d.tape_code = nullptr;
        launch_pressure_B(d, p, bs, 0ull, 0, 0, s);
    }
    ADJ_TRY(cudaMemcpyAsync(tu + size_t(K) * S, h->vel[h->cur], S * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    launch_solver_finish(d, p, mode == 0 ? 0 : 2, s);
    ADJ_TRY(cudaGetLastError());
    return MPS_OK;
}

template <class T>
cudaError_t save(T* dst, const T* src, size_t count, cudaStream_t s) {
    return cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDeviceToDevice, s);
}

// The step of mps_step, run phase by phase with recording into slot t (bit-identical to the
// plain step); the handle advances to the step's output.
int taped_step(mps_handle* h, const Slot& t, cudaStream_t s) {
    AdjointStore& A = *h->adj;
    const size_t S = size_t(h->slots);
    int r;
    if ((r = host::run_phase(h, MPS_PHASE_SORT, s))) return r;
    if ((r = host::run_phase(h, MPS_PHASE_NEIGHBORS, s))) return r;
    if ((r = host::run_phase(h, MPS_PHASE_BVOLUME, s))) return r;
    if ((r = host::run_phase(h, MPS_PHASE_DENSITY_ALPHA, s))) return r;
    if ((r = taped_pressure(h, 0, t.udf, t.kdf, t.cdf, s))) return r;
    {
        const Params p = host::make_params(h);
        const Dev d = host::make_dev(h, h->cur);
        const int bs = host::block_size(h);
        launch_st_factor(d, p, bs, s);
        launch_cg_b(d, p, bs, s);
        ADJ_TRY(save(t.q, h->cg_x, S, s));
        launch_solver_init(d, p, s);
        for (int k = 0; k < A.K; ++k)
            launch_jacobi(d, p, bs, 0ull, 0, 0, t.q + size_t(k) * S, t.q + size_t(k + 1) * S, s);
        launch_solver_finish(d, p, 1, s);
        launch_jacobi_finish(d, p, t.q + size_t(A.K) * S, s);
        ADJ_TRY(cudaGetLastError());
    }
    if ((r = taped_pressure(h, 1, t.ucd, t.kcd, t.ccd, s))) return r;
    {
        const Params p = host::make_params(h);
        Dev d = host::make_dev(h, h->cur);
        ADJ_TRY(save(t.x, h->pos[h->cur], S, s));
        d.tape_adv = t.adv;
        launch_advect(d, p, s);
        ADJ_TRY(cudaGetLastError());
    }
    // what the reverse kernels read of this step
    ADJ_TRY(save(t.nbrf, h->nbr_f, S * size_t(A.cap), s));
    ADJ_TRY(save(t.nbrb, h->nbr_b, S * size_t(A.capb), s));
    ADJ_TRY(save(t.cnt, h->cnt, S, s));
    ADJ_TRY(save(t.ids, h->ids[h->cur], S, s));
    ADJ_TRY(save(t.coef, h->cg_coef, S * size_t(A.cap), s));
    ADJ_TRY(save(t.aux, h->aux, S, s));
    ADJ_TRY(save(t.jd, h->cg_ap, S, s));
    ADJ_TRY(save(t.jd2, h->cg_r, S, s));
    ADJ_TRY(save(t.rho, h->rho, S, s));
    ADJ_TRY(save(t.alpha, h->alpha, S, s));
    return MPS_OK;
}

// Reverse of the step recorded in slot t: cotangents of its output (ID order, A.gx_id / A.gv_id)
// are replaced by those of its input.
int adjoint_step(mps_handle* h, const Slot& t, cudaStream_t s) {
    AdjointStore& A = *h->adj;
    const Params p = host::make_params(h);
    Dev d = host::make_dev(h, h->cur);
    d.nbr_f = t.nbrf;
    d.nbr_b = t.nbrb;
    d.cnt = t.cnt;
    d.ids = t.ids;
    d.cg_coef = t.coef;
    d.aux = t.aux;
    d.jac_d = t.jd;
    d.jac_d2 = t.jd2;
    d.rho = t.rho;
    d.alpha = t.alpha;
    d.vel = t.udf;   // masses (w) in slot order of this step
    const size_t S = size_t(h->slots), cap = size_t(A.cap);
    const int K = A.K;
    const int nb = nb_of(h->slots);
    k_adj_gather<<<nb, kAB, 0, s>>>(d, p, A.gx_id, A.gv_id, A.gx, A.gv, A.grho, A.galpha);
    k_adj_rev<<<nb, kAB, 0, s>>>(d, p, A.rev, A.flag);
    k_adj_advect<<<nb, kAB, 0, s>>>(d, p, t.adv, A.gx, A.gv);
    // constant-density solve
    for (int k = K - 1; k >= 0; --k) {
        k_adj_pack_a<<<nb, kAB, 0, s>>>(d, p, A.gv, t.kcd + size_t(k) * S, A.pa);
        k_adj_pA<<<nb, kAB, 0, s>>>(d, p, t.x, t.kcd + size_t(k) * S, t.ccd + size_t(k) * S, A.gv, A.pa,
                                     t.ucd + size_t(k) * S, A.pb, A.grho, A.galpha, A.gx);
        k_adj_pB<<<nb, kAB, 0, s>>>(d, p, t.x, A.pb, A.gv, A.gx);
    }
    // viscosity + surface tension (Jacobi)
    ADJ_TRY(cudaMemsetAsync(A.pc, 0, cap * S * sizeof(float2), s));
    ADJ_TRY(cudaMemsetAsync(A.px, 0, cap * S * sizeof(float4), s));
    ADJ_TRY(cudaMemsetAsync(A.bbar, 0, S * sizeof(float4), s));
    ADJ_TRY(cudaMemsetAsync(A.Dbar, 0, S * sizeof(float4), s));
    ADJ_TRY(cudaMemsetAsync(A.Dbar2, 0, S * sizeof(float4), s));
    ADJ_TRY(cudaMemcpyAsync(A.qbar0, A.gv, S * sizeof(float4), cudaMemcpyDeviceToDevice, s));
    float4* qa = A.qbar0;
    float4* qb = A.qbar1;
    float4* ya = A.y0;
    float4* yb = A.y1;
    k_adj_y<<<nb, kAB, 0, s>>>(d, p, qa, ya);
    for (int k = K - 1; k >= 0; --k) {
        k_adj_jacobi<<<nb, kAB, 0, s>>>(d, p, t.x, A.rev, t.q + size_t(k) * S, t.q + size_t(k + 1) * S, qa, qb,
                                         ya, yb, A.bbar, A.Dbar, A.Dbar2, A.pc, A.px);
        std::swap(qa, qb);
        std::swap(ya, yb);
    }
    const float4* V0 = t.udf + size_t(K) * S;   // pre-solve velocity = DF output
    k_adj_visc_coef<<<nb, kAB, 0, s>>>(d, p, t.x, V0, A.rev, qa, A.bbar, A.Dbar, A.Dbar2, A.pc, A.px, A.gv, A.gx,
                                        A.grho, A.gsf, A.gsig, A.gmu);
    k_adj_stfac<<<nb, kAB, 0, s>>>(d, p, t.x, V0, A.gsf, A.gv, A.gx);
    // divergence-free solve
    for (int k = K - 1; k >= 0; --k) {
        k_adj_pack_a<<<nb, kAB, 0, s>>>(d, p, A.gv, t.kdf + size_t(k) * S, A.pa);
        k_adj_pA<<<nb, kAB, 0, s>>>(d, p, t.x, t.kdf + size_t(k) * S, t.cdf + size_t(k) * S, A.gv, A.pa,
                                     t.udf + size_t(k) * S, A.pb, A.grho, A.galpha, A.gx);
        k_adj_pB<<<nb, kAB, 0, s>>>(d, p, t.x, A.pb, A.gv, A.gx);
    }
    // gravity is the identity; density and alpha
    k_adj_dens_a<<<nb, kAB, 0, s>>>(d, p, t.x, A.galpha, A.gg);
    k_adj_dens_b<<<nb, kAB, 0, s>>>(d, p, t.x, A.grho, A.gg, A.gx);
    k_adj_scatter<<<nb, kAB, 0, s>>>(d, p, A.gx, A.gv, A.gx_id, A.gv_id);
    k_adj_param_reduce<<<h->nscenes, 256, 0, s>>>(d, p, A.gsig, A.gmu, A.gparam);
    ADJ_TRY(cudaMemsetAsync(A.gsig, 0, S * sizeof(double), s));
    ADJ_TRY(cudaMemsetAsync(A.gmu, 0, S * sizeof(double), s));
    ADJ_TRY(cudaGetLastError());
    return MPS_OK;
}

int check_adjoint_config(mps_handle* h) {
    if (h->cfg.fixed_iters <= 0) return fail(MPS_E_INVALID, "adjoint needs fixed_iters > 0");
    if (h->cfg.visc_solver != MPS_VISC_JACOBI) return fail(MPS_E_INVALID, "adjoint needs visc_solver = MPS_VISC_JACOBI");
    if (h->cfg.volume_accumulate) return fail(MPS_E_INVALID, "adjoint needs volume_accumulate = 0");
    if (h->cfg.max_fluid_neighbors > 255) return fail(MPS_E_INVALID, "adjoint needs max_fluid_neighbors <= 255");
    return MPS_OK;
}

}  // namespace

namespace host {
void adjoint_release(mps_handle* h) {
    if (!h->adj) return;
    h->adj->free_all();
    delete h->adj;
    h->adj = nullptr;
}
}  // namespace host

}  // namespace mpsg

using namespace mpsg;

extern "C" {

int64_t mps_adjoint_memory(mps_handle* h, int32_t nsteps, int32_t every) {
    if (!h || !h->layout_ready || nsteps <= 0 || every <= 0) return -1;
    return int64_t(store_bytes(h, nsteps, every));
}

int mps_adjoint_reserve(mps_handle* h, int32_t nsteps, int32_t every) {
    int r = host::check_ready(h);
    if (r) return r;
    if ((r = check_adjoint_config(h))) return r;
    if (nsteps <= 0 || every <= 0) return fail(MPS_E_INVALID, "nsteps and checkpoint_every must be positive");
    Guard g(h->device);
    return ensure_store(h, nsteps, every);
}

int mps_adjoint_forward(mps_handle* h, int32_t nsteps, int32_t every, void* stream) {
    int r = host::check_ready(h);
    if (r) return r;
    if ((r = check_adjoint_config(h))) return r;
    if (nsteps <= 0 || every <= 0) return fail(MPS_E_INVALID, "nsteps and checkpoint_every must be positive");
    Guard g(h->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if ((r = ensure_store(h, nsteps, every))) return r;
    AdjointStore& A = *h->adj;
    A.nsteps = nsteps;
    A.every = every;
    A.ready = false;
    const size_t S = size_t(h->slots);
    for (int t = 0; t < nsteps; ++t) {
        if (t % every == 0) {
            const int c = t / every;
            ADJ_TRY(copy_state(h, h->cur, A.cp_pos + size_t(c) * S, A.cp_vel + size_t(c) * S, A.cp_ids + size_t(c) * S,
                               true, s));
            A.cp_cur[size_t(c)] = h->cur;
        }
        if ((r = host::step_n(h, 1, s))) return r;
    }
    ADJ_TRY(copy_state(h, h->cur, A.fin_pos, A.fin_vel, A.fin_ids, true, s));
    A.fin_cur = h->cur;
    A.fin_steps = h->steps;
    A.ready = true;
    return MPS_OK;
}

int mps_adjoint_backward(mps_handle* h, const float* g_pos4, const float* g_vel4, float* g_pos0, float* g_vel0,
                         double* g_param2, void* stream) {
    int r = host::check_ready(h);
    if (r) return r;
    if ((r = check_adjoint_config(h))) return r;
    if (!h->adj || !h->adj->ready) return fail(MPS_E_STATE, "mps_adjoint_forward first");
    Guard g(h->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    AdjointStore& A = *h->adj;
    const size_t S = size_t(h->slots), N = size_t(h->n);
    ADJ_TRY(cudaMemcpyAsync(A.ctr_save, h->ctr, sizeof(StepCounters), cudaMemcpyDeviceToDevice, s));
    if (g_pos4) ADJ_TRY(cudaMemcpyAsync(A.gx_id, g_pos4, N * sizeof(float4), cudaMemcpyHostToDevice, s));
    else ADJ_TRY(cudaMemsetAsync(A.gx_id, 0, N * sizeof(float4), s));
    if (g_vel4) ADJ_TRY(cudaMemcpyAsync(A.gv_id, g_vel4, N * sizeof(float4), cudaMemcpyHostToDevice, s));
    else ADJ_TRY(cudaMemsetAsync(A.gv_id, 0, N * sizeof(float4), s));
    ADJ_TRY(cudaMemsetAsync(A.gparam, 0, 2 * size_t(h->nscenes) * sizeof(double), s));
    ADJ_TRY(cudaMemsetAsync(A.flag, 0, sizeof(int), s));
    const int nseg = (A.nsteps + A.every - 1) / A.every;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int t0 = seg * A.every, t1 = std::min(A.nsteps, t0 + A.every);
        // record the segment's steps from its checkpoint, then reverse them
        h->cur = A.cp_cur[size_t(seg)];
        ADJ_TRY(copy_state(h, h->cur, A.cp_pos + size_t(seg) * S, A.cp_vel + size_t(seg) * S, A.cp_ids + size_t(seg) * S,
                           false, s));
        for (int k = 0; k < t1 - t0; ++k)
            if ((r = taped_step(h, slot_of(A, k), s))) return r;
        for (int k = t1 - t0 - 1; k >= 0; --k)
            if ((r = adjoint_step(h, slot_of(A, k), s))) return r;
    }
    int flag = 0, ctr_flags = 0;
    ADJ_TRY(cudaMemcpyAsync(&flag, A.flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    ADJ_TRY(cudaMemcpyAsync(&ctr_flags, &h->ctr->flags, sizeof(int), cudaMemcpyDeviceToHost, s));
    ADJ_TRY(cudaStreamSynchronize(s));
    if (g_pos0) ADJ_TRY(cudaMemcpy(g_pos0, A.gx_id, N * sizeof(float4), cudaMemcpyDeviceToHost));
    if (g_vel0) ADJ_TRY(cudaMemcpy(g_vel0, A.gv_id, N * sizeof(float4), cudaMemcpyDeviceToHost));
    if (g_param2) ADJ_TRY(cudaMemcpy(g_param2, A.gparam, 2 * size_t(h->nscenes) * sizeof(double), cudaMemcpyDeviceToHost));
    // leave the handle at the final state with its counters as they were
    h->cur = A.fin_cur;
    ADJ_TRY(copy_state(h, h->cur, A.fin_pos, A.fin_vel, A.fin_ids, false, s));
    ADJ_TRY(cudaMemcpyAsync(h->ctr, A.ctr_save, sizeof(StepCounters), cudaMemcpyDeviceToDevice, s));
    h->steps = A.fin_steps;
    ADJ_TRY(cudaStreamSynchronize(s));
    if (ctr_flags & 1) return fail(MPS_E_OVERFLOW, "neighbour list capacity exceeded during the adjoint");
    if (flag & 1) return fail(MPS_E_STATE, "asymmetric neighbour lists: the gather-form adjoint needs symmetric lists");
    return MPS_OK;
}

}  // extern "C"
