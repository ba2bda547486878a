// Internal declarations of the GB300 DFSPH step: device data layout, FP32 SPH kernel math,
// launch wrappers.  Layout in HBM (all SoA, 16-byte aligned, "slot" = position in the
// per-step cell-sorted order, scenes padded to a multiple of kPad slots so that every
// thread block belongs to exactly one scene):
//   pos4[slot]  = (x, y, z, h)      h = 4 r support radius, 0 for padding slots
//   vel4[slot]  = (vx, vy, vz, m)
//   ids[slot]   = particle ID given at set time
//   nbr_f[k * slots + slot], nbr_b[k * slots + slot]  neighbour lists (interleaved so that a
//                 warp reading its k-th neighbours touches one 128-byte line)
//   cell tables: uint2 {start, end} per cell of each scene's grid (dense, validated against
//                 slot_key so that stale entries need no clearing between steps)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mpsg {

constexpr int kPad = 256;          // slot padding unit per scene
constexpr int kChunk = 64;         // granularity of the slot -> scene table
constexpr float kHRatio = 4.0f;    // support radius = 4 x particle radius
constexpr float kFltEps = 1.1920928955078125e-07f;   // FLT_EPSILON (viscosity denominator)

// Per-scene constants.
struct Scene {
    float ox, oy, oz;               // grid origin
    float cell, inv_cell;           // grid cell size (>= largest support radius) and 1/cell
    int nx, ny, nz;                 // grid dims
    unsigned long long key_base;    // first cell key of this scene
    float bminx, bminy, bminz, bmaxx, bmaxy, bmaxz;   // collision box
    int slot_begin, slot_end;       // padded fluid slots
    int n;                          // real fluid particles (slots [slot_begin, slot_begin + n))
    int coff;                       // compact offset (prefix of n over scenes)
    int bbegin, bend;               // boundary particles of this scene (sorted order)
};

// Cell keys.  Cells are grouped in columns of kBrick x kBrick rows (y, z) that run along x; a
// column's keys run over x, and for each x over its kBrick x kBrick rows (y fastest).  A run of
// consecutive slots so covers a compact box of cells (a 128-slot block: about 4 x 2 x 2 cells at
// 8 particles a cell) instead of a 16-cell stretch of one row, which shrinks the neighbourhood a
// thread block gathers from from about 10x to about 6x its own cells.  grid_key is the key inside
// one grid (ny and nz padded to whole columns); cell_key adds the scene's key base.
constexpr unsigned kBrick = 2;
#ifndef MPSG_KEY_ORDER
#define MPSG_KEY_ORDER 1   // 1: neighbour lists in ascending cell-key (slot) order; 0: (dz, dy, dx) order
#endif
__host__ __device__ __forceinline__ unsigned long long grid_key(int nx, int ny, int cx, int cy, int cz) {
    const unsigned nyb = (unsigned(ny) + kBrick - 1) / kBrick;
    const unsigned long long col = (unsigned long long)(unsigned(cz) / kBrick) * nyb + unsigned(cy) / kBrick;
    return ((col * unsigned(nx) + unsigned(cx)) * kBrick + unsigned(cz) % kBrick) * kBrick + unsigned(cy) % kBrick;
}
__host__ __device__ __forceinline__ unsigned long long cell_key(const Scene& sc, int cx, int cy, int cz) {
    return sc.key_base + grid_key(sc.nx, sc.ny, cx, cy, cz);
}
// Keys of an nx x ny x nz grid.
__host__ __device__ __forceinline__ unsigned long long cell_key_count(int nx, int ny, int nz) {
    const unsigned long long B = kBrick;
    return (unsigned long long)nx * ((unsigned long long)(ny + B - 1) / B * B) * ((unsigned long long)(nz + B - 1) / B * B);
}

// Device-resident solver state of one scene.
struct SceneSolve {
    int active;       // still iterating
    int do_update;    // run the second pass of this iteration
    int iter;         // reference loop counter l
    int blocks_done;  // blocks of this scene finished in the current pass
    double err;       // last mean error (pressure) or r.r (CG)
    double rr;        // CG: r.r of the last operator pass
    double cg_alpha;  // CG step length of the last iteration
    double cg_beta;   // CG direction coefficient of the last iteration
};

struct StepCounters {
    unsigned int scenes_done;   // scenes whose last block finished this pass
    int nactive;                // scenes active at the start of the pass
    int nactive_next;           // scenes still active after their decision in the current pass
    int flags;                  // bit0 overflow, bit1 non-finite, bit2 loop guard, bit3 tile rank out of range
    int passes;                 // loop bodies run in the current solve (hard guard)
    unsigned long long fluid_pairs, boundary_pairs;
    unsigned long long tile_blocks[2];  // neighbourhood tiles of the step: blocks with a tile, blocks without
    unsigned long long iters_total[3];  // sum over steps and scenes of the loop counter (DF, CG, CD)
    unsigned long long runs_total[3];   // solver passes that ran (one per iteration; max over scenes)
    unsigned long long passes_total[3]; // solver passes launched (a graph body holds cg_unroll CG passes)
};

// Uniform parameters, passed by value to every kernel.
struct Params {
    float dt, inv_dt;
    float gx, gy, gz;
    float rho0, inv_rho0, V;      // rest density, particle volume
    float V_lo;                   // volume - V (the float-float density deviation)
    float visc, xsph, sigma;
    float cg_factor;
    int cubic;
    int cap_f, cap_b;             // neighbour list capacities
    int slots;                    // total padded slots
    int nscenes;
    int fixed_iters;
    int min_iter_df, min_iter_cd, max_iter, cg_max_iter;
    int visc_solver;              // 0 CG, 1 Jacobi
    int cg_form;                  // 0 three-pass (reference), 1 two-pass
    int stage;                    // 1: the three-pass CG operator gathers from per-block neighbourhood tiles
    float df_tol, cd_tol, cg_tol; // stored as float for the kernel args; compared in FP64
    double df_tol_d, cd_tol_d, cg_tol_d;
};

// Loop-sum accumulators (sph.cu): lanes a scene, and 64-bit words a lane (one 128-byte line;
// eight are used, four for each of two components).
#ifndef MPSG_ACC_LANES
#define MPSG_ACC_LANES 128
#endif
constexpr int kAccLanes = MPSG_ACC_LANES;   // a multiple of 32
constexpr int kAccStride = 16;
// Neighbourhood tiles of the CG operator (mps_config.stage = 1): capacity in records per slot of
// an operator block (a 128-slot block holds up to 640 distinct neighbour slots).
constexpr int kTilePerSlot = 5;

// Device pointers of one step (buffer a is read, buffer b written by the reorder).
struct Dev {
    float4 *pos, *vel;            // current (sorted) state
    unsigned int* ids;
    float4 *pos_in, *vel_in;      // previous order (reorder source)
    unsigned int* ids_in;
    unsigned long long* slot_key;
    uint2* ftable;                // fluid cell table
    uint2* btable;                // boundary cell table
    const Scene* scenes;
    const int* chunk_scene;       // slot/kChunk -> scene
    unsigned int* nbr_f;
    unsigned int* nbr_b;
    unsigned int* cnt;            // nf | nb << 16
    float* rho;
    float* rdev;                  // rho / rho0 - 1 from the compensated sums (the stiffness reads this)
    float* alpha;
    float* kappa;
    float4* xk;                   // (x, y, z, kappa) of each slot from pressure pass A, gathered by pass B
    float* delta;
    float2* aux;                  // (rho, st factor) packed for the CG gathers
    float4* color;
    float4 *cg_x, *cg_r, *cg_p, *cg_ap, *cg_b;
    float4* cg_s;                 // CG: s = A p kept by recurrence
    float2* cg_coef;              // per fluid pair, interleaved like nbr_f: (c_ij, cv_ij) of the CG operator
    float4* jac_d;                // Jacobi: inverse of the 3x3 diagonal block of A_0 + f I: (xx, yy, zz, xy) (aliases cg_ap)
    float4* jac_d2;               //   (xz, yz, 1 if the block was replaced by (1 + f) I, 0) (aliases cg_r)
    unsigned char* tape_code;     // adjoint recording (null in plain steps): stiffness branch per slot
    unsigned char* tape_adv;      // adjoint recording: collision branch per slot (2 bits per axis)
    const float4* bpos;           // boundary (x, y, z, h)
    float* bvol;
    float* bvol_lo;               // bvol + bvol_lo = the volume to about 48 bits (the density deviation)
    double* partial;              // per-block partial sums of the CG operator pass and the Jacobi sweep
    unsigned long long* acc;      // loop-sum accumulators: (scenes + 1) x kAccLanes x kAccStride words
    unsigned short* nbr_t;        // stage 1: tile rank of each fluid neighbour, interleaved like nbr_f
    unsigned int* tile_j;         // stage 1: per operator block, its distinct neighbour slots (ascending)
    int* tile_n;                  // stage 1: per operator block, the tile's size, or -1 (global gathers)
    SceneSolve* solve;
    StepCounters* ctr;
    int* scene_iters;             // 3 per scene (DF, CG, CD) of the last step
    double* scene_err;            // 3 per scene
    unsigned long long* keys;     // compact keys (sorted in place by the radix sort)
    unsigned int* vals;
};

// ------------------------------------------------------------------ FP32 kernel math
// Constants of MPSSPHKernel.cuh:9-14 written from their formulas.
#define MPSG_PI_F 3.14159265358979323846f
struct KC {
    static constexpr float w = 315.0f / (64.0f * MPSG_PI_F);
    static constexpr float g = 45.0f / MPSG_PI_F;
    static constexpr float cw = 8.0f / MPSG_PI_F;
    static constexpr float cg = 48.0f / MPSG_PI_F;
    static constexpr float stw = 8.0f / MPSG_PI_F * 10.0f / 7.0f * 2.0f;
    static constexpr float stg = 48.0f / MPSG_PI_F * 10.0f / 7.0f;
};

// W(d) with q = d / h (poly6 or cubic spline), MPSSPHKernel.cuh:28-45.
__device__ __forceinline__ float kW(float d, float invh, int cubic) {
    const float q = d * invh;
    if (q >= 1.0f) return 0.0f;
    if (cubic) {
        if (q >= 0.5f) {
            const float t = (1.0f - q) * invh;
            return KC::cw * 2.0f * t * t * t;
        }
        return KC::cw * invh * invh * invh * ((6.0f * q - 6.0f) * q * q + 1.0f);
    }
    const float t = (1.0f - q * q) * invh;
    return KC::w * t * t * t;
}
// G(d) with grad W = G x_ij, MPSSPHKernel.cuh:46-65.  invd = 1/d.
__device__ __forceinline__ float kG(float d, float invd, float invh, int cubic) {
    const float q = d * invh;
    if (q < 1.0e-20f || q >= 1.0f) return 0.0f;
    const float invh2 = invh * invh;
    if (cubic) {
        if (q > 0.5f) {
            const float t = (1.0f - q) * invh2;
            return -KC::cg * invd * t * t;
        }
        return KC::cg * invd * invh2 * invh2 * (3.0f * q - 2.0f) * q;
    }
    const float t = (1.0f - q) * invh2;
    return -KC::g * invd * t * t;
}
// Surface-tension kernels, MPSSPHKernel.cuh:67-84.
__device__ __forceinline__ float kSTW(float d, float invh) {
    const float q = fmaxf(d * invh, 0.5f);
    if (q >= 1.0f) return 0.0f;
    const float t = (1.0f - q) * invh;
    return KC::stw * t * t * t;
}
__device__ __forceinline__ float kSTG(float d, float invd, float invh) {
    const float q = d * invh;
    if (q <= 0.5f || q >= 1.0f) return 0.0f;
    const float t = (1.0f - q) * invh * invh;
    return -KC::stg * invd * t * t;
}

// Squared distance with an explicit operation order (no implicit contraction), shared with
// the oracle's FP32 neighbour test: fma(dz,dz,fma(dy,dy,dx*dx)).
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// 1/d for a pair; 0 for coincident particles so that d = d2 * (1/d) = 0 and G(0) = 0.
__device__ __forceinline__ float safe_rsqrt(float d2) { return d2 > 0.0f ? rsqrtf(d2) : 0.0f; }

// Kahan-compensated FP32 accumulator.
struct Kahan {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float y = __fsub_rn(x, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
};

// Float-float ("double-float") arithmetic: a value is hi + lo with |lo| <= ulp(hi) / 2, about 48
// significant bits, from error-free transformations in FP32 (explicit round-to-nearest intrinsics,
// so that no contraction changes them).  Used where FP32 loses the result in a cancellation and
// FP64, a small fraction of FP32's rate on GB300, would be the slow part: the density deviation
// rho/rho0 - 1 that the stiffness reads.
struct ff {
    float hi, lo;
};
__device__ __forceinline__ ff ff_two_sum(float a, float b) {   // a + b exactly
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {   // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const ff s = ff_two_sum(a.hi, b.hi);
    return ff_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = __fmaf_rn(a.hi, b.hi, -p);
    return ff_fast_two_sum(p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e)));
}
__device__ __forceinline__ ff ff_mul(ff a, float b) {
    const float p = __fmul_rn(a.hi, b);
    return ff_fast_two_sum(p, __fmaf_rn(a.lo, b, __fmaf_rn(a.hi, b, -p)));
}
__device__ __forceinline__ ff ff_sqr_diff(float a, float b) {   // (a - b)^2 with a - b exact as a pair
    const ff d = ff_two_sum(a, -b);
    return ff_mul(d, d);
}
__device__ __forceinline__ float ff_val(ff a) { return __fadd_rn(a.hi, a.lo); }
// 1/h as a pair: hi the rounded reciprocal, lo its residual (1 - h hi) / h.
__device__ __forceinline__ ff ff_recip(float h) {
    const float r = 1.0f / h;
    return {r, __fmul_rn(__fmaf_rn(-h, r, 1.0f), r)};
}
// Constants of the kernels as pairs (hi = the FP32 rounding of c, lo = c - hi), from FP64.
#define MPSG_FF_CONST(c) ff{float(c), float((c) - double(float(c)))}
constexpr double kPiD = 3.14159265358979323846;
// Per-particle scales of ff_VW: V c invh^3 for the kernel's branches (cubic: c = 16/pi for q >= 1/2,
// 8/pi below; poly6: c = 315 / (64 pi)), so that a pair needs one product for them.
struct FFScale {
    ff outer, inner;
};
__device__ __forceinline__ FFScale ff_scales(ff invh, ff V, int cubic) {
    const ff v3 = ff_mul(ff_mul(ff_mul(invh, invh), invh), V);
    if (cubic) return {ff_mul(v3, MPSG_FF_CONST(16.0 / kPiD)), ff_mul(v3, MPSG_FF_CONST(8.0 / kPiD))};
    const ff w = ff_mul(v3, MPSG_FF_CONST(315.0 / (64.0 * kPiD)));
    return {w, w};
}
// V W(|x_i - x_j|) in float-float, with invh = 1/h_i and the scales of ff_scales: the squared
// distance exactly from the FP32 positions, its square root to about 48 bits, then the kernel
// polynomial (MPSSPHKernel.cuh:28-45) in pairs.
__device__ __forceinline__ ff ff_VW(float4 xi, float4 xj, ff invh, const FFScale& sc, int cubic) {
    const ff d2 = ff_add(ff_add(ff_sqr_diff(xi.x, xj.x), ff_sqr_diff(xi.y, xj.y)), ff_sqr_diff(xi.z, xj.z));
    if (cubic) {
        // d = sqrt(d2): hi the rounded root, lo = (d2 - hi^2) / (2 hi)
        ff d{0.0f, 0.0f};
        if (d2.hi > 0.0f) {
            const float r = sqrtf(d2.hi);
            d = ff_fast_two_sum(r, __fmul_rn(__fadd_rn(__fmaf_rn(-r, r, d2.hi), d2.lo), __fdividef(0.5f, r)));
        }
        const ff q = ff_mul(d, invh);
        if (q.hi >= 1.0f) return ff{0.0f, 0.0f};
        if (q.hi >= 0.5f) {   // V 2 cw invh^3 (1 - q)^3; 1 - q.hi is exact for q in [0.5, 1]
            const ff t = ff_fast_two_sum(__fsub_rn(1.0f, q.hi), -q.lo);
            return ff_mul(ff_mul(ff_mul(t, t), t), sc.outer);
        }
        // V cw invh^3 ((6 q - 6) q^2 + 1)
        const ff q6 = ff_add(ff_mul(q, 6.0f), ff{-6.0f, 0.0f});
        return ff_mul(ff_add(ff_mul(ff_mul(q6, q), q), ff{1.0f, 0.0f}), sc.inner);
    }
    // poly6: V w invh^3 (1 - q^2)^3 with q^2 = d2 invh^2
    const ff q2 = ff_mul(ff_mul(d2, invh), invh);
    if (q2.hi >= 1.0f) return ff{0.0f, 0.0f};
    const ff t = ff_add(ff{1.0f, 0.0f}, ff{-q2.hi, -q2.lo});
    return ff_mul(ff_mul(ff_mul(t, t), t), sc.outer);
}

// Neighbour loops are latency-bound (a dependent index load, then gathers).  visit_batched walks
// the interleaved list of slot i (item k at list[k * stride + i]) in batches of B: phase 1 loads
// the batch's indices and the per-pair data streamed in the same layout (stream(k)), phase 2
// issues every gather (gather(j, k)), phase 3 runs use(gathered, streamed, k) in k order.  A
// thread so keeps B index + stream loads, then B gathers, in flight, and sums in the same order as
// a plain loop (results are bit-identical for every B and PF).  PF != 0 pipelines the loop: the next
// batch's indices and streamed data load while this batch's gathers are in flight.
struct NoStream {};

// Loads of the per-pair streams (neighbour indices, CG coefficients).  Each item is read once per
// pass, so the loads skip L1 allocation (L1::no_allocate) and leave L1 to the neighbour gathers,
// which the warp's other lanes reuse.  MPSG_STREAM_HINT=0 restores plain loads.
#ifndef MPSG_STREAM_HINT
#define MPSG_STREAM_HINT 1
#endif
__device__ __forceinline__ unsigned ld_stream(const unsigned* p) {
#if MPSG_STREAM_HINT
    unsigned v;
    asm("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
#else
    return *p;
#endif
}
__device__ __forceinline__ unsigned ld_stream(const unsigned short* p) {
#if MPSG_STREAM_HINT
    unsigned short v;
    asm("ld.global.nc.L1::no_allocate.u16 %0, [%1];" : "=h"(v) : "l"(p));
    return v;
#else
    return *p;
#endif
}
__device__ __forceinline__ float2 ld_stream(const float2* p) {
#if MPSG_STREAM_HINT
    float2 v;
    asm("ld.global.nc.L1::no_allocate.v2.f32 {%0,%1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
    return v;
#else
    return *p;
#endif
}
template <int B, class S, class T, int PF = 0, class Stream, class Gather, class Use>
__device__ __forceinline__ void visit_batched(const unsigned* __restrict__ list, size_t stride, int i, int n,
                                              Stream stream, Gather gather, Use use) {
    int k = 0;
    if constexpr (PF != 0) {
        unsigned jj[B];
        S ss[B];
        if (n >= B) {
#pragma unroll
            for (int u = 0; u < B; ++u) {
                jj[u] = ld_stream(list + size_t(u) * stride + size_t(i));
                ss[u] = stream(u);
            }
        }
        for (; k + B <= n; k += B) {
            T v[B];
            S sc[B];
#pragma unroll
            for (int u = 0; u < B; ++u) {
                v[u] = gather(jj[u], k + u);
                sc[u] = ss[u];
            }
            if (k + 2 * B <= n) {
#pragma unroll
                for (int u = 0; u < B; ++u) {
                    jj[u] = ld_stream(list + size_t(k + B + u) * stride + size_t(i));
                    ss[u] = stream(k + B + u);
                }
            }
#pragma unroll
            for (int u = 0; u < B; ++u) use(v[u], sc[u], k + u);
        }
    } else {
        for (; k + B <= n; k += B) {
            unsigned jj[B];
            S ss[B];
#pragma unroll
            for (int u = 0; u < B; ++u) {
                jj[u] = ld_stream(list + size_t(k + u) * stride + size_t(i));
                ss[u] = stream(k + u);
            }
            T v[B];
#pragma unroll
            for (int u = 0; u < B; ++u) v[u] = gather(jj[u], k + u);
#pragma unroll
            for (int u = 0; u < B; ++u) use(v[u], ss[u], k + u);
        }
    }
    for (; k < n; ++k) {
        const S sk = stream(k);
        use(gather(ld_stream(list + size_t(k) * stride + size_t(i)), k), sk, k);
    }
}

// Batch sizes per loop (template arguments of visit_batched), set from GB300 sweeps.
// Software-pipelined index loads per loop (PF of visit_batched), set from the same sweeps.
#ifndef MPSG_PF_AP
#define MPSG_PF_AP 0
#endif
#ifndef MPSG_PF_PA
#define MPSG_PF_PA 1
#endif
#ifndef MPSG_PF_PB
#define MPSG_PF_PB 0
#endif
#ifndef MPSG_PF_DENS
#define MPSG_PF_DENS 0
#endif
#ifndef MPSG_PF_SETUP
#define MPSG_PF_SETUP 0
#endif
#ifndef MPSG_B_AP
#define MPSG_B_AP 4      // CG / Jacobi operator
#endif
#ifndef MPSG_B_PA
#define MPSG_B_PA 2      // density change rate (pressure pass A)
#endif
#ifndef MPSG_B_PB
#define MPSG_B_PB 4      // pressure force (pass B)
#endif
#ifndef MPSG_B_DENS
#define MPSG_B_DENS 2    // density and alpha
#endif
#ifndef MPSG_B_SETUP
#define MPSG_B_SETUP 2   // surface-tension factor and the solve's coefficients (once per step)
#endif

__device__ __forceinline__ int cell_coord(float x, float o, float inv, int dim) {
    const float t = __fmul_rn(__fsub_rn(x, o), inv);
    if (!(t >= 0.0f)) return 0;
    if (t >= float(dim)) return dim - 1;
    const int c = int(t);
    return c < dim ? c : dim - 1;
}

// ------------------------------------------------------------------ launch wrappers
// Radix sort of (key, val) pairs by the low `bits` bits of key; stable.  Uses tmp buffers of
// the same size; the result ends in keys/vals.  Returns cudaError_t.
cudaError_t radix_sort_pairs(unsigned long long* keys, unsigned int* vals,
                             unsigned long long* keys_tmp, unsigned int* vals_tmp,
                             unsigned int* counts, int n, int bits, int digit_bits,
                             cudaStream_t s);
size_t radix_counts_size(int n);

void launch_keys(const Dev& d, const Params& p, cudaStream_t s);
void launch_reorder(const Dev& d, const Params& p, int n_real, cudaStream_t s);
void launch_build_nbrs(const Dev& d, const Params& p, int bs, cudaStream_t s);
void launch_bvolume(const Dev& d, const Params& p, int nb, int accumulate, cudaStream_t s);
void launch_density_alpha(const Dev& d, const Params& p, int bs, cudaStream_t s);
// One part of the fused density pass (what: 1 density, 2 colour, 4 alpha, 8 gravity) over the
// neighbour sets in `parts` (1 fluid, 2 boundary); returns -1 for an unknown part.
int launch_density_part(const Dev& d, const Params& p, int bs, int what, int parts, cudaStream_t s);
void launch_solver_init(const Dev& d, const Params& p, cudaStream_t s);
void launch_set_cond(const Dev& d, unsigned long long cond, cudaStream_t s);
void launch_load_state(const Dev& d, const Params& p, const float4* pos4, const float4* vel4, int n,
                       cudaStream_t s);
void launch_store_state(const Dev& d, const Params& p, float4* pos4, float4* vel4, cudaStream_t s);
void launch_pressure_A(const Dev& d, const Params& p, int mode, int bs,
                       unsigned long long cond, int use_cond, cudaStream_t s);
void launch_pressure_B(const Dev& d, const Params& p, int bs, unsigned long long cond, int use_cond, int limit,
                       cudaStream_t s);
void launch_pressure_B_profile(const Dev& d, const Params& p, int bs, cudaStream_t s);
void launch_solver_finish(const Dev& d, const Params& p, int which, cudaStream_t s);
void launch_st_factor(const Dev& d, const Params& p, int bs, cudaStream_t s);
void launch_cg_b(const Dev& d, const Params& p, int bs, cudaStream_t s);
void launch_cg_ap(const Dev& d, const Params& p, int bs, unsigned long long cond, int use_cond,
                  cudaStream_t s);
void launch_cg_update(const Dev& d, const Params& p, int bs, unsigned long long cond, int use_cond, int limit,
                      cudaStream_t s);
// three-pass form: A p + dots, x/r update + r.r, direction update (with the loop guard)
void launch_cg_ap3(const Dev& d, const Params& p, int bs, unsigned long long cond, int use_cond, cudaStream_t s);
void launch_cg_update3(const Dev& d, const Params& p, int bs, cudaStream_t s);
// The three-pass update and direction passes in their profiling form (no loop decision).
void launch_cg_vector_profile(const Dev& d, const Params& p, cudaStream_t s);
void launch_cg_dir3(const Dev& d, const Params& p, int bs, unsigned long long cond, int use_cond, int limit,
                    cudaStream_t s);
void launch_cg_finish(const Dev& d, const Params& p, cudaStream_t s);
// Jacobi sweep of the viscosity/surface-tension system; src/dst null = the two iterate buffers
// chosen by the scene's loop counter (graph form), else explicit (adjoint recording).
void launch_jacobi(const Dev& d, const Params& p, int bs, unsigned long long cond, int use_cond, int limit,
                   const float4* src, float4* dst, cudaStream_t s);
void launch_jacobi_finish(const Dev& d, const Params& p, const float4* src, cudaStream_t s);
void launch_advect(const Dev& d, const Params& p, cudaStream_t s);
// what: 1 boundary collision (velocities), 2 position update
void launch_advect_part(const Dev& d, const Params& p, int what, cudaStream_t s);
void launch_stats(const Dev& d, const Params& p, cudaStream_t s);

}  // namespace mpsg
