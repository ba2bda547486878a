// SPH kernels of the GB300 DFSPH step.  One thread per slot (cell-sorted particle).
// Reference counterparts (moonsh5009/MPS_CUDA):
//   k_keys / k_reorder     SpatialHash::UpdateHash, InitHash_kernel, ReorderHash_kernel
//                          (src/MPS_Object/MPSSpatialHash.cu:53-77, .cuh:83-145); new scheme:
//                          clamped floor cells, 64-bit keys, stable radix sort, SoA reorder.
//   k_build_nbrs           BuildNeighorhood x3 (MPSSpatialHash.cu:142-218, .cuh:147-271);
//                          one pass over the 27 cells in key order instead of count+scan+fill.
//   k_bvolume              ComputeBoundaryParticleVolume* (MPSSPHBaseUtil.cuh:10-86)
//   k_density_alpha        ComputeDensity*, DensityColorTest, ComputeDFSPHFactor*, ResetForce,
//                          ApplyGravity, UpdateVelocity (MPSSystem.cpp:240-255) fused.
//   k_pressure_A / _B      ComputeDensityDelta* + Compute{DF,CD}Stiffness + residual
//                          (MPSSPHDFSPHUtil.cuh:139-340) / ApplyDFSPH* + UpdateVelocity
//                          (:342-468); loop control of MPSSPHDFSPHUtil.cu:270-441 on the device
//                          (k_pressure_decide between the two passes).
//   k_st_factor, k_cg_*    ComputeSurfaceTensionFactor/CGb/CGAp, ComputeCGViscosityAp,
//                          ComputeFinalCGAp (MPSSPHNonPressureUtil.cuh:425-648) and CGSolver
//                          (MPSSolver.cuh:12-73, MPSCGKernel.cuh:5-133) with device-side dots
//                          (k_cg_decide3 / k_cg_beta3 / k_cg_decide2: the solver's scalars).
//   k_advect               BoundaryCollision + UpdatePosition (MPSAdvectUtil.cuh:36-77).
#include "mps_internal.cuh"

namespace mpsg {

namespace {

constexpr unsigned kFull = 0xffffffffu;

// gathered neighbour records of the batched loops
struct XV { float4 x, v; };
struct XVA { float4 x, v; float2 a; };
struct XQ { float4 x, q; };
struct XB { float4 x; float lo; };   // boundary position + volume, and the volume's low part

// Programmatic dependent launch between a decide kernel and the vector pass after it: the decide
// kernel releases its dependent as it starts; the vector pass loads its vectors (written by kernels
// that completed before the decide kernel started) and waits for the decide kernel's result
// (griddepcontrol.wait: the primary grid complete and its memory visible) only before it reads
// alpha or beta and before its first store.  Both instructions are no-ops in a plain launch.
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launch bounds of the neighbour passes that gather through L1 (CG operator, pressure A and B):
// with MPSG_MINW_* > 0 the register allocator is asked for at least that many resident warps a SM
// (MINW / (BS / 32) blocks); 0 leaves its default (48 registers, 40 warps at 128 threads).
#ifndef MPSG_MINW_AP
#define MPSG_MINW_AP 0
#endif
#ifndef MPSG_MINW_PA
#define MPSG_MINW_PA 0
#endif
#ifndef MPSG_MINW_PB
#define MPSG_MINW_PB 0
#endif
#if MPSG_MINW_AP > 0
#define MPSG_BOUNDS_AP(BS) __launch_bounds__(BS, MPSG_MINW_AP / ((BS) / 32))
#else
#define MPSG_BOUNDS_AP(BS) __launch_bounds__(BS)
#endif
#if MPSG_MINW_PA > 0
#define MPSG_BOUNDS_PA(BS) __launch_bounds__(BS, MPSG_MINW_PA / ((BS) / 32))
#else
#define MPSG_BOUNDS_PA(BS) __launch_bounds__(BS)
#endif
#if MPSG_MINW_PB > 0
#define MPSG_BOUNDS_PB(BS) __launch_bounds__(BS, MPSG_MINW_PB / ((BS) / 32))
#else
#define MPSG_BOUNDS_PB(BS) __launch_bounds__(BS)
#endif
// The same for the once-a-step passes: solve set-up (k_cg_b), density (k_density_alpha) and
// neighbour build (k_build_nbrs).
#ifndef MPSG_MINW_SETUP
#define MPSG_MINW_SETUP 0
#endif
#ifndef MPSG_MINW_DENS
#define MPSG_MINW_DENS 0
#endif
#ifndef MPSG_MINW_BUILD
#define MPSG_MINW_BUILD 0
#endif
#if MPSG_MINW_SETUP > 0
#define MPSG_BOUNDS_SETUP(BS) __launch_bounds__(BS, MPSG_MINW_SETUP / ((BS) / 32))
#else
#define MPSG_BOUNDS_SETUP(BS) __launch_bounds__(BS)
#endif
#if MPSG_MINW_DENS > 0
#define MPSG_BOUNDS_DENS(BS) __launch_bounds__(BS, MPSG_MINW_DENS / ((BS) / 32))
#else
#define MPSG_BOUNDS_DENS(BS) __launch_bounds__(BS)
#endif
#if MPSG_MINW_BUILD > 0
#define MPSG_BOUNDS_BUILD(BS) __launch_bounds__(BS, MPSG_MINW_BUILD / ((BS) / 32))
#else
#define MPSG_BOUNDS_BUILD(BS) __launch_bounds__(BS)
#endif

__device__ __forceinline__ int block_scene(const Dev& d, int bs) {
    return d.chunk_scene[(blockIdx.x * bs) / kChunk];
}

template <int BS>
__device__ __forceinline__ double block_sum(double v, double* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < BS / 32 ? sh[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
        if (lane == 0) sh[0] = v;
    }
    __syncthreads();
    const double r = sh[0];
    __syncthreads();
    return r;
}

// Block sums of two per-thread FP32 values: FP32 within a warp (32 terms), FP64 across warps.
// GB300's FP64 rate is a small fraction of FP32, so per-thread products and shuffles stay FP32;
// the result is valid in thread 0 only.
template <int BS>
__device__ __forceinline__ double2 block_sum2_f(float a, float b, double2* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(kFull, a, o);
        b += __shfl_down_sync(kFull, b, o);
    }
    __syncthreads();
    if (lane == 0) sh[warp] = make_double2(double(a), double(b));
    __syncthreads();
    double2 r = make_double2(0.0, 0.0);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 0; w < BS / 32; ++w) { r.x += sh[w].x; r.y += sh[w].y; }
    }
    return r;
}

// Per-block partials are stored as FP32 (hi, lo) pairs, hi + lo = the block's FP64 sum to 48 bits
// (16 bytes a block: two components), and the one-block scene sums add them as compensated
// FP32 pairs (TwoSum, then renormalised): with GB300's FP64 rate, adding a 1M scene's 7800
// partials in FP64 on one SM was most of a decide kernel.  Sums are deterministic (fixed order)
// and relative errors stay near 1e-12, far below the FP32 rounding of alpha and beta.
__device__ __forceinline__ float2 df_from(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - double(h)));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float s = __fadd_rn(a.x, b.x);
    const float v = __fsub_rn(s, a.x);
    const float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, v)), __fsub_rn(b.x, v));
    const float t = __fadd_rn(e, __fadd_rn(a.y, b.y));
    const float h = __fadd_rn(s, t);
    return make_float2(h, __fsub_rn(t, __fsub_rn(h, s)));
}
__device__ __forceinline__ double df_to(float2 a) { return double(a.x) + double(a.y); }
// Thread 0 of block b stores its partials (components 0 and 1).
__device__ __forceinline__ void put_partial(const Dev& d, int b, double v0, double v1) {
    const float2 a = df_from(v0), c = df_from(v1);
    reinterpret_cast<float4*>(d.partial)[b] = make_float4(a.x, a.y, c.x, c.y);
}
// Block sums of two per-thread FP32 values stored as block b's partials (16 bytes a block, the
// layout of put_partial): FP32 within a warp, then the warps' sums added by thread 0 as
// compensated FP32 pairs (TwoSum: each pair holds the exact sum of the warp sums to about 48
// bits), with no FP64 arithmetic at the end of the block (1M CG operator pass: 112 -> 110 us
// against FP64 block sums).  sh: BS / 32 entries.
template <int BS>
__device__ __forceinline__ void block_partial2(const Dev& d, float a, float b, float2* sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(kFull, a, o);
        b += __shfl_down_sync(kFull, b, o);
    }
    __syncthreads();
    if (lane == 0) sh[warp] = make_float2(a, b);
    __syncthreads();
    if (threadIdx.x == 0) {
        float2 t0 = make_float2(sh[0].x, 0.f), t1 = make_float2(sh[0].y, 0.f);
#pragma unroll
        for (int w = 1; w < BS / 32; ++w) {
            t0 = df_add(t0, make_float2(sh[w].x, 0.f));
            t1 = df_add(t1, make_float2(sh[w].y, 0.f));
        }
        reinterpret_cast<float4*>(d.partial)[blockIdx.x] = make_float4(t0.x, t0.y, t1.x, t1.y);
    }
}

// Loop sums through per-scene integer accumulators (pressure pass A, the two-pass CG operator and
// the three-pass CG update; the three-pass CG operator keeps its per-block partials, below).
// Each warp of a pass kernel adds its FP32 sum, scaled by 2^64 and truncated to an integer, as
// three signed 42-bit limbs (bits 0-41, 42-83, 84-125) into one lane of its scene's accumulator;
// a non-finite sum or one of magnitude 2^62 or more counts in a fourth word and makes the scene
// sum NaN.  Integer adds are exact, so a scene sum does not depend on the order in which warps
// finish nor on how the scene is cut into blocks, and the decide kernel after the pass reads the
// lanes with one warp instead of summing a partial per block.  Limb sums stay below 2^63 for up
// to 2^21 additions a lane.  Layout: one 128-byte line a lane,
// acc[(scene * kAccLanes + lane) * kAccStride + 4 * component + word]; region `nscenes` takes the
// additions of the profiling forms, which no decide kernel reads.  1M dam break, same box:
// 6.409 ms a step with per-block partials everywhere, 6.344 ms with accumulators everywhere
// (the CG operator pass 112.8 -> 118.9 us: its warps end on two components' atomics), 6.272 ms
// with this split (CG update 20.9 -> 19.6 us, the decide kernels after these passes one warp).
__device__ __forceinline__ unsigned long long* acc_at(const Dev& d, int s) {
    return d.acc + size_t(s) * (kAccLanes * kAccStride);
}
constexpr unsigned long long kLimbMask = (1ull << 42) - 1ull;
// Called by every thread of a pass block: each warp sums its threads' values (NC components) in
// FP32 (a butterfly, so every lane holds the sums), and lanes 4c + k add word k of component c to
// accumulator lane (warp index in the grid % kAccLanes) of scene s, or of the unread region when
// prof is set.  Word k < 3 is limb k of floor(|v| 2^64) for the warp sum v, from its FP32 bits
// (v = m 2^(e - 150) with the 24-bit significand m and biased exponent e, so |v| 2^64 =
// m 2^(e - 86)), negated for v < 0; word 3 counts sums that are infinite, NaN or 2^62 or more.
// Warps add their own sums and retire independently: an FP64 block sum split into limbs by one
// thread lengthened the end of every block (operator pass +10 us at 1M with integer shifts, more
// with FP64 steps), and a shared-memory merge of the warps' limbs with one set of atomics a block
// was no faster than this.
template <int NC>
__device__ __forceinline__ void warp_acc_put(const Dev& d, const Params& p, int s, bool prof, float a, float b) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(kFull, a, o);
        if (NC == 2) b += __shfl_xor_sync(kFull, b, o);
    }
    const int lane = threadIdx.x & 31;
    if (lane >= 4 * NC) return;
    const int k = lane & 3;
    const unsigned bits = __float_as_uint(lane < 4 ? a : b);
    const unsigned e = (bits >> 23) & 0xffu;
    const bool bad = e >= 189u;   // |v| >= 2^62, infinity or NaN
    unsigned long long w;
    if (k == 3) {
        w = bad ? 1ull : 0ull;
    } else {
        const unsigned long long m = e ? ((bits & 0x7fffffu) | 0x800000u) : 0u;   // subnormal: below 2^-64
        const int t = int(e) - 86 - 42 * k;   // limb k holds bits [42 k, 42 k + 42) of m 2^(e - 86)
        const unsigned long long l = bad ? 0ull : t >= 0 ? (t < 42 ? (m << t) & kLimbMask : 0ull)
                                                         : (t > -24 ? m >> (-t) : 0ull);
        w = (bits >> 31) ? 0ull - l : l;
    }
    if (w) {
        const unsigned wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
        unsigned long long* g = acc_at(d, prof ? p.nscenes : s) + size_t(wid & (kAccLanes - 1)) * kAccStride;
        atomicAdd(g + 4 * (lane >> 2) + k, w);
    }
}
// Moves the carries up so that limbs 0 and 1 lie in [0, 2^42) (arithmetic shifts: floor division).
__device__ __forceinline__ void limb_carry(long long& l0, long long& l1, long long& l2) {
    long long cy = l0 >> 42;
    l0 -= cy * (1ll << 42);
    l1 += cy;
    cy = l1 >> 42;
    l1 -= cy * (1ll << 42);
    l2 += cy;
}
// Run by one full warp: the sum of scene s's component c, which it then zeroes for the next pass.
// The limbs are summed and normalised in integers to the magnitude of the sum (all three
// non-negative), so the only roundings are the two additions of the final FP64 sum, which add
// terms of one sign, the same on every run.
__device__ __forceinline__ double acc_take(const Dev& d, int s, int c) {
    constexpr int U = kAccLanes / 32;
    const int lane = threadIdx.x & 31;
    unsigned long long* a = acc_at(d, s) + 4 * c;
    ulonglong2 q[U][2];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const ulonglong2* w = reinterpret_cast<const ulonglong2*>(a + (lane + 32 * u) * kAccStride);
        q[u][0] = __ldcg(w);
        q[u][1] = __ldcg(w + 1);
    }
    long long l0 = 0, l1 = 0, l2 = 0;
    unsigned long long bad = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) {
        ulonglong2* w = reinterpret_cast<ulonglong2*>(a + (lane + 32 * u) * kAccStride);
        w[0] = make_ulonglong2(0ull, 0ull);
        w[1] = make_ulonglong2(0ull, 0ull);
        l0 += static_cast<long long>(q[u][0].x);
        l1 += static_cast<long long>(q[u][0].y);
        l2 += static_cast<long long>(q[u][1].x);
        bad += q[u][1].y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        l0 += __shfl_xor_sync(kFull, l0, o);
        l1 += __shfl_xor_sync(kFull, l1, o);
        l2 += __shfl_xor_sync(kFull, l2, o);
        bad += __shfl_xor_sync(kFull, bad, o);
    }
    if (bad) return __longlong_as_double(0x7ff8000000000000ll);
    limb_carry(l0, l1, l2);
    const bool neg = l2 < 0;   // limbs 0 and 1 are non-negative now, so the sign is limb 2's
    if (neg) {
        l0 = -l0;
        l1 = -l1;
        l2 = -l2;
        limb_carry(l0, l1, l2);
    }
    const double r = double(l2) * 0x1p20 + (double(l1) * 0x1p-22 + double(l0) * 0x1p-64);
    return neg ? -r : r;
}

// Deterministic sum of this scene's per-block partials (component c of 2), run by one block of
// NT threads over blocks of SPB slots.
template <int NT, int SPB>
__device__ double scene_partial_sum(const Dev& d, const Scene& sc, int c, double* sh) {
    const int b0 = sc.slot_begin / SPB, b1 = sc.slot_end / SPB;
    double v = 0.0;
    const float4* P = reinterpret_cast<const float4*>(d.partial);
    for (int b = b0 + threadIdx.x; b < b1; b += NT) {
        const float4 q = __ldcg(P + b);
        v += c == 0 ? df_to(make_float2(q.x, q.y)) : df_to(make_float2(q.z, q.w));
    }
    return block_sum<NT>(v, sh);
}

#ifndef MPSG_DECIDE_NT
#define MPSG_DECIDE_NT 1024
#endif
#ifndef MPSG_SUM_ILP
#define MPSG_SUM_ILP 4
#endif
constexpr int kAccDecideThreads = 32;   // one warp reads a scene's accumulator lanes
constexpr int kDecideThreads = MPSG_DECIDE_NT;   // a decide kernel over per-block partials
constexpr int kSumILP = MPSG_SUM_ILP;
// Deterministic sums of scene sc's per-block partials (blocks of spb slots; component 0, or both
// when NC = 2) by one block of NT threads: kSumILP loads in flight per thread, combined in a fixed
// order.
template <int NT, int NC>
__device__ double2 scene_partials(const Dev& d, const Scene& sc, int spb, double2* sh) {
    const int b0 = sc.slot_begin / spb, b1 = sc.slot_end / spb;
    const float4* P = reinterpret_cast<const float4*>(d.partial);
    float2 ax[kSumILP], ay[kSumILP];
#pragma unroll
    for (int u = 0; u < kSumILP; ++u) { ax[u] = make_float2(0.f, 0.f); ay[u] = make_float2(0.f, 0.f); }
    int b = b0 + int(threadIdx.x);
    for (; b + (kSumILP - 1) * NT < b1; b += kSumILP * NT) {
        float4 v[kSumILP];
#pragma unroll
        for (int u = 0; u < kSumILP; ++u) v[u] = __ldcg(P + b + u * NT);
#pragma unroll
        for (int u = 0; u < kSumILP; ++u) {
            ax[u] = df_add(ax[u], make_float2(v[u].x, v[u].y));
            if (NC == 2) ay[u] = df_add(ay[u], make_float2(v[u].z, v[u].w));
        }
    }
    for (; b < b1; b += NT) {
        const float4 v = __ldcg(P + b);
        ax[0] = df_add(ax[0], make_float2(v.x, v.y));
        if (NC == 2) ay[0] = df_add(ay[0], make_float2(v.z, v.w));
    }
    float2 tx = ax[0], ty = ay[0];
#pragma unroll
    for (int u = 1; u < kSumILP; ++u) {
        tx = df_add(tx, ax[u]);
        if (NC == 2) ty = df_add(ty, ay[u]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        tx = df_add(tx, make_float2(__shfl_down_sync(kFull, tx.x, o), __shfl_down_sync(kFull, tx.y, o)));
        if (NC == 2) ty = df_add(ty, make_float2(__shfl_down_sync(kFull, ty.x, o), __shfl_down_sync(kFull, ty.y, o)));
    }
    float4* sw = reinterpret_cast<float4*>(sh);
    if (lane == 0) sw[warp] = make_float4(tx.x, tx.y, ty.x, ty.y);
    __syncthreads();
    if (warp == 0) {
        const float4 w = lane < NT / 32 ? sw[lane] : make_float4(0.f, 0.f, 0.f, 0.f);
        tx = make_float2(w.x, w.y);
        ty = make_float2(w.z, w.w);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            tx = df_add(tx, make_float2(__shfl_down_sync(kFull, tx.x, o), __shfl_down_sync(kFull, tx.y, o)));
            if (NC == 2) ty = df_add(ty, make_float2(__shfl_down_sync(kFull, ty.x, o), __shfl_down_sync(kFull, ty.y, o)));
        }
    }
    return make_double2(df_to(tx), NC == 2 ? df_to(ty) : 0.0);   // valid in thread 0
}

// Returns true in every thread of the block that is the last of its scene to finish.  Callers
// write the block's partials from thread 0 just before; the last block reads only those partials,
// so only thread 0 fences (its partial write before its ticket).  A fence in every thread would
// make each wait for its own data stores to become visible device-wide.
template <int BS>
__device__ bool last_block_of_scene(const Dev& d, int s, const Scene& sc) {
    __shared__ int am_last;
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned nblk = unsigned((sc.slot_end - sc.slot_begin) / BS);
        const unsigned t = atomicAdd(reinterpret_cast<unsigned*>(&d.solve[s].blocks_done), 1u);
        am_last = (t == nblk - 1u);
        if (am_last) d.solve[s].blocks_done = 0;
    }
    __syncthreads();
    return am_last != 0;
}

// Called by thread 0 of the block that decided a scene, after the decision: a scene still active
// counts itself, and the last scene to decide takes the count (resetting it for the next pass)
// and sets the loop condition.  (Counting the active flags of every scene there instead was a
// serial chain of one load per scene, 256 a pass for the batched workload.)
__device__ void finish_scene_decision(const Dev& d, const Params& p, unsigned long long cond, int use_cond,
                                      int still_active) {
    if (p.nscenes == 1) {   // the only scene is the last to decide; kernel boundaries order the rest
        d.ctr->nactive = still_active;
        if (use_cond) cudaGraphSetConditional(cond, still_active ? 1u : 0u);
        return;
    }
    if (still_active) atomicAdd(&d.ctr->nactive_next, 1);
    __threadfence();
    const unsigned t = atomicAdd(&d.ctr->scenes_done, 1u);
    const int nact = *reinterpret_cast<volatile int*>(&d.ctr->nactive);
    if (t == unsigned(nact) - 1u) {
        __threadfence();
        const int cnt = atomicExch(&d.ctr->nactive_next, 0);
        d.ctr->nactive = cnt;
        d.ctr->scenes_done = 0;
        if (use_cond) cudaGraphSetConditional(cond, cnt > 0 ? 1u : 0u);
    }
}

// Run by one thread in the last kernel of a loop body: counts the bodies of this solve and ends
// the loop (flag bit 2) if it ran past its limit, whatever the per-scene decisions said.
__device__ void loop_guard(const Dev& d, unsigned long long cond, int limit) {
    const int passes = atomicAdd(&d.ctr->passes, 1) + 1;
    if (passes >= limit) {
        atomicOr(&d.ctr->flags, 4);
        cudaGraphSetConditional(cond, 0u);
    }
}

// Pair distance d and 1/d from d^2.  The fast form takes rsqrtf (MUFU, about 2 ulp) and
// d = d^2 / sqrt(d^2); the exact form correctly rounded sqrt and division (0.5 ulp each), for the
// passes whose sums are small differences (the density deviation and the density change rate).
#ifndef MPSG_EXACT_DIST_DENS
#define MPSG_EXACT_DIST_DENS 1
#endif
#ifndef MPSG_EXACT_DIST_PA
#define MPSG_EXACT_DIST_PA 0
#endif
template <int EXACT>
__device__ __forceinline__ void pair_dist(float d2, float& dist, float& invd) {
    if (EXACT) {
        dist = sqrtf(d2);
        invd = d2 > 0.0f ? 1.0f / dist : 0.0f;
    } else {
        invd = safe_rsqrt(d2);
        dist = d2 * invd;
    }
}
// Density sums of the density pass as float-float pairs (ff_VW): the deviation rho/rho0 - 1, which
// the stiffness reads, to about 1e-8 instead of the 2e-7 of FP32 kernel values and distances.
#ifndef MPSG_DENSITY_FF
#define MPSG_DENSITY_FF 1
#endif
// Compensated (Kahan) sums of the density change rate in pressure pass A: delta is a sum of terms
// of both signs whose result is small against them, and the stiffness is delta against rho/rho0 - 1.
#ifndef MPSG_DELTA_KAHAN
#define MPSG_DELTA_KAHAN 1
#endif

// ------------------------------------------------------------------ sort / reorder
__global__ void k_keys(Dev d, Params p) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= p.slots) return;
    const Scene& sc = d.scenes[d.chunk_scene[slot / kChunk]];
    if (slot >= sc.slot_begin + sc.n) return;
    const float4 x = d.pos_in[slot];
    if (!(isfinite(x.x) && isfinite(x.y) && isfinite(x.z))) atomicOr(&d.ctr->flags, 2);
    const int cx = cell_coord(x.x, sc.ox, sc.inv_cell, sc.nx);
    const int cy = cell_coord(x.y, sc.oy, sc.inv_cell, sc.ny);
    const int cz = cell_coord(x.z, sc.oz, sc.inv_cell, sc.nz);
    const int k = sc.coff + (slot - sc.slot_begin);
    d.keys[k] = cell_key(sc, cx, cy, cz);
    d.vals[k] = unsigned(slot);
}

__global__ void k_reorder(Dev d, Params p, int n_real) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_real) return;
    const unsigned long long key = d.keys[k];
    const unsigned src = d.vals[k];
    int lo = 0, hi = p.nscenes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (d.scenes[mid].coff <= k) lo = mid; else hi = mid - 1;
    }
    const Scene& sc = d.scenes[lo];
    const unsigned dst = unsigned(sc.slot_begin + (k - sc.coff));
    d.pos[dst] = d.pos_in[src];
    d.vel[dst] = d.vel_in[src];
    d.ids[dst] = d.ids_in[src];
    d.slot_key[dst] = key;
    if (k == 0 || d.keys[k - 1] != key) d.ftable[key].x = dst;
    if (k == n_real - 1 || d.keys[k + 1] != key) d.ftable[key].y = dst + 1u;
}

// Fluid cell lookup; stale entries of cells emptied since an earlier step fail the key check.
// Runs test(x[j], j) for j in [b, e) in order, loading kScan candidates before testing them.
constexpr int kScan = 4;
template <class Test>
__device__ __forceinline__ void scan_range(const float4* __restrict__ x, unsigned b, unsigned e, Test test) {
    unsigned j = b;
    for (; j + kScan <= e; j += kScan) {
        float4 v[kScan];
#pragma unroll
        for (int u = 0; u < kScan; ++u) v[u] = x[j + u];
#pragma unroll
        for (int u = 0; u < kScan; ++u) test(v[u], j + u);
    }
    for (; j < e; ++j) test(x[j], j);
}

__device__ __forceinline__ bool fluid_cell(const Dev& d, int slots, unsigned long long key, uint2& e) {
    e = d.ftable[key];
    return e.x < e.y && e.x < unsigned(slots) && d.slot_key[e.x] == key;
}

// ------------------------------------------------------------------ neighbour lists
// The 27 neighbour cells of a cell in ascending key order, for the four positions of the cell in
// its 2 x 2 column (case = (cy & 1) | (cz & 1) << 1); entry = (dx + 1) | (dy + 1) << 2 | (dz + 1) << 4.
// Keys order by column, then x, then row within the column.
static_assert(kBrick == 2, "kKeyOrder is written for columns of 2 x 2 rows");
__constant__ unsigned char kKeyOrder[4][27] = {
    {0, 1, 2, 4, 8, 5, 9, 6, 10, 16, 32, 17, 33, 18, 34, 20, 24, 36, 40, 21, 25, 37, 41, 22, 26, 38, 42},
    {0, 4, 1, 5, 2, 6, 8, 9, 10, 16, 20, 32, 36, 17, 21, 33, 37, 18, 22, 34, 38, 24, 40, 25, 41, 26, 42},
    {0, 16, 1, 17, 2, 18, 4, 8, 20, 24, 5, 9, 21, 25, 6, 10, 22, 26, 32, 33, 34, 36, 40, 37, 41, 38, 42},
    {0, 4, 16, 20, 1, 5, 17, 21, 2, 6, 18, 22, 8, 24, 9, 25, 10, 26, 32, 36, 33, 37, 34, 38, 40, 41, 42},
};

template <int BS>
__global__ void MPSG_BOUNDS_BUILD(BS) k_build_nbrs(Dev d, Params p) {
    const int i = blockIdx.x * BS + threadIdx.x;
    const Scene& sc = d.scenes[block_scene(d, BS)];
    __shared__ unsigned long long s_pf, s_pb;
    if (threadIdx.x == 0) { s_pf = 0; s_pb = 0; }
    __syncthreads();
    unsigned nf = 0, nb = 0;
    if (i < sc.slot_begin + sc.n) {
        const float4 xi = d.pos[i];
        const int cx = cell_coord(xi.x, sc.ox, sc.inv_cell, sc.nx);
        const int cy = cell_coord(xi.y, sc.oy, sc.inv_cell, sc.ny);
        const int cz = cell_coord(xi.z, sc.oz, sc.inv_cell, sc.nz);
        const int x0 = max(cx - 1, 0), x1 = min(cx + 1, sc.nx - 1);
        const size_t stride = size_t(p.slots);
        bool over = false;
        // candidates cell by cell in (dz, dy, x) order, loaded kScan at a time (the loads do not
        // depend on the tests, so a batch is in flight together)
        auto fluid_test = [&](const float4& xj, unsigned j) {
            if (j == unsigned(i)) return;
            const float d2 = dist2(__fsub_rn(xi.x, xj.x), __fsub_rn(xi.y, xj.y), __fsub_rn(xi.z, xj.z));
            const float hij = __fmul_rn(0.5f, __fadd_rn(xi.w, xj.w));
            if (d2 < __fmul_rn(hij, hij)) {
                if (nf < unsigned(p.cap_f)) d.nbr_f[size_t(nf) * stride + size_t(i)] = j; else over = true;
                nf++;
            }
        };
        auto bnd_test = [&](const float4& xj, unsigned j) {
            const float d2 = dist2(__fsub_rn(xi.x, xj.x), __fsub_rn(xi.y, xj.y), __fsub_rn(xi.z, xj.z));
            const float hij = __fmul_rn(0.5f, __fadd_rn(xi.w, xj.w));
            if (d2 < __fmul_rn(hij, hij)) {
                if (nb < unsigned(p.cap_b)) d.nbr_b[size_t(nb) * stride + size_t(i)] = j; else over = true;
                nb++;
            }
        };
#if MPSG_KEY_ORDER
        // the 27 cells in ascending key order, so that every list is sorted by slot: the order
        // depends only on the cell's row within its 2 x 2 column (kKeyOrder[case])
        const int kc = (cy & 1) | ((cz & 1) << 1);
#pragma unroll 1
        for (int t = 0; t < 27; ++t) {
            const int code = kKeyOrder[kc][t];
            const int x = cx + (code & 3) - 1, y = cy + ((code >> 2) & 3) - 1, z = cz + (code >> 4) - 1;
            if (x < 0 || x >= sc.nx || y < 0 || y >= sc.ny || z < 0 || z >= sc.nz) continue;
            const unsigned long long key = cell_key(sc, x, y, z);
            uint2 e;
            if (fluid_cell(d, p.slots, key, e)) scan_range(d.pos, e.x, e.y, fluid_test);
            const uint2 eb = d.btable[key];
            if (eb.x < eb.y) scan_range(d.bpos, eb.x, eb.y, bnd_test);
        }
#else
        for (int dz = -1; dz <= 1; ++dz) {
            const int z = cz + dz;
            if (z < 0 || z >= sc.nz) continue;
            for (int dy = -1; dy <= 1; ++dy) {
                const int y = cy + dy;
                if (y < 0 || y >= sc.ny) continue;
                for (int x = x0; x <= x1; ++x) {
                    const unsigned long long key = cell_key(sc, x, y, z);
                    uint2 e;
                    if (fluid_cell(d, p.slots, key, e)) scan_range(d.pos, e.x, e.y, fluid_test);
                    const uint2 eb = d.btable[key];
                    if (eb.x < eb.y) scan_range(d.bpos, eb.x, eb.y, bnd_test);
                }
            }
        }
#endif
        if (over) atomicOr(&d.ctr->flags, 1);
        nf = min(nf, unsigned(p.cap_f));
        nb = min(nb, unsigned(p.cap_b));
        atomicAdd(&s_pf, (unsigned long long)nf);
        atomicAdd(&s_pb, (unsigned long long)nb);
    }
    d.cnt[i] = nf | (nb << 16);
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicAdd(&d.ctr->fluid_pairs, s_pf);
        atomicAdd(&d.ctr->boundary_pairs, s_pb);
    }
}

// ------------------------------------------------------------------ boundary volume
// V_b = 1 / (prev + W(0) + sum_k W(|x_b - x_k|)) over boundary neighbours (Akinci,
// MPSSPHBaseUtil.cuh:10-86), with the sums and the reciprocal in float-float pairs: the volume is
// stored as bvol + bvol_lo, which the density deviation reads.
__global__ void k_bvolume(Dev d, Params p, int nb, int accumulate) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    int lo = 0, hi = p.nscenes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (d.scenes[mid].bbegin <= b) lo = mid; else hi = mid - 1;
    }
    const Scene& sc = d.scenes[lo];
    const float4 xi = d.bpos[b];
    const ff invh = ff_recip(xi.w);
    const FFScale scl = ff_scales(invh, ff{1.0f, 0.0f}, p.cubic);
    const int cx = cell_coord(xi.x, sc.ox, sc.inv_cell, sc.nx);
    const int cy = cell_coord(xi.y, sc.oy, sc.inv_cell, sc.ny);
    const int cz = cell_coord(xi.z, sc.oz, sc.inv_cell, sc.nz);
    ff sum = ff_VW(xi, xi, invh, scl, p.cubic);
    for (int z = max(cz - 1, 0); z <= min(cz + 1, sc.nz - 1); ++z)
        for (int y = max(cy - 1, 0); y <= min(cy + 1, sc.ny - 1); ++y)
            for (int x = max(cx - 1, 0); x <= min(cx + 1, sc.nx - 1); ++x) {
                const uint2 e = d.btable[cell_key(sc, x, y, z)];
                for (unsigned j = e.x; j < e.y; ++j) {
                    if (j == unsigned(b)) continue;
                    const float4 xj = d.bpos[j];
                    const float dx = __fsub_rn(xi.x, xj.x), dy = __fsub_rn(xi.y, xj.y), dz = __fsub_rn(xi.z, xj.z);
                    const float d2 = dist2(dx, dy, dz);
                    const float hij = __fmul_rn(0.5f, __fadd_rn(xi.w, xj.w));
                    if (d2 < __fmul_rn(hij, hij)) sum = ff_add(sum, ff_VW(xi, xj, invh, scl, p.cubic));
                }
            }
    if (accumulate) sum = ff_add(sum, ff{d.bvol[b], d.bvol_lo[b]});
    // 1 / sum as a pair: r = 1 / hi, then the residual (1 - sum r) r
    const float r = 1.0f / sum.hi;
    const float e = __fsub_rn(__fmaf_rn(-sum.hi, r, 1.0f), __fmul_rn(sum.lo, r));
    const ff v = ff_fast_two_sum(r, __fmul_rn(e, r));
    d.bvol[b] = v.hi;
    d.bvol_lo[b] = v.lo;
}

// ------------------------------------------------------------------ density + alpha + gravity
// What one launch of k_density_alpha computes: the step fuses all four (W_ALL); the drop-in API
// of the reference's functions (ComputeDensityFinal, DensityColorTest, ComputeDFSPHFactorFinal,
// UpdateVelocity after ApplyGravity) runs them one at a time with the same arithmetic, so the
// results are the same bits.  `parts` selects the neighbour sets of the sums (1 fluid, 2 boundary).
constexpr int W_DENSITY = 1, W_COLOR = 2, W_ALPHA = 4, W_GRAVITY = 8, W_ALL = 15;
template <int BS, int WHAT>
__global__ void MPSG_BOUNDS_DENS(BS) k_density_alpha(Dev d, Params p, int parts) {
    const int i = blockIdx.x * BS + threadIdx.x;
    const Scene& sc = d.scenes[block_scene(d, BS)];
    if (i >= sc.slot_begin + sc.n) return;
    constexpr bool kSums = (WHAT & (W_DENSITY | W_ALPHA)) != 0;
    float rho = 0.0f;
    if (kSums) {
        const size_t stride = size_t(p.slots);
        const float4 xi = d.pos[i];
        const float invh = 1.0f / xi.w;
        const unsigned c = d.cnt[i];
        const int nf = (parts & 1) ? int(c & 0xffffu) : 0, nb = (parts & 2) ? int(c >> 16) : 0;
        Kahan rf, gx, gy, gz, sq;
#if MPSG_DENSITY_FF
        // the density sums as float-float pairs (the deviation rho/rho0 - 1 is a small difference)
        const ff invh2 = ff_recip(xi.w);
        const FFScale scf = ff_scales(invh2, ff{p.V, p.V_lo}, p.cubic);   // fluid terms
        const FFScale scb = ff_scales(invh2, ff{1.0f, 0.0f}, p.cubic);    // boundary terms (times V_b)
        ff sf{0.0f, 0.0f}, sb{0.0f, 0.0f};
        if ((WHAT & W_DENSITY) && (parts & 1)) sf = ff_VW(xi, xi, invh2, scf, p.cubic);
#else
        if (parts & 1) rf.add(p.V * kW(0.0f, invh, p.cubic));
#endif
        visit_batched<MPSG_B_DENS, NoStream, float4, MPSG_PF_DENS>(d.nbr_f, stride, i, nf, [&](int) { return NoStream{}; }, [&](unsigned j, int) { return d.pos[j]; },
                              [&](const float4& xj, NoStream, int) {
            const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const float d2 = dx * dx + dy * dy + dz * dz;
            float dist, invd;
            pair_dist<MPSG_EXACT_DIST_DENS>(d2, dist, invd);
#if MPSG_DENSITY_FF
            if (WHAT & W_DENSITY) sf = ff_add(sf, ff_VW(xi, xj, invh2, scf, p.cubic));
#else
            if (WHAT & W_DENSITY) rf.add(p.V * kW(dist, invh, p.cubic));
#endif
            if (WHAT & W_ALPHA) {
                const float g = p.V * kG(dist, invd, invh, p.cubic);
                const float ax = g * dx, ay = g * dy, az = g * dz;
                gx.add(ax); gy.add(ay); gz.add(az);
                sq.add(ax * ax + ay * ay + az * az);
            }
        });
        Kahan rb;
        visit_batched<MPSG_B_DENS, NoStream, XB, MPSG_PF_DENS>(d.nbr_b, stride, i, nb, [&](int) { return NoStream{}; },
                              [&](unsigned j, int) {
                                  float4 x = d.bpos[j];
                                  x.w = d.bvol[j];
                                  return XB{x, (WHAT & W_DENSITY) ? d.bvol_lo[j] : 0.0f};
                              },
                              [&](const XB& xb, NoStream, int) {
            const float4 xj = xb.x;
            const float vb = xj.w;
            const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const float d2 = dx * dx + dy * dy + dz * dz;
            float dist, invd;
            pair_dist<MPSG_EXACT_DIST_DENS>(d2, dist, invd);
#if MPSG_DENSITY_FF
            if (WHAT & W_DENSITY) sb = ff_add(sb, ff_mul(ff_VW(xi, xj, invh2, scb, p.cubic), ff{vb, xb.lo}));
#else
            if (WHAT & W_DENSITY) rb.add(vb * kW(dist, invh, p.cubic));
#endif
            if (WHAT & W_ALPHA) {
                const float g = vb * kG(dist, invd, invh, p.cubic);
                gx.add(g * dx); gy.add(g * dy); gz.add(g * dz);
            }
        });
        if (WHAT & W_DENSITY) {
#if MPSG_DENSITY_FF
            const ff tot = ff_add(sf, sb);
            rho = ff_val(tot) * p.rho0;
            d.rho[i] = rho;
            d.rdev[i] = ff_val(ff_add(tot, ff{-1.0f, 0.0f}));
#else
            rho = (rf.s + rb.s) * p.rho0;
            d.rho[i] = rho;
            // rho / rho0 - 1 without the rounding of rho itself: rf.s - 1 is exact (Sterbenz), and
            // the Kahan sums carry their lost low parts in c (true sum = s - c)
            d.rdev[i] = __fsub_rn(__fadd_rn(__fsub_rn(rf.s, 1.0f), rb.s), __fadd_rn(rf.c, rb.c));
#endif
        }
        if (WHAT & W_ALPHA) {
            // alpha denominator in FP64: |sum grad|^2 + sum |grad|^2, clamp at 1e-20
            // (MPSSPHDFSPHUtil.cuh:127-137)
            const double sx = gx.s, sy = gy.s, sz = gz.s;
            const double f = double(sq.s) + (sx * sx + sy * sy + sz * sz);
            d.alpha[i] = f > 1.0e-20 ? float(1.0 / f) : 0.0f;
        }
    }
    if (WHAT & W_COLOR) {
        if (!(WHAT & W_DENSITY)) rho = d.rho[i];
        const float ratio = rho * p.inv_rho0;
        float4 col;
        col.x = fminf(fmaxf(ratio - 1.0f, 0.0f), 1.0f);
        col.y = fminf(fmaxf(ratio < 1.0f ? ratio : 1.0f - (ratio - 1.0f), 0.0f), 1.0f);
        col.z = fminf(fmaxf(1.0f - ratio, 0.0f), 1.0f);
        col.w = 1.0f;
        d.color[i] = col;
    }
    if (WHAT & W_GRAVITY) {
        float4 v = d.vel[i];
        if (v.w > 1.0e-10f) { v.x += p.dt * p.gx; v.y += p.dt * p.gy; v.z += p.dt * p.gz; }
        d.vel[i] = v;
    }
}

// ------------------------------------------------------------------ pressure solves
__global__ void k_solver_init(Dev d, Params p) {
    __shared__ int cnt;
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    for (int s = threadIdx.x; s < p.nscenes; s += blockDim.x) {
        SceneSolve& S = d.solve[s];
        S.active = d.scenes[s].n > 0 ? 1 : 0;
        S.do_update = 0;
        S.iter = 1;
        S.blocks_done = 0;
        S.err = 0.0;
        S.rr = 0.0;
        S.cg_alpha = 0.0;
        S.cg_beta = 0.0;
        if (S.active) atomicAdd(&cnt, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        d.ctr->nactive = cnt;
        d.ctr->nactive_next = 0;
        d.ctr->scenes_done = 0;
        d.ctr->passes = 0;
    }
}

__global__ void k_set_cond(Dev d, unsigned long long cond) {
    cudaGraphSetConditional(cond, d.ctr->nactive > 0 ? 1u : 0u);
}

// Pass A: density change rate delta, stiffness kappa, mean-error reduction and loop decision.
// mode 0: divergence-free, kappa = min(dt delta, rho/rho0 + dt delta - 0.8);
// mode 1: constant density, kappa = rho/rho0 + dt delta - 1 (MPSSPHDFSPHUtil.cuh:259-340).
template <int BS>
__global__ void MPSG_BOUNDS_PA(BS) k_pressure_A(Dev d, Params p, int mode, unsigned long long cond, int use_cond) {
    const int i = blockIdx.x * BS + threadIdx.x;
    // the slot's own data loads before the scene and solver-state lookups (the grid covers exactly
    // the allocated slots; padding slots have no neighbours)
    const float4 xi = d.pos[i];
    const float4 vi = d.vel[i];
    const unsigned c = d.cnt[i];
    const int s = block_scene(d, BS);
    if (use_cond != 2 && !d.solve[s].active) return;   // use_cond 2: profiling form (no decision follows)
    const Scene& sc = d.scenes[s];
    float err = 0.0f;
    if (i < sc.slot_begin + sc.n) {
        const size_t stride = size_t(p.slots);
        const float invh = 1.0f / xi.w;
        const int nf = int(c & 0xffffu), nb = int(c >> 16);
#if MPSG_DELTA_KAHAN
        Kahan df, db;
#define MPSG_DELTA_ADD(acc, v) acc.add(v)
#define MPSG_DELTA_VAL(acc) __fsub_rn(acc.s, acc.c)
#else
        float df = 0.0f, db = 0.0f;
#define MPSG_DELTA_ADD(acc, v) acc += (v)
#define MPSG_DELTA_VAL(acc) acc
#endif
        visit_batched<MPSG_B_PA, NoStream, XV, MPSG_PF_PA>(d.nbr_f, stride, i, nf, [&](int) { return NoStream{}; },
                          [&](unsigned j, int) { return XV{d.pos[j], d.vel[j]}; },
                          [&](const XV& t, NoStream, int) {
            const float4 xj = t.x, vj = t.v;
            const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const float d2 = dx * dx + dy * dy + dz * dz;
            float dist, invd;
            pair_dist<MPSG_EXACT_DIST_PA>(d2, dist, invd);
            const float g = kG(dist, invd, invh, p.cubic);
            MPSG_DELTA_ADD(df, g * (dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z)));
        });
        visit_batched<MPSG_B_PA, NoStream, float4, MPSG_PF_PA>(d.nbr_b, stride, i, nb, [&](int) { return NoStream{}; },
                              [&](unsigned j, int) { float4 x = d.bpos[j]; x.w = d.bvol[j]; return x; },
                              [&](const float4& xj, NoStream, int) {
            const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const float d2 = dx * dx + dy * dy + dz * dz;
            float dist, invd;
            pair_dist<MPSG_EXACT_DIST_PA>(d2, dist, invd);
            const float g = kG(dist, invd, invh, p.cubic);
            MPSG_DELTA_ADD(db, xj.w * g * (dx * vi.x + dy * vi.y + dz * vi.z));
        });
        const float delta = p.V * MPSG_DELTA_VAL(df) + MPSG_DELTA_VAL(db);
#undef MPSG_DELTA_ADD
#undef MPSG_DELTA_VAL
        // rho/rho0 + dt delta - 0.8 (DF) and rho/rho0 + dt delta - 1 (CD) from the density deviation
        const float rd = d.rdev[i];
        const float ka = delta * p.dt;
        const float kb = (rd + p.dt * delta) + 0.2f;
        float kap = mode == 0 ? fminf(ka, kb) : rd + p.dt * delta;
        unsigned char code = 0;   // 0 clamped, 1 the dt*delta branch of DF, 2 the density branch
        if (kap > 0.0f) {
            err = kap;
            code = (mode == 0 && ka <= kb) ? 1 : 2;
            kap *= d.alpha[i] * (p.inv_dt * p.inv_dt);
        } else {
            kap = 0.0f;
        }
        d.kappa[i] = kap;
        d.xk[i] = make_float4(xi.x, xi.y, xi.z, kap);   // one 16-byte gather a pair in pass B
        d.delta[i] = delta;
        if (d.tape_code) d.tape_code[i] = code;
    }
    warp_acc_put<1>(d, p, s, use_cond == 2, err, 0.0f);
}

// Loop decision of a DF/CD pass (MPSSPHDFSPHUtil.cu:404-433), one warp per scene after
// k_pressure_A: the scene's error sum from its accumulator, the mean error, the break rule, the
// iteration counter; the last scene to decide sets the loop condition.  Deciding in the pass's
// own last block cost every block a fence and a ticket and left the GPU idle during the last
// block's sum (about 17 us of a 1M CG operator pass); here the pass kernel's warps only add their
// sums.  A stopped scene's do_update is cleared here: a
// scene that reached its cap stopped with its last update still to run, and the passes after it
// in the same loop body must not repeat that update.
__global__ void __launch_bounds__(kAccDecideThreads) k_pressure_decide(Dev d, Params p, int mode, int bs,
                                                                    unsigned long long cond, int use_cond) {
    const int s = blockIdx.x;
    SceneSolve& S = d.solve[s];
    if (!S.active) {
        if (threadIdx.x == 0) S.do_update = 0;
        return;
    }
    const Scene& sc = d.scenes[s];
    (void)bs;
    const double tot = acc_take(d, s, 0);
    if (threadIdx.x == 0) {
        const double mean = tot / double(sc.n);
        const int l = S.iter;
        const double tol = mode == 0 ? p.df_tol_d : p.cd_tol_d;
        const int minl = mode == 0 ? p.min_iter_df : p.min_iter_cd;
        const int cap = p.fixed_iters > 0 ? p.fixed_iters : p.max_iter;
        const bool stop = p.fixed_iters > 0 ? false : (mean < tol && l > minl);
        S.err = mean;
        if (stop) {
            S.active = 0;
            S.do_update = 0;
        } else {
            S.do_update = 1;
            S.iter = l + 1;
            if (l + 1 > cap) S.active = 0;
        }
        finish_scene_decision(d, p, cond, use_cond, S.active);
    }
}

// Pass B: pressure force and velocity update, v += dt * F (ApplyDFSPH* + Final + UpdateVelocity).
template <int BS>
__global__ void MPSG_BOUNDS_PB(BS) k_pressure_B(Dev d, Params p, int profile, unsigned long long cond, int use_cond, int limit) {
    if (use_cond == 1 && blockIdx.x == 0 && threadIdx.x == 0) loop_guard(d, cond, limit);
    const int i = blockIdx.x * BS + threadIdx.x;
    // own data before the scene and solver-state lookups, as in k_pressure_A
    const float4 xi = d.pos[i];
    const float ki = d.kappa[i];
    const unsigned c = d.cnt[i];
    const int s = block_scene(d, BS);
    if (!profile && !d.solve[s].do_update) return;
    const Scene& sc = d.scenes[s];
    if (i >= sc.slot_begin + sc.n) return;
    const size_t stride = size_t(p.slots);
    const float invh = 1.0f / xi.w;
    const int nf = int(c & 0xffffu), nb = int(c >> 16);
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    visit_batched<MPSG_B_PB, NoStream, float4, MPSG_PF_PB>(d.nbr_f, stride, i, nf, [&](int) { return NoStream{}; },
                          [&](unsigned j, int) { return d.xk[j]; },
                          [&](const float4& xj, NoStream, int) {
        const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        const float invd = safe_rsqrt(d2);
        const float g = (ki + xj.w) * kG(d2 * invd, invd, invh, p.cubic);
        fx -= g * dx; fy -= g * dy; fz -= g * dz;
    });
    fx *= 0.5f * p.V; fy *= 0.5f * p.V; fz *= 0.5f * p.V;
    if (ki != 0.0f) {
        float bx = 0.0f, by = 0.0f, bz = 0.0f;
        visit_batched<MPSG_B_PB, NoStream, float4, MPSG_PF_PB>(d.nbr_b, stride, i, nb, [&](int) { return NoStream{}; },
                              [&](unsigned j, int) { float4 x = d.bpos[j]; x.w = d.bvol[j]; return x; },
                              [&](const float4& xj, NoStream, int) {
            const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
            const float d2 = dx * dx + dy * dy + dz * dz;
            const float invd = safe_rsqrt(d2);
            const float g = xj.w * kG(d2 * invd, invd, invh, p.cubic);
            bx -= g * dx; by -= g * dy; bz -= g * dz;
        });
        const float h = 0.5f * ki;
        fx += h * bx; fy += h * by; fz += h * bz;
    }
    float4 v = d.vel[i];
    if (v.w > 1.0e-10f) { v.x += p.dt * fx; v.y += p.dt * fy; v.z += p.dt * fz; }
    d.vel[i] = v;
}

// Records the loop counter and error of solve `which` (0 DF, 1 CG, 2 CD) per scene.
// Also accumulates the loop counters and the number of loop bodies run (max over scenes).
__global__ void k_solver_finish(Dev d, Params p, int which) {
    __shared__ unsigned long long sum;
    __shared__ int runs;
    if (threadIdx.x == 0) { sum = 0; runs = 0; }
    __syncthreads();
    const int cap = p.fixed_iters > 0 ? p.fixed_iters : (which == 1 ? p.cg_max_iter : p.max_iter);
    for (int s = threadIdx.x; s < p.nscenes; s += blockDim.x) {
        const int it = d.solve[s].iter;
        d.scene_iters[3 * s + which] = it;
        d.scene_err[3 * s + which] = d.solve[s].err;
        if (d.scenes[s].n > 0) {
            atomicAdd(&sum, (unsigned long long)it);
            atomicMax(&runs, min(it, cap));
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        d.ctr->iters_total[which] += sum;
        d.ctr->runs_total[which] += (unsigned long long)runs;
        // launched passes: the loop guard's count in graph runs; host-driven loops launch one
        // pass per iteration and do not count
        const int launched = d.ctr->passes > 0 ? d.ctr->passes : runs;
        d.ctr->passes_total[which] += (unsigned long long)launched;
    }
}

// ------------------------------------------------------------------ viscosity + surface tension
template <int BS>
__global__ void __launch_bounds__(BS) k_st_factor(Dev d, Params p) {
    const int i = blockIdx.x * BS + threadIdx.x;
    const Scene& sc = d.scenes[block_scene(d, BS)];
    if (i >= sc.slot_begin + sc.n) return;
    const size_t stride = size_t(p.slots);
    const float4 xi = d.pos[i];
    const float4 vi = d.vel[i];
    const float invh = 1.0f / xi.w;
    const int nf = int(d.cnt[i] & 0xffffu);
    float acc = 0.0f;
    visit_batched<MPSG_B_SETUP, NoStream, XV, MPSG_PF_SETUP>(d.nbr_f, stride, i, nf, [&](int) { return NoStream{}; },
                      [&](unsigned j, int) { return XV{d.pos[j], d.vel[j]}; },
                      [&](const XV& t, NoStream, int) {
        const float4 xj = t.x, vj = t.v;
        const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        const float invd = safe_rsqrt(d2);
        const float g = kG(d2 * invd, invd, invh, p.cubic);
        acc += vj.w * g * (dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z));
    });
    d.aux[i] = make_float2(d.rho[i], acc);
}

// b_i = v_i + dt sigma / m_i sum_j -mbar_ij g_ij x_ij; x0 = v (MPSSPHNonPressureUtil.cuh:467-521).
// The operator's per-pair coefficients depend only on positions, the pre-solve velocities, rho
// and the ST factor, all fixed during the CG solve, so they are computed here once per solve:
//   c_ij  = dt sigma / m_i * mbar_ij g_ij + XSPH / dt * m_j / rho_j W_ij     (ST + XSPH, :577-582)
//   cv_ij = 10 rho0 mu / rho_i * (m_i + m_j) / 2 / rho_j / (d^2 + 0.01 h_i^2) * G_ij / (d + eps)
//                                                                           (viscosity, :628-633)
template <int BS>
__global__ void MPSG_BOUNDS_SETUP(BS) k_cg_b(Dev d, Params p) {
    const int i = blockIdx.x * BS + threadIdx.x;
    const Scene& sc = d.scenes[block_scene(d, BS)];
    if (i >= sc.slot_begin + sc.n) return;
    const size_t stride = size_t(p.slots);
    const float4 xi = d.pos[i];
    const float4 vi = d.vel[i];
    const float2 ai = d.aux[i];
    const float invh = 1.0f / xi.w;
    const float eps_h2 = 0.01f * xi.w * xi.w;
    const float st_scale = p.dt * p.sigma / vi.w;
    const float xs_scale = p.xsph * p.inv_dt;
    const float vs = 10.0f * p.rho0 * p.visc / ai.x;
    const int nf = int(d.cnt[i] & 0xffffu);
    float bx = 0.0f, by = 0.0f, bz = 0.0f;
    float csum = 0.0f, sxx = 0.0f, syy = 0.0f, szz = 0.0f, sxy = 0.0f, sxz = 0.0f, syz = 0.0f;  // Jacobi block sums
    float ax = 0.0f, ay = 0.0f, az = 0.0f;   // sum of the operator's pair terms applied to x0 = v
    visit_batched<MPSG_B_SETUP, NoStream, XVA, MPSG_PF_SETUP>(d.nbr_f, stride, i, nf, [&](int) { return NoStream{}; },
                       [&](unsigned j, int) { return XVA{d.pos[j], d.vel[j], d.aux[j]}; },
                       [&](const XVA& t, NoStream, int k) {
        const float4 xj = t.x, vj = t.v;
        const float2 aj = t.a;
        const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        const float invd = safe_rsqrt(d2);
        const float dist = d2 * invd;
        const float invD = 2.0f / (ai.x + aj.x);
        const float stw = kSTW(dist, invh);
        const float stg = kSTG(dist, invd, invh);
        const float vdot = stg * (dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z));
        const float gij = (stw + p.dt * (vdot - (ai.y + aj.y) * invD * 0.5f * stw)) * invD;
        const float mbar = 0.5f * (vi.w + vj.w);
        const float c = mbar * gij;
        bx -= c * dx; by -= c * dy; bz -= c * dz;
        const float w = kW(dist, invh, p.cubic);
        const float G = kG(dist, invd, invh, p.cubic);
        const float inv_rj = 1.0f / aj.x;
        float2 cf;
        cf.x = st_scale * c + xs_scale * (vj.w * inv_rj) * w;
        cf.y = vs * mbar * inv_rj / (d2 + eps_h2) * G / (dist + kFltEps);
        d.cg_coef[size_t(k) * stride + size_t(i)] = cf;
        csum += cf.x;
        sxx += cf.y * dx * dx; syy += cf.y * dy * dy; szz += cf.y * dz * dz;
        sxy += cf.y * dx * dy; sxz += cf.y * dx * dz; syz += cf.y * dy * dz;
        // apply_A's pair term on x0 = v with these coefficients (the CG's A x0, factor 0)
        const float px = vi.x - vj.x, py = vi.y - vj.y, pz = vi.z - vj.z;
        const float tt = cf.y * (px * dx + py * dy + pz * dz);
        ax += cf.x * px - tt * dx;
        ay += cf.x * py - tt * dy;
        az += cf.x * pz - tt * dz;
    });
    const float4 b = make_float4(vi.x + st_scale * bx, vi.y + st_scale * by, vi.z + st_scale * bz, 0.0f);
    d.cg_b[i] = b;
    d.cg_x[i] = make_float4(vi.x, vi.y, vi.z, 0.0f);
    if (p.visc_solver == 0) {
        // r0 = b - A x0 with factor 0 (MPSSolver.cuh:24-28); p0 = r0 (three-pass form) or p = s = 0
        const float4 r = make_float4(b.x - (vi.x + p.dt * ax), b.y - (vi.y + p.dt * ay), b.z - (vi.z + p.dt * az), 0.0f);
        d.cg_r[i] = r;
        if (p.cg_form == 0) {
            d.cg_p[i] = r;
        } else {
            d.cg_p[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            d.cg_s[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    if (p.visc_solver == 1) {
        // 3x3 diagonal block of A_0 + f I, (1 + f + dt sum c) I - dt sum cv x x^T, inverted by
        // cofactors; a block with det <= 1e-30 (or not finite) is replaced by (1 + f) I and flagged
        const float f1 = 1.0f + p.cg_factor;
        const float dg = f1 + p.dt * csum;
        const float axx = dg - p.dt * sxx, ayy = dg - p.dt * syy, azz = dg - p.dt * szz;
        const float axy = -p.dt * sxy, axz = -p.dt * sxz, ayz = -p.dt * syz;
        const float c00 = ayy * azz - ayz * ayz, c01 = axz * ayz - axy * azz, c02 = axy * ayz - axz * ayy;
        const float det = axx * c00 + axy * c01 + axz * c02;
        if (det > 1.0e-30f && isfinite(det)) {
            const float id = 1.0f / det;
            d.jac_d[i] = make_float4(c00 * id, (axx * azz - axz * axz) * id, (axx * ayy - axy * axy) * id, c01 * id);
            d.jac_d2[i] = make_float4(c02 * id, (axy * axz - axx * ayz) * id, 0.0f, 0.0f);
        } else {
            const float id = 1.0f / f1;
            d.jac_d[i] = make_float4(id, id, id, 0.0f);
            d.jac_d2[i] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
        }
    }
}

// (A q)_i = q_i (1 + f) + dt [sum_j c_ij (q_i - q_j) - sum_j cv_ij ((q_i - q_j).x_ij) x_ij]
// with the coefficients of k_cg_b (MPSSPHNonPressureUtil.cuh:523-648).
__device__ __forceinline__ float3 apply_A(const Dev& d, const Params& p, int i, const float4* q, float factor,
                                          float4 xi, float4 qi, unsigned cnt) {
    const size_t stride = size_t(p.slots);
    const int nf = int(cnt & 0xffffu);
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    visit_batched<MPSG_B_AP, float2, XQ, MPSG_PF_AP>(d.nbr_f, stride, i, nf,
                       [&](int k) { return ld_stream(d.cg_coef + size_t(k) * stride + size_t(i)); },
                       [&](unsigned j, int) { return XQ{d.pos[j], q[j]}; },
                       [&](const XQ& g, const float2& cf, int) {
        const float4 xj = g.x, qj = g.q;
        const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
        const float px = qi.x - qj.x, py = qi.y - qj.y, pz = qi.z - qj.z;
        const float t = cf.y * (px * dx + py * dy + pz * dz);
        sx += cf.x * px - t * dx;
        sy += cf.x * py - t * dy;
        sz += cf.x * pz - t * dz;
    });
    const float f1 = 1.0f + factor;
    return make_float3(qi.x * f1 + p.dt * sx, qi.y * f1 + p.dt * sy, qi.z * f1 + p.dt * sz);
}
__device__ __forceinline__ float3 apply_A(const Dev& d, const Params& p, int i, const float4* q, float factor) {
    return apply_A(d, p, i, q, factor, d.pos[i], q[i], d.cnt[i]);
}

// ---- neighbourhood tiles of the CG operator (mps_config.stage = 1)
// An operator block's pairs reach few distinct slots (1M dam break at rest: 514 on average for a
// 128-slot block's 3,600 pairs, each used about 7 times), while a warp's gather of them touches
// about 15 cache lines for 29 lanes.  k_build_tiles lists each block's distinct neighbour slots in
// ascending order (tile_j) and gives every pair its 16-bit rank in that list (nbr_t); the tiled
// operator loads the block's positions and directions into shared memory once per pass and
// gathers from there.  A block with more than kTilePerSlot records a slot keeps the global gathers
// (tile_n = -1).  Every loop is bounded, and a rank outside the tile is skipped and flagged (bit 3).
__host__ __device__ constexpr int pow2_at_least(int v) {
    int r = 1;
    while (r < v) r <<= 1;
    return r;
}
__host__ __device__ constexpr int log2_exact(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}
template <int BS>
__global__ void __launch_bounds__(BS) k_build_tiles(Dev d, Params p) {
    constexpr int TM = kTilePerSlot * BS;            // tile capacity
    constexpr int HS = pow2_at_least(2 * TM);         // open-addressing set of the block's slots
    constexpr int LH = log2_exact(HS);
    constexpr int PS = pow2_at_least(TM);             // sort width
    constexpr unsigned kEmpty = 0xffffffffu;
    __shared__ unsigned set[HS];
    __shared__ unsigned uniq[PS];
    __shared__ int s_cnt, s_over, s_k;
    const int blk = blockIdx.x;
    const int i = blk * BS + threadIdx.x;
    for (int t = threadIdx.x; t < HS; t += BS) set[t] = kEmpty;
    if (threadIdx.x == 0) {
        s_cnt = 0;
        s_over = 0;
        s_k = 0;
    }
    __syncthreads();
    const int s = block_scene(d, BS);
    const Scene& sc = d.scenes[s];
    const size_t stride = size_t(p.slots);
    const bool live = i < sc.slot_begin + sc.n;
    const int nf = live ? int(d.cnt[i] & 0xffffu) : 0;
    volatile int* over = &s_over;
    for (int k = 0; k < nf; ++k) {
        if (*over) break;   // the block keeps the global gathers: stop inserting
        const unsigned j = ld_stream(d.nbr_f + size_t(k) * stride + size_t(i));
        unsigned h = (j * 0x9E3779B1u) >> (32 - LH);
        bool placed = false;
        for (int probe = 0; probe < HS && !*over; ++probe) {
            const unsigned old = atomicCAS(&set[h], kEmpty, j);
            if (old == kEmpty) {
                if (atomicAdd(&s_cnt, 1) >= TM) *over = 1;
                placed = true;
                break;
            }
            if (old == j) {
                placed = true;
                break;
            }
            h = (h + 1u) & unsigned(HS - 1);
        }
        if (!placed) *over = 1;
    }
    __syncthreads();
    const int T = s_cnt;
    if (s_over || T > TM) {   // uniform: shared values after the barrier
        if (threadIdx.x == 0) {
            d.tile_n[blk] = -1;
            atomicAdd(&d.ctr->tile_blocks[1], 1ull);
        }
        return;
    }
    for (int t = threadIdx.x; t < HS; t += BS) {
        const unsigned v = set[t];
        if (v != kEmpty) {
            const int o = atomicAdd(&s_k, 1);
            if (o < PS) uniq[o] = v;
        }
    }
    __syncthreads();
    for (int t = T + int(threadIdx.x); t < PS; t += BS) uniq[t] = kEmpty;
    __syncthreads();
    // bitonic sort of uniq[0, PS), ascending
    for (int size = 2; size <= PS; size <<= 1) {
        for (int half = size >> 1; half > 0; half >>= 1) {
            for (int t = threadIdx.x; t < PS / 2; t += BS) {
                const int lo = 2 * half * (t / half) + (t % half), hi = lo + half;
                const bool up = (lo & size) == 0;
                const unsigned a = uniq[lo], b = uniq[hi];
                if ((a > b) == up) {
                    uniq[lo] = b;
                    uniq[hi] = a;
                }
            }
            __syncthreads();
        }
    }
    unsigned* tj = d.tile_j + size_t(blk) * TM;
    for (int t = threadIdx.x; t < T; t += BS) tj[t] = uniq[t];
    bool bad = false;
    for (int k = 0; k < nf; ++k) {
        const unsigned j = ld_stream(d.nbr_f + size_t(k) * stride + size_t(i));
        int lo = 0, hi = T;
        while (lo < hi) {   // at most log2(TM) + 1 rounds
            const int mid = (lo + hi) >> 1;
            if (uniq[mid] < j) lo = mid + 1;
            else hi = mid;
        }
        if (lo >= T || uniq[lo] != j) bad = true;
        d.nbr_t[size_t(k) * stride + size_t(i)] = static_cast<unsigned short>(lo < T ? lo : 0);
    }
    if (bad) atomicOr(&d.ctr->flags, 8);
    if (threadIdx.x == 0) {
        d.tile_n[blk] = T;
        atomicAdd(&d.ctr->tile_blocks[0], 1ull);
    }
}

// apply_A with the neighbours' positions and directions read from the block's tile (tx, tq of T
// records); the same pairs, order and arithmetic as apply_A.
__device__ __forceinline__ float3 apply_A_tile(const Dev& d, const Params& p, int i, const float4* tx,
                                               const float4* tq, int T, float factor, float4 xi, float4 qi,
                                               unsigned cnt) {
    constexpr int U = 4;   // stream loads in flight per thread
    const size_t stride = size_t(p.slots);
    const int nf = int(cnt & 0xffffu);
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    bool bad = false;
    for (int k = 0; k < nf; k += U) {
        unsigned r[U];
        float2 cf[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const bool in = k + u < nf;
            r[u] = in ? ld_stream(d.nbr_t + size_t(k + u) * stride + size_t(i)) : 0u;
            cf[u] = in ? ld_stream(d.cg_coef + size_t(k + u) * stride + size_t(i)) : make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (k + u < nf) {
                if (r[u] >= unsigned(T)) {
                    bad = true;
                } else {
                    const float4 xj = tx[r[u]], qj = tq[r[u]];
                    const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
                    const float px = qi.x - qj.x, py = qi.y - qj.y, pz = qi.z - qj.z;
                    const float t = cf[u].y * (px * dx + py * dy + pz * dz);
                    sx += cf[u].x * px - t * dx;
                    sy += cf[u].x * py - t * dy;
                    sz += cf[u].x * pz - t * dz;
                }
            }
        }
    }
    if (bad) atomicOr(&d.ctr->flags, 8);
    const float f1 = 1.0f + factor;
    return make_float3(qi.x * f1 + p.dt * sx, qi.y * f1 + p.dt * sy, qi.z * f1 + p.dt * sz);
}

// Two-pass CG form (cg_form 1): the Chronopoulos-Gear arrangement (the same iterates as the
// reference's CGSolver in exact arithmetic): per iteration one operator pass w = A r with the
// dots r.r and r.w, then one vector pass p = r + beta p, s = w + beta s (s = A p),
// x += alpha p, r -= alpha s, where beta = (r.r) / (r.r)_old and
// alpha = (r.r) / (r.w - beta (r.r) / alpha_old) (first iteration: beta = 0,
// alpha = (r.r) / (r.w)); p and s start at zero.  Both forms keep the reference's stop test
// r.r < tol and loop counter (MPSSolver.cuh:33-60); r0 = b - A x0 comes from k_cg_b.
template <int BS>
__global__ void __launch_bounds__(BS) k_cg_ap(Dev d, Params p, unsigned long long cond, int use_cond) {
    const int s = block_scene(d, BS);
    if (use_cond != 2 && !d.solve[s].active) return;   // use_cond 2: profiling form (no decision follows)
    const Scene& sc = d.scenes[s];
    const int i = blockIdx.x * BS + threadIdx.x;
    float rr = 0.0f, rw = 0.0f;
    if (i < sc.slot_begin + sc.n) {
        const float3 w = apply_A(d, p, i, d.cg_r, p.cg_factor);
        d.cg_ap[i] = make_float4(w.x, w.y, w.z, 0.0f);
        const float4 r = d.cg_r[i];
        rr = r.x * r.x + r.y * r.y + r.z * r.z;
        rw = r.x * w.x + r.y * w.y + r.z * w.z;
    }
    warp_acc_put<2>(d, p, s, use_cond == 2, rr, rw);
}

// The two-pass CG's decision after k_cg_ap (one warp per scene, from the accumulator): r.r and r.w,
// the stop test, beta = (r.r) / (r.r)_old and alpha = (r.r) / (r.w - beta (r.r) / alpha_old)
// (first iteration: beta = 0, alpha = (r.r) / (r.w)).
__global__ void __launch_bounds__(kAccDecideThreads) k_cg_decide2(Dev d, Params p, int bs, unsigned long long cond,
                                                               int use_cond) {
    pdl_release();
    const int s = blockIdx.x;
    SceneSolve& S = d.solve[s];
    if (!S.active) {
        if (threadIdx.x == 0) S.do_update = 0;
        return;
    }
    (void)bs;
    const double2 t = make_double2(acc_take(d, s, 0), acc_take(d, s, 1));
    const double trr = t.x, trw = t.y;
    if (threadIdx.x == 0) {
        const int l = S.iter;
        const int cap = p.fixed_iters > 0 ? p.fixed_iters : p.cg_max_iter;
        const bool stop = p.fixed_iters > 0 ? false : (trr < p.cg_tol_d);
        S.err = trr;
        if (stop) {
            S.active = 0;
            S.do_update = 0;
        } else {
            const double beta = l == 1 ? 0.0 : trr / S.rr;
            const double denom = l == 1 ? trw : trw - beta * trr / S.cg_alpha;
            S.cg_beta = beta;
            S.cg_alpha = trr / denom;
            S.do_update = 1;
            S.iter = l + 1;
            if (l + 1 > cap) S.active = 0;
        }
        S.rr = trr;
        finish_scene_decision(d, p, cond, use_cond, S.active);
    }
}

// p = r + beta p, s = w + beta s, x += alpha p, r -= alpha s (MPSSolver.cuh:49-60,
// MPSCGKernel.cuh:196-207), in one pass with no reduction; the loop guard of the WHILE body.
template <int BS>
__global__ void __launch_bounds__(BS) k_cg_update(Dev d, Params p, unsigned long long cond, int use_cond, int limit) {
    if (use_cond == 1 && blockIdx.x == 0 && threadIdx.x == 0) loop_guard(d, cond, limit);
    const int i = blockIdx.x * BS + threadIdx.x;
    // the vectors load before the wait for k_cg_decide2 (the grid covers exactly the allocated slots)
    const float4 r = d.cg_r[i];
    const float4 w = d.cg_ap[i];
    float4 q = d.cg_p[i];
    float4 sv = d.cg_s[i];
    float4 x = d.cg_x[i];
    pdl_wait();
    const int s = block_scene(d, BS);
    if (!d.solve[s].do_update) return;
    const Scene& sc = d.scenes[s];
    if (i >= sc.slot_begin + sc.n) return;
    const float a = float(d.solve[s].cg_alpha);
    const float b = float(d.solve[s].cg_beta);
    q.x = r.x + b * q.x; q.y = r.y + b * q.y; q.z = r.z + b * q.z;
    sv.x = w.x + b * sv.x; sv.y = w.y + b * sv.y; sv.z = w.z + b * sv.z;
    x.x += a * q.x; x.y += a * q.y; x.z += a * q.z;
    d.cg_p[i] = q;
    d.cg_s[i] = sv;
    d.cg_x[i] = x;
    d.cg_r[i] = make_float4(r.x - a * sv.x, r.y - a * sv.y, r.z - a * sv.z, 0.0f);
}

// ---- three-pass form (the reference's CGSolver arrangement, MPSSolver.cuh:33-60)
// A p, dots r.r and p.Ap, the stop test and alpha = r.r / p.Ap.

// The end of the operator pass for slot i (live: a fluid slot of the scene): stores Ap and the
// block's partial sums of r.r and p.Ap.
template <int BS>
__device__ __forceinline__ void ap3_finish(const Dev& d, int i, bool live, float4 q, float3 a, float2* sh) {
    float rr = 0.0f, pap = 0.0f;
    if (live) {
        d.cg_ap[i] = make_float4(a.x, a.y, a.z, 0.0f);
        const float4 r = d.cg_r[i];
        rr = r.x * r.x + r.y * r.y + r.z * r.z;
        pap = q.x * a.x + q.y * a.y + q.z * a.z;
    }
    block_partial2<BS>(d, rr, pap, sh);
}

template <int BS>
__global__ void MPSG_BOUNDS_AP(BS) k_cg_ap3(Dev d, Params p, unsigned long long cond, int use_cond) {
    __shared__ float2 sh2[BS / 32];
    const int i = blockIdx.x * BS + threadIdx.x;
    const int s = block_scene(d, BS);
    if (use_cond != 2 && !d.solve[s].active) return;   // use_cond 2: profiling form (no decision follows)
    const Scene& sc = d.scenes[s];
    const bool live = i < sc.slot_begin + sc.n;
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
    float3 a = make_float3(0.f, 0.f, 0.f);
    if (live) {
        // (the own-slot loads stay after the check: passes after the stop skip them; issuing them
        // first gained nothing in this kernel)
        const float4 xi = d.pos[i];
        q = d.cg_p[i];
        const unsigned c = d.cnt[i];
        a = apply_A(d, p, i, d.cg_p, p.cg_factor, xi, q, c);
    }
    ap3_finish<BS>(d, i, live, q, a, sh2);
}

// k_cg_ap3 with the neighbours' positions and directions gathered from the block's tile
// (mps_config.stage = 1; a block without a tile uses the global gathers).
template <int BS>
__global__ void __launch_bounds__(BS) k_cg_ap3_tile(Dev d, Params p, unsigned long long cond, int use_cond) {
    constexpr int TM = kTilePerSlot * BS;
    extern __shared__ float4 tile[];   // TM positions, then TM directions
    __shared__ float2 sh2[BS / 32];
    const int i = blockIdx.x * BS + threadIdx.x;
    const int s = block_scene(d, BS);
    if (use_cond != 2 && !d.solve[s].active) return;   // use_cond 2: profiling form (no decision follows)
    const Scene& sc = d.scenes[s];
    const int T = d.tile_n[blockIdx.x];
    const bool tiled = T >= 0 && T <= TM;
    if (tiled) {
        const unsigned* tj = d.tile_j + size_t(blockIdx.x) * TM;
        for (int t = threadIdx.x; t < T; t += BS) {
            const unsigned j = tj[t];
            if (j < unsigned(p.slots)) {
                tile[t] = d.pos[j];
                tile[TM + t] = d.cg_p[j];
            } else {
                atomicOr(&d.ctr->flags, 8);
            }
        }
    }
    __syncthreads();
    const bool live = i < sc.slot_begin + sc.n;
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
    float3 a = make_float3(0.f, 0.f, 0.f);
    if (live) {
        const float4 xi = d.pos[i];
        q = d.cg_p[i];
        const unsigned c = d.cnt[i];
        a = tiled ? apply_A_tile(d, p, i, tile, tile + TM, T, p.cg_factor, xi, q, c)
                  : apply_A(d, p, i, d.cg_p, p.cg_factor, xi, q, c);
    }
    ap3_finish<BS>(d, i, live, q, a, sh2);
}

// The three-pass CG's decision after k_cg_ap3 (one 1024-thread block per scene): r.r and p.Ap
// from the operator pass's per-block partials, the stop test r.r < tol, alpha = r.r / p.Ap, the
// loop counter (MPSSolver.cuh:33-60).
__global__ void __launch_bounds__(kDecideThreads) k_cg_decide3(Dev d, Params p, int bs, unsigned long long cond,
                                                               int use_cond) {
    __shared__ double2 sh[32];
    pdl_release();
    const int s = blockIdx.x;
    SceneSolve& S = d.solve[s];
    if (!S.active) {
        if (threadIdx.x == 0) S.do_update = 0;
        return;
    }
    const Scene& sc = d.scenes[s];
    const double2 t = scene_partials<kDecideThreads, 2>(d, sc, bs, sh);
    if (threadIdx.x == 0) {
        const double trr = t.x, tpap = t.y;
        const int l = S.iter;
        const int cap = p.fixed_iters > 0 ? p.fixed_iters : p.cg_max_iter;
        const bool stop = p.fixed_iters > 0 ? false : (trr < p.cg_tol_d);
        S.err = trr;
        S.rr = trr;
        if (stop) {
            S.active = 0;
            S.do_update = 0;
        } else {
            S.do_update = 1;
            S.cg_alpha = trr / tpap;
            S.iter = l + 1;
            if (l + 1 > cap) S.active = 0;
        }
        finish_scene_decision(d, p, cond, use_cond, S.active);
    }
}

// The three-pass CG's vector passes cover kVecSlots slots per block with NT threads (kVecSlots / NT
// slots a thread, their loads issued before any store), which keeps more independent loads in
// flight per thread than one slot a thread.  Blocks keep the 256-slot scene chunks, so a block
// belongs to one scene.
constexpr int kVecSlots = 256;
#ifndef MPSG_VEC_PDL
#define MPSG_VEC_PDL 1
#endif
#ifndef MPSG_VEC_NT
#define MPSG_VEC_NT 128
#endif


// r -= alpha Ap, beta = (r.r)_new / (r.r)_old.  (x += alpha p is left to k_cg_dir3, which reads p
// anyway: the same arithmetic, 16 fewer bytes a slot per iteration.)
template <int NT>
__global__ void __launch_bounds__(NT) k_cg_update3(Dev d, Params p, int profile) {
    constexpr int U = kVecSlots / NT;
    // the grid covers exactly the allocated slots, so the data loads go out before the scene and
    // solver-state lookups (padding slots are loaded and not used)
    const int i0 = blockIdx.x * kVecSlots + threadIdx.x;
    float4 r[U], ap[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int i = i0 + u * NT;
        r[u] = d.cg_r[i];
        ap[u] = d.cg_ap[i];
    }
    pdl_wait();   // alpha and do_update come from k_cg_decide3
    const int s = block_scene(d, kVecSlots);
    if (!profile && !d.solve[s].do_update) return;
    const Scene& sc = d.scenes[s];
    const int end = sc.slot_begin + sc.n;
    const float a = float(d.solve[s].cg_alpha);
    float rr = 0.0f;
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int i = i0 + u * NT;
        if (i < end) {
            r[u].x -= a * ap[u].x; r[u].y -= a * ap[u].y; r[u].z -= a * ap[u].z;
            d.cg_r[i] = r[u];
            rr += r[u].x * r[u].x + r[u].y * r[u].y + r[u].z * r[u].z;
        }
    }
    warp_acc_put<1>(d, p, s, profile != 0, rr, 0.0f);
}

// beta = (r.r)_new / (r.r)_old from k_cg_update3's sums (the scene's accumulator), one warp per
// scene that is updating.
__global__ void __launch_bounds__(kAccDecideThreads) k_cg_beta3(Dev d) {
    pdl_release();
    const int s = blockIdx.x;
    SceneSolve& S = d.solve[s];
    if (!S.do_update) return;
    const double t = acc_take(d, s, 0);
    if (threadIdx.x == 0) S.cg_beta = t / S.rr;
}

// x += alpha p with the old direction, then p = r + beta p (MPSCGKernel.cuh:196-207); the loop
// guard of the WHILE body.
template <int NT>
__global__ void __launch_bounds__(NT) k_cg_dir3(Dev d, Params p, unsigned long long cond, int use_cond, int limit) {
    constexpr int U = kVecSlots / NT;
    if (use_cond == 1 && blockIdx.x == 0 && threadIdx.x == 0) loop_guard(d, cond, limit);
    const int i0 = blockIdx.x * kVecSlots + threadIdx.x;
    float4 x[U], r[U], q[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {   // loads before the lookups, as in k_cg_update3
        x[u] = d.cg_x[i0 + u * NT];
        r[u] = d.cg_r[i0 + u * NT];
        q[u] = d.cg_p[i0 + u * NT];
    }
    pdl_wait();   // beta comes from k_cg_beta3
    const int s = block_scene(d, kVecSlots);
    if (use_cond != 2 && !d.solve[s].do_update) return;   // use_cond 2: profiling form
    const Scene& sc = d.scenes[s];
    const int end = sc.slot_begin + sc.n;
    const float a = float(d.solve[s].cg_alpha);
    const float b = float(d.solve[s].cg_beta);
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int i = i0 + u * NT;
        if (i < end) {
            x[u].x += a * q[u].x; x[u].y += a * q[u].y; x[u].z += a * q[u].z;
            d.cg_x[i] = x[u];
            q[u].x = r[u].x + b * q[u].x; q[u].y = r[u].y + b * q[u].y; q[u].z = r[u].z + b * q[u].z;
            d.cg_p[i] = q[u];
        }
    }
}

// One block-Jacobi sweep: r = b + f x0 - (A_0 + f I) q, q' = q + D^-1 r (D: the particle's 3x3
// diagonal block), with r.r of the input iterate
// reduced per scene for the stop test (r.r < cg_tol, as the CG's, MPSSolver.cuh:33-41).  The
// iterates alternate between cg_x (even) and cg_p (odd) by the scene's loop counter, so that one
// launch per sweep suffices; src/dst given = explicit buffers (adjoint recording).
template <int BS>
__global__ void __launch_bounds__(BS) k_jacobi(Dev d, Params p, unsigned long long cond, int use_cond, int limit,
                                               const float4* src, float4* dst) {
    __shared__ double sh[32];
    __shared__ double2 sh2[BS / 32];
    if (use_cond == 1 && blockIdx.x == 0 && threadIdx.x == 0) loop_guard(d, cond, limit);
    const int s = block_scene(d, BS);
    if (use_cond != 2 && !d.solve[s].active) {
        if (threadIdx.x == 0 && int(blockIdx.x) * BS == d.scenes[s].slot_begin) d.solve[s].do_update = 0;   // as in k_pressure_A
        return;
    }
    const Scene& sc = d.scenes[s];
    const int l = d.solve[s].iter;
    const float4* q = src ? src : (((l - 1) & 1) ? d.cg_p : d.cg_x);
    float4* qn = dst ? dst : ((l & 1) ? d.cg_p : d.cg_x);
    const int i = blockIdx.x * BS + threadIdx.x;
    float rr = 0.0f;
    if (i < sc.slot_begin + sc.n) {
        const float3 a = apply_A(d, p, i, q, p.cg_factor);
        const float4 b = d.cg_b[i];
        const float4 v0 = d.vel[i];
        const float4 qi = q[i];
        const float4 m = d.jac_d[i];
        const float4 m2 = d.jac_d2[i];
        const float f = p.cg_factor;
        const float rx = b.x + f * v0.x - a.x, ry = b.y + f * v0.y - a.y, rz = b.z + f * v0.z - a.z;
        rr = rx * rx + ry * ry + rz * rz;
        qn[i] = make_float4(qi.x + (m.x * rx + m.w * ry + m2.x * rz), qi.y + (m.w * rx + m.y * ry + m2.y * rz),
                            qi.z + (m2.x * rx + m2.y * ry + m.z * rz), 0.0f);
    }
    const double2 bs2 = block_sum2_f<BS>(rr, 0.0f, sh2);
    if (threadIdx.x == 0) put_partial(d, blockIdx.x, bs2.x, 0.0);
    if (use_cond == 2 || !last_block_of_scene<BS>(d, s, sc)) return;
    const double trr = scene_partial_sum<BS, BS>(d, sc, 0, sh);
    if (threadIdx.x == 0) {
        SceneSolve& S = d.solve[s];
        const int cap = p.fixed_iters > 0 ? p.fixed_iters : p.cg_max_iter;
        const bool stop = p.fixed_iters > 0 ? false : (trr < p.cg_tol_d);
        S.err = trr;
        S.rr = trr;
        if (stop) {
            S.active = 0;
            S.do_update = 0;
        } else {
            S.do_update = 1;
            S.iter = l + 1;
            if (l + 1 > cap) S.active = 0;
        }
        finish_scene_decision(d, p, cond, use_cond, S.active);
    }
}

// v = the Jacobi result: the iterate of loop counter l - 1 (buffer (l - 1) & 1), or src.
__global__ void k_jacobi_finish(Dev d, Params p, const float4* src) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    const int s = d.chunk_scene[i / kChunk];
    const Scene& sc = d.scenes[s];
    if (i >= sc.slot_begin + sc.n) return;
    const float4* q = src ? src : (((d.solve[s].iter - 1) & 1) ? d.cg_p : d.cg_x);
    const float4 x = q[i];
    float4 v = d.vel[i];
    v.x = x.x; v.y = x.y; v.z = x.z;
    d.vel[i] = v;
}

// v = x (copy predictVel back, MPSSPHNonPressureUtil.cu:177-180).
__global__ void k_cg_finish(Dev d, Params p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    const Scene& sc = d.scenes[d.chunk_scene[i / kChunk]];
    if (i >= sc.slot_begin + sc.n) return;
    const float4 x = d.cg_x[i];
    float4 v = d.vel[i];
    v.x = x.x; v.y = x.y; v.z = x.z;
    d.vel[i] = v;
}

// ------------------------------------------------------------------ advection
// code: 0 unchanged, 1 reflected (-0.4 v), 2 stopped (|v| < 1e-4).
__device__ __forceinline__ float collide(float pos, float lo, float hi, float v, unsigned& code) {
    if ((pos < lo && v < 0.0f) || (pos > hi && v > 0.0f)) {
        if (fabsf(v) < 1.0e-4f) { code = 2u; return 0.0f; }
        code = 1u;
        return -v * 0.4f;
    }
    code = 0u;
    return v;
}

// BoundaryCollision (WHAT bit 1: the velocity against the box) and UpdatePosition (bit 2:
// x += dt v), fused in the step, one at a time in the drop-in API (same arithmetic).
template <int WHAT>
__global__ void k_advect(Dev d, Params p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    const Scene& sc = d.scenes[d.chunk_scene[i / kChunk]];
    if (i >= sc.slot_begin + sc.n) return;
    float4 x = d.pos[i];
    float4 v = d.vel[i];
    if (WHAT & 1) {
        unsigned cx, cy, cz;
        v.x = collide(x.x + v.x * p.dt, sc.bminx, sc.bmaxx, v.x, cx);
        v.y = collide(x.y + v.y * p.dt, sc.bminy, sc.bmaxy, v.y, cy);
        v.z = collide(x.z + v.z * p.dt, sc.bminz, sc.bmaxz, v.z, cz);
        d.vel[i] = v;
        if (d.tape_adv) d.tape_adv[i] = (unsigned char)(cx | (cy << 2) | (cz << 4));
    }
    if (WHAT & 2) {
        x.x += p.dt * v.x; x.y += p.dt * v.y; x.z += p.dt * v.z;
        d.pos[i] = x;
    }
}

// Loads a state given in particle-ID order (pos4.w = particle radius) into the slot layout.
__global__ void k_load_state(Dev d, Params p, const float4* __restrict__ pos4, const float4* __restrict__ vel4, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int lo = 0, hi = p.nscenes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (d.scenes[mid].coff <= k) lo = mid; else hi = mid - 1;
    }
    const Scene& sc = d.scenes[lo];
    const int slot = sc.slot_begin + (k - sc.coff);
    float4 x = pos4[k];
    x.w *= kHRatio;
    d.pos[slot] = x;
    d.vel[slot] = vel4[k];
    d.ids[slot] = unsigned(k);
}

// Stores the state in particle-ID order (pos4.w = particle radius).
__global__ void k_store_state(Dev d, Params p, float4* __restrict__ pos4, float4* __restrict__ vel4) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.slots) return;
    const Scene& sc = d.scenes[d.chunk_scene[i / kChunk]];
    if (i >= sc.slot_begin + sc.n) return;
    const unsigned id = d.ids[i];
    float4 x = d.pos[i];
    x.w *= (1.0f / kHRatio);
    if (pos4) pos4[id] = x;
    if (vel4) vel4[id] = d.vel[i];
}

int nblocks_for(int n, int bs) { return (n + bs - 1) / bs; }

}  // namespace

// ------------------------------------------------------------------ launchers
// Launch with the programmatic-serialisation attribute (see pdl_wait).
template <class... KArgs, class... Args>
void launch_after_decide(void (*k)(KArgs...), int grid, int block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(unsigned(grid));
    cfg.blockDim = dim3(unsigned(block));
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, args...);
}
#define MPSG_BS_SWITCH(bs, KERNEL, ...)                                                      \
    do {                                                                                     \
        if ((bs) == 128) KERNEL<128><<<p.slots / 128, 128, 0, s>>>(__VA_ARGS__);             \
        else if ((bs) == 64) KERNEL<64><<<p.slots / 64, 64, 0, s>>>(__VA_ARGS__);            \
        else KERNEL<256><<<p.slots / 256, 256, 0, s>>>(__VA_ARGS__);                         \
    } while (0)

void launch_keys(const Dev& d, const Params& p, cudaStream_t s) {
    k_keys<<<nblocks_for(p.slots, 256), 256, 0, s>>>(d, p);
}
void launch_reorder(const Dev& d, const Params& p, int n_real, cudaStream_t s) {
    if (n_real > 0) k_reorder<<<nblocks_for(n_real, 256), 256, 0, s>>>(d, p, n_real);
}
void launch_build_nbrs(const Dev& d, const Params& p, int bs, cudaStream_t s) {
    MPSG_BS_SWITCH(bs, k_build_nbrs, d, p);
    // neighbourhood tiles of the step's neighbour passes: built from the lists they index, so that
    // lists and tiles always change together
    if (p.stage == 1) MPSG_BS_SWITCH(bs, k_build_tiles, d, p);
}
void launch_bvolume(const Dev& d, const Params& p, int nb, int accumulate, cudaStream_t s) {
    if (nb > 0) k_bvolume<<<nblocks_for(nb, 256), 256, 0, s>>>(d, p, nb, accumulate);
}
#define MPSG_BS_SWITCH_W(bs, KERNEL, W, ...)                                                 \
    do {                                                                                     \
        if ((bs) == 128) KERNEL<128, W><<<p.slots / 128, 128, 0, s>>>(__VA_ARGS__);          \
        else if ((bs) == 64) KERNEL<64, W><<<p.slots / 64, 64, 0, s>>>(__VA_ARGS__);         \
        else KERNEL<256, W><<<p.slots / 256, 256, 0, s>>>(__VA_ARGS__);                      \
    } while (0)
void launch_density_alpha(const Dev& d, const Params& p, int bs, cudaStream_t s) {
    MPSG_BS_SWITCH_W(bs, k_density_alpha, W_ALL, d, p, 3);
}
int launch_density_part(const Dev& d, const Params& p, int bs, int what, int parts, cudaStream_t s) {
    switch (what) {
        case W_DENSITY: MPSG_BS_SWITCH_W(bs, k_density_alpha, W_DENSITY, d, p, parts); return 0;
        case W_COLOR: MPSG_BS_SWITCH_W(bs, k_density_alpha, W_COLOR, d, p, parts); return 0;
        case W_ALPHA: MPSG_BS_SWITCH_W(bs, k_density_alpha, W_ALPHA, d, p, parts); return 0;
        case W_GRAVITY: MPSG_BS_SWITCH_W(bs, k_density_alpha, W_GRAVITY, d, p, parts); return 0;
        default: return -1;
    }
}
void launch_solver_init(const Dev& d, const Params& p, cudaStream_t s) {
    k_solver_init<<<1, 256, 0, s>>>(d, p);
}
void launch_set_cond(const Dev& d, unsigned long long cond, cudaStream_t s) {
    k_set_cond<<<1, 1, 0, s>>>(d, cond);
}
void launch_pressure_A(const Dev& d, const Params& p, int mode, int bs, unsigned long long cond, int use_cond,
                       cudaStream_t s) {
    MPSG_BS_SWITCH(bs, k_pressure_A, d, p, mode, cond, use_cond);
    if (use_cond != 2) k_pressure_decide<<<p.nscenes, kAccDecideThreads, 0, s>>>(d, p, mode, bs, cond, use_cond);
}
void launch_pressure_B(const Dev& d, const Params& p, int bs, unsigned long long cond, int use_cond, int limit,
                       cudaStream_t s) {
    MPSG_BS_SWITCH(bs, k_pressure_B, d, p, 0, cond, use_cond, limit);
}
void launch_pressure_B_profile(const Dev& d, const Params& p, int bs, cudaStream_t s) {
    MPSG_BS_SWITCH(bs, k_pressure_B, d, p, 1, 0ull, 0, 0);
}
void launch_solver_finish(const Dev& d, const Params& p, int which, cudaStream_t s) {
    k_solver_finish<<<1, 256, 0, s>>>(d, p, which);
}
void launch_st_factor(const Dev& d, const Params& p, int bs, cudaStream_t s) {
    MPSG_BS_SWITCH(bs, k_st_factor, d, p);
}
void launch_cg_b(const Dev& d, const Params& p, int bs, cudaStream_t s) {
    MPSG_BS_SWITCH(bs, k_cg_b, d, p);
}
void launch_cg_ap(const Dev& d, const Params& p, int bs, unsigned long long cond, int use_cond, cudaStream_t s) {
    MPSG_BS_SWITCH(bs, k_cg_ap, d, p, cond, use_cond);
    if (use_cond != 2) k_cg_decide2<<<p.nscenes, kAccDecideThreads, 0, s>>>(d, p, bs, cond, use_cond);
}
// The CG's vector passes stream their arrays; they run with 256-thread blocks whatever the
// neighbour passes use (scenes are padded to 256 slots, so a block still belongs to one scene).
void launch_cg_update(const Dev& d, const Params& p, int bs, unsigned long long cond, int use_cond, int limit,
                      cudaStream_t s) {
    (void)bs;
    launch_after_decide(k_cg_update<256>, p.slots / 256, 256, s, d, p, cond, use_cond, limit);
}
// Preferred shared-memory carveout (percent) of the plain CG operator, which uses almost no shared
// memory: -1 leaves the driver's choice.
#ifndef MPSG_CG_CARVEOUT
#define MPSG_CG_CARVEOUT -1
#endif
void launch_cg_ap3(const Dev& d, const Params& p, int bs, unsigned long long cond, int use_cond, cudaStream_t s) {
#if MPSG_CG_CARVEOUT >= 0
    static bool carveout_set = false;
    if (!carveout_set) {
        cudaFuncSetAttribute(k_cg_ap3<64>, cudaFuncAttributePreferredSharedMemoryCarveout, MPSG_CG_CARVEOUT);
        cudaFuncSetAttribute(k_cg_ap3<128>, cudaFuncAttributePreferredSharedMemoryCarveout, MPSG_CG_CARVEOUT);
        cudaFuncSetAttribute(k_cg_ap3<256>, cudaFuncAttributePreferredSharedMemoryCarveout, MPSG_CG_CARVEOUT);
        carveout_set = true;
    }
#endif
    if (p.stage == 1) {
        const size_t sm = size_t(2 * kTilePerSlot) * size_t(bs) * sizeof(float4);   // 40 KB at most (256 slots)
        if (bs == 128) k_cg_ap3_tile<128><<<p.slots / 128, 128, sm, s>>>(d, p, cond, use_cond);
        else if (bs == 64) k_cg_ap3_tile<64><<<p.slots / 64, 64, sm, s>>>(d, p, cond, use_cond);
        else k_cg_ap3_tile<256><<<p.slots / 256, 256, sm, s>>>(d, p, cond, use_cond);
    } else {
        MPSG_BS_SWITCH(bs, k_cg_ap3, d, p, cond, use_cond);
    }
    if (use_cond != 2) k_cg_decide3<<<p.nscenes, kDecideThreads, 0, s>>>(d, p, bs, cond, use_cond);
}
void launch_cg_update3(const Dev& d, const Params& p, int bs, cudaStream_t s) {
    (void)bs;
#if MPSG_VEC_PDL
    launch_after_decide(k_cg_update3<MPSG_VEC_NT>, p.slots / kVecSlots, MPSG_VEC_NT, s, d, p, 0);
#else
    k_cg_update3<MPSG_VEC_NT><<<p.slots / kVecSlots, MPSG_VEC_NT, 0, s>>>(d, p, 0);
#endif
    k_cg_beta3<<<p.nscenes, kAccDecideThreads, 0, s>>>(d);
}
void launch_cg_vector_profile(const Dev& d, const Params& p, cudaStream_t s) {
    k_cg_update3<MPSG_VEC_NT><<<p.slots / kVecSlots, MPSG_VEC_NT, 0, s>>>(d, p, 1);
    k_cg_dir3<MPSG_VEC_NT><<<p.slots / kVecSlots, MPSG_VEC_NT, 0, s>>>(d, p, 0ull, 2, 0);
}
void launch_cg_dir3(const Dev& d, const Params& p, int bs, unsigned long long cond, int use_cond, int limit,
                    cudaStream_t s) {
    (void)bs;
#if MPSG_VEC_PDL
    launch_after_decide(k_cg_dir3<MPSG_VEC_NT>, p.slots / kVecSlots, MPSG_VEC_NT, s, d, p, cond, use_cond, limit);
#else
    k_cg_dir3<MPSG_VEC_NT><<<p.slots / kVecSlots, MPSG_VEC_NT, 0, s>>>(d, p, cond, use_cond, limit);
#endif
}
void launch_jacobi(const Dev& d, const Params& p, int bs, unsigned long long cond, int use_cond, int limit,
                   const float4* src, float4* dst, cudaStream_t s) {
    MPSG_BS_SWITCH(bs, k_jacobi, d, p, cond, use_cond, limit, src, dst);
}
void launch_jacobi_finish(const Dev& d, const Params& p, const float4* src, cudaStream_t s) {
    k_jacobi_finish<<<nblocks_for(p.slots, 256), 256, 0, s>>>(d, p, src);
}
void launch_cg_finish(const Dev& d, const Params& p, cudaStream_t s) {
    k_cg_finish<<<nblocks_for(p.slots, 256), 256, 0, s>>>(d, p);
}
void launch_load_state(const Dev& d, const Params& p, const float4* pos4, const float4* vel4, int n, cudaStream_t s) {
    if (n > 0) k_load_state<<<nblocks_for(n, 256), 256, 0, s>>>(d, p, pos4, vel4, n);
}
void launch_store_state(const Dev& d, const Params& p, float4* pos4, float4* vel4, cudaStream_t s) {
    k_store_state<<<nblocks_for(p.slots, 256), 256, 0, s>>>(d, p, pos4, vel4);
}
void launch_advect(const Dev& d, const Params& p, cudaStream_t s) {
    k_advect<3><<<nblocks_for(p.slots, 256), 256, 0, s>>>(d, p);
}
void launch_advect_part(const Dev& d, const Params& p, int what, cudaStream_t s) {
    if (what == 1) k_advect<1><<<nblocks_for(p.slots, 256), 256, 0, s>>>(d, p);
    else k_advect<2><<<nblocks_for(p.slots, 256), 256, 0, s>>>(d, p);
}

}  // namespace mpsg
