/*
 * FP64 CPU oracle for the DFSPH step -- TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, in plain C++ with FP64 arithmetic, the per-frame step of
 * moonsh5009/MPS_CUDA (`mps::System::OnUpdate`, src/MPS_System/MPSSystem.cpp:191-291)
 * and everything it calls.  It is the checker for the CUDA path in mps_cuda_gb300: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  The product
 * never links or calls it.
 *
 * Pinned by: golden vectors produced by the reference's own CUDA step rebuilt headless
 * (oracle/build_ref.sh -> oracle/_ref/) on the same inputs (tests/golden/).
 *
 * Two families of entry points:
 *  - orc_*      : a stateful replay of the reference step (reference hash scheme, CSR
 *                 neighbour lists in the reference's order, FP64 kernels, host-side solver
 *                 loops with the reference's break rules).
 *  - orc_new_*  : restatements of the NEW integer scheme of the CUDA path (64-bit cell keys,
 *                 stable sort, cell ranges, FP32 neighbour test) for bit-exact checks.
 */
#ifndef MPS_ORACLE_H
#define MPS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
    /* PhysicsParam (src/MPS_Object/MPSUniformDef.h:19-25) */
    double dt;
    double gravity[3];
    double bmin[3];
    double bmax[3];
    /* SPHMaterialParam (src/MPS_Object/MPSSPHMaterial.h:9-21) */
    double mat_radius;       /* support radius h of the material (SetRadius(4 r)) */
    double mat_mass;
    double mat_density;      /* rest density rho0 */
    double mat_volume;       /* particle volume V used by every fluid sum */
    double viscosity;
    double xsph;
    double surface_tension;
    /* Spatial hash of the reference (MPSSpatialHash.cu:18-42) */
    double hash_cell;        /* SetCeilSize */
    uint32_t hash_size[3];   /* SetHashSize, powers of two */
    /* Kernel switch: 0 = poly6/spiky (shipped), 1 = cubic spline (USE_CUBIC_KERNEL 1) */
    int32_t cubic;
    /* Solver rules (MPSSPHDFSPHUtil.cu:299-333, :405-419; MPSSolver.cuh:31-41) */
    double df_tol;           /* shipped 1e-3 */
    double cd_tol;           /* shipped 1e-4 */
    int32_t df_min_iter;     /* shipped: break only when l > 1 */
    int32_t cd_min_iter;     /* shipped: break only when l > 2 */
    int32_t max_iter;        /* shipped 100 */
    double cg_tol;           /* shipped 1e-2 (absolute r.r) */
    int32_t cg_max_iter;     /* shipped 100 */
    /* Quirks */
    int32_t volume_accumulate; /* 1: boundary volume not reset between frames (MPSSystem.cpp:237-238) */
    int32_t zsort;             /* 1: Morton re-sort when frame % 50 == 1 (MPSSystem.cpp:220-224) */
    int32_t threads;           /* OpenMP threads, 0 = default */
    int32_t fixed_iters;       /* > 0: DF, CD and CG run exactly this many iterations (no early exit) */
    int32_t visc_solver;       /* 0 CG (the reference's), 1 block-Jacobi sweeps on the same system */
} orc_params;

typedef struct orc_stats {
    int32_t df_iters, cg_iters, cd_iters;
    double df_err, cd_err, cg_rr;
    int64_t nei_ff, nei_fb, nei_bb;  /* total neighbour pairs of the three lists */
    int32_t frame;
} orc_stats;

typedef struct orc_sim orc_sim;

orc_sim* orc_create(const orc_params* p);
void orc_destroy(orc_sim* s);
/* arrays are AoS double [n][3] for vectors, double[n] for scalars; ids optional (NULL = 0..n-1) */
int orc_set_fluid(orc_sim* s, int64_t n, const double* pos, const double* vel,
                  const double* mass, const double* radius, const uint32_t* ids);
int orc_set_boundary(orc_sim* s, int64_t nb, const double* pos, const double* radius,
                     const double* volume /* may be NULL = zeros */);
void orc_set_frame(orc_sim* s, int32_t frame);

/* Phases of OnUpdate, in order. */
enum {
    ORC_ZSORT = 0,          /* MPSSystem.cpp:220-224 */
    ORC_NEIGHBORS = 1,      /* :226-235 */
    ORC_BVOLUME = 2,        /* :237-238 */
    ORC_DENSITY = 3,        /* :240-245 (density + colour) */
    ORC_ALPHA = 4,          /* :247-251 */
    ORC_GRAVITY = 5,        /* :253-255 */
    ORC_DF = 6,             /* :257-264 */
    ORC_VISCST = 7,         /* :266 */
    ORC_CD = 8,             /* :268-275 */
    ORC_ADVECT = 9          /* :277-278, frame++ */
};
int orc_phase(orc_sim* s, int32_t phase);
int orc_step(orc_sim* s, int32_t nsteps);
void orc_get_stats(const orc_sim* s, orc_stats* out);

/* Array access by name: "pos","vel","mass","radius","ids","density","alpha","pressure",
 * "delta","stfac","color"(float[4n]),"bpos","bradius","bvol","nei_ff_idx"(uint32 n+1),
 * "nei_fb_idx","nei_bb_idx"(nb+1),"nei_ff","nei_fb","nei_bb","force","gradsum","cg_b".
 * Returns element count (doubles/u32/floats) or -1. out may be NULL to query size. */
int64_t orc_get(const orc_sim* s, const char* name, void* out);
int orc_put(orc_sim* s, const char* name, const void* in, int64_t count);

/* ---------------- restatement of the NEW integer scheme (CUDA path) ---------------- */
typedef struct orc_grid {
    float origin[3];
    float cell;          /* cell size (>= max support radius) */
    float inv_cell;      /* 1.0f / cell, as computed in FP32 */
    int32_t dims[3];
    uint64_t key_base;   /* offset of this grid's cells in the global key space */
} orc_grid;

/* key = key_base + ((((cz/2)*ceil(ny/2) + cy/2)*nx + cx)*2 + cz%2)*2 + cy%2 with clamped FP32 cell
 * coordinates (columns of 2 x 2 rows along x). */
void orc_new_keys(int64_t n, const float* pos4, const orc_grid* g, uint64_t* keys);
/* Stable sort of (key, value) pairs by key (LSD semantics: ties keep input order). */
void orc_new_stable_sort(int64_t n, uint64_t* keys, uint32_t* vals);
/* For sorted keys: start/end of each occupied cell, written as (cell, start, end) triples. */
int64_t orc_new_cell_ranges(int64_t n, const uint64_t* sorted_keys, uint64_t* cells,
                            uint32_t* starts, uint32_t* ends);
/* FP32 neighbour counts of sorted points q against sorted points p on grid g:
 * d2 = fma(dz,dz,fma(dy,dy,dx*dx)) < (0.5f*(hi+hj))^2, self (same index, same set) excluded. */
void orc_new_nbr_counts(int64_t nq, const float* q4, int64_t np, const float* p4,
                        const uint64_t* p_sorted_keys, const orc_grid* g, int same_set,
                        uint32_t* counts);

#ifdef __cplusplus
}
#endif
#endif
