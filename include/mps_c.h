/*
 * mps_c.h -- C ABI of the GB300-native DFSPH step (libmps_gb300.so).
 *
 * Replaces the per-frame step of moonsh5009/MPS_CUDA: `mps::System::OnUpdate`
 * (src/MPS_System/MPSSystem.cpp:191-291) and the free functions it calls in
 * `mps::kernel::SPH::*` / `mps::kernel::Advect::*` (src/MPS_Computer/MPSSPHBaseUtil.h:9-38,
 * MPSSPHDFSPHUtil.h:9-87, MPSSPHNonPressureUtil.h:29-65, MPSAdvectUtil.h:12-20) plus the
 * neighbour search of `mps::SpatialHash` (src/MPS_Object/MPSSpatialHash.h:20-57).
 *
 * Conventions
 *  - Plain C types only; every call returns MPS_OK (0) or a negative MPS_E* code, and
 *    mps_last_error() returns a message for the calling thread's last failure.
 *  - "particle radius" r is what the reference stores per particle (pRadius); the support
 *    radius is h = 4 r (H_RATIO, src/MPS_Object/MPSDef.h:25-27).
 *  - Work is queued on the stream passed in (a cudaStream_t as void*, NULL = legacy default).
 *  - One handle is used from one host thread at a time.
 */
#ifndef MPS_C_H
#define MPS_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#define MPS_ABI_VERSION 1

enum mps_status {
    MPS_OK = 0,
    MPS_E_INVALID = -1,       /* bad argument or handle */
    MPS_E_CUDA = -2,          /* CUDA runtime error (message in mps_last_error) */
    MPS_E_NOMEM = -3,         /* device allocation failed */
    MPS_E_STATE = -4,         /* call out of order (e.g. step before set_fluid) */
    MPS_E_OVERFLOW = -5,      /* neighbour list capacity exceeded during the last step */
    MPS_E_NONFINITE = -6      /* NaN/Inf met in particle positions during the last step */
};

/* SPHMaterialParam (src/MPS_Object/MPSSPHMaterial.h:9-21). */
typedef struct mps_material {
    double radius;           /* support radius h of the material (reference: SetRadius(4 r)) */
    double mass;             /* particle mass (reference: density * volume) */
    double density;          /* rest density rho0 */
    double volume;           /* particle volume V used by the fluid sums */
    double viscosity;
    double xsph;
    double surface_tension;
} mps_material;

/* PhysicsParam (src/MPS_Object/MPSUniformDef.h:19-25). */
typedef struct mps_physics {
    double dt;
    double gravity[3];
    double min[3];           /* collision box (BoundaryCollision, MPSAdvectUtil.cuh:48-77) */
    double max[3];
} mps_physics;

enum mps_kernel_kind { MPS_KERNEL_POLY6_SPIKY = 0, MPS_KERNEL_CUBIC_SPLINE = 1 };

/* Solver rules.  Defaults (mps_default_config) reproduce the reference's literals:
 * MPSSPHDFSPHUtil.cu:333 (CD 1e-4, l > 2), :419 (DF 1e-3, l > 1), :299/:405 (<= 100
 * iterations), MPSSolver.cuh:31-41 (CG r.r < 1e-2, <= 100 iterations),
 * MPSSPHNonPressureUtil.cu:165-169 (operator factor 0 for A x0, 0.01 afterwards). */
typedef struct mps_config {
    int32_t kernel;              /* mps_kernel_kind */
    double df_tol;
    double cd_tol;
    int32_t df_min_iter;
    int32_t cd_min_iter;
    int32_t max_iter;
    double cg_tol;
    int32_t cg_max_iter;
    double cg_factor;
    int32_t fixed_iters;         /* > 0: DF, CD and CG each run exactly this many iterations */
    int32_t max_fluid_neighbors; /* list capacity per particle (overflow -> MPS_E_OVERFLOW); 0 = 96,
                                    above 65535 (16-bit counts) mps_create returns MPS_E_INVALID */
    int32_t max_boundary_neighbors;
    int32_t volume_accumulate;   /* 1: reproduce the un-reset boundary volume (MPSSystem.cpp:237-238) */
    int32_t use_graph;           /* 1: whole step as one CUDA graph with device-side loops */
    int32_t block_size;          /* threads per block of the neighbour-sum kernels (64..256) */
    int32_t stage;               /* 0 (default): the neighbour passes gather neighbour data from global
                                    memory; 1: the three-pass CG operator gathers from a shared-memory tile
                                    of each block's distinct neighbours, built with the neighbour lists
                                    (16-bit ranks: 2 bytes a neighbour slot and 20 bytes a particle more
                                    memory) */
    int32_t sort_digit_bits;     /* radix digit width of the cell sort (1..8) */
    int32_t visc_solver;         /* mps_visc_solver: implicit viscosity/surface-tension solve */
    int32_t cg_form;             /* mps_cg_form: arrangement of the CG iteration (same iterates) */
    int32_t cg_unroll;           /* CG iterations per body of the device-side loop (1..8, default 4): the
                                    iterations after the stop return at once, so more save loop
                                    evaluations and fewer save empty launches; results do not change */
} mps_config;

/* MPS_CG_THREE_PASS (default): the reference's arrangement (MPSSolver.cuh:33-60): A p with r.r
 * and p.Ap, then the r update with the new r.r, then x and the direction.  MPS_CG_TWO_PASS: the
 * Chronopoulos-Gear arrangement: A r with r.r and r.w, then one vector pass updating p, s = A p
 * (by recurrence), x and r.  Equal in exact arithmetic; in FP32 the
 * recurrence for s adds rounding: against the FP64 oracle from an identical state, single
 * particles' velocities then differ by up to ~1e-4 (max-norm) where the three-pass form stays
 * below ~3e-6 (RMS ~2e-7 for both). */
enum mps_cg_form { MPS_CG_THREE_PASS = 0, MPS_CG_TWO_PASS = 1 };

/* MPS_VISC_CG: the reference's CGSolver (MPSSolver.cuh:12-73).  MPS_VISC_JACOBI: block-Jacobi
 * sweeps on the same system, the alternative of the reference's legacy Jacobi viscosity
 * (MPSSPHNonPressureUtil.cuh:90-195, commented out there, which also inverts each particle's 3x3
 * block).  The CG's converged point satisfies (A_0 + f I) x = b + f x0 (f = cg_factor, x0 =
 * pre-solve velocity); Jacobi iterates x += D^-1 (b + f x0 - (A_0 + f I) x), D = the 3x3 diagonal
 * blocks of A_0 + f I, from x0, stopping when the residual's r.r < cg_tol (at most cg_max_iter
 * sweeps) or after fixed_iters sweeps. */
enum mps_visc_solver { MPS_VISC_CG = 0, MPS_VISC_JACOBI = 1 };

/* Per-step statistics, written by the device at the end of each step. */
typedef struct mps_stats {
    int32_t df_iters;        /* reference loop counter l at exit (MPSSPHDFSPHUtil.cu:404-433) */
    int32_t cg_iters;        /* CGSolver return value (MPSSolver.cuh:30-72) */
    int32_t cd_iters;
    int32_t flags;           /* bit0 neighbour overflow, bit1 non-finite position */
    double df_err;           /* last mean divergence error */
    double cd_err;           /* last mean density error */
    double cg_rr;            /* last r.r */
    int64_t fluid_pairs;     /* fluid-fluid neighbour pairs of the step */
    int64_t boundary_pairs;  /* fluid-boundary neighbour pairs of the step */
    int64_t steps;           /* steps taken since creation */
    int64_t iters_total[3];  /* DF, CG, CD loop counters summed over steps (and scenes) */
    int64_t runs_total[3];   /* DF, CG, CD solver passes that ran since creation (one per iteration) */
    int64_t passes_total[3]; /* DF, CG, CD solver passes launched since creation (>= runs_total: a
                              * graph loop body holds several CG passes; the ones after the stop
                              * return at once) */
    int64_t tile_blocks[2];  /* stage 1: blocks of the last neighbour build with a neighbourhood tile,
                              * and blocks whose neighbourhood exceeded the tile (global gathers) */
    int64_t sort_passes;     /* radix passes of the step's cell sort (significant key bits / digit) */
} mps_stats;

typedef struct mps_handle mps_handle;

const char* mps_last_error(void);
int mps_abi_version(void);
void mps_default_config(mps_config* cfg);
/* Reference defaults: SPHMaterial() then SetRadius(h) (MPSSPHMaterial.cpp:4-19). */
void mps_reference_material(double h, double density, mps_material* out);

/* Object lifetime: replaces SPHModel/ObstacleModel construction (MPSSystem.cpp:22-84). */
int mps_create(const mps_material* mat, const mps_physics* phys, const mps_config* cfg,
               int device, mps_handle** out);
int mps_destroy(mps_handle* h);
int mps_set_physics(mps_handle* h, const mps_physics* phys);
int mps_set_material(mps_handle* h, const mps_material* mat);

/* Fluid particles, host FP64 AoS as the reference stores them (REAL3 pos/vel, REAL mass,
 * REAL radius; MPSSystem.cpp:586-623).  ids may be NULL (0..n-1). */
int mps_set_fluid(mps_handle* h, int64_t n, const double* pos3, const double* vel3,
                  const double* mass, const double* radius, const uint32_t* ids);
/* Boundary particles: positions and particle radii; volume NULL = Akinci volume computed on
 * the device (ComputeBoundaryParticleVolumeSub/Final, MPSSPHBaseUtil.cu:9-53). */
int mps_set_boundary(mps_handle* h, int64_t nb, const double* pos3, const double* radius,
                     const double* volume);

/* Native FP32 layout: pos4 = (x, y, z, particle radius), vel4 = (vx, vy, vz, mass).
 * on_device != 0: pointers are device memory.  Order: as given (becomes particle IDs). */
int mps_set_fluid_f32(mps_handle* h, int64_t n, const float* pos4, const float* vel4,
                      int on_device, void* stream);
/* Reads the fluid back in ID order (particle k of mps_set_fluid* at index k). */
int mps_get_fluid_f32(mps_handle* h, float* pos4, float* vel4, int on_device, void* stream);
int mps_get_fluid(mps_handle* h, double* pos3, double* vel3);

/* One frame of System::OnUpdate (MPSSystem.cpp:191-291), nsteps times, queued on stream. */
int mps_step(mps_handle* h, int32_t nsteps, void* stream);
/* Host-buffer form: copies pos4/vel4 in, steps, copies them back (ID order). */
int mps_step_host(mps_handle* h, float* pos4, float* vel4, int32_t nsteps, void* stream);
int mps_get_stats(mps_handle* h, mps_stats* out, void* stream);

/* Fine-grained phases of the step, in OnUpdate order (for parity tests and tools). */
enum mps_phase {
    MPS_PHASE_SORT = 0,          /* UpdateHash / ZSort: keys, radix sort, reorder, cell ranges */
    MPS_PHASE_NEIGHBORS = 1,     /* BuildNeighorhood x3 (MPSSpatialHash.cu:142-218) */
    MPS_PHASE_BVOLUME = 2,       /* ComputeBoundaryParticleVolume* (MPSSystem.cpp:237-238) */
    MPS_PHASE_DENSITY_ALPHA = 3, /* density, colour, DFSPH factor, gravity (:240-255) */
    MPS_PHASE_DF = 4,            /* ComputeDFSPHDivergenceFree (:257-264) */
    MPS_PHASE_VISCST = 5,        /* ApplyImplicitViscosityNSurfaceTension (:266) */
    MPS_PHASE_CD = 6,            /* ComputeDFSPHConstantDensity (:268-275) */
    MPS_PHASE_ADVECT = 7         /* BoundaryCollision + UpdatePosition (:277-278) */
};
int mps_phase(mps_handle* h, int32_t phase, void* stream);

/* Per-particle fields by name: "density","alpha","pressure","delta","density_deviation" (rho/rho0 - 1
 * from the compensated density sums, which the stiffness reads),"aux"(2: rho, ST factor),"color"(4),
 * "pos"(4),"vel"(4),"ids"(u32),"bvol"(boundary),"bpos"(boundary, 4),
 * "nbr_count"(u32: fluid + boundary * 65536),"cell_key"(u64),"cg_b"(4),"cg_x"(4).
 * order: 0 = current slot order (sorted by cell), 1 = particle ID order.
 * Values are copied to/from host memory; count is in elements of the field's type. */
int64_t mps_field_size(mps_handle* h, const char* name);
int mps_get_field(mps_handle* h, const char* name, void* host_dst, int order);
int mps_put_field(mps_handle* h, const char* name, const void* host_src, int order);

/* Kernels that mps_profile_kernel can time. */
enum mps_kernel_id {
    MPS_K_PRESSURE_A = 0,     /* density change rate + stiffness pass of a DF/CD iteration */
    MPS_K_PRESSURE_B = 1,     /* pressure force + velocity pass of a DF/CD iteration */
    MPS_K_CG_AP = 2,          /* viscosity + surface tension + XSPH operator pass of a CG iteration */
    MPS_K_DENSITY_ALPHA = 3,  /* density, colour, alpha, gravity */
    MPS_K_BUILD_NBRS = 4,     /* neighbour lists */
    MPS_K_SORT = 5,           /* cell keys + radix sort + reorder */
    MPS_K_CG_VECTOR = 6       /* the three-pass CG's update + direction passes of a CG iteration */
};
/* Times `reps` (1..1000) launches of one kernel of the step on the current state with CUDA events
 * recorded on `stream`; *ms = mean milliseconds per launch.  A solver pass is timed with its loop
 * partner run (untimed) between the timed launches -- pressure A with B, the CG operator with the
 * CG vector passes, and the reverse -- so that the caches are as inside the solver loop.  Solver
 * passes run in their profiling form (no loop decision) and change the velocities and CG state,
 * so call this after the work being measured.  No counterpart in the reference (it has no device
 * timers). */
int mps_profile_kernel(mps_handle* h, int32_t kernel, int32_t reps, void* stream, double* ms);

/* Allocation-free cell sort (no counterpart in the reference).  For callers that cannot
 * allocate device memory -- an application recording a stream capture, a plugin whose host owns
 * the GPU allocator, a real-time loop that cannot afford an allocation's implicit device
 * synchronisation.  Computes the step's 64-bit cell keys of n caller-owned particles (device
 * float4 x,y,z,w; w unused) on the grid (origin, cell, dims) and stable-sorts them: keys_out[k]
 * is the k-th smallest key, order_out[k] the index of that particle.  Scratch lives in one fixed
 * device array inside the library (about 3.1 MB, held by every GPU that loads it until exit);
 * n > MPS_NOALLOC_MAX_PARTICLES returns MPS_E_INVALID, and so does pos4 not 16-byte aligned
 * (keys_out and order_out need 8- and 4-byte alignment).  The first call on a device looks up that
 * array with the device current: make it before any stream capture.  Calls that overlap on the
 * GPU share the array and race; serialise them. */
#define MPS_NOALLOC_MAX_PARTICLES 262144
int mps_cell_sort_noalloc(const float* pos4, int64_t n, const float origin[3], float cell,
                          const int32_t dims[3], uint64_t* keys_out, uint32_t* order_out, void* stream);

/* Cell grid of the step (one scene): origin, cell size, dims. */
int mps_get_grid(mps_handle* h, float origin[3], float* cell, int32_t dims[3]);

/* ---- Function-granular calls (the building blocks of the C++ drop-in API, mps_reference.hpp) ----
 * One call per function of the reference's step API that mps::System::OnUpdate calls
 * (MPSSystem.cpp:220-278), for single-scene handles.  The step fuses some of them into one kernel;
 * each op here runs alone with the same arithmetic, so a frame driven op by op (with mps_phase for
 * the hash, lists and solver drivers) gives the same bits as mps_step.
 *   MPS_OP_DENSITY_SUB    ComputeDensitySub (MPSSPHBaseUtil.h:19-31): names the neighbour set
 *                         (`parts`: MPS_PART_FLUID, MPS_PART_BOUNDARY) of the next DENSITY_FINAL
 *   MPS_OP_DENSITY_FINAL  ComputeDensityFinal (:32-34): one pass over the named sets (Kahan sums)
 *   MPS_OP_COLOR          DensityColorTest (:35-37)
 *   MPS_OP_FACTOR_SUB / MPS_OP_FACTOR_FINAL  ComputeDFSPHFactorSub / Final (MPSSPHDFSPHUtil.h:10-25)
 *   MPS_OP_GRAVITY        ApplyGravity (MPSAdvectUtil.h:16): names gravity for the next UPDATE_VELOCITY
 *   MPS_OP_UPDATE_VELOCITY UpdateVelocity (:17): v += dt g where m > 1e-10
 *   MPS_OP_COLLISION      BoundaryCollision (:19)
 *   MPS_OP_POSITION       UpdatePosition (:18); completes the frame (the step counter advances)
 *   MPS_OP_ST_FACTOR      ComputeSurfaceTensionFactor (MPSSPHNonPressureUtil.h:34-37)
 * A Final without its Sub calls returns MPS_E_STATE. */
enum mps_op_id {
    MPS_OP_DENSITY_SUB = 0,
    MPS_OP_DENSITY_FINAL = 1,
    MPS_OP_COLOR = 2,
    MPS_OP_FACTOR_SUB = 3,
    MPS_OP_FACTOR_FINAL = 4,
    MPS_OP_GRAVITY = 5,
    MPS_OP_UPDATE_VELOCITY = 6,
    MPS_OP_COLLISION = 7,
    MPS_OP_POSITION = 8,
    MPS_OP_ST_FACTOR = 9
};
#define MPS_PART_FLUID 1
#define MPS_PART_BOUNDARY 2
int mps_op(mps_handle* h, int32_t op, int32_t parts, void* stream);

/* Device addresses of the library's per-particle arrays, in the current slot order (cell-sorted;
 * slot k holds particle ids[k]; arrays are padded to `slots`).  The fluid's position and velocity
 * arrays alternate between two buffers at every cell sort (MPS_PHASE_SORT / mps_step): views
 * taken before a sort name the previous order.  Neighbour lists are interleaved: the k-th
 * neighbour slot of slot i is at nbr_*[k * nbr_stride + i]; nbr_count[i] = fluid count | boundary
 * count << 16. */
typedef struct mps_device_views {
    int64_t n, nb, slots;
    float* pos4;          /* (x, y, z, support radius h = 4 r) */
    float* vel4;          /* (vx, vy, vz, mass) */
    uint32_t* ids;
    float* density;
    float* pressure;      /* stiffness kappa of the last solver iteration */
    float* alpha;         /* DFSPH factor */
    float* delta;         /* density change rate of the last pressure iteration */
    float* color4;
    float* scratch4;      /* 4 floats a slot of scratch (overwritten by the viscosity solve) */
    float* bpos4;         /* boundary (x, y, z, h), cell-sorted at set time */
    float* bvol;
    uint32_t* nbr_fluid;
    uint32_t* nbr_boundary;
    uint32_t* nbr_count;
    int64_t nbr_stride;
    int32_t cap_fluid, cap_boundary;
    int32_t volume_accumulate;
} mps_device_views;
int mps_get_device_views(mps_handle* h, mps_device_views* out);

/* cudaMemsetAsync of a device range to zero (ResetREAL of the drop-in API). */
int mps_device_zero(void* dev_ptr, int64_t bytes, void* stream);

/* ---- Batched scenes (many independent scenes, one set of launches per pass) ---- */
/* Scenes are concatenated: fluid of scene s is particles [fluid_offsets[s], fluid_offsets[s+1])
 * of pos4/vel4, boundary of scene s is [boundary_offsets[s], boundary_offsets[s+1]).
 * boxes: 6 doubles per scene (min xyz, max xyz) for collision and the cell grid. */
int mps_create_batched(const mps_material* mat, const mps_physics* phys, const mps_config* cfg,
                       int device, int32_t nscenes, const int64_t* fluid_offsets,
                       const int64_t* boundary_offsets, const double* boxes, mps_handle** out);
int mps_set_batched(mps_handle* h, const float* pos4, const float* vel4, const float* bpos4,
                    void* stream);
int mps_get_batched(mps_handle* h, float* pos4, float* vel4, void* stream);
/* Per-scene iteration counts of the last step: 3 int32 per scene (DF, CG, CD). */
int mps_get_scene_iters(mps_handle* h, int32_t* out3);

/* ---- Scene generation (host only, deterministic across platforms) ---- */
/* Jittered lattice block: nx*ny*nz particles at lower corner origin + spacing*(i+1).
 * Writes pos4 (x,y,z,radius) and vel4 (0,0,0,mass).  jitter: uniform in [-jitter, jitter]. */
int mps_gen_block(int32_t nx, int32_t ny, int32_t nz, const double origin[3], double spacing,
                  double radius, double mass, double jitter, uint64_t seed, float* pos4,
                  float* vel4);
/* Single-layer walls of an axis-aligned box at spacing (open_mask bit k: skip face k,
 * faces ordered -x,+x,-y,+y,-z,+z).  Returns particle count; pos4 may be NULL to count. */
int64_t mps_gen_box_walls(const double lo[3], const double hi[3], double spacing, double radius,
                          int32_t open_mask, float* pos4);
/* Sphere surface sampled at about spacing (Fibonacci lattice).  Returns count; pos4 may be NULL. */
int64_t mps_gen_sphere(const double center[3], double R, double spacing, double radius, float* pos4);

/* ---- Mesh boundaries (scene set-up; replaces MeshObject::LoadMesh + ParticleSampling) ---- */
/* Reads "v x y z" and "f a b c ..." records of an OBJ file (1-based indices, polygons fanned into
 * triangles) and, when center/size are given, fits the mesh's bounding box to that box per axis
 * (MPSMeshObject.cu:58-103).  Two-call form: pass NULL arrays to get the counts. */
int mps_mesh_load_obj(const char* path, const double center[3], const double size[3], int64_t* nverts,
                      int64_t* nfaces, double* verts3, uint32_t* faces3);
/* Boundary particles on a triangle mesh, sampled on the GPU as the reference's ParticleSampling
 * (MPSParticleSamplingUtil.cu:42-133): each face writes the vertices and edges it owns and its
 * scanlines at spacing mesh_radius / 2; particle radius mesh_radius / 4.  Returns the count (or a
 * negative MPS_E_* code); pos4 NULL = count only; face_id optional. */
int64_t mps_mesh_sample(const double* verts3, int64_t nv, const uint32_t* faces3, int64_t nf,
                        double mesh_radius, float* pos4, uint32_t* face_id);

/* ---- Adjoint (reverse-mode gradient of a rollout) ----
 * No counterpart in the reference, which has no differentiation.  Requirements: fixed_iters > 0
 * (every solve runs a fixed count), visc_solver = MPS_VISC_JACOBI, volume_accumulate = 0.
 * mps_adjoint_forward runs nsteps steps from the current state exactly like mps_step and keeps
 * a checkpoint (slot-order state) every checkpoint_every steps on the device.
 * mps_adjoint_backward takes the cotangents of the final state (host, particle-ID order, 4
 * floats per particle, the 4th ignored; either may be NULL = zero) and returns, per particle in
 * ID order, d/d(initial position) and d/d(initial velocity) (4 floats each, 4th = 0), and per
 * scene d/d(viscosity) and d/d(surface_tension) (2 doubles per scene).  Steps between
 * checkpoints are recomputed with neighbour lists rebuilt; each step's solves are reversed as
 * transposed Jacobi sweeps of the same fixed count.  The handle is left at the final state.
 * The neighbour lists are assumed symmetric (MPS_E_STATE otherwise). */
int mps_adjoint_forward(mps_handle* h, int32_t nsteps, int32_t checkpoint_every, void* stream);
int mps_adjoint_backward(mps_handle* h, const float* g_pos4, const float* g_vel4, float* g_pos0,
                         float* g_vel0, double* g_param2, void* stream);
/* Device bytes the adjoint holds for the current layout (checkpoints + one step's tape). */
int64_t mps_adjoint_memory(mps_handle* h, int32_t nsteps, int32_t checkpoint_every);
/* Allocates those buffers now (mps_adjoint_forward otherwise allocates on first use). */
int mps_adjoint_reserve(mps_handle* h, int32_t nsteps, int32_t checkpoint_every);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif /* MPS_C_H */
