/*
 * jetgpu — GB300-native pressure projection for the Jet fluid engine.
 *
 * C ABI of libjetgpu.so. Plain C types only: no C++ types, no exceptions, no
 * torch types cross this boundary. Every function returns a jetgpu_status;
 * jetgpu_last_error() gives the message of the last failure on a context.
 *
 * Array conventions follow Jet: 3-D arrays are i-fastest,
 * index = i + nx*(j + ny*k) (include/jet/detail/array_accessor3-inl.h:197-200).
 * A face-centred velocity grid of resolution (nx,ny,nz) stores
 * u:(nx+1,ny,nz), v:(nx,ny+1,nz), w:(nx,ny,nz+1) doubles whose data origins
 * are origin + h/2 on the two tangential axes
 * (src/jet/face_centered_grid3.cpp:428-445).
 *
 * Threading: one context per solver instance, used by one host thread at a
 * time. Each context owns one CUDA stream and its device buffers; buffers are
 * reallocated only when the resolution changes. Every call is synchronous on
 * return, as the reference's solvers are.
 */
#ifndef JETGPU_H_
#define JETGPU_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum jetgpu_status {
    JETGPU_OK = 0,
    /* The iteration cap was reached before the tolerance. The outputs hold
     * the last iterate, as the reference's FdmMgpcgSolver3 does
     * (src/jet/fdm_mgpcg_solver3.cpp:54-80). */
    JETGPU_NOT_CONVERGED = 1,
    /* The flexible-PCG iteration with the learned preconditioner stalled and
     * the solve finished with the plain multigrid preconditioner. */
    JETGPU_STALLED_FALLBACK_USED = 2,
    JETGPU_BAD_INPUT = 3,
    JETGPU_CUDA_ERROR = 4,
    JETGPU_OUT_OF_MEMORY = 5,
    /* A NaN or Inf appeared in a reduction (input or breakdown). */
    JETGPU_NUMERICAL_ERROR = 6,
    /* The problem is larger than the fixed capacity of an entry point that
     * works without allocating (jetgpu_p2g_device_noalloc). */
    JETGPU_CAPACITY_EXCEEDED = 7
} jetgpu_status;

/* Arithmetic of the Krylov iteration. In every mode the global r.z and p.Ap
 * reductions and the final true-residual check are FP64, and the true
 * residual is taken against the FP64 operator the reference builds. */
typedef enum jetgpu_precision {
    /* FP32 Krylov vectors and FP32 V-cycle; FP64 iterative refinement
     * accumulates the solution and checks the true residual. */
    JETGPU_PRECISION_FP32 = 0,
    /* FP64 Krylov vectors and operator; FP32 V-cycle. */
    JETGPU_PRECISION_FP64 = 1,
    /* As FP32, with BF16 storage of the V-cycle's vectors and coefficients. */
    JETGPU_PRECISION_MIXED_BF16 = 2
} jetgpu_precision;

typedef enum jetgpu_preconditioner {
    JETGPU_PRECOND_MULTIGRID = 0,
    /* Learned preconditioner in flexible PCG: a multigrid V-cycle plus a
     * U-Net's coarse-level correction of its error (jetgpu_learned_apply),
     * with plain multigrid PCG as fallback when iterations stall. Requires
     * weights loaded with jetgpu_load_unet(). */
    JETGPU_PRECOND_LEARNED = 1,
    /* No preconditioner (plain CG); for comparisons. */
    JETGPU_PRECOND_NONE = 2
} jetgpu_preconditioner;

/* Solver configuration. The first nine fields mirror the FdmMgpcgSolver3
 * constructor (include/jet/fdm_mgpcg_solver3.h:35-41):
 * FdmMgpcgSolver3(numberOfCgIter, maxNumberOfLevels, numberOfRestrictionIter,
 *                 numberOfCorrectionIter, numberOfCoarsestIter,
 *                 numberOfFinalIter, maxTolerance, sorFactor,
 *                 useRedBlackOrdering).
 * Differences, by design: `tolerance` is the relative true residual
 * ||b - A x||_2 / ||b||_2 (the reference stops on the absolute
 * sqrt(r.M^-1 r), include/jet/detail/cg-inl.h:48); smoothing is always
 * red-black (the lexicographic sweep is serial by construction); and the
 * V-cycle is made symmetric (post-smoothing runs the colours in reverse order)
 * with a zero initial guess, so that it is a fixed SPD preconditioner. */
typedef struct jetgpu_config {
    int device;                 /* CUDA device ordinal */
    unsigned int max_cg_iter;   /* numberOfCgIter */
    unsigned int max_levels;    /* maxNumberOfLevels */
    unsigned int restrict_iter; /* pre-smoothing sweeps */
    unsigned int correct_iter;  /* post-smoothing sweeps, coarse levels */
    unsigned int coarsest_iter; /* sweeps on the coarsest level */
    unsigned int final_iter;    /* post-smoothing sweeps, finest level */
    double tolerance;           /* relative true residual target */
    double sor;                 /* SOR factor of the red-black smoother */
    int red_black;              /* must be nonzero */
    int precision;              /* jetgpu_precision */
    int preconditioner;         /* jetgpu_preconditioner */
    unsigned int max_refinements; /* FP32 modes: FP64 refinement passes */
    /* P2G (jetgpu_p2g[_device], the FLIP/PIC sub-step): nonzero sums every
     * face's contributions in particle order, as the reference's serial loop
     * does (pic_solver3.cpp:118-193), so the grids are bit-exact and the same
     * from run to run; zero scatters with FP64 atomics (faster; the sums
     * differ from the reference's in rounding only). */
    int ordered_p2g;
    /* Host-pointer fractional solves (jetgpu_solve_pressure[_collider]):
     * nonzero moves only the velocity faces inside the bounding box of the
     * fluid cells (fluid_sdf < 0), widened by the faces that close it, in
     * both directions, and leaves the output's faces outside that box as
     * they are. The reference reads and writes velocities only at faces
     * next to fluid cells (buildSystem, applyPressureGradient), so this
     * gives its result whenever the output already holds the input's
     * values outside the box — as in GridFluidSolver3::computePressure,
     * whose input is a clone of the output grid. Inside the box, faces the
     * projection leaves alone get the input's values (as with zero). */
    int fluid_box_io;
} jetgpu_config;

/* Fills `cfg` with defaults: FdmMgpcgSolver3(100, 6, 2, 2, 5, 2, 1e-6, 1.2,
 * true), FP32, multigrid, 6 refinements, device 0. Two symmetric red-black
 * SOR sweeps with omega 1.2 per level converge in 7 iterations on the 256^3
 * FLIP scene (8 with omega 1.0, at the same cost per iteration). */
void jetgpu_config_default(jetgpu_config* cfg);

/* A scalar-field argument of GridPressureSolver3::solve
 * (include/jet/grid_pressure_solver3.h:58-64): a ConstantScalarField3
 * (kind 0) or a grid sampled with Jet's trilinear rule (kind 1), e.g. a
 * CellCenteredScalarGrid3 whose data point (0,0,0) sits at `origin`
 * (its dataOrigin()). */
typedef struct jetgpu_scalar_field {
    int kind;            /* 0 = constant, 1 = grid */
    double value;        /* kind 0 */
    const double* data;  /* kind 1: res[0]*res[1]*res[2] doubles */
    int res[3];
    double origin[3];
    double spacing[3];
} jetgpu_scalar_field;

/* Geometry of a FaceCenteredGrid3: resolution, grid spacing, origin. */
typedef struct jetgpu_grid {
    int res[3];
    double spacing[3];
    double origin[3];
} jetgpu_grid;

typedef struct jetgpu_solve_stats {
    unsigned int iterations;     /* Krylov iterations, all passes */
    unsigned int refinements;    /* FP64 refinement passes (FP32 modes) */
    unsigned int levels;         /* multigrid levels used */
    double residual;             /* ||b - A x||_2, FP64, reference operator */
    double relative_residual;    /* residual / ||b||_2 */
    double b_norm;               /* ||b||_2 */
    double setup_ms;             /* weights + system build (device time) */
    double solve_ms;             /* Krylov solve (device time) */
    double total_ms;             /* whole call, including copies */
    int fallback_used;           /* learned preconditioner fell back */
    unsigned long long h2d_bytes; /* host-pointer solves: bytes uploaded */
    unsigned long long d2h_bytes; /* ... and downloaded */
} jetgpu_solve_stats;

/* Context lifetime. */
jetgpu_status jetgpu_create(const jetgpu_config* cfg, struct jetgpu_ctx** out);
void jetgpu_destroy(struct jetgpu_ctx* ctx);
const char* jetgpu_last_error(const struct jetgpu_ctx* ctx);
jetgpu_status jetgpu_set_config(struct jetgpu_ctx* ctx,
                                const jetgpu_config* cfg);

/* GridFractionalSinglePhasePressureSolver3::solve
 * (src/jet/grid_fractional_single_phase_pressure_solver3.cpp:456-484) with
 * an MGPCG linear solver installed: buildWeights (:520-636), buildSystem
 * (:651-713), the multigrid-preconditioned CG solve
 * (src/jet/fdm_mgpcg_solver3.cpp:54-80) and applyPressureGradient (:715-765).
 *
 * HOST pointers. u/v/w: the input velocity. boundary_sdf: collider SDF
 * (negative inside solids). fluid_sdf: liquid SDF (negative inside liquid).
 * solid_u/v/w: the collider velocity's normal component sampled at every
 * u/v/w face position, or NULL for a static collider (boundaryVelocity).
 * out_u/v/w: the projected velocity; faces the reference leaves untouched
 * keep the input values (out may alias the input). out_pressure: the level-0
 * pressure (GridFractionalSinglePhasePressureSolver3::pressure(), :512-518),
 * or NULL. stats may be NULL. */
jetgpu_status jetgpu_solve_pressure(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, const double* u,
    const double* v, const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, const double* solid_u,
    const double* solid_v, const double* solid_w, double* out_u,
    double* out_v, double* out_w, double* out_pressure,
    jetgpu_solve_stats* stats);

/* Same as jetgpu_solve_pressure with every array (including the SDF grids'
 * data) in DEVICE memory of the context's device. For solvers that keep the
 * simulation resident on the GPU. */
jetgpu_status jetgpu_solve_pressure_device(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, const double* u,
    const double* v, const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, const double* solid_u,
    const double* solid_v, const double* solid_w, double* out_u,
    double* out_v, double* out_w, double* out_pressure,
    jetgpu_solve_stats* stats);

/* GridSinglePhasePressureSolver3::solve, the blocked solver
 * (src/jet/grid_single_phase_pressure_solver3.cpp:183-211), with an MGPCG
 * linear solver installed: buildMarkers (:245-322; a cell is boundary,
 * fluid or air by the SDFs at its centre, coarse levels by majority),
 * buildSystem (:341-376), the MGPCG solve and applyPressureGradient
 * (:378-405). The reference ignores boundaryVelocity (:191), so it is not an
 * argument. HOST pointers; arguments otherwise as jetgpu_solve_pressure:
 * faces the reference leaves untouched keep the input values, out_pressure
 * is GridSinglePhasePressureSolver3::pressure() (:229-235) or NULL. */
jetgpu_status jetgpu_solve_pressure_blocked(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, const double* u,
    const double* v, const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, double* out_u, double* out_v,
    double* out_w, double* out_pressure, jetgpu_solve_stats* stats);

/* jetgpu_solve_pressure_blocked with every array in DEVICE memory. */
jetgpu_status jetgpu_solve_pressure_blocked_device(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, const double* u,
    const double* v, const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, double* out_u, double* out_v,
    double* out_w, double* out_pressure, jetgpu_solve_stats* stats);

/* FdmMgpcgSolver3::solve(FdmMgLinearSystem3*)
 * (src/jet/fdm_mgpcg_solver3.cpp:54-80) on a caller-built multigrid system.
 * HOST pointers. Levels are concatenated finest first; level l has
 * resolution res0 >> l. A: FdmMatrixRow3 {center,right,up,front} doubles per
 * cell (include/jet/fdm_linear_system3.h:18-30); b: doubles per cell, only
 * level 0 is read; x: level-0 solution out. */
jetgpu_status jetgpu_mgpcg_solve_system(struct jetgpu_ctx* ctx,
                                        const int res0[3], int levels,
                                        const double* A, const double* b,
                                        double* x, jetgpu_solve_stats* stats);

/* PicSolver3::transferFromParticlesToGrids (src/jet/pic_solver3.cpp:118-193)
 * and, when snap_* are non-NULL, FlipSolver3's float snapshot of the result
 * (src/jet/flip_solver3.cpp:27-48). DEVICE pointers. pos/vel: AoS xyz
 * doubles (particle_system_data3.h:114-123). u/v/w: velocity out. mu/mv/mw:
 * face markers out (1 where a particle contributed). */
jetgpu_status jetgpu_p2g_device(struct jetgpu_ctx* ctx,
                                const jetgpu_grid* grid, long num_particles,
                                const double* pos, const double* vel,
                                double* u, double* v, double* w,
                                unsigned char* mu, unsigned char* mv,
                                unsigned char* mw, float* snap_u,
                                float* snap_v, float* snap_w);

/* FlipSolver3::transferFromGridsToParticles (src/jet/flip_solver3.cpp:50-99).
 * DEVICE pointers. snap_* hold the P2G snapshot on entry and the float delta
 * on exit; vel is updated in place. */
jetgpu_status jetgpu_g2p_flip_device(struct jetgpu_ctx* ctx,
                                     const jetgpu_grid* grid,
                                     long num_particles, const double* pos,
                                     double* vel, const double* u,
                                     const double* v, const double* w,
                                     float* snap_u, float* snap_v,
                                     float* snap_w, double pic_blending);

/* PicSolver3::transferFromGridsToParticles (src/jet/pic_solver3.cpp:195-204).
 * DEVICE pointers. */
jetgpu_status jetgpu_g2p_pic_device(struct jetgpu_ctx* ctx,
                                    const jetgpu_grid* grid,
                                    long num_particles, const double* pos,
                                    double* vel, const double* u,
                                    const double* v, const double* w);

/* P2G that allocates nothing. No counterpart in the reference.
 *
 * For callers that must not allocate device memory while they run: a host
 * engine or plugin that owns the GPU's memory budget and forbids hidden
 * allocations, or a real-time loop in which cudaMalloc's implicit device
 * synchronisation is not allowed. It computes the same result as
 * jetgpu_p2g_device (same DEVICE-pointer arguments) but needs no context:
 * its only scratch, the per-face weight sums, lives in a fixed array in the
 * library's device memory of JETGPU_P2G_NOALLOC_MAX_FACES doubles (6.4 MB),
 * which every GPU that loads the library holds until the process exits.
 * The limit is on the face count, not on each axis: a grid (nx, ny, nz) is
 * accepted when (nx+1)*ny*nz + nx*(ny+1)*nz + nx*ny*(nz+1) <=
 * JETGPU_P2G_NOALLOC_MAX_FACES (a 64^3 grid fits exactly; so does
 * 100 x 40 x 40) and rejected with JETGPU_CAPACITY_EXCEEDED, before any GPU
 * work, otherwise. Grids with a non-finite origin or spacing, a spacing
 * <= 0 or 2^31 cells or more get JETGPU_BAD_INPUT.
 *
 * The work is queued on `stream` (a cudaStream_t; NULL = the default
 * stream) and the call returns without waiting for it. The first call on a
 * device, with that device current, looks up the scratch array's device
 * address; make that first call before any stream capture. All calls share
 * the one array: calls that overlap on the GPU (different streams, or
 * different host threads, without ordering between them) race on it. Each
 * call clears the part it uses before accumulating. No cudaMalloc, cudaFree
 * or allocating library routine is called. */
#define JETGPU_P2G_NOALLOC_MAX_FACES (3u * 65u * 64u * 64u)
jetgpu_status jetgpu_p2g_device_noalloc(void* stream, const jetgpu_grid* grid,
                                        long num_particles, const double* pos,
                                        const double* vel, double* u,
                                        double* v, double* w,
                                        unsigned char* mu, unsigned char* mv,
                                        unsigned char* mw, float* snap_u,
                                        float* snap_v, float* snap_w);

/* A rigid collider: surface velocity linear + angular x (p - centre)
 * (RigidBodyCollider3::velocityAt, src/jet/rigid_body_collider3.cpp:25-28;
 * centre = the surface transform's translation) and the friction
 * coefficient (Collider3::frictionCoefficient, src/jet/collider3.h). */
typedef struct jetgpu_collider {
    double linear_velocity[3];
    double angular_velocity[3];
    double centre[3];
    double friction;
} jetgpu_collider;

/* jetgpu_solve_pressure with the collider velocity given as a rigid body's
 * motion instead of sampled face arrays: the boundaryVelocity that
 * GridFractionalBoundaryConditionSolver3::colliderVelocityField() hands the
 * pressure solver (src/jet/grid_fractional_boundary_condition_solver3.cpp:
 * 265-278) is RigidBodyCollider3::velocityAt
 * (src/jet/rigid_body_collider3.cpp:25-28), which is evaluated here on the
 * device at every face position. collider NULL, or one with zero linear and
 * angular velocity, is a static collider (no moving-boundary term, as
 * solid_u/v/w = NULL). HOST pointers; otherwise as jetgpu_solve_pressure. */
jetgpu_status jetgpu_solve_pressure_collider(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, const double* u,
    const double* v, const double* w, const jetgpu_scalar_field* boundary_sdf,
    const jetgpu_scalar_field* fluid_sdf, const jetgpu_collider* collider,
    double* out_u, double* out_v, double* out_w, double* out_pressure,
    jetgpu_solve_stats* stats);

/* Closed-domain bits of closedDomainBoundaryFlag()
 * (include/jet/constants.h:312-335). */
#define JETGPU_DIRECTION_LEFT 1
#define JETGPU_DIRECTION_RIGHT 2
#define JETGPU_DIRECTION_DOWN 4
#define JETGPU_DIRECTION_UP 8
#define JETGPU_DIRECTION_BACK 16
#define JETGPU_DIRECTION_FRONT 32
#define JETGPU_DIRECTION_ALL 63

/* GridFractionalBoundaryConditionSolver3::constrainVelocity
 * (src/jet/grid_fractional_boundary_condition_solver3.cpp:26-233), in place
 * on the face velocity u/v/w. DEVICE pointers (collider_sdf->data too).
 * collider_sdf: the solver's colliderSdf() (a cell-centred grid of the
 * velocity grid's resolution; kind 0 = no collider). collider: NULL = none.
 * closed_domain_flags: JETGPU_DIRECTION_* bits. extrapolation_depth: the
 * free-slip extrapolation depth (GridFluidSolver3 passes ceil(maxCfl)).
 * Bit-identical to the reference. Queued on the context's stream; returns
 * without waiting. */
jetgpu_status jetgpu_constrain_velocity_device(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, double* u, double* v,
    double* w, const jetgpu_scalar_field* collider_sdf,
    const jetgpu_collider* collider, int closed_domain_flags,
    unsigned int extrapolation_depth);

/* Host-pointer form of jetgpu_constrain_velocity_device (copies inside the
 * call; synchronous). */
jetgpu_status jetgpu_constrain_velocity(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, double* u, double* v,
    double* w, const jetgpu_scalar_field* collider_sdf,
    const jetgpu_collider* collider, int closed_domain_flags,
    unsigned int extrapolation_depth);

/* GridBlockedBoundaryConditionSolver3::constrainVelocity
 * (src/jet/grid_blocked_boundary_condition_solver3.cpp:23-67), the
 * boundary-condition solver GridSinglePhasePressureSolver3 suggests: the
 * fractional constraint above, then every face between a collider cell
 * (collider_sdf < 0 at the cell, :79-90) and a non-collider cell takes the
 * collider velocity's normal component at the face position. collider_sdf,
 * when a grid, must have the velocity grid's resolution. DEVICE pointers;
 * queued on the context's stream. Bit-identical to the reference. */
jetgpu_status jetgpu_constrain_velocity_blocked_device(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, double* u, double* v,
    double* w, const jetgpu_scalar_field* collider_sdf,
    const jetgpu_collider* collider, int closed_domain_flags,
    unsigned int extrapolation_depth);

/* Host-pointer form of jetgpu_constrain_velocity_blocked_device. */
jetgpu_status jetgpu_constrain_velocity_blocked(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, double* u, double* v,
    double* w, const jetgpu_scalar_field* collider_sdf,
    const jetgpu_collider* collider, int closed_domain_flags,
    unsigned int extrapolation_depth);

/* extrapolateToRegion (include/jet/detail/array_utils-inl.h:172-244), as
 * PicSolver3::extrapolateVelocityToAir (src/jet/pic_solver3.cpp:284-294)
 * applies it to each face array with the P2G markers: `iterations` passes
 * in place on data (res[0]*res[1]*res[2] doubles, i fastest) from the cells
 * whose valid byte is non-zero. DEVICE pointers; valid is not modified.
 * Bit-identical to the reference. */
jetgpu_status jetgpu_extrapolate_to_region_device(
    struct jetgpu_ctx* ctx, const int res[3], double* data,
    const unsigned char* valid, unsigned int iterations);

/* A Sphere3 collider surface (src/jet/sphere3.cpp) under its Transform3
 * (include/jet/detail/transform3-inl.h): local centre and radius, normal
 * flip (Surface3::isNormalFlipped), and the transform's orientation matrix
 * and its inverse, row-major (Transform3 keeps both; identity for an
 * unrotated sphere). The translation is the collider's `centre`. */
typedef struct jetgpu_sphere {
    double center[3];
    double radius;
    int normal_flipped;
    double orientation[9];
    double inverse_orientation[9];
} jetgpu_sphere;

/* PicSolver3::moveParticles (src/jet/pic_solver3.cpp:206-282): per
 * particle, max(1, floor(max_cfl)) RK2 midpoint sub-steps of dt through the
 * face velocity u/v/w, clamping to the closed domain walls
 * (closed_domain_flags, JETGPU_DIRECTION_* bits) with the velocity component
 * zeroed there; then, when both collider and sphere are non-NULL,
 * Collider3::resolveCollision (src/jet/collider3.cpp:19-73) with radius 0
 * and restitution 0 against the sphere. pos/vel: AoS xyz doubles, updated in
 * place. DEVICE pointers. Bit-identical to the reference. */
jetgpu_status jetgpu_move_particles_device(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, long num_particles,
    double* pos, double* vel, const double* u, const double* v,
    const double* w, double dt, double max_cfl, int closed_domain_flags,
    const jetgpu_collider* collider, const jetgpu_sphere* sphere);

/* Host-pointer form of jetgpu_move_particles_device (synchronous). */
jetgpu_status jetgpu_move_particles(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, long num_particles,
    double* pos, double* vel, const double* u, const double* v,
    const double* w, double dt, double max_cfl, int closed_domain_flags,
    const jetgpu_collider* collider, const jetgpu_sphere* sphere);

/* PicSolver3::buildSignedDistanceField (src/jet/pic_solver3.cpp:296-317)
 * and GridFluidSolver3::extrapolateIntoCollider
 * (src/jet/grid_fluid_solver3.cpp:423-438): the liquid SDF the pressure
 * solve takes, at the cell centres of `grid` (res cells, i fastest) — the
 * distance to the nearest particle within 2r minus r, r = 1.2 max(h) /
 * sqrt(2) — then extrapolated ceil(max_cfl) cells into the collider
 * (collider_sdf negative; kind 0 = no collider). pos: AoS xyz doubles.
 * DEVICE pointers. Bit-identical to the reference. */
jetgpu_status jetgpu_build_particle_sdf_device(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, long num_particles,
    const double* pos, const jetgpu_scalar_field* collider_sdf,
    double max_cfl, double* sdf_out);

/* Host-pointer form of jetgpu_build_particle_sdf_device (synchronous). */
jetgpu_status jetgpu_build_particle_sdf(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, long num_particles,
    const double* pos, const jetgpu_scalar_field* collider_sdf,
    double max_cfl, double* sdf_out);

/* Settings of a FLIP / PIC step (GridFluidSolver3 / FlipSolver3). */
typedef struct jetgpu_flip_params {
    double gravity[3];        /* GridFluidSolver3::gravity */
    double max_cfl;           /* GridFluidSolver3::maxCfl */
    int closed_domain_flags;  /* JETGPU_DIRECTION_* bits */
    int flip;                 /* 1: FlipSolver3, 0: PicSolver3,
                                 2: ApicSolver3 */
    double pic_blending;      /* FlipSolver3::picBlendingFactor */
} jetgpu_flip_params;

/* Fills the reference defaults (grid_fluid_solver3.h:269,
 * flip_solver3.h:67): gravity (0,-9.8,0), maxCfl 5, all walls closed, FLIP,
 * no PIC blending. */
void jetgpu_flip_params_default(jetgpu_flip_params* params);

/* GridFluidSolver3::cfl (src/jet/grid_fluid_solver3.cpp:360-378): the
 * largest component (or 0) of the cell-centre velocity plus dt * gravity,
 * times dt, over the smallest grid spacing; the adaptive sub-stepping of
 * PhysicsAnimation::onUpdate (src/jet/physics_animation.cpp:98-122) takes
 * max(ceil(cfl / maxCfl), 1) sub-steps. DEVICE velocity; synchronous. */
jetgpu_status jetgpu_fluid_cfl_device(struct jetgpu_ctx* ctx,
                                      const jetgpu_grid* grid, const double* u,
                                      const double* v, const double* w,
                                      double dt, const double gravity[3],
                                      double* cfl);

/* One GridFluidSolver3::onAdvanceTimeStep of FlipSolver3 / PicSolver3
 * (src/jet/grid_fluid_solver3.cpp:179-210, src/jet/pic_solver3.cpp:63-112,
 * src/jet/flip_solver3.cpp:27-99) on device-resident state: boundary
 * conditions, P2G (+ FLIP snapshot), the particle SDF, extrapolation to air,
 * gravity, the pressure projection of this library (its configured solver),
 * G2P and particle advection with collisions, each stage in the
 * reference's order. DEVICE pointers. pos/vel: AoS xyz doubles; affine:
 * the APIC particles' cX, cY, cZ (9 doubles each; read and written; NULL
 * unless params->flip == 2); u/v/w: the grid velocity (the solver's grid
 * state, read and written); fluid_sdf: the
 * particle SDF out (res cells). collider_sdf: colliderSdf() of the boundary
 * solver (kind 0 = none); collider / sphere: NULL = none. stats: the
 * pressure solve's. Returns the first error, or the pressure solve's status. */
jetgpu_status jetgpu_flip_substep_device(
    struct jetgpu_ctx* ctx, const jetgpu_grid* grid, long num_particles,
    double* pos, double* vel, double* affine, double* u, double* v, double* w,
    double* fluid_sdf, const jetgpu_scalar_field* collider_sdf,
    const jetgpu_collider* collider, const jetgpu_sphere* sphere,
    const jetgpu_flip_params* params, double dt, jetgpu_solve_stats* stats);

/* ApicSolver3::transferFromParticlesToGrids (src/jet/apic_solver3.cpp:
 * 26-146): the affine particle-to-grid transfer. affine: each particle's
 * cX, cY, cZ (9 doubles: cX.x, cX.y, cX.z, cY.x, ...). u/v/w and markers out
 * as jetgpu_p2g_device. DEVICE pointers. The FP64 atomic scatter reorders the
 * reference's serial sums (rounding only). */
jetgpu_status jetgpu_apic_p2g_device(struct jetgpu_ctx* ctx,
                                     const jetgpu_grid* grid,
                                     long num_particles, const double* pos,
                                     const double* vel, const double* affine,
                                     double* u, double* v, double* w,
                                     unsigned char* mu, unsigned char* mv,
                                     unsigned char* mw);

/* ApicSolver3::transferFromGridsToParticles (:148-228): vel (the PIC
 * sample) and affine (the velocity gradients, 9 doubles per particle) out.
 * DEVICE pointers. Bit-identical to the reference. */
jetgpu_status jetgpu_apic_g2p_device(struct jetgpu_ctx* ctx,
                                     const jetgpu_grid* grid,
                                     long num_particles, const double* pos,
                                     double* vel, double* affine,
                                     const double* u, const double* v,
                                     const double* w);

/* Host-pointer forms of the three transfers (copies inside the call). */
jetgpu_status jetgpu_p2g(struct jetgpu_ctx* ctx, const jetgpu_grid* grid,
                         long num_particles, const double* pos,
                         const double* vel, double* u, double* v, double* w,
                         unsigned char* mu, unsigned char* mv,
                         unsigned char* mw, float* snap_u, float* snap_v,
                         float* snap_w);
jetgpu_status jetgpu_g2p_flip(struct jetgpu_ctx* ctx, const jetgpu_grid* grid,
                              long num_particles, const double* pos,
                              double* vel, const double* u, const double* v,
                              const double* w, float* snap_u, float* snap_v,
                              float* snap_w, double pic_blending);
jetgpu_status jetgpu_g2p_pic(struct jetgpu_ctx* ctx, const jetgpu_grid* grid,
                             long num_particles, const double* pos,
                             double* vel, const double* u, const double* v,
                             const double* w);

/* Copies internal state of the last pressure solve to HOST memory, for
 * checking against the reference's private members
 * (grid_fractional_single_phase_pressure_solver3.h:103-115).
 * what: 0 fluid SDF (float, cells), 1/2/3 u/v/w weights (float, faces),
 *       4 matrix rows (4 doubles per cell; level 0 exact FP64, coarse levels
 *       as stored in FP32 and widened), 5 rhs b (doubles, level 0 only),
 *       6 the pressure of the last solve (doubles, level 0 only; after a
 *       jetgpu_flip_substep_device, that sub-step's pressure).
 * Returns the element count via *count. */
jetgpu_status jetgpu_get_level(struct jetgpu_ctx* ctx, int level, int what,
                               void* dst, size_t capacity, size_t* count);

/* The context's CUDA stream (a cudaStream_t), so callers can order their
 * own work and time the library's kernels with events on it. No
 * counterpart in the reference, which has no device. */
jetgpu_status jetgpu_get_stream(struct jetgpu_ctx* ctx, void** stream);

/* Live per-kernel profile: while enabled, every kernel launch of the
 * context is bracketed by CUDA events on its stream and filed under its
 * kernel class with the launch's algorithmic bytes. Enabling (or disabling)
 * clears the record. Replaces the reference's Timer logs around each phase
 * (src/jet/grid_fluid_solver3.cpp:189-207). */
typedef struct jetgpu_kernel_stat {
    char name[32];
    unsigned int launches;
    double total_ms;   /* sum of event-timed launch durations */
    double bytes;      /* sum of algorithmic bytes of those launches */
} jetgpu_kernel_stat;

jetgpu_status jetgpu_profile(struct jetgpu_ctx* ctx, int enable);
/* Fills up to `capacity` entries (one per kernel class seen) and returns the
 * number of classes through *count. */
jetgpu_status jetgpu_profile_read(struct jetgpu_ctx* ctx,
                                  jetgpu_kernel_stat* out, int capacity,
                                  int* count);

/* ---- Learned preconditioner building blocks (no counterpart in the
 * reference; Jet has no learned components). DEVICE pointers, queued on
 * `stream` (a cudaStream_t) without waiting. Activations are BF16,
 * channels-last ([cell][channel], cells i-fastest). */

/* 3x3x3 convolution, stride 1, zero padding 1, on the tcgen05 tensor cores:
 * out[v][co] = act(bias[co] + sum_{tap,ci} in[v+tap][ci] * w[tap][co][ci])
 * with FP32 accumulation; tap = (dz+1)*9 + (dy+1)*3 + (dx+1). ci and co are
 * multiples of 16 in [16, 128]. relu != 0 applies max(0, .). out (BF16)
 * and/or out32 (FP32) receive the result. *err is or-ed with 1 if an
 * internal wait gave up (it never should). */
jetgpu_status jetgpu_conv3d(void* stream, const void* in, int ci,
                            const void* w, const float* bias, int co,
                            const int res[3], int relu, void* out,
                            float* out32, unsigned int* err);

/* Weight gradient of jetgpu_conv3d (no bias, no activation):
 * dw[tap][co][ci] += sum_v dy[v][co] * in[v+tap][ci], FP32, on the tensor
 * cores. The caller zeroes dw first. The input gradient is jetgpu_conv3d of
 * dy with the weights flipped in tap and transposed in (co, ci). */
jetgpu_status jetgpu_conv3d_wgrad(void* stream, const void* in, int ci,
                                  const void* dy, int co, const int res[3],
                                  float* dw, unsigned int* err);

/* Number of FP32 parameters of the preconditioner network: per layer,
 * w[27][co][ci] then b[co], for the 14 layers of the 4-level U-Net
 * (16/32/48/64 channels). */
size_t jetgpu_net_param_count(void);

/* Loads network parameters (HOST pointer, FP32, the order above) into the
 * context; stored as BF16 weights and FP32 biases. Enables
 * preconditioner = JETGPU_PRECOND_LEARNED (flexible PCG). */
jetgpu_status jetgpu_load_unet(struct jetgpu_ctx* ctx, const float* params,
                               size_t count);

/* Training data from the solver itself: runs multigrid PCG on the system of
 * the context's last pressure solve and records, for each of up to
 * max_pairs iterations, the residual r_k and the V-cycle correction
 * z_k = M r_k (DEVICE arrays of max_pairs * cells floats each). */
jetgpu_status jetgpu_harvest(struct jetgpu_ctx* ctx, unsigned int max_pairs,
                             float* r_out, float* z_out,
                             unsigned int* count);

/* z = M r: one multigrid V-cycle preconditioner application (the
 * preconditioner of FdmMgpcgSolver3, fdm_mgpcg_solver3.cpp:15-36, with this
 * library's masked symmetric V-cycle) for residual r on the finest level of
 * the last solved system, FP32 DEVICE arrays of cells floats (r and z may
 * alias). For Krylov methods and training outside the library;
 * synchronous. */
jetgpu_status jetgpu_vcycle_apply(struct jetgpu_ctx* ctx, const float* r,
                                  float* z);

/* The level of the multigrid hierarchy of the last solved system that the
 * network works on: the finest level at most 64 cells wide on every axis
 * (the coarsest level when none is). */
unsigned int jetgpu_net_level(const struct jetgpu_ctx* ctx);

/* The network's 16 input channels (BF16, channels-last) for residual r on
 * level `level` of the last solved system, and the network's output
 * e = net(r) there (cells of that level). DEVICE pointers; synchronous. */
jetgpu_status jetgpu_net_features(struct jetgpu_ctx* ctx, unsigned int level,
                                  const float* r, void* feat);
jetgpu_status jetgpu_net_apply(struct jetgpu_ctx* ctx, unsigned int level,
                               const float* r, float* e);

/* z = M r with the learned preconditioner of JETGPU_PRECOND_LEARNED, for
 * residual r on the finest level (FP32 DEVICE arrays of cells floats; r and
 * z must not alias): one V-cycle z0 = V r, then the network's correction of
 * its error from the residual it leaves, on level k = jetgpu_net_level():
 * z = z0 + mask P^k net(R^k (r - A z0)), R the V-cycle's masked
 * restriction, P its trilinear prolongation, mask zero outside the fluid.
 * Synchronous. */
jetgpu_status jetgpu_learned_apply(struct jetgpu_ctx* ctx, const float* r,
                                   float* z);

/* Library version string. */
const char* jetgpu_version(void);

#ifdef __cplusplus
}
#endif

#endif /* JETGPU_H_ */
