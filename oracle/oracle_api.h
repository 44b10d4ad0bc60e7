/*
 * Oracle C API — TEST INFRASTRUCTURE ONLY.
 *
 * Two libraries export this same set of functions:
 *   - liboracle_port.so : a CPU restatement (C++/OpenMP) of the Jet pressure
 *     projection written in this repository (oracle/port/jet_port.cpp);
 *   - _ref/libjet_ref_harness.so : a thin harness that drives the real Jet
 *     reference classes compiled from their own sources (oracle/ref_harness.cpp).
 * Tests use them to check the CUDA product against the reference algorithm;
 * the product never links or calls either.
 *
 * Conventions follow Jet: arrays are i-fastest (index = i + nx*(j + ny*k),
 * include/jet/detail/array_accessor3-inl.h:197-200); face-centred velocity
 * has u:(nx+1,ny,nz), v:(nx,ny+1,nz), w:(nx,ny,nz+1)
 * (src/jet/face_centered_grid3.cpp:428-445).
 */
#ifndef ORACLE_ORACLE_API_H_
#define ORACLE_ORACLE_API_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A scalar field argument of GridPressureSolver3::solve
 * (include/jet/grid_pressure_solver3.h:58-64): either a constant
 * (ConstantScalarField3) or a CellCenteredScalarGrid3 whose data point (0,0,0)
 * sits at `origin` (the grid's dataOrigin()). */
typedef struct orc_field {
    int kind;            /* 0 = constant, 1 = grid */
    double value;        /* constant value when kind == 0 */
    const double* data;  /* res[0]*res[1]*res[2] doubles when kind == 1 */
    int res[3];
    double origin[3];
    double spacing[3];
} orc_field;

/* FdmMgpcgSolver3 constructor arguments (include/jet/fdm_mgpcg_solver3.h:35-41). */
typedef struct orc_mg_params {
    unsigned int max_cg_iter;
    unsigned int max_levels;
    unsigned int restrict_iter;
    unsigned int correct_iter;
    unsigned int coarsest_iter;
    unsigned int final_iter;
    double tolerance;
    double sor;
    int red_black;
} orc_mg_params;

/* Face-centred grid geometry: resolution, spacing, origin. */
typedef struct orc_grid {
    int res[3];
    double spacing[3];
    double origin[3];
} orc_grid;

/* GridFractionalSinglePhasePressureSolver3::solve with an FdmMgpcgSolver3
 * installed. solid_{u,v,w} are the collider velocity's normal component at
 * each face position (NULL = static collider). out_p receives the level-0
 * pressure (may be NULL). Returns the MGPCG solver's bool result. */
int orc_pressure_solve(const orc_grid* g, const double* u, const double* v,
                       const double* w, const orc_field* boundary_sdf,
                       const orc_field* fluid_sdf, const double* solid_u,
                       const double* solid_v, const double* solid_w,
                       const orc_mg_params* p, double* out_u, double* out_v,
                       double* out_w, double* out_p, unsigned int* iters,
                       double* resid);

/* Number of multigrid levels built by the last orc_pressure_solve. */
int orc_level_count(void);

/* Copies a level of the last solve's internal state into dst (capacity
 * bytes). what: 0 fluid SDF (float), 1/2/3 u/v/w weights (float),
 *       4 matrix rows (4 doubles per cell: center,right,up,front), 5 rhs b.
 * Returns the number of elements copied (cells or faces), -1 for an
 * unknown level or array, -2 when the array does not fit (nothing copied). */
long orc_get_level(int level, int what, void* dst, size_t capacity);

/* FdmMgpcgSolver3::solve on a caller-built multigrid system. Levels are
 * concatenated finest first; level l has resolution res0 >> l.
 * A: 4 doubles per cell; b: 1 double per cell; x0: finest solution out. */
int orc_mgpcg_system(const int res0[3], int levels, const double* A,
                     const double* b, const orc_mg_params* p, double* x0,
                     unsigned int* iters, double* resid);

/* FdmGaussSeidelSolver3::relaxRedBlack (red_black=1) or ::relax (0),
 * `sweeps` times, in place on x. */
void orc_relax(const int res[3], const double* A, const double* b,
               double sor, int red_black, int sweeps, double* x);

/* FdmMgUtils3::restrict and ::correct; fine resolution = 2 * coarse. */
void orc_mg_restrict(const int coarse_res[3], const double* finer,
                     double* coarser);
void orc_mg_correct(const int coarse_res[3], const double* coarser,
                    double* finer);

/* FdmBlas3::residual and ::dot. */
void orc_residual(const int res[3], const double* A, const double* x,
                  const double* b, double* r);
double orc_dot(long n, const double* a, const double* b);

/* PicSolver3::transferFromParticlesToGrids (pic_solver3.cpp:118-193) followed
 * by the FlipSolver3 float snapshot (flip_solver3.cpp:27-48).
 * pos/vel: AoS xyz doubles. markers: char per face (may be NULL).
 * snap: float per face (may be NULL). */
void orc_p2g(const orc_grid* g, long np, const double* pos, const double* vel,
             double* u, double* v, double* w, char* mu, char* mv, char* mw,
             float* snap_u, float* snap_v, float* snap_w);

/* FlipSolver3::transferFromGridsToParticles (flip_solver3.cpp:50-99).
 * snap_* hold the P2G snapshot on entry and the float delta on exit.
 * vel is updated in place. */
void orc_g2p_flip(const orc_grid* g, long np, const double* pos, double* vel,
                  const double* u, const double* v, const double* w,
                  float* snap_u, float* snap_v, float* snap_w,
                  double pic_blend);

/* PicSolver3::transferFromGridsToParticles (pic_solver3.cpp:195-204). */
void orc_g2p_pic(const orc_grid* g, long np, const double* pos, double* vel,
                 const double* u, const double* v, const double* w);

/* A rigid collider's surface velocity v(p) = lin + ang x (p - centre)
 * (RigidBodyCollider3::velocityAt, src/jet/rigid_body_collider3.cpp:25-28)
 * and its friction coefficient (Collider3::frictionCoefficient). */
typedef struct orc_collider {
    double lin[3];
    double ang[3];
    double centre[3];
    double friction;
} orc_collider;

/* GridFractionalBoundaryConditionSolver3::constrainVelocity
 * (src/jet/grid_fractional_boundary_condition_solver3.cpp:26-233) in place on
 * u/v/w. sdf: the solver's collider SDF (a cell-centred grid of the velocity
 * grid's resolution, colliderSdf()). col: the collider (NULL = none).
 * closed: closedDomainBoundaryFlag() bits (kDirectionLeft = 1 ... Front = 32,
 * include/jet/constants.h:312-335). depth: extrapolation depth. */
void orc_constrain_velocity(const orc_grid* g, double* u, double* v,
                            double* w, const orc_field* sdf,
                            const orc_collider* col, int closed,
                            unsigned int depth);

/* extrapolateToRegion (include/jet/detail/array_utils-inl.h:172-244) in
 * place on data (res cells) from the cells whose valid byte is non-zero. */
void orc_extrapolate(const int res[3], double* data, const char* valid,
                     unsigned int iterations);

/* A Sphere3 collider surface (src/jet/sphere3.cpp) under its Transform3
 * (include/jet/detail/transform3-inl.h): local centre and radius, normal
 * flip, the orientation matrix and its inverse (row-major; Transform3 keeps
 * both), and the orientation quaternion (w, x, y, z) they came from (used by
 * the reference harness to build the same transform). The translation is the
 * collider's `centre`. */
typedef struct orc_sphere {
    double center[3];
    double radius;
    int normal_flipped;
    double orient[9];
    double inv_orient[9];
    double quat[4];
} orc_sphere;

/* PicSolver3::moveParticles (src/jet/pic_solver3.cpp:206-282): RK2
 * midpoint sub-steps through the face velocity, clamping to closed domain
 * walls, then Collider3::resolveCollision (src/jet/collider3.cpp:19-73) of
 * every particle against the sphere collider (col and sphere both non-NULL).
 * pos/vel: AoS xyz doubles, updated in place. */
void orc_move_particles(const orc_grid* g, long np, double* pos, double* vel,
                        const double* u, const double* v, const double* w,
                        double dt, double max_cfl, int closed,
                        const orc_collider* col, const orc_sphere* sphere);

/* PicSolver3::buildSignedDistanceField (src/jet/pic_solver3.cpp:296-317):
 * at every cell centre the distance to the nearest particle within the band
 * 2r (r = 1.2 max(h) / sqrt(2)) minus r (the band value where none is
 * near), then extrapolateIntoCollider (src/jet/grid_fluid_solver3.cpp:
 * 423-438) with depth ceil(max_cfl) from the cells outside collider_sdf.
 * out: res cells. */
void orc_build_particle_sdf(const orc_grid* g, long np, const double* pos,
                            const orc_field* collider_sdf, double max_cfl,
                            double* out);

/* Reference harness only: FlipSolver3 (flip = 1), PicSolver3 (0) or
 * ApicSolver3 (2) with
 * GridFractionalSinglePhasePressureSolver3 + FdmMgpcgSolver3(p), gravity g,
 * maxCfl, closed walls and no collider, run for `frames` frames of 1/fps
 * (update(Frame(i, 1/fps)), adaptive sub-steps) from the particles
 * pos/vel, which are updated in place. */
void orc_flip_run(const orc_grid* g, long np, double* pos, double* vel,
                  int frames, double fps, double max_cfl, int closed,
                  const double gravity[3], int flip, const orc_mg_params* p);
/* orc_flip_run that also copies the pressure solver's pressure() (the last
 * sub-step's pressure, cells) after each frame listed in rec_frames (frame
 * counts 1..frames, ascending) into p_out (nrec x cells). */
void orc_flip_run_record(const orc_grid* g, long np, double* pos, double* vel,
                         int frames, double fps, double max_cfl, int closed,
                         const double gravity[3], int flip,
                         const orc_mg_params* p, int nrec,
                         const int* rec_frames, double* p_out);

/* orc_flip_run with a static sphere collider: a RigidBodyCollider3 over a
 * Sphere3 of `radius` translated to `centre`, friction coefficient
 * `friction` (GridFluidSolver3::setCollider). */
void orc_flip_run_sphere(const orc_grid* g, long np, double* pos, double* vel,
                         int frames, double fps, double max_cfl, int closed,
                         const double gravity[3], int flip,
                         const orc_mg_params* p, const double centre[3],
                         double radius, double friction);

/* Reference harness only: Transform3's orientation matrix and its inverse
 * for quaternion q = (w, x, y, z), row-major. */
void orc_quaternion_matrices(const double q[4], double orient[9],
                             double inv_orient[9]);

/* Reference harness only: the collider SDF that
 * GridFractionalBoundaryConditionSolver3::onColliderUpdated (:244-281)
 * builds for a sphere collider (cell-centred samples of the surface's signed
 * distance). out: res cells. */
void orc_sphere_collider_sdf(const orc_grid* g, const double centre[3],
                             double radius, double* out);

/* ApicSolver3::transferFromParticlesToGrids (src/jet/apic_solver3.cpp:
 * 26-146). affine: the particles' cX, cY, cZ as 9 doubles each (cX.x, cX.y,
 * cX.z, cY.x, ...). Grids and markers out as orc_p2g. */
void orc_apic_p2g(const orc_grid* g, long np, const double* pos,
                  const double* vel, const double* affine, double* u,
                  double* v, double* w, char* mu, char* mv, char* mw);

/* ApicSolver3::transferFromGridsToParticles (:148-228): vel and affine out. */
void orc_apic_g2p(const orc_grid* g, long np, const double* pos, double* vel,
                  double* affine, const double* u, const double* v,
                  const double* w);

/* GridBlockedBoundaryConditionSolver3::constrainVelocity
 * (src/jet/grid_blocked_boundary_condition_solver3.cpp:23-67): as
 * orc_constrain_velocity, then the faces between a collider cell (sdf < 0
 * at the cell) and a non-collider cell take the collider velocity. With cells
 * inside the collider, col must be given (the reference dereferences it). */
void orc_constrain_velocity_blocked(const orc_grid* g, double* u, double* v,
                                    double* w, const orc_field* sdf,
                                    const orc_collider* col, int closed,
                                    unsigned int depth);

/* GridSinglePhasePressureSolver3::solve (the blocked solver,
 * src/jet/grid_single_phase_pressure_solver3.cpp:183-211) with an
 * FdmMgpcgSolver3 installed. The boundary velocity is not an argument: the
 * reference ignores it (:191). Output and return value as orc_pressure_solve. */
int orc_blocked_pressure_solve(const orc_grid* g, const double* u,
                               const double* v, const double* w,
                               const orc_field* boundary_sdf,
                               const orc_field* fluid_sdf,
                               const orc_mg_params* p, double* out_u,
                               double* out_v, double* out_w, double* out_p,
                               unsigned int* iters, double* resid);

/* A level of the last orc_blocked_pressure_solve: what 0 = cell markers
 * (char: 0 fluid, 1 air, 2 boundary), 4 = matrix rows (4 doubles per cell),
 * 5 = rhs b. Returns the number of cells copied, or -1. */
long orc_blocked_get_level(int level, int what, void* dst);

/* Port only: additionally stop MGPCG once the true relative residual
 * ||b - A x|| / ||b|| falls to `rel` (0 disables). Used to state the CPU
 * baseline at the GPU solver's accuracy. */
void orc_set_relative_stop(double rel);

/* Sets the number of host threads the library may use (0 = all). */
void orc_set_threads(int n);

#ifdef __cplusplus
}
#endif

#endif /* ORACLE_ORACLE_API_H_ */
