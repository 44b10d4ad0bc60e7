// Host-side context of libjetgpu: device buffers, stream, launch helpers.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <mutex>
#include <functional>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/jetgpu.h"
#include "common.cuh"

namespace jg {

// One multigrid level.
struct Level {
    Dims n{0, 0, 0};
    double h[3] = {0, 0, 0};
    float* phi = nullptr;        // fluid SDF at cell centres
    float* uw = nullptr;         // face weights
    float* vw = nullptr;
    float* ww = nullptr;
    // Matrix rows as a structure of arrays: the center, right, up and front
    // coefficients in four planes of N values each (FP32 in A; BF16 in Ah
    // for the mixed-precision V-cycle).
    float* A = nullptr;
    float* x = nullptr;          // V-cycle solution
    float* x2 = nullptr;         // ping-pong partner of x (fused smoother)
    float* b = nullptr;          // V-cycle rhs
    float* r = nullptr;          // residual scratch
    unsigned short* Ah = nullptr;
};

// Kernel classes of the live per-kernel profile (jetgpu_profile_read).
enum KernelClass : int {
    K_SWEEP_L0 = 0,   // fused red-black sweep, finest level
    K_SWEEP_COARSE,   // fused red-black sweep, coarse levels
    K_HALF_L0,        // red or black half-sweep, finest level
    K_HALF_COARSE,    // red or black half-sweep, coarse levels
    K_COARSEST,       // one-CTA coarsest-level sweeps
    K_RESIDUAL,       // FP32 residual (V-cycle)
    K_RESTRICT,       // residual restriction
    K_CORRECT,        // prolongation + correction
    K_SPMV,           // q = A d, d.q
    K_UPDATE_XR,      // x += a d, r -= a q, r.r
    K_DOT_RZ,         // r.z
    K_UPDATE_D,       // d = z + b d
    K_RESIDUAL64,     // FP64 true residual
    K_ACCUMULATE,     // x += e (double-float) / x64 += e
    K_WEIGHTS,        // fluid SDF sampling + face weights
    K_PYRAMID,        // restriction of the weight/SDF pyramid
    K_SYSTEM,         // matrix rows + rhs
    K_GRADIENT,       // pressure gradient
    K_P2G,
    K_G2P,
    K_UNET,
    K_BOUNDARY,       // boundary conditions / extrapolation
    K_SDF,            // particle signed-distance field
    K_MOVE,           // particle advection
    K_CLASS_COUNT
};
const char* kernel_class_name(int cls);

// Per-axis exact sampling tables of buildWeights (see build.cu), cached per
// grid/field geometry.
struct SampleTables {
    bool valid = false;
    bool use_nodes = false;
    // The fluid SDF lies on the grid's cells: every cell centre's table
    // entry is (its own index, fraction +0), the last (n - 2, 1).
    bool fluid_on_cells = false;
    int* irregular = nullptr;  // device flag: a zero or non-finite SDF value
    GridDesc g{};
    FieldDesc B{}, F{};
    int off[3][4] = {};   // entry offsets [axis][N,M,P,C]
    int total = 0;
    int soff[3] = {}, nslot[3] = {};
    size_t cap = 0;       // entries allocated
    int* idx = nullptr;
    double* frac = nullptr;
    int* slot = nullptr;
    int* sidx = nullptr;
    double* sfrac = nullptr;
    size_t node_cap = 0;
    double* node = nullptr;
};

struct ProfRec {
    int cls;
    int e0, e1;
    double bytes;
};

struct Ctx {
    jetgpu_config cfg;
    int device = 0;
    int num_sms = 0;
    int tma_blocks_per_sm[2] = {0, 0};  // fused sweep blocks/SM, FP32 / BF16
                                        // rows (0: not usable on this device)
    std::unordered_map<const void*, int> occupancy;  // blocks/SM per kernel
    cudaStream_t stream = nullptr;
    // Host-pointer solves move data on copy_stream, ordered against the
    // compute stream by io_ev (see SolveIo).
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t io_ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    // Fluid-box transfers: the box on the device and in pinned host memory,
    // and the event that says it has arrived.
    int* box_dev = nullptr;
    int* box_host = nullptr;
    cudaEvent_t box_ev = nullptr;
    // One event per slab of cell planes of the pressure gradient, so that
    // the download of the faces a slab completes runs under the next slab.
    static constexpr int kGradSlabs = 4;
    cudaEvent_t grad_ev[kGradSlabs] = {nullptr, nullptr, nullptr, nullptr};
    // High-priority stream for the coarse levels' set-up, which runs beside
    // the finest level's (fork and join events).
    cudaStream_t side_stream = nullptr;
    cudaEvent_t side_ev[2] = {nullptr, nullptr};
    std::string err;

    // Allocated geometry.
    Dims n0{0, 0, 0};
    unsigned built_levels = 0;
    std::vector<Level> levels;

    // Finest-level FP64 system and solution.
    double* A64 = nullptr;  // 4 doubles per cell
    double* b64 = nullptr;
    double* x64 = nullptr;
    double* r64 = nullptr;
    // Double-float image of the finest-level system and iterate (FP32
    // modes): the exact rows and rhs as hi + lo FP32 pairs (hi = the FP32
    // rows of level 0), and the solution accumulated as a pair.
    float4* Alo = nullptr;
    float2* bdf = nullptr;
    float2* xdf = nullptr;

    // Krylov vectors (FP32 modes).
    float* kx = nullptr;
    float* kr = nullptr;
    float* kd = nullptr;
    float* kq = nullptr;
    float* kz = nullptr;
    float* kz2 = nullptr;  // previous z (flexible PCG)
    // Krylov vectors (FP64 mode).
    double* dx = nullptr;
    double* dr = nullptr;
    double* dd = nullptr;
    double* dq = nullptr;
    double* dz = nullptr;

    // Reductions.
    double* scal = nullptr;
    double* partials = nullptr;
    unsigned* counters = nullptr;
    double* h_scal = nullptr;  // pinned mirror

    // Staging for the host-pointer API (device copies of inputs/outputs).
    size_t stage_bytes = 0;
    unsigned char* stage = nullptr;
    size_t host_stage_bytes = 0;
    unsigned char* host_stage = nullptr;  // pinned

    // Particle-transfer scratch.
    size_t pscratch_bytes = 0;
    unsigned char* pscratch = nullptr;
    // Ordered P2G scratch (transfer.cu): bin keys, bin counts / offsets /
    // cursors, scan totals and the particles listed by bin (ints); each
    // particle's fractions on the face lattice (doubles).
    size_t p2g_int_cap = 0, p2g_dbl_cap = 0;
    int* p2g_int = nullptr;
    double* p2g_dbl = nullptr;

    // Boundary-condition scratch (boundary.cu): bc_cap doubles and 2 x bc_cap
    // validity bytes.
    size_t bc_cap = 0;
    double* bc_tmp = nullptr;
    unsigned char* bc_valid = nullptr;
    size_t bc_cls_cap = 0;
    unsigned char* bc_cls = nullptr;  // face classes of the last bc_classify
    int* bc_list = nullptr;           // its invalid / inside face lists
    unsigned* bc_cnt = nullptr;       // their lengths per axis
    int* bc_flag = nullptr;           // the classification's regular SDF
    size_t rflag_cap = 0;             // build_system0_rows: rhs cells
    unsigned char* rflag = nullptr;
    size_t bc_nrm_cap = 0;            // collider normals of inside faces
    double4_32a* bc_nrm = nullptr;
    // extrapolate_region(s): stamps and two front lists (xp_cap entries
    // each), two front lengths per array.
    size_t xp_cap = 0;
    int* xp_int = nullptr;
    unsigned* xp_cnt = nullptr;

    // Device-resident FLIP step scratch (flip.cu): P2G markers, FLIP
    // snapshot, collider face velocities, the CFL maximum.
    size_t flip_marks_cap = 0, flip_snap_cap = 0, flip_solid_cap = 0,
           flip_cfl_cap = 0;
    unsigned char* flip_marks = nullptr;
    float* flip_snap = nullptr;
    double* flip_solid = nullptr;
    unsigned long long* flip_cfl = nullptr;

    // Particle-SDF scratch (sdf.cu): bins, keys, sorted particles, validity.
    size_t sdf_int_cap = 0, sdf_dbl_cap = 0, sdf_valid_cap = 0;
    int* sdf_int = nullptr;
    double* sdf_dbl = nullptr;
    unsigned char* sdf_valid = nullptr;

    // The FP32 PCG's V-cycle captured as a CUDA graph (mgpcg.cu,
    // vcycle_graph), with what it was captured for: its vectors, the level
    // count and the smoother settings. Destroyed with the buffers.
    cudaGraphExec_t vc_exec = nullptr;
    const void* vc_key[3] = {nullptr, nullptr, nullptr};
    unsigned vc_levels = 0;
    unsigned vc_iters[4] = {0, 0, 0, 0};
    double vc_sor = 0.0;
    int vc_precision = -1;
    float* vc_result = nullptr;
    bool vc_disabled = false;
    // The whole FP32 PCG loop as one graph with a device-side while node
    // (mgpcg.cu, pcg_loop_graph): V-cycle, Krylov updates and the stopping
    // test per iteration, no host round trip. Captured for the same key as
    // vc_exec; destroyed with the buffers.
    cudaGraphExec_t loop_exec = nullptr;
    bool loop_disabled = false;

    // Compaction list of the two-pass face-weight build (build.cu): the
    // faces whose FP64 marching-squares work runs in a second, full-warp
    // pass.
    size_t build_cap = 0;
    int* build_list = nullptr;
    unsigned* build_cnt = nullptr;

    // Blocked pressure solver (blocked.cu): cell markers of every level,
    // finest first.
    size_t blk_cap = 0;
    unsigned char* blk_marks = nullptr;

    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};

    // Learned preconditioner (opaque; see unet.cu).
    void* unet = nullptr;

    // Exact sampling tables of the weights build.
    SampleTables tabs;

    // Live per-kernel profile: CUDA events recorded on `stream` around
    // launches while enabled.
    bool prof_on = false;
    std::vector<cudaEvent_t> prof_ev;
    size_t prof_used = 0;
    std::vector<ProfRec> prof_recs;
};

// Records an event before a launch; returns its index or -1.
int prof_begin(Ctx* c);
// Records the closing event and files the launch under `cls`.
void prof_end(Ctx* c, int cls, int e0, double bytes);

// Brackets one launch for the live per-kernel profile (no-op unless on).
struct Prof {
    Ctx* c;
    int cls;
    double bytes;
    int e0;
    Prof(Ctx* c_, int cls_, double bytes_) : c(c_), cls(cls_), bytes(bytes_) {
        e0 = prof_begin(c);
    }
    ~Prof() { prof_end(c, cls, e0, bytes); }
};

// Sets ctx->err and returns the status.
jetgpu_status fail(Ctx* c, jetgpu_status s, const std::string& msg);

#define JG_CUDA(c, call)                                                    \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) {                                            \
            return ::jg::fail((c), e_ == cudaErrorMemoryAllocation          \
                                       ? JETGPU_OUT_OF_MEMORY               \
                                       : JETGPU_CUDA_ERROR,                 \
                              std::string(#call) + ": " +                   \
                                  cudaGetErrorString(e_));                  \
        }                                                                   \
    } while (0)

// Runs a set-up step (a kernel attribute, which CUDA keeps per device) once
// on each device: the first call with a device current runs `f` and records
// success for that device; later calls on it do nothing.
class DeviceOnce {
  public:
    template <typename F>
    bool run(F&& f) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMax)
            return false;
        std::lock_guard<std::mutex> lock(mu_);
        if (done_[dev]) return true;
        if (f() != cudaSuccess) return false;
        done_[dev] = true;
        return true;
    }

  private:
    static constexpr int kMax = 64;
    std::mutex mu_;
    bool done_[kMax] = {};
};

// Number of blocks for a grid-stride kernel over n elements.
inline int blocks_for(long n, int threads = kThreads, int cap = 1 << 30) {
    long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}

// Reduction grid size: fixed per resolution, at most kMaxRedBlocks.
inline int red_blocks(const Ctx* c, long n) {
    int cap = c->num_sms * 6;
    if (cap > kMaxRedBlocks) cap = kMaxRedBlocks;
    return blocks_for(n, kThreads, cap);
}

// ---- build.cu -------------------------------------------------------------
// The finest level's face weights and fluid SDF, then (with `pyramid`) the
// coarser levels' (build_pyramid). With `fluid_ready`, the fluid SDF's part
// waits for that event (the face weights need only the collider SDF).
jetgpu_status build_weights(Ctx* c, const GridDesc& g, const FieldDesc& bsdf,
                            const FieldDesc& fsdf, bool pyramid = true,
                            cudaEvent_t fluid_ready = nullptr);
jetgpu_status build_pyramid(Ctx* c);
// Levels [lo, hi) of the hierarchy; only level 0 reads the velocities.
jetgpu_status build_system(Ctx* c, const GridDesc& g, const double* u,
                           const double* v, const double* w,
                           const double* su, const double* sv,
                           const double* sw, unsigned lo = 0,
                           unsigned hi = ~0u);
// The finest level's system in two parts, for host-pointer solves: the rows
// (no velocity needed; marks the cells whose rhs is filled), then the rhs
// once the velocities are in. Together the same as build_system's level 0.
jetgpu_status build_system0_rows(Ctx* c, const GridDesc& g);
jetgpu_status build_system0_rhs(Ctx* c, const GridDesc& g, const double* u,
                                const double* v, const double* w,
                                const double* su, const double* sv,
                                const double* sw);
// Low parts of a caller-built finest-level system (jetgpu_mgpcg_solve_system).
jetgpu_status split_system(Ctx* c);
// The pressure gradient of the cells in planes [kz0, kz1) (kz1 < 0: to
// the last plane); each cell writes the faces it owns.
jetgpu_status apply_gradient(Ctx* c, const GridDesc& g, const double* u,
                             const double* v, const double* w, double* ou,
                             double* ov, double* ow, int kz0 = 0,
                             int kz1 = -1);

// ---- blocked.cu ------------------------------------------------------------
// GridSinglePhasePressureSolver3: markers of every level (and phi = -1 for
// fluid, +1 otherwise, for the V-cycle's masked restriction), the rows of
// every level with the finest-level rhs, and the pressure gradient.
jetgpu_status blocked_markers(Ctx* c, const GridDesc& g, const FieldDesc& bsdf,
                              const FieldDesc& fsdf);
jetgpu_status blocked_system(Ctx* c, const GridDesc& g, const double* u,
                             const double* v, const double* w);
jetgpu_status blocked_gradient(Ctx* c, const GridDesc& g, const double* u,
                               const double* v, const double* w, double* ou,
                               double* ov, double* ow);

// ---- mgpcg.cu -------------------------------------------------------------
// The driver's cuTensorMapEncodeTiled (null when the driver lacks it).
PFN_cuTensorMapEncodeTiled_v12000 tma_encoder();
// Allocates the multigrid hierarchy and solver buffers for resolution n.
jetgpu_status ensure_buffers(Ctx* c, Dims n, unsigned max_levels);
// Derives FP32 (and BF16) matrices of levels [lo, hi) from the built system.
jetgpu_status prepare_levels(Ctx* c, unsigned lo = 0, unsigned hi = ~0u);
// Solves A64 x64 = b64 on the finest level; fills stats.
jetgpu_status mgpcg_solve(Ctx* c, jetgpu_solve_stats* st);
// Computes level count for resolution n (FdmMgUtils3::resizeArrayWithFinest).
unsigned level_count(Dims n, unsigned max_levels);

// Applies one V-cycle z = M r on FP32 vectors; the result lands in z or
// alt (returned through *result).
jetgpu_status vcycle(Ctx* c, const float* r, float* z, float* alt,
                     float** result);
// One-time kernel attributes (dynamic shared memory limits).
jetgpu_status init_kernels(Ctx* c);

// ---- unet.cu --------------------------------------------------------------
struct NetLayer {
    int ci, co, relu, level;
};
constexpr int kNetLayerCount = 14;
extern const NetLayer kNetLayers[kNetLayerCount];
size_t net_param_count();
jetgpu_status net_load(Ctx* c, const float* params, size_t count);
// The multigrid level the network works on: the finest level at most 64
// cells wide on every axis (the coarsest level when none is).
unsigned net_level(const Ctx* c);
// A loaded network and a net_level() whose extents are multiples of 8.
bool net_supported(const Ctx* c);
jetgpu_status net_features(Ctx* c, unsigned level, const float* r,
                           const double* rr, void* feat);
jetgpu_status net_apply(Ctx* c, unsigned level, const float* r,
                        const double* rr, float* z);
void net_destroy(void* net);
jetgpu_status conv3d(cudaStream_t st, const __nv_bfloat16* in, int ci,
                     const __nv_bfloat16* w, const float* bias, int co,
                     Dims n, int relu, __nv_bfloat16* out, float* out32,
                     unsigned* err);

// ---- mgpcg.cu (learned path) ----------------------------------------------
// Records up to max_pairs (r_k, z_k = V-cycle(r_k)) pairs of an MGPCG run on
// the current system into device arrays of max_pairs * N floats.
jetgpu_status harvest_pairs(Ctx* c, unsigned max_pairs, float* r_out,
                            float* z_out, unsigned* count);
// sum(r^2) of an FP32 vector into scal[target] (device).
jetgpu_status norm2f(Ctx* c, const float* r, long n, int target);
// z = M r with the learned preconditioner (a V-cycle plus the network's
// coarse-level correction of its error).
jetgpu_status learned_precond(Ctx* c, const float* r, float* z);

// ---- sdf.cu (shared scan) --------------------------------------------------
// Exclusive scan of n int counts into off[0..n] (off[n] = the total; also in
// *grand); tile_sum holds scan_tiles(n) ints of scratch.
long scan_tiles(long n);
jetgpu_status scan_counts(Ctx* c, const int* count, int* off, long n,
                          int* tile_sum, int* grand);

// ---- transfer.cu ----------------------------------------------------------
jetgpu_status constrain_velocity(Ctx* c, const GridDesc& g, double* u,
                                 double* v, double* w, const FieldDesc& sdf,
                                 const jetgpu_collider* col, int closed,
                                 unsigned depth);
// GridBlockedBoundaryConditionSolver3::constrainVelocity: constrain_velocity
// plus the no-flux pass on the faces of collider cells (boundary.cu).
jetgpu_status constrain_velocity_blocked(Ctx* c, const GridDesc& g, double* u,
                                         double* v, double* w,
                                         const FieldDesc& sdf,
                                         const jetgpu_collider* col,
                                         int closed, unsigned depth);
// The two halves of constrain_velocity: bc_classify evaluates the collider
// SDF at every face (cached in ctx->bc_cls), bc_apply does the rest with
// those classes; a caller whose collider does not move between calls
// classifies once.
jetgpu_status bc_classify(Ctx* c, const GridDesc& g, const FieldDesc& sdf);
jetgpu_status bc_apply(Ctx* c, const GridDesc& g, double* u, double* v,
                       double* w, const FieldDesc& sdf,
                       const jetgpu_collider* col, int closed, unsigned depth);
jetgpu_status extrapolate_region(Ctx* c, Dims s, double* data,
                                 const unsigned char* valid, unsigned iters);
// Up to three arrays extrapolated together, one launch per step.
jetgpu_status extrapolate_regions(Ctx* c, int na, const Dims* s,
                                  double* const* data,
                                  const unsigned char* const* valid,
                                  unsigned iters);

// Overlap of a host-pointer solve's copies with its kernels. The compute
// stream waits for sdf_in before the weights build (which needs only the
// SDFs) and for vel_in before the system build, so the velocity upload runs
// under the weights; once the solve is final, x_final is recorded and the
// pressure is downloaded on `copy` straight into host_p while the gradient
// kernel runs.
struct SolveIo {
    // bsdf_in: the collider SDF is in; sdf_in: both SDFs are.
    cudaEvent_t bsdf_in = nullptr, sdf_in = nullptr, vel_in = nullptr,
                x_final = nullptr;
    cudaStream_t copy = nullptr;
    double* host_p = nullptr;
    // Called once the set-up that needs no velocity is queued, before the
    // level-0 system waits for vel_in (issues the velocity uploads when
    // they depend on something the host must first read back).
    std::function<jetgpu_status()> before_vel;
    // When *grad_slabs > 0, the gradient runs as that many launches over
    // the cell planes [grad_cuts[s], grad_cuts[s + 1]), each followed by
    // Ctx::grad_ev[s] on the compute stream (the caller sets both, up to
    // the point where before_vel returns).
    const int* grad_cuts = nullptr;
    const int* grad_slabs = nullptr;
    // Called once the gradient is queued, before the host waits for it
    // (issues the downloads of the projected velocity).
    std::function<jetgpu_status()> after_grad;
};

// GridFractionalSinglePhasePressureSolver3::solve on device arrays (api.cu):
// the SDF descriptors' data pointers are replaced by bdata / fdata. With
// `blocked`, GridSinglePhasePressureSolver3::solve instead (blocked.cu; the
// solid velocities are ignored, as the reference ignores boundaryVelocity).
jetgpu_status solve_pressure_dev(
    Ctx* c, const jetgpu_grid* grid, const double* u, const double* v,
    const double* w, const jetgpu_scalar_field* bsdf, const double* bdata,
    const jetgpu_scalar_field* fsdf, const double* fdata, const double* su,
    const double* sv, const double* sw, double* ou, double* ov, double* ow,
    double* op, jetgpu_solve_stats* st, const SolveIo* io = nullptr,
    bool blocked = false);

// True when a rigid collider has a non-zero linear or angular velocity.
bool collider_moves(const jetgpu_collider* col);
// RigidBodyCollider3::velocityAt at every face of the grid: the u, v and w
// face components one after the other in `out` (flip.cu).
jetgpu_status solid_face_velocities(Ctx* c, const GridDesc& g,
                                    const jetgpu_collider& col, double* out);

jetgpu_status fluid_cfl(Ctx* c, const GridDesc& g, const double* u,
                        const double* v, const double* w, double dt,
                        const double gravity[3], double* cfl);
jetgpu_status flip_substep(Ctx* c, const GridDesc& g, long np, double* pos,
                           double* vel, double* affine, double* u, double* v,
                           double* w,
                           double* fluid_sdf, const FieldDesc& col_sdf,
                           const jetgpu_collider* col,
                           const jetgpu_sphere* sph,
                           const jetgpu_flip_params& prm, double dt,
                           jetgpu_solve_stats* stats);

jetgpu_status build_particle_sdf(Ctx* c, const GridDesc& g, long np,
                                 const double* pos, const FieldDesc& col,
                                 double max_cfl, double* out);

jetgpu_status apic_p2g(Ctx* c, const GridDesc& g, long np, const double* pos,
                       const double* vel, const double* aff, double* u,
                       double* v, double* w, unsigned char* mu,
                       unsigned char* mv, unsigned char* mw);
jetgpu_status apic_g2p(Ctx* c, const GridDesc& g, long np, const double* pos,
                       double* vel, double* aff, const double* u,
                       const double* v, const double* w);

jetgpu_status move_particles(Ctx* c, const GridDesc& g, long np, double* pos,
                             double* vel, const double* u, const double* v,
                             const double* w, double dt, double max_cfl,
                             int closed, const jetgpu_collider* col,
                             const jetgpu_sphere* sph);

jetgpu_status p2g(Ctx* c, const GridDesc& g, long np, const double* pos,
                  const double* vel, double* u, double* v, double* w,
                  unsigned char* mu, unsigned char* mv, unsigned char* mw,
                  float* su, float* sv, float* sw);
jetgpu_status g2p_flip(Ctx* c, const GridDesc& g, long np, const double* pos,
                       double* vel, const double* u, const double* v,
                       const double* w, float* su, float* sv, float* sw,
                       double blend);
jetgpu_status g2p_pic(Ctx* c, const GridDesc& g, long np, const double* pos,
                      double* vel, const double* u, const double* v,
                      const double* w);

}  // namespace jg
