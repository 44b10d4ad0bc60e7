// One device-resident FLIP / PIC / APIC sub-step:
// GridFluidSolver3::onAdvanceTimeStep (src/jet/grid_fluid_solver3.cpp:
// 179-210) as FlipSolver3 / PicSolver3 / ApicSolver3 run it
// (src/jet/pic_solver3.cpp:63-112, src/jet/flip_solver3.cpp:27-99,
// src/jet/apic_solver3.cpp:26-228), with no
// viscosity, emitter or advected scalar fields:
//   beginAdvanceTimeStep        applyBoundaryCondition            (:137-160)
//   onBeginAdvanceTimeStep      P2G (+ FLIP snapshot), particle SDF,
//                               extrapolateVelocityToAir, applyBoundaryCondition
//   computeExternalForces       gravity, applyBoundaryCondition    (:317-344)
//   computePressure             pressure projection, applyBoundaryCondition
//   computeAdvection            extrapolateVelocityToAir, applyBoundaryCondition,
//                               G2P (FLIP delta or PIC), moveParticles
// applyBoundaryCondition is GridFractionalBoundaryConditionSolver3::
// constrainVelocity with depth ceil(maxCfl) (:346-353). Every stage is a
// kernel of this library; the particles and the grid never leave the device.
// The CFL number that drives the reference's adaptive sub-stepping
// (GridFluidSolver3::cfl, :360-378) is a device max-reduction.

#include "ctx.h"
#include "sampling.cuh"

#include <cmath>
#include <cstring>

namespace jg {
namespace {

using namespace smp;

// computeGravity: a(i,j,k) += dt * g (one face array).
__global__ void k_gravity(double* __restrict__ a, long n, double add) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
         c += (long)gridDim.x * blockDim.x)
        a[c] += add;
}

// The collider's surface velocity component `a` at every face of axis `a`
// (the pressure solve's boundaryVelocity samples,
// GridFractionalSinglePhasePressureSolver3::buildSingleSystem :241-255).
__global__ void k_solid_faces(FaceSet fs, int a, double hx, double hy,
                              double hz, jetgpu_collider col,
                              double* __restrict__ out) {
    const Dims s = fs.s[a];
    const long n = s.count();
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n;
         c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, s, i, j, k);
        // RigidBodyCollider3::velocityAt (src/jet/rigid_body_collider3.cpp:
        // 25-28) at the face position (data origin + h * index); the _rn
        // intrinsics keep every product and sum separately rounded, as the
        // reference's double arithmetic is.
        const double p0 = __dadd_rn(fs.o[a][0], __dmul_rn(hx, (double)i));
        const double p1 = __dadd_rn(fs.o[a][1], __dmul_rn(hy, (double)j));
        const double p2 = __dadd_rn(fs.o[a][2], __dmul_rn(hz, (double)k));
        const double* w = col.angular_velocity;
        const double r0 = __dsub_rn(p0, col.centre[0]),
                     r1 = __dsub_rn(p1, col.centre[1]),
                     r2 = __dsub_rn(p2, col.centre[2]);
        const double cr[3] = {
            __dsub_rn(__dmul_rn(w[1], r2), __dmul_rn(r1, w[2])),
            __dsub_rn(__dmul_rn(w[2], r0), __dmul_rn(r2, w[0])),
            __dsub_rn(__dmul_rn(w[0], r1), __dmul_rn(r0, w[1]))};
        out[c] = __dadd_rn(col.linear_velocity[a], cr[a]);
    }
}

// GridFluidSolver3::cfl before the division: max(0, every component of
// valueAtCellCenter(i,j,k) + dt * g) (FaceCenteredGrid3::valueAtCellCenter,
// src/jet/face_centered_grid3.cpp:128-135). Non-negative doubles order like
// their bit patterns, so the block maxima meet in one 64-bit atomicMax.
__global__ void k_cfl_max(Dims n, const double* __restrict__ u,
                          const double* __restrict__ v,
                          const double* __restrict__ w, double gx, double gy,
                          double gz, unsigned long long* __restrict__ out) {
    __shared__ double sm[kThreads / 32];
    double m = 0.0;
    const long N = n.count();
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < N;
         c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(c, n, i, j, k);
        const long cu = lin(i, j, k, n.x + 1, n.y);
        const long cv = lin(i, j, k, n.x, n.y + 1);
        const long cw = lin(i, j, k, n.x, n.y);
        const double vx = 0.5 * (u[cu] + u[cu + 1]) + gx;
        const double vy = 0.5 * (v[cv] + v[cv + n.x]) + gy;
        const double vz = 0.5 * (w[cw] + w[cw + (long)n.x * n.y]) + gz;
        m = m < vx ? vx : m;
        m = m < vy ? vy : m;
        m = m < vz ? vz : m;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_down_sync(0xffffffffu, m, o);
        m = m < y ? y : m;
    }
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < kThreads / 32 ? sm[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_down_sync(0xffffffffu, m, o);
            m = m < y ? y : m;
        }
        if (threadIdx.x == 0)
            atomicMax(out, (unsigned long long)__double_as_longlong(m));
    }
}

template <typename T>
jetgpu_status grow(Ctx* c, T** p, size_t* cap, size_t n) {
    if (*cap >= n) return JETGPU_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    JG_CUDA(c, cudaMalloc((void**)p, n * sizeof(T)));
    *cap = n;
    return JETGPU_OK;
}

bool usable(jetgpu_status s) {
    return s == JETGPU_OK || s == JETGPU_NOT_CONVERGED ||
           s == JETGPU_STALLED_FALLBACK_USED;
}

}  // namespace

bool collider_moves(const jetgpu_collider* col) {
    if (!col) return false;
    for (int d = 0; d < 3; ++d)
        if (col->linear_velocity[d] != 0.0 || col->angular_velocity[d] != 0.0)
            return true;
    return false;
}

jetgpu_status solid_face_velocities(Ctx* c, const GridDesc& g,
                                    const jetgpu_collider& col, double* out) {
    const FaceSet fs = face_set(g);
    for (int a = 0; a < 3; ++a) {
        const long n = fs.s[a].count();
        k_solid_faces<<<blocks_for(n, kThreads, c->num_sms * 8), kThreads, 0,
                        c->stream>>>(fs, a, g.spacing[0], g.spacing[1],
                                     g.spacing[2], col, out);
        out += n;
    }
    JG_CUDA(c, cudaGetLastError());
    return JETGPU_OK;
}

jetgpu_status fluid_cfl(Ctx* c, const GridDesc& g, const double* u,
                        const double* v, const double* w, double dt,
                        const double gravity[3], double* cfl) {
    if (jetgpu_status s = grow(c, &c->flip_cfl, &c->flip_cfl_cap, 1)) return s;
    JG_CUDA(c, cudaMemsetAsync(c->flip_cfl, 0, sizeof(unsigned long long),
                               c->stream));
    const Dims n{g.res[0], g.res[1], g.res[2]};
    k_cfl_max<<<blocks_for(n.count(), kThreads, c->num_sms * 8), kThreads, 0,
                c->stream>>>(n, u, v, w, dt * gravity[0], dt * gravity[1],
                             dt * gravity[2], c->flip_cfl);
    unsigned long long bits = 0;
    JG_CUDA(c, cudaMemcpyAsync(&bits, c->flip_cfl, sizeof(bits),
                               cudaMemcpyDeviceToHost, c->stream));
    JG_CUDA(c, cudaStreamSynchronize(c->stream));
    double maxVel;
    std::memcpy(&maxVel, &bits, sizeof(double));
    const double minH = std::min(std::min(g.spacing[0], g.spacing[1]),
                                 g.spacing[2]);
    *cfl = maxVel * dt / minH;
    return JETGPU_OK;
}

jetgpu_status flip_substep(Ctx* c, const GridDesc& g, long np, double* pos,
                           double* vel, double* affine, double* u, double* v,
                           double* w,
                           double* fluid_sdf, const FieldDesc& col_sdf,
                           const jetgpu_collider* col,
                           const jetgpu_sphere* sph,
                           const jetgpu_flip_params& prm, double dt,
                           jetgpu_solve_stats* stats) {
    const FaceSet fs = face_set(g);
    const long nf[3] = {fs.s[0].count(), fs.s[1].count(), fs.s[2].count()};
    const long faces = nf[0] + nf[1] + nf[2];
    const unsigned depth = (unsigned)std::ceil(prm.max_cfl);
    const int closed = prm.closed_domain_flags;
    if (jetgpu_status s = grow(c, &c->flip_marks, &c->flip_marks_cap,
                               (size_t)faces))
        return s;
    if (jetgpu_status s = grow(c, &c->flip_snap, &c->flip_snap_cap,
                               (size_t)faces))
        return s;
    unsigned char* mk[3] = {c->flip_marks, c->flip_marks + nf[0],
                            c->flip_marks + nf[0] + nf[1]};
    float* sn[3] = {c->flip_snap, c->flip_snap + nf[0],
                    c->flip_snap + nf[0] + nf[1]};
    double* vel3[3] = {u, v, w};
    const int res3[3][3] = {{fs.s[0].x, fs.s[0].y, fs.s[0].z},
                            {fs.s[1].x, fs.s[1].y, fs.s[1].z},
                            {fs.s[2].x, fs.s[2].y, fs.s[2].z}};
    // The collider stands still within a sub-step: its faces are classified
    // once for the five boundary-condition passes.
    if (jetgpu_status s = bc_classify(c, g, col_sdf)) return s;
    auto bc = [&]() {
        return bc_apply(c, g, u, v, w, col_sdf, col, closed, depth);
    };
    auto to_air = [&]() -> jetgpu_status {  // extrapolateVelocityToAir
        const Dims ds[3] = {Dims{res3[0][0], res3[0][1], res3[0][2]},
                            Dims{res3[1][0], res3[1][1], res3[1][2]},
                            Dims{res3[2][0], res3[2][1], res3[2][2]}};
        const unsigned char* vm[3] = {mk[0], mk[1], mk[2]};
        return extrapolate_regions(c, 3, ds, vel3, vm, depth);
    };
    jetgpu_status s;
    // beginAdvanceTimeStep
    if ((s = bc()) != JETGPU_OK) return s;
    // onBeginAdvanceTimeStep
    const bool flip = prm.flip == 1, apic = prm.flip == 2;
    if (apic)
        s = apic_p2g(c, g, np, pos, vel, affine, u, v, w, mk[0], mk[1], mk[2]);
    else
        s = p2g(c, g, np, pos, vel, u, v, w, mk[0], mk[1], mk[2],
                flip ? sn[0] : nullptr, flip ? sn[1] : nullptr,
                flip ? sn[2] : nullptr);
    if (s != JETGPU_OK) return s;
    if ((s = build_particle_sdf(c, g, np, pos, col_sdf, prm.max_cfl,
                                fluid_sdf)) != JETGPU_OK)
        return s;
    if ((s = to_air()) != JETGPU_OK) return s;
    if ((s = bc()) != JETGPU_OK) return s;
    // computeExternalForces
    const double* gr = prm.gravity;
    const double eps = 2.220446049250313e-16;  // kEpsilonD
    if (gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2] > eps) {
        for (int a = 0; a < 3; ++a)
            if (std::fabs(gr[a]) > eps)
                k_gravity<<<blocks_for(nf[a], kThreads, c->num_sms * 8),
                            kThreads, 0, c->stream>>>(vel3[a], nf[a],
                                                      dt * gr[a]);
        if ((s = bc()) != JETGPU_OK) return s;
    }
    // computePressure: the collider SDF and velocity, the particle SDF.
    const double* solid[3] = {nullptr, nullptr, nullptr};
    if (collider_moves(col)) {
        if ((s = grow(c, &c->flip_solid, &c->flip_solid_cap,
                      (size_t)faces)) != JETGPU_OK)
            return s;
        if ((s = solid_face_velocities(c, g, *col, c->flip_solid)) !=
            JETGPU_OK)
            return s;
        solid[0] = c->flip_solid;
        solid[1] = solid[0] + nf[0];
        solid[2] = solid[1] + nf[1];
    }
    {
        jetgpu_grid jg_grid;
        jetgpu_scalar_field bsdf, fsdf;
        for (int d = 0; d < 3; ++d) {
            jg_grid.res[d] = g.res[d];
            jg_grid.spacing[d] = g.spacing[d];
            jg_grid.origin[d] = g.origin[d];
        }
        bsdf.kind = col_sdf.kind;
        bsdf.value = col_sdf.value;
        bsdf.data = col_sdf.data;
        fsdf.kind = 1;
        fsdf.value = 0.0;
        fsdf.data = fluid_sdf;
        for (int d = 0; d < 3; ++d) {
            bsdf.res[d] = col_sdf.res[d];
            bsdf.origin[d] = col_sdf.origin[d];
            bsdf.spacing[d] = col_sdf.spacing[d];
            fsdf.res[d] = g.res[d];
            fsdf.origin[d] = g.origin[d] + 0.5 * g.spacing[d];
            fsdf.spacing[d] = g.spacing[d];
        }
        // The reference ignores the solver's result (:466-483); a solve that
        // returns its last iterate is applied the same way.
        s = solve_pressure_dev(c, &jg_grid, u, v, w, &bsdf, bsdf.data, &fsdf,
                               fsdf.data, solid[0], solid[1], solid[2], u, v,
                               w, nullptr, stats);
        if (!usable(s)) return s;
    }
    if ((s = bc()) != JETGPU_OK) return s;
    // computeAdvection
    if ((s = to_air()) != JETGPU_OK) return s;
    if ((s = bc()) != JETGPU_OK) return s;
    if (flip)
        s = g2p_flip(c, g, np, pos, vel, u, v, w, sn[0], sn[1], sn[2],
                     prm.pic_blending);
    else if (apic)
        s = apic_g2p(c, g, np, pos, vel, affine, u, v, w);
    else
        s = g2p_pic(c, g, np, pos, vel, u, v, w);
    if (s != JETGPU_OK) return s;
    return move_particles(c, g, np, pos, vel, u, v, w, dt, prm.max_cfl, closed,
                          col, sph);
}

}  // namespace jg
