// Reference harness — TEST INFRASTRUCTURE ONLY.
//
// Implements oracle/oracle_api.h by driving the Jet reference classes compiled
// from their own sources (oracle/Makefile.ref). It lets tests pin the oracle
// port (oracle/port/jet_port.cpp) and generate golden fixtures from the real
// reference. Only this harness reads solver internals: to reach the private
// weight pyramids and multigrid system of
// GridFractionalSinglePhasePressureSolver3 (include/jet/
// grid_fractional_single_phase_pressure_solver3.h:103-115) and the protected
// transfer methods of PicSolver3/FlipSolver3, the access keywords are widened
// for the Jet headers only, after every standard header they use is in place.

#include "oracle_api.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <fstream>
#include <functional>
#include <future>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#define private public
#define protected public
#include <jet/jet.h>
#undef private
#undef protected

using namespace jet;

namespace {

std::shared_ptr<GridFractionalSinglePhasePressureSolver3> g_solver;

std::shared_ptr<ScalarField3> makeField(const orc_field* f) {
    if (f == nullptr || f->kind == 0) {
        return std::make_shared<ConstantScalarField3>(f ? f->value : kMaxD);
    }
    // dataOrigin = origin + h/2 for a cell-centred grid.
    Vector3D h(f->spacing[0], f->spacing[1], f->spacing[2]);
    Vector3D o(f->origin[0] - 0.5 * h.x, f->origin[1] - 0.5 * h.y,
               f->origin[2] - 0.5 * h.z);
    auto grid = std::make_shared<CellCenteredScalarGrid3>(
        Size3(f->res[0], f->res[1], f->res[2]), h, o);
    auto acc = grid->dataAccessor();
    std::memcpy(acc.data(), f->data,
                sizeof(double) * f->res[0] * f->res[1] * f->res[2]);
    return grid;
}

void fillGrid(FaceCenteredGrid3* g, const double* u, const double* v,
              const double* w) {
    auto ua = g->uAccessor();
    auto va = g->vAccessor();
    auto wa = g->wAccessor();
    std::memcpy(ua.data(), u, sizeof(double) * ua.size().x * ua.size().y * ua.size().z);
    std::memcpy(va.data(), v, sizeof(double) * va.size().x * va.size().y * va.size().z);
    std::memcpy(wa.data(), w, sizeof(double) * wa.size().x * wa.size().y * wa.size().z);
}

void readGrid(const FaceCenteredGrid3& g, double* u, double* v, double* w) {
    auto ua = g.uConstAccessor();
    auto va = g.vConstAccessor();
    auto wa = g.wConstAccessor();
    std::memcpy(u, ua.data(), sizeof(double) * ua.size().x * ua.size().y * ua.size().z);
    std::memcpy(v, va.data(), sizeof(double) * va.size().x * va.size().y * va.size().z);
    std::memcpy(w, wa.data(), sizeof(double) * wa.size().x * wa.size().y * wa.size().z);
}

FdmMgpcgSolver3Ptr makeMgpcg(const orc_mg_params* p) {
    return std::make_shared<FdmMgpcgSolver3>(
        p->max_cg_iter, p->max_levels, p->restrict_iter, p->correct_iter,
        p->coarsest_iter, p->final_iter, p->tolerance, p->sor,
        p->red_black != 0);
}

Size3 sz(const int r[3]) { return Size3(r[0], r[1], r[2]); }

void copyIn(FdmMatrix3* A, const double* src) {
    std::memcpy(A->data(), src,
                sizeof(FdmMatrixRow3) * A->size().x * A->size().y * A->size().z);
}

void copyIn(FdmVector3* v, const double* src) {
    std::memcpy(v->data(), src,
                sizeof(double) * v->size().x * v->size().y * v->size().z);
}

void copyOut(const FdmVector3& v, double* dst) {
    std::memcpy(dst, v.data(),
                sizeof(double) * v.size().x * v.size().y * v.size().z);
}

class HarnessFlip : public FlipSolver3 {
 public:
    HarnessFlip(const Size3& res, const Vector3D& h, const Vector3D& o)
        : FlipSolver3(res, h, o) {}
};

}  // namespace

extern "C" {

void orc_set_threads(int n) {
    unsigned t = n > 0 ? (unsigned)n : std::thread::hardware_concurrency();
    setMaxNumberOfThreads(t);
#ifdef _OPENMP
    omp_set_num_threads((int)t);
#endif
    Logging::mute();
}

int orc_pressure_solve(const orc_grid* g, const double* u, const double* v,
                       const double* w, const orc_field* boundary_sdf,
                       const orc_field* fluid_sdf, const double* solid_u,
                       const double* solid_v, const double* solid_w,
                       const orc_mg_params* p, double* out_u, double* out_v,
                       double* out_w, double* out_p, unsigned int* iters,
                       double* resid) {
    Logging::mute();
    Size3 res(g->res[0], g->res[1], g->res[2]);
    Vector3D h(g->spacing[0], g->spacing[1], g->spacing[2]);
    Vector3D o(g->origin[0], g->origin[1], g->origin[2]);
    FaceCenteredGrid3 in(res, h, o);
    fillGrid(&in, u, v, w);
    FaceCenteredGrid3 out(in);

    auto bsdf = makeField(boundary_sdf);
    auto fsdf = makeField(fluid_sdf);

    // Collider velocity: the reference samples it at face positions
    // (grid_fractional_..._solver3.cpp:241-255). A given per-face normal
    // component is replayed through a lookup keyed by the exact face position.
    std::shared_ptr<VectorField3> bvel;
    if (solid_u || solid_v || solid_w) {
        auto uPos = in.uPosition();
        auto vPos = in.vPosition();
        auto wPos = in.wPosition();
        auto table = std::make_shared<std::map<std::array<double, 3>, Vector3D>>();
        auto put = [&](const Vector3D& x, int axis, double val) {
            auto& e = (*table)[{x.x, x.y, x.z}];
            e[axis] = val;
        };
        for (size_t k = 0; k < res.z; ++k)
            for (size_t j = 0; j < res.y; ++j)
                for (size_t i = 0; i <= res.x; ++i)
                    put(uPos(i, j, k), 0,
                        solid_u ? solid_u[i + (res.x + 1) * (j + res.y * k)] : 0.0);
        for (size_t k = 0; k < res.z; ++k)
            for (size_t j = 0; j <= res.y; ++j)
                for (size_t i = 0; i < res.x; ++i)
                    put(vPos(i, j, k), 1,
                        solid_v ? solid_v[i + res.x * (j + (res.y + 1) * k)] : 0.0);
        for (size_t k = 0; k <= res.z; ++k)
            for (size_t j = 0; j < res.y; ++j)
                for (size_t i = 0; i < res.x; ++i)
                    put(wPos(i, j, k), 2,
                        solid_w ? solid_w[i + res.x * (j + res.y * k)] : 0.0);
        bvel = std::make_shared<CustomVectorField3>(
            [table](const Vector3D& x) -> Vector3D {
                auto it = table->find({x.x, x.y, x.z});
                return it == table->end() ? Vector3D() : it->second;
            });
    } else {
        bvel = std::make_shared<ConstantVectorField3>(Vector3D(0, 0, 0));
    }

    g_solver = std::make_shared<GridFractionalSinglePhasePressureSolver3>();
    auto mg = makeMgpcg(p);
    g_solver->setLinearSystemSolver(mg);
    g_solver->solve(in, 1.0, &out, *bsdf, *bvel, *fsdf, false);

    readGrid(out, out_u, out_v, out_w);
    if (out_p) copyOut(g_solver->pressure(), out_p);
    if (iters) *iters = mg->lastNumberOfIterations();
    if (resid) *resid = mg->lastResidual();
    bool ok = mg->lastResidual() <= mg->tolerance() ||
              mg->lastNumberOfIterations() < mg->maxNumberOfIterations();
    return ok ? 1 : 0;
}

int orc_level_count(void) {
    return g_solver ? (int)g_solver->_fluidSdf.size() : 0;
}

long orc_get_level(int level, int what, void* dst, size_t capacity) {
    if (!g_solver || level < 0 || level >= orc_level_count()) return -1;
    // Copies n elements of `size` bytes if they fit the caller's buffer.
    auto put = [&](const void* src, long n, size_t size) -> long {
        if ((size_t)n * size > capacity) return -2;
        std::memcpy(dst, src, (size_t)n * size);
        return n;
    };
    auto copyF = [&](const Array3<float>& a) {
        return put(a.data(), (long)(a.size().x * a.size().y * a.size().z),
                   sizeof(float));
    };
    switch (what) {
        case 0: return copyF(g_solver->_fluidSdf[level]);
        case 1: return copyF(g_solver->_uWeights[level]);
        case 2: return copyF(g_solver->_vWeights[level]);
        case 3: return copyF(g_solver->_wWeights[level]);
        case 4: {
            const auto& A = g_solver->_mgSystem.A.levels[level];
            return put(A.data(), (long)(A.size().x * A.size().y * A.size().z),
                       sizeof(FdmMatrixRow3));
        }
        case 5: {
            const auto& b = g_solver->_mgSystem.b.levels[level];
            return put(b.data(), (long)(b.size().x * b.size().y * b.size().z),
                       sizeof(double));
        }
        default: return -1;
    }
}

std::shared_ptr<GridSinglePhasePressureSolver3> g_blocked;

int orc_blocked_pressure_solve(const orc_grid* g, const double* u,
                               const double* v, const double* w,
                               const orc_field* boundary_sdf,
                               const orc_field* fluid_sdf,
                               const orc_mg_params* p, double* out_u,
                               double* out_v, double* out_w, double* out_p,
                               unsigned int* iters, double* resid) {
    Logging::mute();
    Size3 res(g->res[0], g->res[1], g->res[2]);
    Vector3D h(g->spacing[0], g->spacing[1], g->spacing[2]);
    Vector3D o(g->origin[0], g->origin[1], g->origin[2]);
    FaceCenteredGrid3 in(res, h, o);
    fillGrid(&in, u, v, w);
    FaceCenteredGrid3 out(in);
    auto bsdf = makeField(boundary_sdf);
    auto fsdf = makeField(fluid_sdf);
    g_blocked = std::make_shared<GridSinglePhasePressureSolver3>();
    auto mg = makeMgpcg(p);
    g_blocked->setLinearSystemSolver(mg);
    g_blocked->solve(in, 1.0, &out, *bsdf, ConstantVectorField3({0, 0, 0}),
                     *fsdf, false);
    readGrid(out, out_u, out_v, out_w);
    if (out_p) copyOut(g_blocked->pressure(), out_p);
    if (iters) *iters = mg->lastNumberOfIterations();
    if (resid) *resid = mg->lastResidual();
    bool ok = mg->lastResidual() <= mg->tolerance() ||
              mg->lastNumberOfIterations() < mg->maxNumberOfIterations();
    return ok ? 1 : 0;
}

long orc_blocked_get_level(int level, int what, void* dst) {
    if (!g_blocked || level < 0 ||
        level >= (int)g_blocked->_markers.size())
        return -1;
    switch (what) {
        case 0: {
            const auto& m = g_blocked->_markers[level];
            long n = (long)(m.size().x * m.size().y * m.size().z);
            std::memcpy(dst, m.data(), n);
            return n;
        }
        case 4: {
            const auto& A = g_blocked->_mgSystem.A.levels[level];
            long n = (long)(A.size().x * A.size().y * A.size().z);
            std::memcpy(dst, A.data(), n * sizeof(FdmMatrixRow3));
            return n;
        }
        case 5: {
            const auto& b = g_blocked->_mgSystem.b.levels[level];
            long n = (long)(b.size().x * b.size().y * b.size().z);
            std::memcpy(dst, b.data(), n * sizeof(double));
            return n;
        }
        default: return -1;
    }
}

int orc_mgpcg_system(const int res0[3], int levels, const double* A,
                     const double* b, const orc_mg_params* p, double* x0,
                     unsigned int* iters, double* resid) {
    Logging::mute();
    FdmMgLinearSystem3 system;
    Size3 coarsest(res0[0] >> (levels - 1), res0[1] >> (levels - 1),
                   res0[2] >> (levels - 1));
    system.resizeWithCoarsest(coarsest, levels);
    long off = 0;
    for (int l = 0; l < levels; ++l) {
        Size3 s = system.A[l].size();
        long n = (long)(s.x * s.y * s.z);
        copyIn(&system.A[l], A + 4 * off);
        copyIn(&system.b[l], b + off);
        system.x[l].set(0.0);
        off += n;
    }
    auto mg = makeMgpcg(p);
    bool ok = mg->solve(&system);
    copyOut(system.x[0], x0);
    if (iters) *iters = mg->lastNumberOfIterations();
    if (resid) *resid = mg->lastResidual();
    return ok ? 1 : 0;
}

void orc_relax(const int res[3], const double* A, const double* b, double sor,
               int red_black, int sweeps, double* x) {
    FdmMatrix3 M(sz(res));
    FdmVector3 B(sz(res)), X(sz(res));
    copyIn(&M, A);
    copyIn(&B, b);
    copyIn(&X, x);
    for (int it = 0; it < sweeps; ++it) {
        if (red_black)
            FdmGaussSeidelSolver3::relaxRedBlack(M, B, sor, &X);
        else
            FdmGaussSeidelSolver3::relax(M, B, sor, &X);
    }
    copyOut(X, x);
}

void orc_mg_restrict(const int coarse_res[3], const double* finer,
                     double* coarser) {
    Size3 c = sz(coarse_res);
    FdmVector3 F(Size3(2 * c.x, 2 * c.y, 2 * c.z)), C(c);
    copyIn(&F, finer);
    FdmMgUtils3::restrict(F, &C);
    copyOut(C, coarser);
}

void orc_mg_correct(const int coarse_res[3], const double* coarser,
                    double* finer) {
    Size3 c = sz(coarse_res);
    FdmVector3 F(Size3(2 * c.x, 2 * c.y, 2 * c.z)), C(c);
    copyIn(&C, coarser);
    copyIn(&F, finer);
    FdmMgUtils3::correct(C, &F);
    copyOut(F, finer);
}

void orc_residual(const int res[3], const double* A, const double* x,
                  const double* b, double* r) {
    FdmMatrix3 M(sz(res));
    FdmVector3 X(sz(res)), B(sz(res)), R(sz(res));
    copyIn(&M, A);
    copyIn(&X, x);
    copyIn(&B, b);
    FdmBlas3::residual(M, X, B, &R);
    copyOut(R, r);
}

double orc_dot(long n, const double* a, const double* b) {
    FdmVector3 A(Size3(n, 1, 1)), B(Size3(n, 1, 1));
    copyIn(&A, a);
    copyIn(&B, b);
    return FdmBlas3::dot(A, B);
}

static std::unique_ptr<HarnessFlip> makeFlip(const orc_grid* g, long np,
                                             const double* pos,
                                             const double* vel) {
    Logging::mute();
    auto s = std::make_unique<HarnessFlip>(
        Size3(g->res[0], g->res[1], g->res[2]),
        Vector3D(g->spacing[0], g->spacing[1], g->spacing[2]),
        Vector3D(g->origin[0], g->origin[1], g->origin[2]));
    auto particles = s->particleSystemData();
    Array1<Vector3D> P(np), V(np), F(np);
    for (long i = 0; i < np; ++i) {
        P[i] = Vector3D(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        V[i] = Vector3D(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
    }
    particles->addParticles(P.constAccessor(), V.constAccessor(),
                            F.constAccessor());
    return s;
}

void orc_p2g(const orc_grid* g, long np, const double* pos, const double* vel,
             double* u, double* v, double* w, char* mu, char* mv, char* mw,
             float* snap_u, float* snap_v, float* snap_w) {
    auto s = makeFlip(g, np, pos, vel);
    s->transferFromParticlesToGrids();
    readGrid(*s->gridSystemData()->velocity(), u, v, w);
    auto cpyc = [](const Array3<char>& a, char* d) {
        if (d) std::memcpy(d, a.data(), a.size().x * a.size().y * a.size().z);
    };
    cpyc(s->_uMarkers, mu);
    cpyc(s->_vMarkers, mv);
    cpyc(s->_wMarkers, mw);
    auto cpyf = [](const Array3<float>& a, float* d) {
        if (d)
            std::memcpy(d, a.data(),
                        sizeof(float) * a.size().x * a.size().y * a.size().z);
    };
    cpyf(s->_uDelta, snap_u);
    cpyf(s->_vDelta, snap_v);
    cpyf(s->_wDelta, snap_w);
}

void orc_g2p_flip(const orc_grid* g, long np, const double* pos, double* vel,
                  const double* u, const double* v, const double* w,
                  float* snap_u, float* snap_v, float* snap_w,
                  double pic_blend) {
    auto s = makeFlip(g, np, pos, vel);
    s->setPicBlendingFactor(pic_blend);
    auto flow = s->gridSystemData()->velocity();
    fillGrid(flow.get(), u, v, w);
    auto setf = [](Array3<float>* a, const Size3& sz, const float* src) {
        a->resize(sz);
        std::memcpy(a->data(), src, sizeof(float) * sz.x * sz.y * sz.z);
    };
    setf(&s->_uDelta, flow->uSize(), snap_u);
    setf(&s->_vDelta, flow->vSize(), snap_v);
    setf(&s->_wDelta, flow->wSize(), snap_w);
    s->transferFromGridsToParticles();
    auto vels = s->particleSystemData()->velocities();
    for (long i = 0; i < np; ++i) {
        vel[3 * i] = vels[i].x;
        vel[3 * i + 1] = vels[i].y;
        vel[3 * i + 2] = vels[i].z;
    }
    auto cpyf = [](const Array3<float>& a, float* d) {
        std::memcpy(d, a.data(),
                    sizeof(float) * a.size().x * a.size().y * a.size().z);
    };
    cpyf(s->_uDelta, snap_u);
    cpyf(s->_vDelta, snap_v);
    cpyf(s->_wDelta, snap_w);
}

void orc_g2p_pic(const orc_grid* g, long np, const double* pos, double* vel,
                 const double* u, const double* v, const double* w) {
    Logging::mute();
    auto s = std::make_unique<PicSolver3>(
        Size3(g->res[0], g->res[1], g->res[2]),
        Vector3D(g->spacing[0], g->spacing[1], g->spacing[2]),
        Vector3D(g->origin[0], g->origin[1], g->origin[2]));
    auto particles = s->particleSystemData();
    Array1<Vector3D> P(np), V(np), F(np);
    for (long i = 0; i < np; ++i) {
        P[i] = Vector3D(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        V[i] = Vector3D(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
    }
    particles->addParticles(P.constAccessor(), V.constAccessor(),
                            F.constAccessor());
    fillGrid(s->gridSystemData()->velocity().get(), u, v, w);
    s->transferFromGridsToParticles();
    auto vels = s->particleSystemData()->velocities();
    for (long i = 0; i < np; ++i) {
        vel[3 * i] = vels[i].x;
        vel[3 * i + 1] = vels[i].y;
        vel[3 * i + 2] = vels[i].z;
    }
}

namespace {
// A rigid sphere collider, so that Collider3::velocityAt and
// frictionCoefficient answer as `col` says (the surface only sets the
// rotation centre; the solver's SDF is replaced by the caller's grid).
std::shared_ptr<RigidBodyCollider3> makeCollider(const orc_collider* col,
                                                 double radius) {
    auto sphere = std::make_shared<Sphere3>(Vector3D(), radius);
    if (col)
        sphere->transform.setTranslation(
            Vector3D(col->centre[0], col->centre[1], col->centre[2]));
    auto c = std::make_shared<RigidBodyCollider3>(sphere);
    if (col) {
        c->linearVelocity = Vector3D(col->lin[0], col->lin[1], col->lin[2]);
        c->angularVelocity = Vector3D(col->ang[0], col->ang[1], col->ang[2]);
        c->setFrictionCoefficient(col->friction);
    }
    return c;
}
}  // namespace

void orc_constrain_velocity(const orc_grid* g, double* u, double* v,
                            double* w, const orc_field* sdf,
                            const orc_collider* col, int closed,
                            unsigned int depth) {
    Logging::mute();
    const Size3 res(g->res[0], g->res[1], g->res[2]);
    const Vector3D h(g->spacing[0], g->spacing[1], g->spacing[2]);
    const Vector3D o(g->origin[0], g->origin[1], g->origin[2]);
    FaceCenteredGrid3 vel(res, h, o);
    fillGrid(&vel, u, v, w);
    GridFractionalBoundaryConditionSolver3 bc;
    bc.updateCollider(col ? makeCollider(col, 0.1) : nullptr, res, h, o);
    // Replace the collider SDF with the caller's samples (same grid).
    if (sdf && sdf->kind == 1) {
        auto acc = bc._colliderSdf->dataAccessor();
        std::memcpy(acc.data(), sdf->data,
                    sizeof(double) * res.x * res.y * res.z);
    } else {
        bc._colliderSdf->fill(sdf ? sdf->value : kMaxD);
    }
    bc.setClosedDomainBoundaryFlag(closed);
    bc.constrainVelocity(&vel, depth);
    readGrid(vel, u, v, w);
}

void orc_constrain_velocity_blocked(const orc_grid* g, double* u, double* v,
                                    double* w, const orc_field* sdf,
                                    const orc_collider* col, int closed,
                                    unsigned int depth) {
    Logging::mute();
    const Size3 res(g->res[0], g->res[1], g->res[2]);
    const Vector3D h(g->spacing[0], g->spacing[1], g->spacing[2]);
    const Vector3D o(g->origin[0], g->origin[1], g->origin[2]);
    FaceCenteredGrid3 vel(res, h, o);
    fillGrid(&vel, u, v, w);
    GridBlockedBoundaryConditionSolver3 bc;
    bc.updateCollider(col ? makeCollider(col, 0.1) : nullptr, res, h, o);
    // Replace the collider SDF with the caller's samples (same grid) and
    // re-derive the cell markers from it with onColliderUpdated's rule
    // (grid_blocked_boundary_condition_solver3.cpp:79-90).
    if (sdf && sdf->kind == 1) {
        auto acc = bc._colliderSdf->dataAccessor();
        std::memcpy(acc.data(), sdf->data,
                    sizeof(double) * res.x * res.y * res.z);
    } else {
        bc._colliderSdf->fill(sdf ? sdf->value : kMaxD);
    }
    const auto grid =
        std::dynamic_pointer_cast<CellCenteredScalarGrid3>(bc.colliderSdf());
    bc._marker.forEachIndex([&](size_t i, size_t j, size_t k) {
        bc._marker(i, j, k) = isInsideSdf((*grid)(i, j, k)) ? 0 : 1;
    });
    bc.setClosedDomainBoundaryFlag(closed);
    bc.constrainVelocity(&vel, depth);
    readGrid(vel, u, v, w);
}

void orc_extrapolate(const int res[3], double* data, const char* valid,
                     unsigned int iterations) {
    const Size3 s(res[0], res[1], res[2]);
    Array3<double> in(s), out(s);
    Array3<char> mk(s);
    std::memcpy(in.data(), data, sizeof(double) * s.x * s.y * s.z);
    std::memcpy(mk.data(), valid, s.x * s.y * s.z);
    extrapolateToRegion(in.constAccessor(), mk.constAccessor(), iterations,
                        out.accessor());
    std::memcpy(data, out.data(), sizeof(double) * s.x * s.y * s.z);
}

void orc_move_particles(const orc_grid* g, long np, double* pos, double* vel,
                        const double* u, const double* v, const double* w,
                        double dt, double max_cfl, int closed,
                        const orc_collider* col, const orc_sphere* sph) {
    Logging::mute();
    auto s = std::make_unique<PicSolver3>(
        Size3(g->res[0], g->res[1], g->res[2]),
        Vector3D(g->spacing[0], g->spacing[1], g->spacing[2]),
        Vector3D(g->origin[0], g->origin[1], g->origin[2]));
    auto particles = s->particleSystemData();
    Array1<Vector3D> P(np), V(np), F(np);
    for (long i = 0; i < np; ++i) {
        P[i] = Vector3D(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        V[i] = Vector3D(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
    }
    particles->addParticles(P.constAccessor(), V.constAccessor(),
                            F.constAccessor());
    fillGrid(s->gridSystemData()->velocity().get(), u, v, w);
    s->setMaxCfl(max_cfl);
    s->setClosedDomainBoundaryFlag(closed);
    if (col && sph) {
        auto sphere = std::make_shared<Sphere3>(
            Vector3D(sph->center[0], sph->center[1], sph->center[2]),
            sph->radius,
            Transform3(Vector3D(col->centre[0], col->centre[1], col->centre[2]),
                       QuaternionD(sph->quat[0], sph->quat[1], sph->quat[2],
                                   sph->quat[3])),
            sph->normal_flipped != 0);
        auto c = std::make_shared<RigidBodyCollider3>(sphere);
        c->linearVelocity = Vector3D(col->lin[0], col->lin[1], col->lin[2]);
        c->angularVelocity = Vector3D(col->ang[0], col->ang[1], col->ang[2]);
        c->setFrictionCoefficient(col->friction);
        // Installed directly: setCollider would also rebuild the boundary
        // solver, which moveParticles does not use.
        s->_collider = c;
    }
    s->moveParticles(dt);
    auto ps = s->particleSystemData()->positions();
    auto vs = s->particleSystemData()->velocities();
    for (long i = 0; i < np; ++i) {
        for (int d = 0; d < 3; ++d) {
            pos[3 * i + d] = ps[i][d];
            vel[3 * i + d] = vs[i][d];
        }
    }
}

void orc_build_particle_sdf(const orc_grid* g, long np, const double* pos,
                            const orc_field* collider_sdf, double max_cfl,
                            double* out) {
    Logging::mute();
    const Size3 res(g->res[0], g->res[1], g->res[2]);
    const Vector3D h(g->spacing[0], g->spacing[1], g->spacing[2]);
    const Vector3D o(g->origin[0], g->origin[1], g->origin[2]);
    auto s = std::make_unique<PicSolver3>(res, h, o);
    auto particles = s->particleSystemData();
    Array1<Vector3D> P(np), V(np), F(np);
    for (long i = 0; i < np; ++i)
        P[i] = Vector3D(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    particles->addParticles(P.constAccessor(), V.constAccessor(),
                            F.constAccessor());
    s->setMaxCfl(max_cfl);
    // The collider SDF the boundary solver holds, replaced by the caller's.
    auto bc = std::dynamic_pointer_cast<GridFractionalBoundaryConditionSolver3>(
        s->_boundaryConditionSolver);
    bc->updateCollider(nullptr, res, h, o);
    if (collider_sdf && collider_sdf->kind == 1) {
        auto acc = bc->_colliderSdf->dataAccessor();
        std::memcpy(acc.data(), collider_sdf->data,
                    sizeof(double) * res.x * res.y * res.z);
    } else {
        bc->_colliderSdf->fill(collider_sdf ? collider_sdf->value : kMaxD);
    }
    s->buildSignedDistanceField();
    auto acc = s->signedDistanceField()->constDataAccessor();
    std::memcpy(out, acc.data(), sizeof(double) * res.x * res.y * res.z);
}

namespace {
std::unique_ptr<ApicSolver3> makeApic(const orc_grid* g, long np,
                                      const double* pos, const double* vel) {
    Logging::mute();
    auto s = std::make_unique<ApicSolver3>(
        Size3(g->res[0], g->res[1], g->res[2]),
        Vector3D(g->spacing[0], g->spacing[1], g->spacing[2]),
        Vector3D(g->origin[0], g->origin[1], g->origin[2]));
    Array1<Vector3D> P(np), V(np), F(np);
    for (long i = 0; i < np; ++i) {
        P[i] = Vector3D(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        V[i] = Vector3D(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
    }
    s->particleSystemData()->addParticles(P.constAccessor(), V.constAccessor(),
                                          F.constAccessor());
    return s;
}
}  // namespace

void orc_apic_p2g(const orc_grid* g, long np, const double* pos,
                  const double* vel, const double* affine, double* u,
                  double* v, double* w, char* mu, char* mv, char* mw) {
    auto s = makeApic(g, np, pos, vel);
    s->_cX.resize(np);
    s->_cY.resize(np);
    s->_cZ.resize(np);
    for (long i = 0; i < np; ++i) {
        const double* c = affine + 9 * i;
        s->_cX[i] = Vector3D(c[0], c[1], c[2]);
        s->_cY[i] = Vector3D(c[3], c[4], c[5]);
        s->_cZ[i] = Vector3D(c[6], c[7], c[8]);
    }
    s->transferFromParticlesToGrids();
    readGrid(*s->gridSystemData()->velocity(), u, v, w);
    auto cpyc = [](const Array3<char>& a, char* d) {
        if (d) std::memcpy(d, a.data(), a.size().x * a.size().y * a.size().z);
    };
    cpyc(s->_uMarkers, mu);
    cpyc(s->_vMarkers, mv);
    cpyc(s->_wMarkers, mw);
}

void orc_apic_g2p(const orc_grid* g, long np, const double* pos, double* vel,
                  double* affine, const double* u, const double* v,
                  const double* w) {
    auto s = makeApic(g, np, pos, vel);
    fillGrid(s->gridSystemData()->velocity().get(), u, v, w);
    s->transferFromGridsToParticles();
    auto vs = s->particleSystemData()->velocities();
    for (long i = 0; i < np; ++i) {
        for (int d = 0; d < 3; ++d) {
            vel[3 * i + d] = vs[i][d];
            affine[9 * i + d] = s->_cX[i][d];
            affine[9 * i + 3 + d] = s->_cY[i][d];
            affine[9 * i + 6 + d] = s->_cZ[i][d];
        }
    }
}

void orc_flip_run(const orc_grid* g, long np, double* pos, double* vel,
                  int frames, double fps, double max_cfl, int closed,
                  const double gravity[3], int flip, const orc_mg_params* p) {
    orc_flip_run_record(g, np, pos, vel, frames, fps, max_cfl, closed,
                        gravity, flip, p, 0, nullptr, nullptr);
}

namespace {
// The harness's FLIP/PIC/APIC run, with an optional static sphere collider
// (RigidBodyCollider3 over Sphere3 of `radius` at `centre`, friction
// `friction`; GridFluidSolver3::setCollider).
void flip_run_impl(const orc_grid* g, long np, double* pos, double* vel,
                   int frames, double fps, double max_cfl, int closed,
                   const double gravity[3], int flip, const orc_mg_params* p,
                   int nrec, const int* rec_frames, double* p_out,
                   const double* centre, double radius, double friction) {
    Logging::mute();
    const Size3 res(g->res[0], g->res[1], g->res[2]);
    const Vector3D h(g->spacing[0], g->spacing[1], g->spacing[2]);
    const Vector3D o(g->origin[0], g->origin[1], g->origin[2]);
    std::shared_ptr<PicSolver3> s;
    if (flip == 1)
        s = std::make_shared<FlipSolver3>(res, h, o);
    else if (flip == 2)
        s = std::make_shared<ApicSolver3>(res, h, o);
    else
        s = std::make_shared<PicSolver3>(res, h, o);
    auto particles = s->particleSystemData();
    Array1<Vector3D> P(np), V(np), F(np);
    for (long i = 0; i < np; ++i) {
        P[i] = Vector3D(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        V[i] = Vector3D(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
    }
    particles->addParticles(P.constAccessor(), V.constAccessor(),
                            F.constAccessor());
    s->setGravity(Vector3D(gravity[0], gravity[1], gravity[2]));
    s->setMaxCfl(max_cfl);
    s->setClosedDomainBoundaryFlag(closed);
    auto ps = std::make_shared<GridFractionalSinglePhasePressureSolver3>();
    ps->setLinearSystemSolver(std::make_shared<FdmMgpcgSolver3>(
        p->max_cg_iter, p->max_levels, p->restrict_iter, p->correct_iter,
        p->coarsest_iter, p->final_iter, p->tolerance, p->sor,
        p->red_black != 0));
    s->setPressureSolver(ps);
    if (centre) {
        orc_collider c{{0, 0, 0}, {0, 0, 0}, {centre[0], centre[1], centre[2]},
                       friction};
        s->setCollider(makeCollider(&c, radius));
    }
    const size_t cells = res.x * res.y * res.z;
    int next = 0;
    for (Frame frame(0, 1.0 / fps); frame.index < frames; ++frame) {
        s->update(frame);
        if (next < nrec && rec_frames[next] == frame.index + 1) {
            const FdmVector3& pr = ps->pressure();
            std::memcpy(p_out + cells * next, pr.data(),
                        sizeof(double) * cells);
            ++next;
        }
    }
    auto pp = s->particleSystemData()->positions();
    auto vv = s->particleSystemData()->velocities();
    for (long i = 0; i < np; ++i)
        for (int d = 0; d < 3; ++d) {
            pos[3 * i + d] = pp[i][d];
            vel[3 * i + d] = vv[i][d];
        }
}
}  // namespace

void orc_flip_run_record(const orc_grid* g, long np, double* pos, double* vel,
                         int frames, double fps, double max_cfl, int closed,
                         const double gravity[3], int flip,
                         const orc_mg_params* p, int nrec,
                         const int* rec_frames, double* p_out) {
    flip_run_impl(g, np, pos, vel, frames, fps, max_cfl, closed, gravity, flip,
                  p, nrec, rec_frames, p_out, nullptr, 0.0, 0.0);
}

void orc_flip_run_sphere(const orc_grid* g, long np, double* pos, double* vel,
                         int frames, double fps, double max_cfl, int closed,
                         const double gravity[3], int flip,
                         const orc_mg_params* p, const double centre[3],
                         double radius, double friction) {
    flip_run_impl(g, np, pos, vel, frames, fps, max_cfl, closed, gravity, flip,
                  p, 0, nullptr, nullptr, centre, radius, friction);
}

void orc_quaternion_matrices(const double q[4], double orient[9],
                             double inv_orient[9]) {
    Transform3 t(Vector3D(), QuaternionD(q[0], q[1], q[2], q[3]));
    for (int i = 0; i < 9; ++i) {
        orient[i] = t._orientationMat3[i];
        inv_orient[i] = t._inverseOrientationMat3[i];
    }
}

void orc_sphere_collider_sdf(const orc_grid* g, const double centre[3],
                             double radius, double* out) {
    const Size3 res(g->res[0], g->res[1], g->res[2]);
    const Vector3D h(g->spacing[0], g->spacing[1], g->spacing[2]);
    const Vector3D o(g->origin[0], g->origin[1], g->origin[2]);
    orc_collider c{{0, 0, 0}, {0, 0, 0}, {centre[0], centre[1], centre[2]}, 0};
    GridFractionalBoundaryConditionSolver3 bc;
    bc.updateCollider(makeCollider(&c, radius), res, h, o);
    auto acc = bc._colliderSdf->constDataAccessor();
    std::memcpy(out, acc.data(), sizeof(double) * res.x * res.y * res.z);
}

}  // extern "C"
