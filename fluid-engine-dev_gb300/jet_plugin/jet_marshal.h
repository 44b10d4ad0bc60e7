// Argument marshalling shared by the C++ drop-ins: Jet grids and fields to
// the plain structs of the C ABI (include/jetgpu.h), and the GPU
// constrainVelocity call of both boundary-condition solvers.
#ifndef JETGPU_JET_MARSHAL_H_
#define JETGPU_JET_MARSHAL_H_

#include <jet/cell_centered_scalar_grid3.h>
#include <jet/constant_scalar_field3.h>
#include <jet/face_centered_grid3.h>
#include <jet/grid_fractional_boundary_condition_solver3.h>
#include <jet/rigid_body_collider3.h>

#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "jetgpu.h"

namespace jetgpu_jet {

//! Resolution, spacing and origin of a face-centred grid.
inline jetgpu_grid grid_of(const jet::FaceCenteredGrid3& grid) {
    jetgpu_grid g;
    const jet::Size3 res = grid.resolution();
    const jet::Vector3D h = grid.gridSpacing(), o = grid.origin();
    for (int d = 0; d < 3; ++d) {
        g.res[d] = (int)res[d];
        g.spacing[d] = h[d];
        g.origin[d] = o[d];
    }
    return g;
}

//! A ScalarField3 argument of GridPressureSolver3::solve. Constants and
//! CellCenteredScalarGrid3 pass as they are, the grid's own data pointer
//! included (nothing is copied on the host; the GPU samples grids with Jet's
//! exact trilinear rule); any other field is rasterised at the velocity
//! grid's cell centres into `raster`, which keeps that data alive.
inline jetgpu_scalar_field describe_field(const jet::ScalarField3& field,
                                          const jet::FaceCenteredGrid3& grid,
                                          std::vector<double>* raster) {
    using namespace jet;
    jetgpu_scalar_field f;
    std::memset(&f, 0, sizeof(f));
    if (auto c = dynamic_cast<const ConstantScalarField3*>(&field)) {
        f.kind = 0;
        f.value = c->sample(Vector3D());
        return f;
    }
    const CellCenteredScalarGrid3* g =
        dynamic_cast<const CellCenteredScalarGrid3*>(&field);
    std::shared_ptr<CellCenteredScalarGrid3> owned;
    if (!g) {
        owned = std::make_shared<CellCenteredScalarGrid3>(
            grid.resolution(), grid.gridSpacing(), grid.origin());
        owned->fill([&](const Vector3D& x) { return field.sample(x); });
        g = owned.get();
    }
    const Size3 r = g->resolution();
    auto acc = g->constDataAccessor();
    f.kind = 1;
    if (owned) {
        raster->assign(acc.data(), acc.data() + r.x * r.y * r.z);
        f.data = raster->data();
    } else {
        f.data = acc.data();
    }
    const Vector3D o = g->dataOrigin(), h = g->gridSpacing();
    for (int d = 0; d < 3; ++d) {
        f.res[d] = (int)r[d];
        f.origin[d] = o[d];
        f.spacing[d] = h[d];
    }
    return f;
}

//! The motion of a rigid collider as the C ABI takes it (velocityAt =
//! linear + angular x (p - translation), src/jet/rigid_body_collider3.cpp:
//! 25-28).
inline jetgpu_collider rigid_motion(const jet::RigidBodyCollider3& rigid) {
    jetgpu_collider col{};
    const jet::Vector3D t = rigid.surface()->transform.translation();
    for (int d = 0; d < 3; ++d) {
        col.linear_velocity[d] = rigid.linearVelocity[d];
        col.angular_velocity[d] = rigid.angularVelocity[d];
        col.centre[d] = t[d];
    }
    col.friction = rigid.frictionCoefficient();
    return col;
}

//! Creates the context on first use; throws when that fails.
inline void ensure_context(const jetgpu_config& cfg, jetgpu_ctx** ctx,
                           jetgpu_status* status) {
    if (*ctx) return;
    *status = jetgpu_create(&cfg, ctx);
    if (*status != JETGPU_OK) {
        *ctx = nullptr;
        throw std::runtime_error("jetgpu_create failed with status " +
                                 std::to_string(*status));
    }
}

//! constrainVelocity of a fractional (blocked = false) or blocked boundary
//! solver on the GPU: the collider SDF is the solver's colliderSdf(),
//! rebuilt as the reference does when the resolution changes
//! (grid_fractional_boundary_condition_solver3.cpp:29-36); the collider must
//! be a RigidBodyCollider3 (or none).
inline void constrain_on_gpu(jet::GridFractionalBoundaryConditionSolver3& bc,
                             const jetgpu_config& cfg, jetgpu_ctx** ctx,
                             jetgpu_status* status,
                             jet::FaceCenteredGrid3* velocity,
                             unsigned int depth, bool blocked) {
    using namespace jet;
    const Size3 size = velocity->resolution();
    auto sdf = std::dynamic_pointer_cast<CellCenteredScalarGrid3>(bc.colliderSdf());
    if (!sdf || sdf->resolution() != size) {
        bc.updateCollider(bc.collider(), size, velocity->gridSpacing(),
                          velocity->origin());
        sdf = std::dynamic_pointer_cast<CellCenteredScalarGrid3>(bc.colliderSdf());
    }
    jetgpu_collider col{};
    const jetgpu_collider* colp = nullptr;
    if (bc.collider()) {
        auto rigid = std::dynamic_pointer_cast<RigidBodyCollider3>(bc.collider());
        if (!rigid)
            throw std::invalid_argument(
                "the GPU boundary-condition solvers take rigid colliders "
                "(RigidBodyCollider3) only");
        col = rigid_motion(*rigid);
        colp = &col;
    }
    ensure_context(cfg, ctx, status);
    const jetgpu_grid g = grid_of(*velocity);
    jetgpu_scalar_field f;
    std::memset(&f, 0, sizeof(f));
    const Vector3D d0 = sdf->dataOrigin();
    f.kind = 1;
    f.data = sdf->constDataAccessor().data();
    for (int d = 0; d < 3; ++d) {
        f.res[d] = (int)size[d];
        f.origin[d] = d0[d];
        f.spacing[d] = sdf->gridSpacing()[d];
    }
    auto u = velocity->uAccessor();
    auto v = velocity->vAccessor();
    auto w = velocity->wAccessor();
    *status = (blocked ? jetgpu_constrain_velocity_blocked
                       : jetgpu_constrain_velocity)(
        *ctx, &g, u.data(), v.data(), w.data(), &f, colp,
        bc.closedDomainBoundaryFlag(), depth);
    if (*status != JETGPU_OK)
        throw std::runtime_error(std::string("constrainVelocity on the GPU: ") +
                                 jetgpu_last_error(*ctx));
}

}  // namespace jetgpu_jet

#endif  // JETGPU_JET_MARSHAL_H_
