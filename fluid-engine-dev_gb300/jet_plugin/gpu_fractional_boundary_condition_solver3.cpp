// GPU drop-in for Jet's GridFractionalBoundaryConditionSolver3: argument
// marshalling onto jetgpu_constrain_velocity. See
// gpu_fractional_boundary_condition_solver3.h.
#include "gpu_fractional_boundary_condition_solver3.h"

#include <jet/cell_centered_scalar_grid3.h>
#include <jet/face_centered_grid3.h>
#include <jet/rigid_body_collider3.h>

#include <memory>
#include <stdexcept>
#include <string>

namespace jetgpu_jet {

using namespace jet;

GpuFractionalBoundaryConditionSolver3::GpuFractionalBoundaryConditionSolver3(
    const jetgpu_config* cfg) {
    jetgpu_config_default(&_config);
    if (cfg) _config = *cfg;
}

GpuFractionalBoundaryConditionSolver3::
    ~GpuFractionalBoundaryConditionSolver3() {
    if (_ctx) jetgpu_destroy(_ctx);
}

void GpuFractionalBoundaryConditionSolver3::constrainVelocity(
    FaceCenteredGrid3* velocity, unsigned int extrapolationDepth) {
    const Size3 size = velocity->resolution();
    // The collider SDF on this grid, rebuilt as the reference does when the
    // resolution changes (:29-36).
    auto sdf = std::dynamic_pointer_cast<CellCenteredScalarGrid3>(colliderSdf());
    if (!sdf || sdf->resolution() != size) {
        updateCollider(collider(), size, velocity->gridSpacing(),
                       velocity->origin());
        sdf = std::dynamic_pointer_cast<CellCenteredScalarGrid3>(colliderSdf());
    }
    jetgpu_collider col{};
    const jetgpu_collider* colp = nullptr;
    if (collider()) {
        auto rigid = std::dynamic_pointer_cast<RigidBodyCollider3>(collider());
        if (!rigid)
            throw std::invalid_argument(
                "GpuFractionalBoundaryConditionSolver3: the GPU takes rigid "
                "colliders (RigidBodyCollider3) only");
        const Vector3D t = rigid->surface()->transform.translation();
        for (int d = 0; d < 3; ++d) {
            col.linear_velocity[d] = rigid->linearVelocity[d];
            col.angular_velocity[d] = rigid->angularVelocity[d];
            col.centre[d] = t[d];
        }
        col.friction = rigid->frictionCoefficient();
        colp = &col;
    }
    if (!_ctx) {
        _status = jetgpu_create(&_config, &_ctx);
        if (_status != JETGPU_OK) {
            _ctx = nullptr;
            throw std::runtime_error("jetgpu_create failed with status " +
                                     std::to_string(_status));
        }
    }
    jetgpu_grid g;
    jetgpu_scalar_field f;
    const Vector3D h = velocity->gridSpacing(), o = velocity->origin();
    const Vector3D d0 = sdf->dataOrigin();
    f.kind = 1;
    f.value = 0.0;
    f.data = sdf->constDataAccessor().data();
    for (int d = 0; d < 3; ++d) {
        g.res[d] = (int)size[d];
        g.spacing[d] = h[d];
        g.origin[d] = o[d];
        f.res[d] = (int)size[d];
        f.origin[d] = d0[d];
        f.spacing[d] = sdf->gridSpacing()[d];
    }
    auto u = velocity->uAccessor();
    auto v = velocity->vAccessor();
    auto w = velocity->wAccessor();
    _status = jetgpu_constrain_velocity(
        _ctx, &g, u.data(), v.data(), w.data(), &f, colp,
        closedDomainBoundaryFlag(), extrapolationDepth);
    if (_status != JETGPU_OK)
        throw std::runtime_error(std::string("jetgpu_constrain_velocity: ") +
                                 jetgpu_last_error(_ctx));
}

}  // namespace jetgpu_jet
