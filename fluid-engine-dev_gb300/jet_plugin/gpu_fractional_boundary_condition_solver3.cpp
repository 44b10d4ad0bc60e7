// GPU drop-in for Jet's GridFractionalBoundaryConditionSolver3: argument
// marshalling onto jetgpu_constrain_velocity. See
// gpu_fractional_boundary_condition_solver3.h.
#include "gpu_fractional_boundary_condition_solver3.h"

#include "jet_marshal.h"

#include <jet/rigid_body_collider3.h>

namespace jetgpu_jet {

jet::Vector3D GpuColliderVelocityField3::sample(const jet::Vector3D& x) const {
    const jet::Collider3Ptr& c = collider();
    return c ? c->velocityAt(x) : jet::Vector3D();
}

double GpuColliderVelocityField3::divergence(const jet::Vector3D& x) const {
    const jet::Collider3Ptr& c = collider();
    if (!c || std::dynamic_pointer_cast<jet::RigidBodyCollider3>(c))
        return 0.0;
    // Central differences at a small step, as a field without an analytic
    // derivative is differentiated.
    const double h = 1e-4;
    double d = 0.0;
    for (int a = 0; a < 3; ++a) {
        jet::Vector3D e;
        e[a] = h;
        d += (sample(x + e)[a] - sample(x - e)[a]) / (2.0 * h);
    }
    return d;
}

jet::Vector3D GpuColliderVelocityField3::curl(const jet::Vector3D& x) const {
    const jet::Collider3Ptr& c = collider();
    if (!c) return jet::Vector3D();
    if (auto r = std::dynamic_pointer_cast<jet::RigidBodyCollider3>(c))
        return 2.0 * r->angularVelocity;
    const double h = 1e-4;
    auto d = [&](int comp, int axis) {
        jet::Vector3D e;
        e[axis] = h;
        return (sample(x + e)[comp] - sample(x - e)[comp]) / (2.0 * h);
    };
    return jet::Vector3D(d(2, 1) - d(1, 2), d(0, 2) - d(2, 0),
                         d(1, 0) - d(0, 1));
}

std::function<jet::Vector3D(const jet::Vector3D&)>
GpuColliderVelocityField3::sampler() const {
    return [this](const jet::Vector3D& x) { return sample(x); };
}

GpuFractionalBoundaryConditionSolver3::GpuFractionalBoundaryConditionSolver3(
    const jetgpu_config* cfg)
    : _velocityField(std::make_shared<GpuColliderVelocityField3>(this)) {
    jetgpu_config_default(&_config);
    if (cfg) _config = *cfg;
}

jet::VectorField3Ptr
GpuFractionalBoundaryConditionSolver3::colliderVelocityField() const {
    return _velocityField;
}

GpuFractionalBoundaryConditionSolver3::
    ~GpuFractionalBoundaryConditionSolver3() {
    if (_ctx) jetgpu_destroy(_ctx);
}

void GpuFractionalBoundaryConditionSolver3::constrainVelocity(
    jet::FaceCenteredGrid3* velocity, unsigned int extrapolationDepth) {
    constrain_on_gpu(*this, _config, &_ctx, &_status, velocity,
                     extrapolationDepth, false);
}

}  // namespace jetgpu_jet
