// GPU drop-in for Jet's GridBlockedBoundaryConditionSolver3: argument
// marshalling onto jetgpu_constrain_velocity_blocked. See
// gpu_blocked_boundary_condition_solver3.h.
#include "gpu_blocked_boundary_condition_solver3.h"

#include "jet_marshal.h"

namespace jetgpu_jet {

GpuBlockedBoundaryConditionSolver3::GpuBlockedBoundaryConditionSolver3(
    const jetgpu_config* cfg) {
    jetgpu_config_default(&_config);
    if (cfg) _config = *cfg;
}

GpuBlockedBoundaryConditionSolver3::~GpuBlockedBoundaryConditionSolver3() {
    if (_ctx) jetgpu_destroy(_ctx);
}

void GpuBlockedBoundaryConditionSolver3::onColliderUpdated(
    const jet::Size3& gridSize, const jet::Vector3D& gridSpacing,
    const jet::Vector3D& gridOrigin) {
    GridFractionalBoundaryConditionSolver3::onColliderUpdated(
        gridSize, gridSpacing, gridOrigin);
    const auto sdf =
        std::dynamic_pointer_cast<jet::CellCenteredScalarGrid3>(colliderSdf());
    _marker.resize(gridSize);
    _marker.parallelForEachIndex([&](size_t i, size_t j, size_t k) {
        _marker(i, j, k) = (*sdf)(i, j, k) < 0.0 ? 0 : 1;
    });
}

void GpuBlockedBoundaryConditionSolver3::constrainVelocity(
    jet::FaceCenteredGrid3* velocity, unsigned int extrapolationDepth) {
    constrain_on_gpu(*this, _config, &_ctx, &_status, velocity,
                     extrapolationDepth, true);
}

}  // namespace jetgpu_jet
