// GPU drop-in for Jet's GridFractionalBoundaryConditionSolver3: argument
// marshalling onto jetgpu_constrain_velocity. See
// gpu_fractional_boundary_condition_solver3.h.
#include "gpu_fractional_boundary_condition_solver3.h"

#include "jet_marshal.h"

namespace jetgpu_jet {

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
    jet::FaceCenteredGrid3* velocity, unsigned int extrapolationDepth) {
    constrain_on_gpu(*this, _config, &_ctx, &_status, velocity,
                     extrapolationDepth, false);
}

}  // namespace jetgpu_jet
