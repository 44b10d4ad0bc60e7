// GPU drop-in for Jet's GridSinglePhasePressureSolver3: argument marshalling
// onto jetgpu_solve_pressure_blocked. See gpu_single_phase_pressure_solver3.h.
#include "gpu_single_phase_pressure_solver3.h"

#include <jet/logging.h>

#include "gpu_blocked_boundary_condition_solver3.h"
#include "jet_marshal.h"

namespace jetgpu_jet {

using namespace jet;

GpuSinglePhasePressureSolver3::GpuSinglePhasePressureSolver3(
    const jetgpu_config* cfg) {
    jetgpu_config_default(&_config);
    if (cfg) _config = *cfg;
}

GpuSinglePhasePressureSolver3::~GpuSinglePhasePressureSolver3() {
    if (_ctx) jetgpu_destroy(_ctx);
}

GridBoundaryConditionSolver3Ptr
GpuSinglePhasePressureSolver3::suggestedBoundaryConditionSolver() const {
    return std::make_shared<GpuBlockedBoundaryConditionSolver3>(&_config);
}

void GpuSinglePhasePressureSolver3::solve(
    const FaceCenteredGrid3& input, double timeIntervalInSeconds,
    FaceCenteredGrid3* output, const ScalarField3& boundarySdf,
    const VectorField3& boundaryVelocity, const ScalarField3& fluidSdf,
    bool useCompressed) {
    (void)timeIntervalInSeconds;  // unused, as in the reference (:189-191)
    (void)boundaryVelocity;
    (void)useCompressed;  // the GPU system is row based either way
    if (!_ctx) {
        _status = jetgpu_create(&_config, &_ctx);
        if (_status != JETGPU_OK) {
            _ctx = nullptr;
            JET_ERROR << "jetgpu_create failed with status " << _status;
            return;
        }
    }
    const jetgpu_grid g = grid_of(input);
    const jetgpu_scalar_field bsdf =
        describe_field(boundarySdf, input, &_boundaryRaster);
    const jetgpu_scalar_field fsdf =
        describe_field(fluidSdf, input, &_fluidRaster);
    _pressure.resize(input.resolution());
    auto u = input.uConstAccessor();
    auto v = input.vConstAccessor();
    auto w = input.wConstAccessor();
    auto ou = output->uAccessor();
    auto ov = output->vAccessor();
    auto ow = output->wAccessor();
    _status = jetgpu_solve_pressure_blocked(
        _ctx, &g, u.data(), v.data(), w.data(), &bsdf, &fsdf, ou.data(),
        ov.data(), ow.data(), _pressure.data(), &_stats);
    if (_status != JETGPU_OK) {
        // The reference ignores its linear solver's result (:193-210): the
        // gradient of the last iterate has been applied.
        JET_WARN << "jetgpu_solve_pressure_blocked: status " << _status << ": "
                 << jetgpu_last_error(_ctx);
    }
}

}  // namespace jetgpu_jet
