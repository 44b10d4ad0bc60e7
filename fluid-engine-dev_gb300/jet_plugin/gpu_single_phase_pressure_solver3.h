// GPU drop-in for Jet's GridSinglePhasePressureSolver3, the blocked pressure
// solver (host side, C++).
//
// Derives from jet::GridPressureSolver3
// (include/jet/grid_pressure_solver3.h:29-75) and forwards solve() to
// jetgpu_solve_pressure_blocked (include/jetgpu.h): cells are marked
// boundary, fluid or air by the SDFs at their centres, the system is the
// 7-point Laplacian on those markers, and an MGPCG solve on the GPU replaces
// the reference's default ICCG (grid_single_phase_pressure_solver3.cpp:
// 173-175). Install it like the reference class:
//
//   solver->setPressureSolver(
//       std::make_shared<jetgpu_jet::GpuSinglePhasePressureSolver3>());
//
// GridFluidSolver3::setPressureSolver (src/jet/grid_fluid_solver3.cpp:
// 110-121) then installs the suggested GpuBlockedBoundaryConditionSolver3.
#ifndef JETGPU_JET_GPU_SINGLE_PHASE_PRESSURE_SOLVER3_H_
#define JETGPU_JET_GPU_SINGLE_PHASE_PRESSURE_SOLVER3_H_

#include <jet/fdm_linear_system3.h>
#include <jet/grid_pressure_solver3.h>

#include <vector>

#include "jetgpu.h"

namespace jetgpu_jet {

class GpuSinglePhasePressureSolver3 : public jet::GridPressureSolver3 {
 public:
    //! Uses jetgpu_config_default() when cfg is null. The CUDA context is
    //! created on the first solve.
    explicit GpuSinglePhasePressureSolver3(const jetgpu_config* cfg = nullptr);
    ~GpuSinglePhasePressureSolver3() override;

    GpuSinglePhasePressureSolver3(const GpuSinglePhasePressureSolver3&) = delete;
    GpuSinglePhasePressureSolver3& operator=(
        const GpuSinglePhasePressureSolver3&) = delete;

    //! GridSinglePhasePressureSolver3::solve (:183-211). The boundary
    //! velocity is ignored, as the reference ignores it (:191).
    void solve(const jet::FaceCenteredGrid3& input,
               double timeIntervalInSeconds, jet::FaceCenteredGrid3* output,
               const jet::ScalarField3& boundarySdf =
                   jet::ConstantScalarField3(jet::kMaxD),
               const jet::VectorField3& boundaryVelocity =
                   jet::ConstantVectorField3({0, 0, 0}),
               const jet::ScalarField3& fluidSdf =
                   jet::ConstantScalarField3(-jet::kMaxD),
               bool useCompressed = false) override;

    //! GpuBlockedBoundaryConditionSolver3, as the reference suggests its CPU
    //! GridBlockedBoundaryConditionSolver3 (:213-216).
    jet::GridBoundaryConditionSolver3Ptr suggestedBoundaryConditionSolver()
        const override;

    //! Pressure of the last solve (cf. :229-235).
    const jet::FdmVector3& pressure() const { return _pressure; }

    unsigned int lastNumberOfIterations() const { return _stats.iterations; }
    double lastResidual() const { return _stats.relative_residual; }
    const jetgpu_solve_stats& lastStats() const { return _stats; }
    jetgpu_status lastStatus() const { return _status; }

 private:
    jetgpu_config _config;
    struct jetgpu_ctx* _ctx = nullptr;
    jet::FdmVector3 _pressure;
    jetgpu_solve_stats _stats{};
    jetgpu_status _status = JETGPU_OK;
    std::vector<double> _fluidRaster, _boundaryRaster;
};

}  // namespace jetgpu_jet

#endif  // JETGPU_JET_GPU_SINGLE_PHASE_PRESSURE_SOLVER3_H_
