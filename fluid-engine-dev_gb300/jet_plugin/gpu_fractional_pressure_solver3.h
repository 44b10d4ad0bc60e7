// GPU drop-in for Jet's GridPressureSolver3 (host side, C++).
//
// Derives from jet::GridPressureSolver3
// (include/jet/grid_pressure_solver3.h:29-75) and forwards solve() to the
// C ABI of libjetgpu (include/jetgpu.h). Install it like the reference's
// GridFractionalSinglePhasePressureSolver3:
//
//   auto solver = jet::FlipSolver3::builder()....makeShared();
//   solver->setPressureSolver(
//       std::make_shared<jetgpu_jet::GpuFractionalSinglePhasePressureSolver3>());
//
// GridFluidSolver3::setPressureSolver (src/jet/grid_fluid_solver3.cpp:110-121)
// then installs the suggested boundary-condition solver, as for the
// reference class. Builds only where the Jet headers are available; link
// with libjet and libjetgpu.so.
#ifndef JETGPU_JET_GPU_FRACTIONAL_PRESSURE_SOLVER3_H_
#define JETGPU_JET_GPU_FRACTIONAL_PRESSURE_SOLVER3_H_

#include <jet/fdm_linear_system3.h>
#include <jet/grid_pressure_solver3.h>

#include <vector>

#include "jetgpu.h"

namespace jetgpu_jet {

class GpuFractionalSinglePhasePressureSolver3 : public jet::GridPressureSolver3 {
 public:
    //! Uses jetgpu_config_default() when cfg is null. The CUDA context is
    //! created on the first solve.
    explicit GpuFractionalSinglePhasePressureSolver3(
        const jetgpu_config* cfg = nullptr);
    ~GpuFractionalSinglePhasePressureSolver3() override;

    GpuFractionalSinglePhasePressureSolver3(
        const GpuFractionalSinglePhasePressureSolver3&) = delete;
    GpuFractionalSinglePhasePressureSolver3& operator=(
        const GpuFractionalSinglePhasePressureSolver3&) = delete;

    //! GridPressureSolver3::solve (grid_pressure_solver3.h:58-64).
    //! CellCenteredScalarGrid3 and ConstantScalarField3 SDFs go to the GPU
    //! as they are (the grid's own data, not a copy) and are sampled there
    //! with Jet's exact trilinear rule; other field types are rasterised at
    //! cell centres first. The collider velocity of the GPU
    //! boundary-condition solver (GpuColliderVelocityField3) costs nothing
    //! on the host: a missing or resting collider adds no moving-boundary
    //! term, a moving RigidBodyCollider3 is evaluated on the GPU. Any other
    //! velocity field is sampled at every face position on the host.
    void solve(const jet::FaceCenteredGrid3& input,
               double timeIntervalInSeconds, jet::FaceCenteredGrid3* output,
               const jet::ScalarField3& boundarySdf =
                   jet::ConstantScalarField3(jet::kMaxD),
               const jet::VectorField3& boundaryVelocity =
                   jet::ConstantVectorField3({0, 0, 0}),
               const jet::ScalarField3& fluidSdf =
                   jet::ConstantScalarField3(-jet::kMaxD),
               bool useCompressed = false) override;

    //! GpuFractionalBoundaryConditionSolver3 (a
    //! GridFractionalBoundaryConditionSolver3 whose constrainVelocity runs on
    //! the GPU), as the reference's fractional solver suggests its CPU class
    //! (grid_fractional_single_phase_pressure_solver3.cpp:486-490).
    jet::GridBoundaryConditionSolver3Ptr suggestedBoundaryConditionSolver()
        const override;

    //! Level-0 pressure of the last solve (cf. :512-518), read from the
    //! device on first use after a solve.
    const jet::FdmVector3& pressure() const;

    unsigned int lastNumberOfIterations() const { return _stats.iterations; }
    double lastResidual() const { return _stats.relative_residual; }
    const jetgpu_solve_stats& lastStats() const { return _stats; }
    jetgpu_status lastStatus() const { return _status; }

 private:
    jetgpu_config _config;
    struct jetgpu_ctx* _ctx = nullptr;
    mutable jet::FdmVector3 _pressure;
    mutable bool _pressureStale = false;
    jetgpu_solve_stats _stats{};
    jetgpu_status _status = JETGPU_OK;
    std::vector<double> _fluidRaster, _boundaryRaster;
    std::vector<double> _solidU, _solidV, _solidW;
};

}  // namespace jetgpu_jet

#endif  // JETGPU_JET_GPU_FRACTIONAL_PRESSURE_SOLVER3_H_
