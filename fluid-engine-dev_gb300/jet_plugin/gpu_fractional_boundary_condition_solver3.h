// GPU drop-in for Jet's GridFractionalBoundaryConditionSolver3 (host side,
// C++).
//
// Derives from jet::GridFractionalBoundaryConditionSolver3
// (include/jet/grid_fractional_boundary_condition_solver3.h:27-66), keeps its
// collider SDF (built on the host from the collider's surface, as the
// reference does in onColliderUpdated), and runs constrainVelocity on the GPU
// through jetgpu_constrain_velocity (include/jetgpu.h), bit for bit the
// reference's result. GpuFractionalSinglePhasePressureSolver3 suggests it,
// so GridFluidSolver3::setPressureSolver installs both. Colliders must be
// RigidBodyCollider3 (or none): the GPU evaluates the collider velocity as
// linear + angular x (p - centre); other colliders are refused loudly.
#ifndef JETGPU_JET_GPU_FRACTIONAL_BOUNDARY_CONDITION_SOLVER3_H_
#define JETGPU_JET_GPU_FRACTIONAL_BOUNDARY_CONDITION_SOLVER3_H_

#include <jet/grid_fractional_boundary_condition_solver3.h>

#include "jetgpu.h"

namespace jetgpu_jet {

class GpuFractionalBoundaryConditionSolver3
    : public jet::GridFractionalBoundaryConditionSolver3 {
 public:
    //! The CUDA context is created on the first call (device 0 unless cfg
    //! says otherwise).
    explicit GpuFractionalBoundaryConditionSolver3(
        const jetgpu_config* cfg = nullptr);
    ~GpuFractionalBoundaryConditionSolver3() override;

    GpuFractionalBoundaryConditionSolver3(
        const GpuFractionalBoundaryConditionSolver3&) = delete;
    GpuFractionalBoundaryConditionSolver3& operator=(
        const GpuFractionalBoundaryConditionSolver3&) = delete;

    //! GridFractionalBoundaryConditionSolver3::constrainVelocity
    //! (src/jet/grid_fractional_boundary_condition_solver3.cpp:26-233) on the
    //! GPU. Throws std::invalid_argument for a collider that is not a
    //! RigidBodyCollider3 and std::runtime_error when the GPU call fails.
    void constrainVelocity(jet::FaceCenteredGrid3* velocity,
                           unsigned int extrapolationDepth = 5) override;

    jetgpu_status lastStatus() const { return _status; }

 private:
    jetgpu_config _config;
    struct jetgpu_ctx* _ctx = nullptr;
    jetgpu_status _status = JETGPU_OK;
};

}  // namespace jetgpu_jet

#endif  // JETGPU_JET_GPU_FRACTIONAL_BOUNDARY_CONDITION_SOLVER3_H_
