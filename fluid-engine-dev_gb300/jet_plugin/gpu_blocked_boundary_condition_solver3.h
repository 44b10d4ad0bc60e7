// GPU drop-in for Jet's GridBlockedBoundaryConditionSolver3 (host side,
// C++).
//
// The reference class is final, so this one derives from its base,
// jet::GridFractionalBoundaryConditionSolver3, and offers the same interface
// (include/jet/grid_blocked_boundary_condition_solver3.h:27-57): the collider
// SDF is built on the host by the base, the cell markers (marker()) by
// onColliderUpdated with the reference's rule, and constrainVelocity runs on
// the GPU through jetgpu_constrain_velocity_blocked (include/jetgpu.h), bit
// for bit the reference's result.
// GpuSinglePhasePressureSolver3 suggests it. Colliders must be
// RigidBodyCollider3 (or none); other colliders are refused loudly.
#ifndef JETGPU_JET_GPU_BLOCKED_BOUNDARY_CONDITION_SOLVER3_H_
#define JETGPU_JET_GPU_BLOCKED_BOUNDARY_CONDITION_SOLVER3_H_

#include <jet/array3.h>
#include <jet/grid_fractional_boundary_condition_solver3.h>

#include "jetgpu.h"

namespace jetgpu_jet {

class GpuBlockedBoundaryConditionSolver3
    : public jet::GridFractionalBoundaryConditionSolver3 {
 public:
    //! The CUDA context is created on the first call.
    explicit GpuBlockedBoundaryConditionSolver3(
        const jetgpu_config* cfg = nullptr);
    ~GpuBlockedBoundaryConditionSolver3() override;

    GpuBlockedBoundaryConditionSolver3(
        const GpuBlockedBoundaryConditionSolver3&) = delete;
    GpuBlockedBoundaryConditionSolver3& operator=(
        const GpuBlockedBoundaryConditionSolver3&) = delete;

    //! GridBlockedBoundaryConditionSolver3::constrainVelocity
    //! (src/jet/grid_blocked_boundary_condition_solver3.cpp:23-67) on the
    //! GPU. Throws std::invalid_argument for a collider that is not a
    //! RigidBodyCollider3 and std::runtime_error when the GPU call fails.
    void constrainVelocity(jet::FaceCenteredGrid3* velocity,
                           unsigned int extrapolationDepth = 5) override;

    //! Cell markers: 0 inside the collider, 1 elsewhere (:69-71).
    const jet::Array3<char>& marker() const { return _marker; }

    jetgpu_status lastStatus() const { return _status; }

 protected:
    //! The base's collider SDF, then the markers from it (:73-91).
    void onColliderUpdated(const jet::Size3& gridSize,
                           const jet::Vector3D& gridSpacing,
                           const jet::Vector3D& gridOrigin) override;

 private:
    jet::Array3<char> _marker;
    jetgpu_config _config;
    struct jetgpu_ctx* _ctx = nullptr;
    jetgpu_status _status = JETGPU_OK;
};

}  // namespace jetgpu_jet

#endif  // JETGPU_JET_GPU_BLOCKED_BOUNDARY_CONDITION_SOLVER3_H_
