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
#include <jet/vector_field3.h>

#include <memory>

#include "jetgpu.h"

namespace jetgpu_jet {

//! The collider velocity field a GPU boundary-condition solver hands the
//! pressure solver (GridFluidSolver3::computePressure passes
//! colliderVelocityField(), src/jet/grid_fluid_solver3.cpp:243-253). It
//! samples exactly as the reference's field does
//! (grid_fractional_boundary_condition_solver3.cpp:265-278: the collider's
//! velocityAt(x), zero without a collider), and it tells the GPU pressure
//! solver which collider it stands for, so that a static collider costs no
//! per-face host sampling and a moving rigid one is evaluated on the GPU.
class GpuColliderVelocityField3 : public jet::VectorField3 {
 public:
    explicit GpuColliderVelocityField3(
        const jet::GridBoundaryConditionSolver3* owner)
        : _owner(owner) {}

    jet::Vector3D sample(const jet::Vector3D& x) const override;
    //! Zero for a rigid motion; a finite difference otherwise.
    double divergence(const jet::Vector3D& x) const override;
    //! Twice the angular velocity for a rigid motion.
    jet::Vector3D curl(const jet::Vector3D& x) const override;
    std::function<jet::Vector3D(const jet::Vector3D&)> sampler()
        const override;

    //! The owner's current collider (null when there is none).
    const jet::Collider3Ptr& collider() const { return _owner->collider(); }

 private:
    const jet::GridBoundaryConditionSolver3* _owner;
};

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

    //! The collider's velocity as GpuColliderVelocityField3 (samples as the
    //! reference's colliderVelocityField does).
    jet::VectorField3Ptr colliderVelocityField() const override;

    jetgpu_status lastStatus() const { return _status; }

 private:
    std::shared_ptr<GpuColliderVelocityField3> _velocityField;
    jetgpu_config _config;
    struct jetgpu_ctx* _ctx = nullptr;
    jetgpu_status _status = JETGPU_OK;
};

}  // namespace jetgpu_jet

#endif  // JETGPU_JET_GPU_FRACTIONAL_BOUNDARY_CONDITION_SOLVER3_H_
