// GPU drop-in for Jet's GridPressureSolver3: argument marshalling onto the
// C ABI of libjetgpu. See gpu_fractional_pressure_solver3.h.
#include "gpu_fractional_pressure_solver3.h"
#include "gpu_fractional_boundary_condition_solver3.h"
#include "jet_marshal.h"

#include <jet/cell_centered_scalar_grid3.h>
#include <jet/constant_scalar_field3.h>
#include <jet/constant_vector_field3.h>
#include <jet/face_centered_grid3.h>
#include <jet/grid_fractional_boundary_condition_solver3.h>
#include <jet/logging.h>
#include <jet/rigid_body_collider3.h>

#include <cstring>
#include <memory>

namespace jetgpu_jet {

using namespace jet;

GpuFractionalSinglePhasePressureSolver3::GpuFractionalSinglePhasePressureSolver3(
    const jetgpu_config* cfg) {
    jetgpu_config_default(&_config);
    if (cfg) _config = *cfg;
    // applyPressureGradient writes only the faces next to fluid cells, and
    // GridFluidSolver3::computePressure hands in a clone of the output grid
    // as the input: only the velocity faces around the fluid cells need to
    // cross the host link, and the output's other faces keep their values,
    // as the reference leaves them.
    _config.fluid_box_io = 1;
}

GpuFractionalSinglePhasePressureSolver3::
    ~GpuFractionalSinglePhasePressureSolver3() {
    if (_ctx) jetgpu_destroy(_ctx);
}

GridBoundaryConditionSolver3Ptr
GpuFractionalSinglePhasePressureSolver3::suggestedBoundaryConditionSolver()
    const {
    // The fractional boundary solver the reference suggests (:486-490),
    // with constrainVelocity on the GPU.
    return std::make_shared<GpuFractionalBoundaryConditionSolver3>(&_config);
}

void GpuFractionalSinglePhasePressureSolver3::solve(
    const FaceCenteredGrid3& input, double timeIntervalInSeconds,
    FaceCenteredGrid3* output, const ScalarField3& boundarySdf,
    const VectorField3& boundaryVelocity, const ScalarField3& fluidSdf,
    bool useCompressed) {
    (void)timeIntervalInSeconds;  // unused, as in the reference (:461)
    (void)useCompressed;          // the GPU system is row based either way
    if (!_ctx) {
        _status = jetgpu_create(&_config, &_ctx);
        if (_status != JETGPU_OK) {
            JET_ERROR << "jetgpu_create failed with status " << _status;
            return;
        }
    }
    const Size3 res = input.resolution();
    const jetgpu_grid g = grid_of(input);
    const jetgpu_scalar_field bsdf =
        describe_field(boundarySdf, input, &_boundaryRaster);
    const jetgpu_scalar_field fsdf =
        describe_field(fluidSdf, input, &_fluidRaster);

    // Collider velocity: only the normal component at each face is used
    // (grid_fractional_single_phase_pressure_solver3.cpp:241-255). The GPU
    // boundary-condition solver (which setPressureSolver installs with this
    // solver) passes a GpuColliderVelocityField3: no collider, or a rigid
    // one standing still, means no moving-boundary term at all; a moving
    // rigid collider's velocityAt is evaluated on the GPU. Any other field
    // is sampled at every face position on the host.
    const double* su = nullptr;
    const double* sv = nullptr;
    const double* sw = nullptr;
    jetgpu_collider motion{};
    bool moving_rigid = false;
    bool sample_on_host = true;
    if (auto gv = dynamic_cast<const GpuColliderVelocityField3*>(
            &boundaryVelocity)) {
        const Collider3Ptr& collider = gv->collider();
        auto rigid = std::dynamic_pointer_cast<RigidBodyCollider3>(collider);
        if (!collider) {
            sample_on_host = false;
        } else if (rigid) {
            motion = rigid_motion(*rigid);
            sample_on_host = false;
            for (int d = 0; d < 3; ++d)
                moving_rigid = moving_rigid ||
                               motion.linear_velocity[d] != 0.0 ||
                               motion.angular_velocity[d] != 0.0;
        }
    } else if (auto cv = dynamic_cast<const ConstantVectorField3*>(
                   &boundaryVelocity)) {
        sample_on_host = cv->sample(Vector3D()).lengthSquared() != 0.0;
    }
    if (sample_on_host) {
        auto sample = [&](std::vector<double>* out, const Size3& s,
                          VectorGrid3::DataPositionFunc pos, int axis) {
            out->resize(s.x * s.y * s.z);
            size_t c = 0;
            for (size_t k = 0; k < s.z; ++k)
                for (size_t j = 0; j < s.y; ++j)
                    for (size_t i = 0; i < s.x; ++i)
                        (*out)[c++] = boundaryVelocity.sample(pos(i, j, k))[axis];
        };
        sample(&_solidU, input.uSize(), input.uPosition(), 0);
        sample(&_solidV, input.vSize(), input.vPosition(), 1);
        sample(&_solidW, input.wSize(), input.wPosition(), 2);
        su = _solidU.data();
        sv = _solidV.data();
        sw = _solidW.data();
    }

    // The pressure stays on the device until pressure() asks for it
    // (FlipSolver3 never does): no 8-byte-per-cell download per solve.
    _pressure.resize(res);
    _pressureStale = true;
    auto u = input.uConstAccessor();
    auto v = input.vConstAccessor();
    auto w = input.wConstAccessor();
    auto ou = output->uAccessor();
    auto ov = output->vAccessor();
    auto ow = output->wAccessor();
    if (moving_rigid)
        _status = jetgpu_solve_pressure_collider(
            _ctx, &g, u.data(), v.data(), w.data(), &bsdf, &fsdf, &motion,
            ou.data(), ov.data(), ow.data(), nullptr, &_stats);
    else
        _status = jetgpu_solve_pressure(_ctx, &g, u.data(), v.data(),
                                        w.data(), &bsdf, &fsdf, su, sv, sw,
                                        ou.data(), ov.data(), ow.data(),
                                        nullptr, &_stats);
    if (_status != JETGPU_OK) {
        // The reference ignores its linear solver's result
        // (grid_fractional_single_phase_pressure_solver3.cpp:466-483); the
        // projected velocity of the last iterate has been applied.
        JET_WARN << "jetgpu_solve_pressure: status " << _status << ": "
                 << jetgpu_last_error(_ctx);
    }
}

const jet::FdmVector3& GpuFractionalSinglePhasePressureSolver3::pressure()
    const {
    if (_pressureStale && _ctx) {
        size_t count = 0;
        const jetgpu_status s = jetgpu_get_level(
            _ctx, 0, 6, _pressure.data(),
            _pressure.width() * _pressure.height() * _pressure.depth() *
                sizeof(double),
            &count);
        if (s != JETGPU_OK)
            JET_WARN << "jetgpu_get_level: status " << s << ": "
                     << jetgpu_last_error(_ctx);
        _pressureStale = false;
    }
    return _pressure;
}

}  // namespace jetgpu_jet
