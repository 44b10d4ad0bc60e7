"""The C++ drop-in compiles against the reference and installs (CPU only).

Builds the C++ drop-ins of fluid-engine-dev_gb300/jet_plugin/ (the fractional
and blocked pressure solvers and their boundary-condition solvers) against the reference's own headers, links it with the reference library
(oracle/_ref/libjet_ref.a) and libjetgpu.so, and runs a program that
installs the GPU solver with setPressureSolver() on FlipSolver3, PicSolver3,
GridSmokeSolver3 and LevelSetLiquidSolver3 — the reference's install point
(src/jet/grid_fluid_solver3.cpp:110-121) — and checks that the GPU
boundary-condition solver is the one it suggests (setPressureSolver installs
the suggestion). No solve runs (no GPU here); the
CUDA context is created lazily on the first solve. Skipped where the
reference sources are absent.
"""
import os
import subprocess

import pytest

from conftest import PKG, REPO

REF = "/root/reference"

MAIN = r"""
#include <jet/jet.h>
#include "gpu_fractional_pressure_solver3.h"
#include "gpu_fractional_boundary_condition_solver3.h"
#include "gpu_single_phase_pressure_solver3.h"
#include "gpu_blocked_boundary_condition_solver3.h"
#include <cstdio>
#include <memory>

template <typename P, typename B, typename S>
bool install(S solver) {
    auto gpu = std::make_shared<P>();
    solver->setPressureSolver(gpu);
    // setPressureSolver installs gpu->suggestedBoundaryConditionSolver()
    // (grid_fluid_solver3.cpp:110-121); Jet has no getter for it, so the
    // suggestion's type is checked on the solver itself.
    return solver->pressureSolver() == gpu &&
           std::dynamic_pointer_cast<B>(gpu->suggestedBoundaryConditionSolver()) !=
               nullptr;
}

template <typename S>
bool install(S solver) {
    return install<jetgpu_jet::GpuFractionalSinglePhasePressureSolver3,
                   jetgpu_jet::GpuFractionalBoundaryConditionSolver3>(solver);
}

template <typename S>
bool installBlocked(S solver) {
    return install<jetgpu_jet::GpuSinglePhasePressureSolver3,
                   jetgpu_jet::GpuBlockedBoundaryConditionSolver3>(solver);
}

int main() {
    jet::Logging::mute();
    bool ok = true;
    ok &= install(jet::FlipSolver3::builder().withResolution({8, 8, 8}).makeShared());
    ok &= install(jet::PicSolver3::builder().withResolution({8, 8, 8}).makeShared());
    ok &= install(jet::GridSmokeSolver3::builder().withResolution({8, 8, 8}).makeShared());
    ok &= install(jet::LevelSetLiquidSolver3::builder().withResolution({8, 8, 8}).makeShared());
    ok &= installBlocked(jet::FlipSolver3::builder().withResolution({8, 8, 8}).makeShared());
    ok &= installBlocked(jet::GridSmokeSolver3::builder().withResolution({8, 8, 8}).makeShared());
    jetgpu_jet::GpuSinglePhasePressureSolver3 sb;
    ok &= std::dynamic_pointer_cast<jetgpu_jet::GpuBlockedBoundaryConditionSolver3>(
              sb.suggestedBoundaryConditionSolver()) != nullptr;
    ok &= std::dynamic_pointer_cast<jet::GridFractionalBoundaryConditionSolver3>(
              sb.suggestedBoundaryConditionSolver()) != nullptr;
    jetgpu_jet::GpuFractionalSinglePhasePressureSolver3 s;
    ok &= std::dynamic_pointer_cast<jet::GridFractionalBoundaryConditionSolver3>(
              s.suggestedBoundaryConditionSolver()) != nullptr;
    ok &= std::dynamic_pointer_cast<jetgpu_jet::GpuFractionalBoundaryConditionSolver3>(
              s.suggestedBoundaryConditionSolver()) != nullptr;

    std::printf("%s %s\n", ok ? "installed" : "FAILED", jetgpu_version());
    return ok ? 0 : 1;
}
"""


def test_cpp_adapter_installs_into_jet_solvers(tmp_path):
    if not os.path.isdir(os.path.join(REF, "include", "jet")):
        pytest.skip("reference headers not present on this machine")
    import oracle
    from jetgpu import _build
    lib = _build.build()
    oracle.build_reference()
    ref_a = os.path.join(REPO, "oracle", "_ref", "libjet_ref.a")
    assert os.path.exists(ref_a)
    main = tmp_path / "main.cpp"
    main.write_text(MAIN)
    exe = tmp_path / "install"
    plugin = os.path.join(PKG, "jet_plugin")
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", "-DJET_TASKING_OPENMP",
           "-include", "cstdint", "-w",
           "-I" + os.path.join(REF, "include"),
           "-I" + os.path.join(REF, "external"),
           "-I" + os.path.join(REPO, "include"), "-I" + plugin,
           str(main), os.path.join(plugin, "gpu_fractional_pressure_solver3.cpp"),
           os.path.join(plugin, "gpu_fractional_boundary_condition_solver3.cpp"),
           os.path.join(plugin, "gpu_single_phase_pressure_solver3.cpp"),
           os.path.join(plugin, "gpu_blocked_boundary_condition_solver3.cpp"),
           ref_a, lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "installed" in r.stdout, r.stdout + r.stderr


FLIP_MAIN = r"""
#include <jet/jet.h>
#include "gpu_fractional_pressure_solver3.h"
#include "gpu_fractional_boundary_condition_solver3.h"
#include <cstdio>
#include <memory>

struct jetgpu_stub_record_t {
    int solve_calls, solve_collider_calls, blocked_calls, constrain_calls;
    const double* solid[3];
    const double* boundary_data;
    const double* fluid_data;
    int boundary_kind, fluid_kind;
    int had_collider;
    jetgpu_collider collider;
};
extern "C" const jetgpu_stub_record_t* jetgpu_stub_record(void);
extern "C" void jetgpu_stub_reset(void);

using namespace jet;

// FlipSolver3 with the fields GridFluidSolver3 hands the pressure solver
// made visible (they are protected members).
struct ProbeFlip : FlipSolver3 {
    ProbeFlip() : FlipSolver3({16, 16, 16}, {1.0 / 16, 1.0 / 16, 1.0 / 16},
                              {0, 0, 0}) {}
    const double* colliderSdfData() const {
        auto g = std::dynamic_pointer_cast<CellCenteredScalarGrid3>(colliderSdf());
        return g ? g->constDataAccessor().data() : nullptr;
    }
    const double* fluidSdfData() const {
        auto g = std::dynamic_pointer_cast<CellCenteredScalarGrid3>(fluidSdf());
        return g ? g->constDataAccessor().data() : nullptr;
    }
};

static bool run(const Vector3D& linear, const Vector3D& angular) {
    jetgpu_stub_reset();
    auto solver = std::make_shared<ProbeFlip>();
    solver->setPressureSolver(
        std::make_shared<jetgpu_jet::GpuFractionalSinglePhasePressureSolver3>());
    auto sphere = Sphere3::builder().withCenter({0.5, 0.3, 0.5})
                      .withRadius(0.15).makeShared();
    auto collider = RigidBodyCollider3::builder().withSurface(sphere)
                        .makeShared();
    collider->linearVelocity = linear;
    collider->angularVelocity = angular;
    solver->setCollider(collider);
    Array1<Vector3D> pos;
    const double h = 1.0 / 16;
    for (int k = 0; k < 16; ++k)
        for (int j = 0; j < 8; ++j)
            for (int i = 0; i < 6; ++i)
                for (int s = 0; s < 8; ++s)
                    pos.append(Vector3D((i + 0.125 + 0.25 * (s & 1)) * h,
                                        (j + 0.125 + 0.25 * ((s >> 1) & 1)) * h,
                                        (k + 0.125 + 0.25 * (s >> 2)) * h));
    solver->particleSystemData()->addParticles(pos);
    Frame frame(0, 1.0 / 60.0);
    solver->update(frame);
    const jetgpu_stub_record_t* r = jetgpu_stub_record();
    const bool moving = linear.lengthSquared() + angular.lengthSquared() > 0;
    bool ok = r->constrain_calls > 0 && r->blocked_calls == 0;
    ok &= r->solid[0] == nullptr && r->solid[1] == nullptr &&
          r->solid[2] == nullptr;
    ok &= r->boundary_kind == 1 && r->fluid_kind == 1;
    ok &= r->boundary_data == solver->colliderSdfData();
    ok &= r->fluid_data == solver->fluidSdfData();
    if (moving) {
        ok &= r->solve_calls == 0 && r->solve_collider_calls > 0;
        const Vector3D t = sphere->transform.translation();
        for (int d = 0; d < 3; ++d)
            ok &= r->had_collider && r->collider.linear_velocity[d] == linear[d] &&
                  r->collider.angular_velocity[d] == angular[d] &&
                  r->collider.centre[d] == t[d];
    } else {
        ok &= r->solve_calls > 0 && r->solve_collider_calls == 0;
    }
    std::printf("%s collider: solves %d / %d with collider motion, "
                "constrain %d, sdf pointers %s\n",
                moving ? "moving" : "static", r->solve_calls,
                r->solve_collider_calls, r->constrain_calls,
                (r->boundary_data == solver->colliderSdfData() &&
                 r->fluid_data == solver->fluidSdfData()) ? "original" : "COPIED");
    return ok;
}

int main() {
    Logging::mute();
    bool ok = run({0, 0, 0}, {0, 0, 0});
    ok &= run({0.1, 0, 0}, {0, 0.5, 0});
    std::printf("%s\n", ok ? "adapter ok" : "FAILED");
    return ok ? 0 : 1;
}
"""


def test_cpp_adapter_flip_substep_reaches_abi(tmp_path):
    """A Jet FlipSolver3 frame with the GPU pressure solver installed, the
    adapters linked against a recording stand-in for libjetgpu
    (tests/native/jetgpu_recording_stub.cpp): the pressure solve reaches the
    C ABI with NULL solid velocities (a static collider costs no per-face
    host sampling), a moving rigid collider reaches
    jetgpu_solve_pressure_collider with its motion, and both SDFs arrive as
    the solver's own grid data pointers (no host copy)."""
    if not os.path.isdir(os.path.join(REF, "include", "jet")):
        pytest.skip("reference headers not present on this machine")
    import oracle
    oracle.build_reference()
    ref_a = os.path.join(REPO, "oracle", "_ref", "libjet_ref.a")
    assert os.path.exists(ref_a)
    main = tmp_path / "flip_main.cpp"
    main.write_text(FLIP_MAIN)
    exe = tmp_path / "flip_probe"
    plugin = os.path.join(PKG, "jet_plugin")
    stub = os.path.join(REPO, "tests", "native", "jetgpu_recording_stub.cpp")
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", "-DJET_TASKING_OPENMP",
           "-include", "cstdint", "-w",
           "-I" + os.path.join(REF, "include"),
           "-I" + os.path.join(REF, "external"),
           "-I" + os.path.join(REPO, "include"), "-I" + plugin,
           str(main), stub,
           os.path.join(plugin, "gpu_fractional_pressure_solver3.cpp"),
           os.path.join(plugin, "gpu_fractional_boundary_condition_solver3.cpp"),
           ref_a, "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0 and "adapter ok" in r.stdout, r.stdout + r.stderr
