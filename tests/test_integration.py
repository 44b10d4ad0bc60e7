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
