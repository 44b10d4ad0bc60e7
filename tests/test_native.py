"""Host checks of device helpers that must agree bit for bit with the FP64
arithmetic they replace (CPU only; builds small host programs with nvcc)."""
import os
import shutil
import subprocess

import pytest

from conftest import PKG, REPO


def run_check(tmp_path, name):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = tmp_path / name
    src = os.path.join(REPO, "tests", "native", name + ".cu")
    r = subprocess.run([nvcc, "-x", "cu", "-O2", "-std=c++17", "-Xcompiler",
                        "-ffp-contract=off", "-I" + os.path.join(PKG, "csrc"),
                        src, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout


def test_bary_bits_matches_fp64_floor(tmp_path):
    """smp::bary_bits, the integer-pipe getBarycentric used by every exact
    FP64 trilinear sample on the GPU."""
    run_check(tmp_path, "bary_bits_check")


def test_lerp_fast_matches_reference_lerp(tmp_path):
    """smp::lerp_fast, the integer-pipe shortcuts of the reference's lerp
    for the fractions 0, 1/2 and 1 of grid-aligned samples."""
    run_check(tmp_path, "lerp_fast_check")

