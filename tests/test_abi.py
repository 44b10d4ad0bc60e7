"""The C-ABI library loads and exports every declared symbol (CPU only).

No compute call runs here; calls that must fail before touching the device
(argument validation) are checked, and a context creation without a GPU must
fail with a status, not crash.
"""
import ctypes as C
import os
import re

import pytest

import jetgpu
from conftest import REPO


def declared_functions():
    text = open(os.path.join(REPO, "include", "jetgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(jetgpu_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from jetgpu import _build
    _build.build()
    return jetgpu.library()


def test_header_lists_match_bindings():
    assert sorted(jetgpu.EXPORTS) == declared_functions()


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_version(lib):
    assert b"sm_103a" in lib.jetgpu_version()


def test_default_config_mirrors_constructor(lib):
    cfg = jetgpu.Config()
    lib.jetgpu_config_default(C.byref(cfg))
    assert cfg.max_cg_iter == 100 and cfg.red_black == 1
    assert cfg.tolerance == 1e-6
    assert 0.0 < cfg.sor < 2.0


@pytest.mark.parametrize("field,value", [("sor", 2.5), ("red_black", 0),
                                         ("max_levels", 0),
                                         ("precision", 9),
                                         ("tolerance", -1.0)])
def test_bad_config_rejected_before_device(lib, field, value):
    cfg = jetgpu.Config()
    lib.jetgpu_config_default(C.byref(cfg))
    setattr(cfg, field, value)
    h = C.c_void_p()
    assert lib.jetgpu_create(C.byref(cfg), C.byref(h)) == 3  # BAD_INPUT
    assert not h.value


def test_null_context_is_bad_input(lib):
    g = jetgpu.Grid()
    assert lib.jetgpu_solve_pressure(None, C.byref(g), None, None, None, None,
                                     None, None, None, None, None, None, None,
                                     None, None) == 3


def test_create_without_gpu_fails_cleanly(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    cfg = jetgpu.Config()
    lib.jetgpu_config_default(C.byref(cfg))
    h = C.c_void_p()
    st = lib.jetgpu_create(C.byref(cfg), C.byref(h))
    assert st == 4 and not h.value  # CUDA_ERROR, no context


def test_lexicographic_ordering_refused():
    with pytest.raises(ValueError):
        jetgpu.FdmMgpcgSolver3(useRedBlackOrdering=False)
