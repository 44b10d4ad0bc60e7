"""Learned-preconditioner layers on the tensor cores vs the FP64 CPU oracle
(oracle/conv_ref.py). Inputs are BF16-representable, so the only error is
the FP32 accumulation: tolerance 1e-4 of the output scale."""
import ctypes as C

import numpy as np
import pytest

import jetgpu
from oracle import conv_ref

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def to_bf16(t):
    return torch.from_numpy(np.ascontiguousarray(t, np.float32)).to(
        torch.bfloat16)


def run_conv(x, w, bias, relu):
    L = jetgpu.library()
    dev = torch.device("cuda", 0)
    nz, ny, nx, ci = x.shape
    co = w.shape[1]
    xin = to_bf16(x).to(dev)
    wt = to_bf16(w).to(dev)
    b = torch.from_numpy(np.asarray(bias, np.float32)).to(dev)
    out32 = torch.zeros((nz, ny, nx, co), dtype=torch.float32, device=dev)
    out = torch.zeros((nz, ny, nx, co), dtype=torch.bfloat16, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    res = (C.c_int * 3)(nx, ny, nz)
    st = L.jetgpu_conv3d(None, xin.data_ptr(), ci, wt.data_ptr(), b.data_ptr(),
                         co, res, int(relu), out.data_ptr(), out32.data_ptr(),
                         err.data_ptr())
    assert st == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return out32.cpu().numpy(), out.float().cpu().numpy()


# Shapes are (nz, ny, nx). Rows of 128 or 256 cells run on the brick kernel
# (the input brick of a 128-cell row staged by TMA once, all taps from shared
# memory), the others on the per-tap gather kernel.
@pytest.mark.parametrize("ci,co,shape", [(16, 16, (9, 10, 12)),
                                         (32, 16, (8, 8, 8)),
                                         (16, 48, (5, 7, 11)),
                                         (112, 48, (6, 6, 6)),
                                         (64, 64, (16, 16, 16)),
                                         (16, 16, (3, 4, 128)),
                                         (48, 16, (4, 3, 128)),
                                         (16, 32, (2, 3, 256)),
                                         (80, 32, (3, 2, 128)),
                                         (32, 80, (2, 2, 128))])
def test_conv3d_matches_oracle(ci, co, shape):
    rng = np.random.default_rng(ci * 7 + co)
    x = conv_ref.bf16_round(rng.standard_normal(shape + (ci,)))
    w = conv_ref.bf16_round(rng.standard_normal((27, co, ci)) * 0.1)
    bias = rng.standard_normal(co).astype(np.float32)
    for relu in (False, True):
        got32, got16 = run_conv(x, w, bias, relu)
        ref = conv_ref.conv3d(x, w, bias, relu)
        scale = np.abs(ref).max()
        assert np.abs(got32 - ref).max() <= 1e-4 * scale, (ci, co, relu)
        assert np.abs(got16 - ref).max() <= 1e-2 * scale


def test_conv3d_gradients_match_oracle():
    """dgrad = forward conv with flipped/transposed weights; wgrad on the
    tensor cores. Both against the FP64 oracle (BF16-exact inputs)."""
    L = jetgpu.library()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(3)
    for ci, co, shape in ((16, 16, (9, 10, 12)), (48, 32, (6, 7, 8)),
                          (112, 48, (5, 6, 7)), (64, 64, (8, 8, 8)),
                          (48, 16, (3, 2, 128)), (32, 80, (2, 3, 128))):
        x = conv_ref.bf16_round(rng.standard_normal(shape + (ci,)))
        w = conv_ref.bf16_round(rng.standard_normal((27, co, ci)) * 0.1)
        dy = conv_ref.bf16_round(rng.standard_normal(shape + (co,)))
        nz, ny, nx = shape
        res = (C.c_int * 3)(nx, ny, nz)
        err = torch.zeros(1, dtype=torch.int32, device=dev)
        # dgrad through the forward kernel
        wT = np.ascontiguousarray(w[::-1].transpose(0, 2, 1))
        dyd, wTd = to_bf16(dy).to(dev), to_bf16(wT).to(dev)
        dx = torch.zeros(shape + (ci,), dtype=torch.float32, device=dev)
        st = L.jetgpu_conv3d(None, dyd.data_ptr(), co, wTd.data_ptr(), None, ci,
                             res, 0, None, dx.data_ptr(), err.data_ptr())
        assert st == 0
        # wgrad
        xd = to_bf16(x).to(dev)
        dw = torch.zeros((27, co, ci), dtype=torch.float32, device=dev)
        st = L.jetgpu_conv3d_wgrad(None, xd.data_ptr(), ci, dyd.data_ptr(), co,
                                   res, dw.data_ptr(), err.data_ptr())
        assert st == 0
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        ref_dx = conv_ref.conv3d_dgrad(dy, w)
        ref_dw = conv_ref.conv3d_wgrad(x, dy)
        assert np.abs(dx.cpu().numpy() - ref_dx).max() <= 1e-4 * np.abs(ref_dx).max()
        assert np.abs(dw.cpu().numpy() - ref_dw).max() <= 1e-4 * np.abs(ref_dw).max(), (ci, co)
