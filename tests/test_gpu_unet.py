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


@pytest.mark.parametrize("ci,co,shape", [(16, 16, (9, 10, 12)),
                                         (32, 16, (8, 8, 8)),
                                         (16, 48, (5, 7, 11)),
                                         (112, 48, (6, 6, 6)),
                                         (64, 64, (16, 16, 16))])
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
