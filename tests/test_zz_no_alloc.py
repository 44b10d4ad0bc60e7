"""The allocation-free P2G entry point matches the regular one (GPU).

jetgpu_p2g_device_noalloc serves callers that must not allocate device
memory while they run (an engine that owns the GPU memory budget, a
real-time loop where cudaMalloc's implicit synchronisation is not allowed).
Its scratch is a fixed array inside the library, shared by every call, so
this test calls it twice in a row and checks both results against
jetgpu_p2g_device, the entry point that uses context scratch, at the same
tolerance as the other P2G tests. It sits in a file of its own that pytest
collects last.
"""
import ctypes as C

import numpy as np
import pytest

import jetgpu
from conftest import golden

pytestmark = pytest.mark.gpu


def _grid(n, h):
    g = jetgpu.Grid()
    g.res[:] = (n, n, n)
    g.spacing[:] = (h, h, h)
    g.origin[:] = (0.0, 0.0, 0.0)
    return g


def _buffers(torch, n, dev):
    shapes = [(n, n, n + 1), (n, n + 1, n), (n + 1, n, n)]
    grids = [torch.zeros(s, dtype=torch.float64, device=dev) for s in shapes]
    marks = [torch.zeros(s, dtype=torch.uint8, device=dev) for s in shapes]
    snaps = [torch.zeros(s, dtype=torch.float32, device=dev) for s in shapes]
    return grids, marks, snaps


def _ptrs(ts):
    return [t.data_ptr() for t in ts]


def test_noalloc_p2g_matches_context_p2g_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = jetgpu.library()
    dev = torch.device("cuda", 0)
    g = golden("transfer_16.npz")
    cases = [(16, g["pos"], g["vel"])]
    rng = np.random.default_rng(5)
    # The largest grid the fixed scratch holds, with more particles.
    cases.append((64, rng.uniform(0, 1, (200_000, 3)),
                  rng.uniform(-1, 1, (200_000, 3))))
    solver = jetgpu.FdmMgpcgSolver3()
    for n, pos, vel in cases:
        h = 1.0 / n
        grid = _grid(n, h)
        dpos = torch.from_numpy(np.ascontiguousarray(pos)).to(dev)
        dvel = torch.from_numpy(np.ascontiguousarray(vel)).to(dev)
        ref = _buffers(torch, n, dev)
        st = L.jetgpu_p2g_device(solver.context(), C.byref(grid), dpos.shape[0],
                                 dpos.data_ptr(), dvel.data_ptr(),
                                 *_ptrs(ref[0]), *_ptrs(ref[1]), *_ptrs(ref[2]))
        assert st == 0
        stream = torch.cuda.current_stream(dev)
        for call in range(2):
            out = _buffers(torch, n, dev)
            st = L.jetgpu_p2g_device_noalloc(
                C.c_void_p(stream.cuda_stream), C.byref(grid), dpos.shape[0],
                dpos.data_ptr(), dvel.data_ptr(), *_ptrs(out[0]),
                *_ptrs(out[1]), *_ptrs(out[2]))
            assert st == 0, (n, call, st)
            stream.synchronize()
            for a in range(3):
                got, want = out[0][a].cpu().numpy(), ref[0][a].cpu().numpy()
                assert np.allclose(got, want, rtol=1e-12, atol=1e-13), (n, call, a)
                assert torch.equal(out[1][a], ref[1][a]), (n, call, a)
                assert np.allclose(out[2][a].cpu().numpy(),
                                   ref[2][a].cpu().numpy(), rtol=2e-7,
                                   atol=1e-30), (n, call, a)
    solver.close()


def test_noalloc_p2g_rejects_grids_beyond_capacity():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = jetgpu.library()
    grid = _grid(65, 1.0 / 65)
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = dummy.data_ptr()
    st = L.jetgpu_p2g_device_noalloc(None, C.byref(grid), 0, None, None, p, p,
                                     p, None, None, None, None, None, None)
    assert st == 7  # JETGPU_CAPACITY_EXCEEDED
