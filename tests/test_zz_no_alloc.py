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


def _grid(res, h):
    g = jetgpu.Grid()
    g.res[:] = tuple(res)
    g.spacing[:] = (h, h, h)
    g.origin[:] = (0.0, 0.0, 0.0)
    return g


def _buffers(torch, res, dev):
    nx, ny, nz = res
    shapes = [(nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx)]
    grids = [torch.zeros(s, dtype=torch.float64, device=dev) for s in shapes]
    marks = [torch.zeros(s, dtype=torch.uint8, device=dev) for s in shapes]
    snaps = [torch.zeros(s, dtype=torch.float32, device=dev) for s in shapes]
    return grids, marks, snaps


def _ptrs(ts):
    return [t.data_ptr() for t in ts]


def _cases():
    g = golden("transfer_16.npz")
    rng = np.random.default_rng(5)
    big = (rng.uniform(0, 1, (200_000, 3)), rng.uniform(-1, 1, (200_000, 3)))
    # 64^3 fills the fixed scratch exactly; the 16^3 case after it checks
    # that clearing only the faces a call uses is enough when the previous
    # call left larger sums behind; 100 x 40 x 40 is a non-cubic grid with
    # one axis beyond 64 that still fits by face count.
    return [((16, 16, 16), g["pos"], g["vel"], True),
            ((64, 64, 64), *big, True),
            ((16, 16, 16), g["pos"], g["vel"], False),
            ((100, 40, 40), *big, True)]


def test_noalloc_p2g_matches_context_p2g_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = jetgpu.library()
    dev = torch.device("cuda", 0)
    solver = jetgpu.FdmMgpcgSolver3()
    stream = torch.cuda.current_stream(dev)
    for res, pos, vel, with_marks in _cases():
        h = 1.0 / max(res)
        grid = _grid(res, h)
        dpos = torch.from_numpy(np.ascontiguousarray(pos)).to(dev)
        dvel = torch.from_numpy(np.ascontiguousarray(vel)).to(dev)
        ref = _buffers(torch, res, dev)
        st = L.jetgpu_p2g_device(solver.context(), C.byref(grid), dpos.shape[0],
                                 dpos.data_ptr(), dvel.data_ptr(),
                                 *_ptrs(ref[0]), *_ptrs(ref[1]), *_ptrs(ref[2]))
        assert st == 0
        torch.cuda.synchronize()
        for call in range(2):
            out = _buffers(torch, res, dev)
            # Marker and snapshot outputs are optional (NULL skips them).
            marks = _ptrs(out[1]) if with_marks else [None] * 3
            snaps = _ptrs(out[2]) if with_marks else [None] * 3
            st = L.jetgpu_p2g_device_noalloc(
                C.c_void_p(stream.cuda_stream), C.byref(grid), dpos.shape[0],
                dpos.data_ptr(), dvel.data_ptr(), *_ptrs(out[0]), *marks,
                *snaps)
            assert st == 0, (res, call, st)
            stream.synchronize()
            for a in range(3):
                got, want = out[0][a].cpu().numpy(), ref[0][a].cpu().numpy()
                assert np.allclose(got, want, rtol=1e-12, atol=1e-13), (res, call, a)
                if not with_marks:
                    continue
                assert torch.equal(out[1][a], ref[1][a]), (res, call, a)
                assert np.allclose(out[2][a].cpu().numpy(),
                                   ref[2][a].cpu().numpy(), rtol=2e-7,
                                   atol=1e-30), (res, call, a)
    solver.close()


def test_noalloc_p2g_rejects_grids_beyond_capacity():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = jetgpu.library()
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = dummy.data_ptr()

    def call(grid):
        return L.jetgpu_p2g_device_noalloc(None, C.byref(grid), 0, None, None,
                                           p, p, p, None, None, None, None,
                                           None, None)

    assert call(_grid((65, 65, 65), 1.0 / 65)) == 7  # CAPACITY_EXCEEDED
    assert call(_grid((16, 16, 1000), 1.0 / 16)) == 7
    bad = _grid((16, 16, 16), 1.0 / 16)
    bad.origin[1] = float("nan")
    assert call(bad) == 3  # BAD_INPUT: non-finite origin
    bad = _grid((16, 16, 16), float("inf"))
    assert call(bad) == 3  # BAD_INPUT: non-finite spacing
    assert call(_grid((1 << 11, 1 << 10, 1 << 10), 1e-3)) == 3  # >= 2^31 cells
