"""The GPU V-cycle preconditioner against a float64 numpy model of the same
symmetric, masked V-cycle.

The GPU applies z = M r with fused single-pass red-black sweeps (tile plus
ring recomputation, ping-pong buffers), half-sweep kernels on small levels,
the residual / masked restriction / correction kernels and the one-CTA
coarsest solve. The model below restates that cycle with whole-array numpy
operations on the FP32 rows the library built (read back through
jetgpu_get_level): red-black SOR in the order the library documents (pre-
smoothing red first, post-smoothing black first), restriction with the
(1,3,3,1)/8 filter clamped at the edges
(src/jet/fdm_mg_linear_system3.cpp:43-98) with coarse non-fluid cells set to
zero, trilinear (1/4, 3/4) correction (:100-179). The pairs (r, z) come from
jetgpu_harvest. In mixed precision the model applies the library's BF16
rounding of the rows (diagonal up, off-diagonals toward zero). Tolerance:
FP32 arithmetic with an approximate division in the smoother against
float64 — 1e-4 relative L2.
"""
import ctypes as C

import numpy as np
import pytest

import jetgpu
from jetgpu import scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

REL = 1e-4


def nbr_sum(A, x):
    s = np.zeros_like(x)
    s[:, :, 1:] += A[:, :, :-1, 1] * x[:, :, :-1]
    s[:, :, :-1] += A[:, :, :-1, 1] * x[:, :, 1:]
    s[:, 1:, :] += A[:, :-1, :, 2] * x[:, :-1, :]
    s[:, :-1, :] += A[:, :-1, :, 2] * x[:, 1:, :]
    s[1:] += A[:-1, :, :, 3] * x[:-1]
    s[:-1] += A[:-1, :, :, 3] * x[1:]
    return s


def parity(shape):
    k, j, i = np.indices(shape)
    return (i + j + k) & 1


def sweep(A, b, x, first, omega):
    par = parity(x.shape)
    for color in (first, 1 - first):
        new = (1.0 - omega) * x + omega * (b - nbr_sum(A, x)) / A[..., 0]
        m = par == color
        x[m] = new[m]
    return x


def smooth(A, b, x, sweeps, reverse, omega):
    for _ in range(sweeps):
        sweep(A, b, x, 1 if reverse else 0, omega)
    return x


def restrict_axis(f, axis, nc):
    i = np.arange(nc)
    idx = [np.where(i > 0, 2 * i - 1, 2 * i), 2 * i, 2 * i + 1,
           np.where(i + 1 < nc, 2 * i + 2, 2 * i + 1)]
    w = (0.125, 0.375, 0.375, 0.125)
    return sum(wk * np.take(f, ik, axis=axis) for wk, ik in zip(w, idx))


def correct_axis(c, axis, nf):
    i = np.arange(nf)
    ci = i >> 1
    even = (i & 1) == 0
    i0 = np.where(even, np.where(i > 1, ci - 1, ci), ci)
    i1 = np.where(even, ci, np.where(i + 1 < nf, ci + 1, ci))
    w0 = np.where(even, 0.25, 0.75)
    w1 = 1.0 - w0
    shape = [1, 1, 1]
    shape[axis] = nf
    return (w0.reshape(shape) * np.take(c, i0, axis=axis) +
            w1.reshape(shape) * np.take(c, i1, axis=axis))


def vcycle(levels, l, b, cfg):
    A, phi = levels[l]
    omega = cfg["sor"]
    if l + 1 == len(levels):
        x = np.zeros_like(b)
        smooth(A, b, x, cfg["coarsest"], False, omega)
        return smooth(A, b, x, cfg["coarsest"], True, omega)
    x = smooth(A, b, np.zeros_like(b), cfg["pre"], False, omega)
    r = b - (A[..., 0] * x + nbr_sum(A, x))
    Ac, phic = levels[l + 1]
    nz, ny, nx = Ac.shape[:3]
    bc = restrict_axis(restrict_axis(restrict_axis(r, 2, nx), 1, ny), 0, nz)
    bc = np.where(phic < 0, bc, 0.0)
    xc = vcycle(levels, l + 1, bc, cfg)
    fz, fy, fx = b.shape
    x += correct_axis(correct_axis(correct_axis(xc, 2, fx), 1, fy), 0, fz)
    return smooth(A, b, x, cfg["final"] if l == 0 else cfg["post"], True,
                  omega)


def bf16_rows(A):
    """The mixed-precision V-cycle rows: FP32 rows rounded to BF16, the
    diagonal up (away from zero for positive values), off-diagonals toward
    zero."""
    a = A.astype(np.float32)
    u = a.view(np.uint32)
    t = u & np.uint32(0xFFFF0000)
    up = (a[..., 0] > 0) & ((u[..., 0] & 0xFFFF) != 0)
    out = t.view(np.float32).astype(np.float64)
    c = t[..., 0].astype(np.uint64) + np.where(up, 0x10000, 0).astype(np.uint64)
    out[..., 0] = c.astype(np.uint32).view(np.float32)
    return out


def scene(res, seed):
    nx, ny, nz = res
    h = 1.0 / max(res)
    rng = np.random.default_rng(seed)
    k, j, i = np.indices((nz, ny, nx))
    x, y, z = (i + 0.5) * h, (j + 0.5) * h, (k + 0.5) * h
    fluid = np.minimum(y - 0.55 * ny * h,
                       np.sqrt((x - 0.4 * nx * h) ** 2 + (y - 0.7 * ny * h) ** 2 +
                               (z - 0.5 * nz * h) ** 2) - 0.2 * ny * h)
    solid = np.sqrt((x - 0.6 * nx * h) ** 2 + (y - 0.2 * ny * h) ** 2 +
                    (z - 0.5 * nz * h) ** 2) - 0.15 * ny * h
    u = rng.uniform(-1, 1, (nz, ny, nx + 1))
    v = rng.uniform(-1, 1, (nz, ny + 1, nx))
    w = rng.uniform(-1, 1, (nz + 1, ny, nx))
    return h, u, v, w, solid, fluid


@pytest.mark.parametrize("res,sor,max_levels,precision",
                         [((64, 64, 64), 1.0, 5, "fp32"),
                          ((96, 40, 48), 1.2, 6, "fp32"),
                          ((128, 128, 128), 1.0, 6, "fp32"),
                          ((72, 36, 40), 1.2, 6, "fp32"),
                          ((72, 36, 40), 1.0, 6, "mixed"),
                          ((96, 40, 48), 1.0, 6, "mixed"),
                          ((128, 128, 128), 1.0, 6, "mixed"),
                          # More 64x8 sweep tiles (512) than resident
                          # blocks: the segment-by-segment work order.
                          ((512, 512, 8), 1.2, 4, "fp32")])
def test_vcycle_matches_numpy_model(res, sor, max_levels, precision):
    cfg = dict(pre=2, post=2, coarsest=10, final=2, sor=sor)
    h, u, v, w, solid, fluid = scene(res, seed=11)
    hh = (h, h, h)
    solver = jetgpu.FdmMgpcgSolver3(200, max_levels, cfg["pre"], cfg["post"],
                                    cfg["coarsest"], cfg["final"], 1e-6, sor,
                                    True, precision=precision)
    ps = jetgpu.GridFractionalSinglePhasePressureSolver3(solver)
    vel = jetgpu.FaceCenteredGrid3(res, hh, (0, 0, 0), u, v, w)
    g = lambda d: jetgpu.CellCenteredScalarGrid3(res, hh, (0, 0, 0), d)
    st = ps.solve(vel, 1 / 60, vel.clone(), g(solid), None, g(fluid))
    assert st in (0, 2)
    nlev = ps.last_stats.levels
    levels = []
    shape = (res[2], res[1], res[0])
    for l in range(nlev):
        A = ps.level(l, "A").reshape(shape + (4,))
        if l == 0:
            A = A.astype(np.float32).astype(np.float64)
        if precision == "mixed":
            A = bf16_rows(A)
        phi = ps.level(l, "fluid").reshape(shape).astype(np.float64)
        levels.append((A, phi))
        shape = tuple(s // 2 for s in shape)
    N = res[0] * res[1] * res[2]
    dev = torch.device("cuda", 0)
    R = torch.empty((2, N), dtype=torch.float32, device=dev)
    Z = torch.empty((2, N), dtype=torch.float32, device=dev)
    cnt = C.c_uint(0)
    L = jetgpu.library()
    solver.check(L.jetgpu_harvest(solver.context(), 2, R.data_ptr(),
                                  Z.data_ptr(), C.byref(cnt)))
    assert cnt.value == 2
    for k in range(2):
        r = R[k].cpu().numpy().astype(np.float64).reshape(res[::-1])
        z = Z[k].cpu().numpy().astype(np.float64).reshape(res[::-1])
        zm = vcycle(levels, 0, r, cfg)
        err = np.linalg.norm(z - zm) / np.linalg.norm(zm)
        assert err < REL, (k, err)
    solver.close()
