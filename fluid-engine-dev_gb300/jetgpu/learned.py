"""Training of the learned preconditioner (3-D U-Net) on the tensor-core
kernels of libjetgpu.

The learned preconditioner of libjetgpu's flexible PCG is a multigrid
V-cycle followed by the network's correction of the error the V-cycle
leaves (``jetgpu_learned_apply``):

    z0 = V r,   rho = r - A z0,   z = z0 + mask P^k e,   e = net(R^k rho)

on level k of the multigrid hierarchy (``jetgpu_net_level``: the finest
level at most 64 cells wide), with the V-cycle's masked restriction R (1/8
of the transposed prolongation) and trilinear prolongation P. The network
sees 16 channels that libjetgpu builds for the restricted residual
(``jetgpu_net_features``: rho_k / rms(rho_k), the level's six face weights,
fluid indicator, scaled diagonal) and predicts NET_GAIN * e / rms(rho_k).

It is trained to minimise the A-norm of the error left after the
correction. With y = mask P^k e and the V-cycle's error e0 = A^-1 rho,
||e0 - y||_A^2 = ||e0||_A^2 - 2 y.rho + y.A y, so the loss
(y.A y - 2 y.rho) needs no solve; it is divided by the energy a steepest-
descent step along rho removes, (rho.rho)^2 / (rho.A rho), so that samples
of every size weigh alike. Residuals r come from the solver's own MGPCG
iterations (``jetgpu_harvest``) on GPU-generated sphere-union scenes. Every
convolution of the forward and backward passes runs on libjetgpu's tcgen05
kernels (``jetgpu_conv3d`` and ``jetgpu_conv3d_wgrad``); PyTorch supplies
device memory, the optimizer and the element-wise glue (pooling,
upsampling, concatenation, ReLU masks, restriction and prolongation),
mirroring the library's inference path (``unet.cu``, ``learned_precond`` in
``mgpcg.cu``) step for step.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import (CellCenteredScalarGrid3, FaceCenteredGrid3, FdmMgpcgSolver3,
               GridFractionalSinglePhasePressureSolver3, library, scenes)

# (ci, co, relu) of the 14 layers, identical to kNetLayers in unet.cu.
LAYERS = [(16, 16, 1), (16, 16, 1), (16, 32, 1), (32, 32, 1), (32, 48, 1),
          (48, 48, 1), (48, 64, 1), (64, 64, 1), (112, 48, 1), (48, 48, 1),
          (80, 32, 1), (32, 32, 1), (48, 16, 1), (16, 16, 0)]

NET_GAIN = 32.0  # kNetGain in unet.cu

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights",
                       "unet_pressure.npz")


def param_count() -> int:
    return sum(27 * ci * co + co for ci, co, _ in LAYERS)


def init_params(seed: int = 0):
    rng = np.random.default_rng(seed)
    params = []
    for l, (ci, co, _) in enumerate(LAYERS):
        std = np.sqrt(2.0 / (27 * ci))
        if l == len(LAYERS) - 1:
            std *= 0.01  # start near z = 0: a large initial loss kills ReLUs
        params.append((rng.standard_normal((27, co, ci)).astype(np.float32) * std,
                       np.zeros(co, np.float32)))
    return params


def flatten(params) -> np.ndarray:
    return np.concatenate([np.concatenate([w.reshape(-1), b.reshape(-1)])
                           for w, b in params]).astype(np.float32)


def unflatten(flat: np.ndarray):
    params, off = [], 0
    for ci, co, _ in LAYERS:
        nw = 27 * co * ci
        w = flat[off:off + nw].reshape(27, co, ci)
        off += nw
        b = flat[off:off + co]
        off += co
        params.append((w, b))
    return params


def save(params, path: str = WEIGHTS) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez_compressed(path, params=flatten(params))


def load(path: str = WEIGHTS):
    return unflatten(np.load(path)["params"])


# ---------------------------------------------------------------------------
# Autograd over the tensor-core kernels.

def _torch():
    import torch
    return torch


def _res(x):
    nz, ny, nx = x.shape[:3]
    return (C.c_int * 3)(nx, ny, nz)


def _conv(x16, w16, bias, co, relu, out32=False):
    torch = _torch()
    L = library()
    nz, ny, nx, ci = x16.shape
    stream = torch.cuda.current_stream().cuda_stream
    err = torch.zeros(1, dtype=torch.int32, device=x16.device)
    if out32:
        out = torch.empty((nz, ny, nx, co), dtype=torch.float32, device=x16.device)
        st = L.jetgpu_conv3d(stream, x16.data_ptr(), ci, w16.data_ptr(),
                             None if bias is None else bias.data_ptr(), co,
                             _res(x16), int(relu), None, out.data_ptr(),
                             err.data_ptr())
    else:
        out = torch.empty((nz, ny, nx, co), dtype=torch.bfloat16, device=x16.device)
        st = L.jetgpu_conv3d(stream, x16.data_ptr(), ci, w16.data_ptr(),
                             None if bias is None else bias.data_ptr(), co,
                             _res(x16), int(relu), out.data_ptr(), None,
                             err.data_ptr())
    if st != 0:
        raise RuntimeError(f"jetgpu_conv3d failed with status {st}")
    return out


def _wgrad(x16, dy16):
    torch = _torch()
    L = library()
    ci, co = x16.shape[3], dy16.shape[3]
    dw = torch.zeros((27, co, ci), dtype=torch.float32, device=x16.device)
    err = torch.zeros(1, dtype=torch.int32, device=x16.device)
    st = L.jetgpu_conv3d_wgrad(torch.cuda.current_stream().cuda_stream,
                               x16.data_ptr(), ci, dy16.data_ptr(), co,
                               _res(x16), dw.data_ptr(), err.data_ptr())
    if st != 0:
        raise RuntimeError(f"jetgpu_conv3d_wgrad failed with status {st}")
    return dw


def make_conv_fn():
    torch = _torch()

    class Conv3dTC(torch.autograd.Function):
        """y = act(conv3d(x, w) + b) on libjetgpu's tensor-core kernels."""

        @staticmethod
        def forward(ctx, x16, w32, b32, relu, out32):
            w16 = w32.to(torch.bfloat16).contiguous()
            y = _conv(x16.contiguous(), w16, b32.contiguous(), w32.shape[1],
                      relu, out32)
            ctx.save_for_backward(x16, w32, y)
            ctx.relu = relu
            return y

        @staticmethod
        def backward(ctx, gy):
            x16, w32, y = ctx.saved_tensors
            g = gy * (y > 0).to(gy.dtype) if ctx.relu else gy
            g16 = g.to(torch.bfloat16).contiguous()
            # Input gradient: forward conv with the taps flipped and
            # (co, ci) transposed.
            wT = w32.flip(0).transpose(1, 2).contiguous().to(torch.bfloat16)
            dx = _conv(g16, wT, None, w32.shape[2], False, out32=True)
            dw = _wgrad(x16.contiguous(), g16)
            db = g.float().sum(dim=(0, 1, 2))
            return dx.to(x16.dtype), dw, db, None, None

    return Conv3dTC.apply


def pool2(x):
    nz, ny, nx, c = x.shape
    return (x.float().reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c)
            .sum(dim=(1, 3, 5)) * 0.125).to(x.dtype)


def up_concat(coarse, skip):
    up = coarse.repeat_interleave(2, 0).repeat_interleave(2, 1).repeat_interleave(2, 2)
    return _torch().cat([up, skip], dim=3)


def forward(conv, params, feat):
    """U-Net forward, mirroring net_apply in unet.cu. feat: (nz,ny,nx,16)
    BF16. params: list of (w FP32, b FP32) torch tensors. Returns the
    FP32 output channel 0."""
    P = params
    t = conv(feat, *P[0], 1, False)
    e0 = conv(t, *P[1], 1, False)
    t = conv(pool2(e0), *P[2], 1, False)
    e1 = conv(t, *P[3], 1, False)
    t = conv(pool2(e1), *P[4], 1, False)
    e2 = conv(t, *P[5], 1, False)
    t = conv(pool2(e2), *P[6], 1, False)
    e3 = conv(t, *P[7], 1, False)
    t = conv(up_concat(e3, e2), *P[8], 1, False)
    d2 = conv(t, *P[9], 1, False)
    t = conv(up_concat(d2, e1), *P[10], 1, False)
    d1 = conv(t, *P[11], 1, False)
    t = conv(up_concat(d1, e0), *P[12], 1, False)
    out = conv(t, *P[13], 0, True)
    return out[..., 0]


# ---------------------------------------------------------------------------
# The multigrid transfers of the V-cycle, on torch tensors.

def prolong(e):
    """Trilinear prolongation by 2 (k_correct: weights 1/4, 3/4 per axis,
    clamped at the edges), differentiable."""
    F = _torch().nn.functional
    return F.interpolate(e[None, None], scale_factor=2, mode="trilinear",
                         align_corners=False)[0, 0]


def restrict(rho, mask_c):
    """The V-cycle's restriction (k_restrict2): 1/8 of the transposed
    prolongation, zero on coarse cells outside the fluid."""
    torch = _torch()
    nz, ny, nx = rho.shape
    with torch.enable_grad():
        x = torch.zeros((nz // 2, ny // 2, nx // 2), dtype=rho.dtype,
                        device=rho.device, requires_grad=True)
        (g,) = torch.autograd.grad(prolong(x), x, grad_outputs=rho)
    return mask_c * (g * 0.125)


def _sync():
    """Orders torch's pending work before a library call on its own
    stream."""
    _torch().cuda.current_stream().synchronize()


# ---------------------------------------------------------------------------
# Data from the solver.

def device_scene(n: int, seed: int, device):
    """The 16-sphere union scene of ``scenes.sphere_union_scene`` built on
    the GPU (torch tensors): sphere centres and radii from the same
    std::mt19937(seed) stream, the SDFs evaluated on the device. The face
    velocities are U[-1, 1] from torch's generator seeded with `seed` (not
    the reference's stream: training data only needs their distribution).
    Returns dict(u, v, w, fluid_sdf, boundary_sdf)."""
    torch = _torch()
    rng = scenes.Mt19937Uniform(seed)
    cs, rs = [], []
    for _ in range(16):
        cs.append(rng.uniform(0.2, 0.8, 3))
        rs.append(rng.uniform(0.05, 0.2, 1)[0])
    f64 = dict(dtype=torch.float64, device=device)
    c = (torch.arange(n, **f64) + 0.5) / n
    Z, Y, X = torch.meshgrid(c, c, c, indexing="ij")
    fluid = torch.full((n, n, n), float("inf"), **f64)
    for cc, r in zip(cs, rs):
        d = torch.sqrt((X - cc[0]) ** 2 + (Y - cc[1]) ** 2 + (Z - cc[2]) ** 2) - r
        fluid = torch.minimum(fluid, d)
    walls = torch.minimum(torch.minimum(torch.minimum(X, 1 - X),
                                        torch.minimum(Y, 1 - Y)),
                          torch.minimum(Z, 1 - Z))
    ball = torch.sqrt((X - 0.5) ** 2 + (Y - 0.3) ** 2 + (Z - 0.5) ** 2) - 0.15
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    u = torch.rand((n, n, n + 1), generator=gen, **f64) * 2 - 1
    v = torch.rand((n, n + 1, n), generator=gen, **f64) * 2 - 1
    w = torch.rand((n + 1, n, n), generator=gen, **f64) * 2 - 1
    return dict(u=u, v=v, w=w, fluid_sdf=fluid.contiguous(),
                boundary_sdf=torch.minimum(walls, ball).contiguous())


def harvest_device(solver: FdmMgpcgSolver3, sc: dict, n: int, pairs: int):
    """Projects a scene already on the device (device_scene) through
    jetgpu_solve_pressure_device, then records up to `pairs` (r_k, V r_k)
    pairs of the MGPCG iterations on that system (jetgpu_harvest). Returns
    (R, Z), each (count, n, n, n) FP32 on the device."""
    torch = _torch()
    from . import Grid, ScalarField, solve_pressure_device
    L = library()
    h = 1.0 / n
    g = Grid()
    g.res[:] = (n, n, n)
    g.spacing[:] = (h, h, h)
    g.origin[:] = (0.0, 0.0, 0.0)

    def field(t):
        f = ScalarField()
        f.kind = 1
        f.data = t.data_ptr()
        f.res[:] = (n, n, n)
        f.origin[:] = (0.5 * h,) * 3
        f.spacing[:] = (h, h, h)
        return f

    out = [torch.empty_like(sc[k]) for k in ("u", "v", "w")]
    _sync()
    solve_pressure_device(solver, g, sc["u"], sc["v"], sc["w"],
                          field(sc["boundary_sdf"]), field(sc["fluid_sdf"]),
                          *out)
    dev = sc["u"].device
    N = n ** 3
    R = torch.empty((pairs, N), dtype=torch.float32, device=dev)
    Z = torch.empty((pairs, N), dtype=torch.float32, device=dev)
    cnt = C.c_uint(0)
    solver.check(L.jetgpu_harvest(solver.context(), pairs, R.data_ptr(),
                                  Z.data_ptr(), C.byref(cnt)))
    k = cnt.value
    return R[:k].reshape(k, n, n, n), Z[:k].reshape(k, n, n, n)


def level0_rows(solver: FdmMgpcgSolver3, n: int, device):
    """The finest level's matrix rows {center, right, up, front} of the
    solver's last system as an FP32 (n, n, n, 4) device tensor."""
    torch = _torch()
    L = library()
    rows = np.zeros(n ** 3 * 4)
    cnt = C.c_size_t(0)
    solver.check(L.jetgpu_get_level(solver.context(), 0, 4,
                                    rows.ctypes.data_as(C.c_void_p),
                                    rows.nbytes, C.byref(cnt)))
    return torch.from_numpy(rows.reshape(n, n, n, 4).astype(np.float32)).to(device)


def level0_rhs(solver: FdmMgpcgSolver3, n: int, device):
    """The finest level's right-hand side of the solver's last system as an
    FP32 (n, n, n) device tensor."""
    torch = _torch()
    L = library()
    b = np.zeros(n ** 3)
    cnt = C.c_size_t(0)
    solver.check(L.jetgpu_get_level(solver.context(), 0, 5,
                                    b.ctypes.data_as(C.c_void_p), b.nbytes,
                                    C.byref(cnt)))
    return torch.from_numpy(b.reshape(n, n, n).astype(np.float32)).to(device)


def fluid_masks(solver: FdmMgpcgSolver3, n: int, levels: int, device):
    """1.0 on fluid cells (fluid SDF < 0), 0.0 elsewhere, for levels
    0..levels of the solver's last system, as (n/2^l)^3 device tensors."""
    torch = _torch()
    L = library()
    out = []
    for l in range(levels + 1):
        m = n >> l
        phi = np.zeros(m ** 3, np.float32)
        cnt = C.c_size_t(0)
        solver.check(L.jetgpu_get_level(solver.context(), l, 0,
                                        phi.ctypes.data_as(C.c_void_p),
                                        phi.nbytes, C.byref(cnt)))
        out.append(torch.from_numpy((phi.reshape(m, m, m) < 0)
                                    .astype(np.float32)).to(device))
    return out


def apply_rows(A, x):
    """y = A x for 7-point rows (FdmBlas3::mvm, fdm_linear_system3.cpp:
    79-96) on torch tensors (differentiable)."""
    y = A[..., 0] * x
    y = y + _torch().nn.functional.pad(A[:, :, :-1, 1] * x[:, :, :-1], (1, 0))
    y = y + _torch().nn.functional.pad(A[:, :, :-1, 1] * x[:, :, 1:], (0, 1))
    y = y + _torch().nn.functional.pad(A[:, :-1, :, 2] * x[:, :-1, :], (0, 0, 1, 0))
    y = y + _torch().nn.functional.pad(A[:, :-1, :, 2] * x[:, 1:, :], (0, 0, 0, 1))
    y = y + _torch().nn.functional.pad(A[:-1, :, :, 3] * x[:-1], (0, 0, 0, 0, 1, 0))
    y = y + _torch().nn.functional.pad(A[:-1, :, :, 3] * x[1:], (0, 0, 0, 0, 0, 1))
    return y


def step_energy(A, r, z):
    """Energy (A-norm squared of the error) that the exact line search
    along z removes from residual r: (r.z)^2 / (z.A z)."""
    return (r * z).sum() ** 2 / (z * apply_rows(A, z)).sum().clamp_min(1e-30)


def vcycle_apply(solver: FdmMgpcgSolver3, r):
    """z = V r with the solver's multigrid V-cycle (jetgpu_vcycle_apply)."""
    torch = _torch()
    r = r.contiguous()
    z = torch.empty_like(r)
    _sync()
    solver.check(library().jetgpu_vcycle_apply(
        solver.context(), r.data_ptr(), z.data_ptr()))
    return z


def learned_apply(solver: FdmMgpcgSolver3, r):
    """z = M r with the library's learned preconditioner
    (jetgpu_learned_apply)."""
    torch = _torch()
    r = r.contiguous()
    z = torch.empty_like(r)
    _sync()
    solver.check(library().jetgpu_learned_apply(
        solver.context(), r.data_ptr(), z.data_ptr()))
    return z


def net_level(solver: FdmMgpcgSolver3) -> int:
    """The hierarchy level the network works on (jetgpu_net_level)."""
    return int(library().jetgpu_net_level(solver.context()))


def coarse_residual(A, masks, r, z0, k):
    """rho = r - A z0 on the finest level and its restriction to level k."""
    rho = r - apply_rows(A, z0)
    rk = rho
    for l in range(1, k + 1):
        rk = restrict(rk, masks[l])
    return rho, rk


def net_input(solver: FdmMgpcgSolver3, k: int, rk):
    """The network's 16 input channels for level-k residual rk
    (jetgpu_net_features) and rms(rk)."""
    torch = _torch()
    m = rk.shape[0]
    feat = torch.empty((m, m, m, 16), dtype=torch.bfloat16, device=rk.device)
    rk = rk.contiguous()
    _sync()
    solver.check(library().jetgpu_net_features(solver.context(), k,
                                               rk.data_ptr(), feat.data_ptr()))
    rms = torch.sqrt(torch.mean(rk.double() ** 2)).float()
    return feat, rms


def correction(conv, P, feat, rms, masks, k):
    """y = mask P^k e with e = net output * rms / NET_GAIN on the level-k
    fluid: the network's correction on the finest level (differentiable in
    the parameters P)."""
    e = forward(conv, P, feat) * (rms / NET_GAIN) * masks[k]
    for _ in range(k):
        e = prolong(e)
    return e * masks[0]


def correction_loss(A, rho, y):
    """(y.A y - 2 y.rho) / ((rho.rho)^2 / (rho.A rho)): the change of the
    error's A-norm squared that the correction y makes, in units of what a
    steepest-descent step along rho removes (negative is better)."""
    sd = (rho * rho).sum() ** 2 / (rho * apply_rows(A, rho)).sum().clamp_min(1e-30)
    return ((y * apply_rows(A, y)).sum() - 2.0 * (y * rho).sum()) / sd.clamp_min(1e-30)


def train_stream(n: int = 128, seeds=range(100, 2100), pairs: int = 2,
                 lr: float = 1e-3, seed: int = 0, init=None, log=print):
    """Training at the scale of the learned-preconditioner workload: one
    sphere-union scene per seed (by default 2,000 scenes at 128^3, seeds
    100-2099), each projected on the GPU; `pairs` residuals of its MGPCG
    iterations (with the V-cycle's z0 = V r) each give one optimiser step
    on correction_loss, then are discarded. Every convolution forward and
    backward runs on libjetgpu's tensor-core kernels. Returns (params, loss
    history)."""
    torch = _torch()
    conv = make_conv_fn()
    solver = FdmMgpcgSolver3(200, 6, 2, 2, 5, 2, 1e-6, 1.2, True)
    dev = torch.device("cuda", solver.config.device)
    start = init if init is not None else init_params(seed)
    P = [(torch.tensor(w, device=dev, requires_grad=True),
          torch.tensor(b, device=dev, requires_grad=True)) for w, b in start]
    flat_params = [t for p in P for t in p]
    seeds = list(seeds)
    steps = len(seeds) * pairs
    opt = torch.optim.Adam(flat_params, lr=lr)
    warm = max(1, min(200, steps // 10))
    sched = torch.optim.lr_scheduler.LambdaLR(
        opt, lambda s: min(1.0, (s + 1) / warm) *
        0.5 * (1.0 + np.cos(np.pi * min(s, steps) / steps)))
    hist = []
    for si, sd in enumerate(seeds):
        sc = device_scene(n, sd, dev)
        R, Z = harvest_device(solver, sc, n, pairs)
        k = net_level(solver)
        A = level0_rows(solver, n, dev)
        masks = fluid_masks(solver, n, k, dev)
        for r, z0 in zip(R, Z):
            with torch.no_grad():
                rho, rk = coarse_residual(A, masks, r, z0, k)
            feat, rms = net_input(solver, k, rk)
            if not float(rms) > 0:
                continue
            y = correction(conv, P, feat, rms, masks, k)
            loss = correction_loss(A, rho, y)
            opt.zero_grad()
            loss.backward()
            torch.nn.utils.clip_grad_norm_(flat_params, 1.0)
            opt.step()
            sched.step()
            hist.append(float(loss.detach()))
        del sc, R, Z
        if si % 100 == 0 or si == len(seeds) - 1:
            log(f"scene {si} (seed {sd}) loss {np.mean(hist[-2 * pairs * 50:]):.4f}")
    params = [(w.detach().cpu().numpy(), b.detach().cpu().numpy()) for w, b in P]
    solver.close()
    return params, hist


def evaluate(params, n: int, seed: int, tolerance: float = 1e-6,
             scene: str = "sphere_union"):
    """Solves one held-out scene (the sphere union of a seed outside the
    training range, or the FLIP dam-break sub-step) with the learned,
    multigrid and no preconditioner; returns {name: dict(status,
    iterations, relative residual, fallback used, ms)}, ms = the solve's
    device time (weights, system and Krylov solve) of a second solve."""
    flat = flatten(params)
    if scene == "sphere_union":
        sc = scenes.sphere_union_scene(n, seed=seed)
    else:
        sc = scenes.flip_first_substep(n, box_hi=(0.3, 0.8, 1.0),
                                       sphere=((0.6, 0.2, 0.5), 0.15))
    h = (1.0 / n,) * 3
    out = {}
    for pre in ("learned", "multigrid", "none"):
        s = FdmMgpcgSolver3(1000, 6, 2, 2, 5, 2, tolerance, 1.2, True,
                            preconditioner=pre, maxRefinements=8)
        if pre == "learned":
            s.load_network(flat)
        ps = GridFractionalSinglePhasePressureSolver3(s)
        vel = FaceCenteredGrid3((n,) * 3, h, (0, 0, 0), sc["u"], sc["v"], sc["w"])
        g = lambda d: CellCenteredScalarGrid3((n,) * 3, h, (0, 0, 0), d)
        for _ in range(2):
            st = ps.solve(vel, 1 / 60, vel.clone(), g(sc["boundary_sdf"]),
                          None, g(sc["fluid_sdf"]))
        t = ps.last_stats
        out[pre] = dict(status=st, iterations=t.iterations,
                        relative_residual=t.relative_residual,
                        fallback=bool(t.fallback_used),
                        ms=round(t.setup_ms + t.solve_ms, 3))
        s.close()
    return out


def coarse_correction_bound(n: int, scene: str = "sphere_union",
                            seed: int = 9001, levels=(1, 2, 3),
                            tolerance: float = 1e-6):
    """How many flexible-PCG iterations any coarse-level correction after the
    V-cycle can save: FPCG (FP64, torch) on the scene's finest-level system
    with M r = V r, and with M r = V r + mask P^k G^-1 (mask P^k)^T rho for
    rho = r - A V r and the Galerkin operator G = (mask P^k)^T A (mask P^k)
    solved by CG to 1e-8 — the best a correction computed on level k from
    rho can do in one step. Returns {"multigrid": (iterations, relative
    residual), "level<k>": ...}."""
    torch = _torch()
    if scene == "sphere_union":
        sc = scenes.sphere_union_scene(n, seed=seed)
    else:
        sc = scenes.flip_first_substep(n, box_hi=(0.3, 0.8, 1.0),
                                       sphere=((0.6, 0.2, 0.5), 0.15))
    h = (1.0 / n,) * 3
    s = FdmMgpcgSolver3(200, 6, 2, 2, 5, 2, tolerance, 1.2, True)
    ps = GridFractionalSinglePhasePressureSolver3(s)
    vel = FaceCenteredGrid3((n,) * 3, h, (0, 0, 0), sc["u"], sc["v"], sc["w"])
    g = lambda d: CellCenteredScalarGrid3((n,) * 3, h, (0, 0, 0), d)
    ps.solve(vel, 1 / 60, vel.clone(), g(sc["boundary_sdf"]), None,
             g(sc["fluid_sdf"]))
    dev = torch.device("cuda", s.config.device)
    A = level0_rows(s, n, dev).double()
    b = level0_rhs(s, n, dev).double()
    mask = fluid_masks(s, n, 0, dev)[0].double()

    def V(r):
        return vcycle_apply(s, r.float()).double()

    def adjoint(y):
        x = torch.zeros(tuple(d // 2 for d in y.shape), dtype=y.dtype,
                        device=y.device, requires_grad=True)
        with torch.enable_grad():
            (gx,) = torch.autograd.grad(prolong(x), x, grad_outputs=y)
        return gx

    def cg(op, rhs, tol=1e-8, maxit=2000):
        x = torch.zeros_like(rhs)
        r = rhs.clone()
        d = r.clone()
        rr = (r * r).sum()
        b2 = rr
        for _ in range(maxit):
            q = op(d)
            a = rr / (d * q).sum()
            x += a * d
            r -= a * q
            rn = (r * r).sum()
            if rn <= tol * tol * b2:
                break
            d = r + (rn / rr) * d
            rr = rn
        return x

    def fpcg(M, maxit=100):
        x = torch.zeros_like(b)
        r = b.clone()
        bn = float(b.norm())
        d = z_old = rz_old = None
        for it in range(1, maxit + 1):
            z = M(r)
            rz = (r * z).sum()
            d = z.clone() if d is None else z + (rz - (r * z_old).sum()) / rz_old * d
            q = apply_rows(A, d)
            a = rz / (d * q).sum()
            x += a * d
            r -= a * q
            z_old, rz_old = z, rz
            rel = float(r.norm()) / bn
            if rel <= tolerance:
                return it, rel
        return maxit, rel

    out = {"multigrid": fpcg(V)}
    for k in levels:
        def MP(e, k=k):
            for _ in range(k):
                e = prolong(e)
            return mask * e

        def MPt(y, k=k):
            y = mask * y
            for _ in range(k):
                y = adjoint(y)
            return y

        def M(r, k=k, MP=MP, MPt=MPt):
            z = V(r)
            rho = r - apply_rows(A, z)
            e = cg(lambda v: MPt(apply_rows(A, MP(v))), MPt(rho))
            return z + MP(e)
        out[f"level{k}"] = fpcg(M)
    s.close()
    return out


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(
        description="Trains the preconditioner network on the GPU: 2,000 "
                    "sphere-union scenes at 128^3 (seeds 100-2099) by default")
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--first-seed", type=int, default=100)
    ap.add_argument("--scenes", type=int, default=2000)
    ap.add_argument("--pairs", type=int, default=2)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--init", default=None,
                    help="start from these weights instead of a random "
                         "initialisation")
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--eval", type=int, nargs="*", default=[128, 256],
                    help="grid sizes of the held-out evaluation solves")
    ap.add_argument("--bound", type=int, nargs="*", default=None,
                    help="instead of training: for these grid sizes, the "
                         "FPCG iterations with an exact coarse-level "
                         "correction after the V-cycle "
                         "(coarse_correction_bound)")
    a = ap.parse_args()
    if a.bound is not None:
        for n in a.bound:
            for scene, seed in (("sphere_union", 9001), ("flip", 0)):
                print(json.dumps({"grid": n, "scene": scene, "seed": seed,
                                  **coarse_correction_bound(n, scene, seed)}),
                      flush=True)
        raise SystemExit(0)
    params, hist = train_stream(a.n, range(a.first_seed,
                                           a.first_seed + a.scenes),
                                a.pairs, lr=a.lr,
                                init=load(a.init) if a.init else None)
    save(params, a.out)
    print("saved", a.out, "final loss", np.mean(hist[-100:]))
    for n in a.eval:
        for seed in (9001, 9002):
            print(json.dumps({"held_out": f"{n}^3 sphere union seed {seed}",
                              **evaluate(params, n, seed)}), flush=True)
        print(json.dumps({"held_out": f"{n}^3 FLIP dam-break sub-step",
                          **evaluate(params, n, 0, scene="flip")}), flush=True)
