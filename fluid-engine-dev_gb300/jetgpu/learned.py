"""Training of the learned preconditioner (3-D U-Net) on the tensor-core
kernels of libjetgpu.

The network maps the 16 input channels libjetgpu builds for a residual r
(``jetgpu_net_features``: r / rms(r), the six face weights of each cell,
fluid indicator, scaled diagonal) to NET_GAIN * z / rms(r), where z = M r is
the multigrid V-cycle's correction. For the smooth modes that dominate a
preconditioned residual z is about r / (3 pi^2) at any grid spacing, so the
target is O(1) and independent of the resolution. Pairs (r_k, z_k) come from the solver's own
MGPCG iterations (``jetgpu_harvest``). Every convolution of the forward and
backward passes runs on libjetgpu's tcgen05 kernels (``jetgpu_conv3d`` and
``jetgpu_conv3d_wgrad``); PyTorch supplies device memory, the optimizer and
the element-wise glue (pooling, upsampling, concatenation, ReLU masks),
mirroring the library's inference path (``unet.cu``) step for step.

The trained parameters are used by the flexible PCG of libjetgpu through
``jetgpu_load_unet`` (``preconditioner = JETGPU_PRECOND_LEARNED``).
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
# Data from the solver.

def harvest(solver: FdmMgpcgSolver3, sc: dict, n: int, pairs: int):
    """Solves the scene's pressure system, then records `pairs` (features,
    target, fluid mask) samples from the solver's MGPCG iterations."""
    torch = _torch()
    L = library()
    h = 1.0 / n
    ps = GridFractionalSinglePhasePressureSolver3(solver)
    vel = FaceCenteredGrid3((n,) * 3, (h,) * 3, (0, 0, 0), sc["u"], sc["v"], sc["w"])
    out = vel.clone()
    g = lambda d: CellCenteredScalarGrid3((n,) * 3, (h,) * 3, (0, 0, 0), d)
    ps.solve(vel, 1 / 60, out, g(sc["boundary_sdf"]), None, g(sc["fluid_sdf"]))
    dev = torch.device("cuda", solver.config.device)
    N = n ** 3
    R = torch.empty((pairs, N), dtype=torch.float32, device=dev)
    Z = torch.empty((pairs, N), dtype=torch.float32, device=dev)
    cnt = C.c_uint(0)
    solver.check(L.jetgpu_harvest(solver.context(), pairs, R.data_ptr(),
                                  Z.data_ptr(), C.byref(cnt)))
    samples = []
    fluid = torch.from_numpy((sc["fluid_sdf"] < 0).astype(np.float32)).to(dev)
    for k in range(cnt.value):
        feat = torch.empty((n, n, n, 16), dtype=torch.bfloat16, device=dev)
        solver.check(L.jetgpu_net_features(solver.context(), R[k].data_ptr(),
                                           feat.data_ptr()))
        rms = torch.sqrt(torch.mean(R[k].double() ** 2)).float()
        if rms <= 0:
            continue
        target = (Z[k] * (NET_GAIN / rms)).reshape(n, n, n)
        mask = feat[..., 7].float()
        samples.append((feat, target, mask))
    del fluid
    return samples


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
    """harvest() for a scene already on the device (device_scene): the
    projection through jetgpu_solve_pressure_device, then `pairs` samples of
    the MGPCG iterations on that system."""
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
    torch.cuda.synchronize()
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
    samples = []
    for k in range(cnt.value):
        feat = torch.empty((n, n, n, 16), dtype=torch.bfloat16, device=dev)
        solver.check(L.jetgpu_net_features(solver.context(), R[k].data_ptr(),
                                           feat.data_ptr()))
        rms = torch.sqrt(torch.mean(R[k].double() ** 2)).float()
        if rms <= 0:
            continue
        target = (Z[k] * (NET_GAIN / rms)).reshape(n, n, n)
        samples.append((feat, target, feat[..., 7].float()))
    return samples


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


def vcycle_apply(solver: FdmMgpcgSolver3, r):
    """z = M r with the solver's multigrid V-cycle (jetgpu_vcycle_apply)."""
    torch = _torch()
    z = torch.empty_like(r).contiguous()
    solver.check(library().jetgpu_vcycle_apply(
        solver.context(), r.contiguous().data_ptr(), z.data_ptr()))
    return z


def fpcg_samples(solver: FdmMgpcgSolver3, conv, P, n: int, iters: int):
    """Samples from the network's own flexible-PCG trajectory on the
    solver's last system: starting from x = 0, each iteration's residual r_k
    becomes a sample (its features, the V-cycle's correction M r_k as the
    target, the fluid mask), and the iteration continues with the network's
    correction, as the library's flexible PCG does (Polak-Ribiere beta).
    The residuals a network meets inside its own solve differ from those of
    multigrid PCG; training on them keeps it useful past the first step."""
    torch = _torch()
    L = library()
    dev = P[0][0].device
    A = level0_rows(solver, n, dev)
    r = level0_rhs(solver, n, dev)
    out = []
    d = z_old = None
    rz_old = 0.0
    with torch.no_grad():
        for k in range(iters):
            rms = torch.sqrt(torch.mean(r.double() ** 2)).float()
            if not float(rms) > 0:
                break
            feat = torch.empty((n, n, n, 16), dtype=torch.bfloat16, device=dev)
            solver.check(L.jetgpu_net_features(solver.context(),
                                               r.contiguous().data_ptr(),
                                               feat.data_ptr()))
            mask = feat[..., 7].float()
            zmg = vcycle_apply(solver, r)
            out.append((feat, (zmg * (NET_GAIN / rms)).reshape(n, n, n), mask))
            z = forward(conv, P, feat) * (rms / NET_GAIN) * mask
            rz = float((r * z).sum())
            if k == 0 or d is None:
                d = z.clone()
            else:
                beta = float((r * (z - z_old)).sum()) / rz_old if rz_old else 0.0
                d = z + beta * d
            q = apply_rows(A, d)
            dq = float((d * q).sum())
            if not (dq > 0 and rz > 0):
                break
            r = r - (rz / dq) * q
            z_old, rz_old = z, rz
    return out


def train_stream(n: int = 128, seeds=range(100, 2100), pairs: int = 2,
                 lr: float = 2e-3, seed: int = 0, init=None, log=print,
                 loss_kind: str = "energy", own: int = 0):
    """Training at the scale of BASELINE's learned-preconditioner config:
    one sphere-union scene per seed (by default 2,000 scenes at 128^3, seeds
    100-2099), each solved on the GPU, `pairs` (residual, V-cycle
    correction) samples harvested from its MGPCG iterations and used for one
    optimiser step each, then discarded (a 128^3 sample is 64 MB of BF16
    features). Every convolution forward and backward runs on libjetgpu's
    tensor-core kernels. With `own` > 0, the residuals of the first `own`
    iterations of the network's own flexible PCG on each scene are added as
    samples (fpcg_samples). Returns (params, loss history)."""
    torch = _torch()
    conv = make_conv_fn()
    solver = FdmMgpcgSolver3(200, 6, 2, 2, 10, 2, 1e-6, 1.0, True)
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
        samples = harvest_device(solver, sc, n, pairs)
        if own > 0:
            samples += fpcg_samples(solver, conv, P, n, own)
        A = level0_rows(solver, n, dev) if loss_kind == "energy" else None
        for feat, target, mask in samples:
            pred = forward(conv, P, feat)
            if loss_kind == "energy":
                # One minus the energy a step along the network's output
                # removes, relative to the V-cycle's step (scale-free).
                r = feat[..., 0].float() * mask
                z = pred * mask
                loss = 1.0 - step_energy(A, r, z) / step_energy(
                    A, r, target * mask).detach()
            else:
                err = (pred - target) * mask
                loss = (err * err).sum() / ((target * mask) ** 2).sum().clamp_min(1e-30)
            opt.zero_grad()
            loss.backward()
            torch.nn.utils.clip_grad_norm_(flat_params, 1.0)
            opt.step()
            sched.step()
            hist.append(float(loss.detach()))
        del sc
        if si % 100 == 0 or si == len(seeds) - 1:
            log(f"scene {si} (seed {sd}) loss {np.mean(hist[-2 * pairs * 50:]):.4f}")
    params = [(w.detach().cpu().numpy(), b.detach().cpu().numpy()) for w, b in P]
    solver.close()
    return params, hist


def training_scenes(n: int, count: int, first_seed: int = 100):
    """Sphere-union scenes (16 spheres, seeds first_seed..) and FLIP first
    sub-step boxes of varying size."""
    out = []
    rng = np.random.default_rng(first_seed)
    for s in range(count):
        if s % 2 == 0:
            out.append(scenes.sphere_union_scene(n, seed=first_seed + s))
        else:
            hi = (rng.uniform(0.2, 0.9), rng.uniform(0.3, 0.9), 1.0)
            c = (rng.uniform(0.3, 0.8), rng.uniform(0.15, 0.5), rng.uniform(0.3, 0.7))
            out.append(scenes.flip_first_substep(n, box_hi=hi,
                                                 sphere=(c, rng.uniform(0.08, 0.2))))
    return out


def train(n: int = 64, scenes_count: int = 24, pairs: int = 6,
          steps: int = 600, lr: float = 2e-3, seed: int = 0, log=print):
    torch = _torch()
    conv = make_conv_fn()
    solver = FdmMgpcgSolver3(200, 6, 2, 2, 10, 2, 1e-6, 1.0, True)
    data = []
    for sc in training_scenes(n, scenes_count):
        data += harvest(solver, sc, n, pairs)
    log(f"harvested {len(data)} samples at {n}^3")
    dev = data[0][0].device
    P = [(torch.tensor(w, device=dev, requires_grad=True),
          torch.tensor(b, device=dev, requires_grad=True))
         for w, b in init_params(seed)]
    flat_params = [t for p in P for t in p]
    opt = torch.optim.Adam(flat_params, lr=lr)
    warm = max(1, min(200, steps // 10))
    sched = torch.optim.lr_scheduler.LambdaLR(
        opt, lambda s: min(1.0, (s + 1) / warm) *
        0.5 * (1.0 + np.cos(np.pi * min(s, steps) / steps)))
    rng = np.random.default_rng(seed)
    hist = []
    for step in range(steps):
        feat, target, mask = data[rng.integers(len(data))]
        pred = forward(conv, P, feat)
        err = (pred - target) * mask
        loss = (err * err).sum() / ((target * mask) ** 2).sum().clamp_min(1e-30)
        opt.zero_grad()
        loss.backward()
        torch.nn.utils.clip_grad_norm_(flat_params, 1.0)
        opt.step()
        sched.step()
        hist.append(float(loss.detach()))
        if step % 50 == 0 or step == steps - 1:
            log(f"step {step} loss {np.mean(hist[-50:]):.4f}")
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
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--loss", default="energy", choices=["energy", "mse"],
                    help="energy: the error energy a step along the output "
                         "removes, relative to the V-cycle's step; mse: "
                         "relative squared error to the V-cycle's output")
    ap.add_argument("--own", type=int, default=6,
                    help="iterations of the network's own flexible PCG whose "
                         "residuals are added as samples per scene")
    ap.add_argument("--init", default=None,
                    help="start from these weights instead of a random "
                         "initialisation")
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--eval", type=int, nargs="*", default=[128, 256],
                    help="grid sizes of the held-out evaluation solves")
    a = ap.parse_args()
    params, hist = train_stream(a.n, range(a.first_seed,
                                           a.first_seed + a.scenes),
                                a.pairs, lr=a.lr, loss_kind=a.loss,
                                own=a.own,
                                init=load(a.init) if a.init else None)
    save(params, a.out)
    print("saved", a.out, "final loss", np.mean(hist[-100:]))
    for n in a.eval:
        for seed in (9001, 9002):
            print(json.dumps({"held_out": f"{n}^3 sphere union seed {seed}",
                              **evaluate(params, n, seed)}), flush=True)
        print(json.dumps({"held_out": f"{n}^3 FLIP dam-break sub-step",
                          **evaluate(params, n, 0, scene="flip")}), flush=True)
