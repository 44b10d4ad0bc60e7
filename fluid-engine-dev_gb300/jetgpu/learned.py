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


def evaluate(params, n: int, seed: int, tolerance: float = 1e-6):
    """Solves one held-out sphere-union scene with the learned, multigrid and
    no preconditioner; returns {name: (status, iterations, relative residual,
    fallback used)}."""
    flat = flatten(params)
    sc = scenes.sphere_union_scene(n, seed=seed)
    h = (1.0 / n,) * 3
    out = {}
    for pre in ("learned", "multigrid", "none"):
        s = FdmMgpcgSolver3(1000, 8, 2, 2, 10, 2, tolerance, 1.0, True,
                            preconditioner=pre, maxRefinements=8)
        if pre == "learned":
            s.load_network(flat)
        ps = GridFractionalSinglePhasePressureSolver3(s)
        vel = FaceCenteredGrid3((n,) * 3, h, (0, 0, 0), sc["u"], sc["v"], sc["w"])
        g = lambda d: CellCenteredScalarGrid3((n,) * 3, h, (0, 0, 0), d)
        st = ps.solve(vel, 1 / 60, vel.clone(), g(sc["boundary_sdf"]), None,
                      g(sc["fluid_sdf"]))
        t = ps.last_stats
        out[pre] = (st, t.iterations, t.relative_residual, t.fallback_used)
        s.close()
    return out


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--scenes", type=int, default=24)
    ap.add_argument("--pairs", type=int, default=6)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--eval", type=int, nargs="*", default=[64],
                    help="grid sizes of the held-out evaluation solves")
    a = ap.parse_args()
    params, hist = train(a.n, a.scenes, a.pairs, a.steps, lr=a.lr)
    save(params, a.out)
    print("saved", a.out, "final loss", np.mean(hist[-50:]))
    for n in a.eval:
        for seed in (9001, 9002):
            print(f"held-out {n}^3 seed {seed}:", evaluate(params, n, seed))
