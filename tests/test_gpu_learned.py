"""Learned preconditioner: inference inside libjetgpu vs the training-time
forward, training on the tensor-core kernels, and flexible PCG with the
trained network (GPU)."""
import ctypes as C
import os

import numpy as np
import pytest

import jetgpu
from jetgpu import learned, scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_library_and_training_forward_agree():
    n = 32
    solver = jetgpu.FdmMgpcgSolver3(200, 5, 2, 2, 10, 2, 1e-6, 1.0, True)
    params = learned.init_params(seed=1)
    solver.load_network(learned.flatten(params))
    sc = scenes.sphere_union_scene(n, seed=7)
    samples = learned.harvest(solver, sc, n, 2)
    assert len(samples) == 2
    feat, target, mask = samples[1]
    dev = feat.device
    # Residual behind the sample: harvest it again to get r itself.
    R = torch.empty((1, n ** 3), dtype=torch.float32, device=dev)
    Z = torch.empty((1, n ** 3), dtype=torch.float32, device=dev)
    cnt = C.c_uint(0)
    L = jetgpu.library()
    solver.check(L.jetgpu_harvest(solver.context(), 1, R.data_ptr(), Z.data_ptr(),
                                  C.byref(cnt)))
    z_lib = torch.empty(n ** 3, dtype=torch.float32, device=dev)
    solver.check(L.jetgpu_net_apply(solver.context(), R[0].data_ptr(),
                                    z_lib.data_ptr()))
    f0 = torch.empty((n, n, n, 16), dtype=torch.bfloat16, device=dev)
    solver.check(L.jetgpu_net_features(solver.context(), R[0].data_ptr(),
                                       f0.data_ptr()))
    conv = learned.make_conv_fn()
    P = [(torch.tensor(w, device=dev), torch.tensor(b, device=dev))
         for w, b in params]
    with torch.no_grad():
        out = learned.forward(conv, P, f0)
    rms = torch.sqrt(torch.mean(R[0].double() ** 2)).float()
    z_py = (out * rms / learned.NET_GAIN * f0[..., 7].float()).reshape(-1)
    err = (z_py - z_lib).abs().max() / z_py.abs().max()
    assert float(err) < 2e-2
    solver.close()


def test_training_on_tensor_core_kernels_reduces_loss():
    params, hist = learned.train(n=32, scenes_count=4, pairs=3, steps=80,
                                 lr=3e-3, log=lambda *a: None)
    assert np.mean(hist[-20:]) < 0.8 * np.mean(hist[:5])
    assert len(learned.flatten(params)) == jetgpu.library().jetgpu_net_param_count()


@pytest.mark.skipif(not os.path.exists(learned.WEIGHTS),
                    reason="trained weights not present")
def test_learned_fpcg_reaches_tolerance_and_beats_no_preconditioner():
    """Held-out scene (seed outside the training range). The trained network
    inside flexible PCG reaches the 1e-6 relative residual (possibly with
    the multigrid fallback) and needs far fewer iterations than CG without
    a preconditioner: what the network gains over the method without it."""
    n = 64
    h = (1.0 / n,) * 3
    sc = scenes.sphere_union_scene(n, seed=9001)
    flat = learned.flatten(learned.load())

    def run(pre):
        s = jetgpu.FdmMgpcgSolver3(400, 6, 2, 2, 10, 2, 1e-6, 1.0, True,
                                   preconditioner=pre, maxRefinements=8)
        if pre == "learned":
            s.load_network(flat)
        ps = jetgpu.GridFractionalSinglePhasePressureSolver3(s)
        vel = jetgpu.FaceCenteredGrid3((n,) * 3, h, (0, 0, 0), sc["u"], sc["v"],
                                       sc["w"])
        g = lambda d: jetgpu.CellCenteredScalarGrid3((n,) * 3, h, (0, 0, 0), d)
        st = ps.solve(vel, 1 / 60, vel.clone(), g(sc["boundary_sdf"]), None,
                      g(sc["fluid_sdf"]))
        stats = ps.last_stats
        s.close()
        return st, stats.iterations, stats.relative_residual, stats.fallback_used

    st_l, it_l, rel_l, fb = run("learned")
    st_n, it_n, rel_n, _ = run("none")
    assert st_l in (0, 2) and rel_l <= 1e-6
    assert it_l < it_n


def _apply_rows(A, x):
    """A x for level rows A[..., (center, right, up, front)] (FdmBlas3::mvm,
    src/jet/fdm_linear_system3.cpp:79-96), in float64."""
    y = A[..., 0] * x
    y[:, :, 1:] += A[:, :, :-1, 1] * x[:, :, :-1]
    y[:, :, :-1] += A[:, :, :-1, 1] * x[:, :, 1:]
    y[:, 1:, :] += A[:, :-1, :, 2] * x[:, :-1, :]
    y[:, :-1, :] += A[:, :-1, :, 2] * x[:, 1:, :]
    y[1:] += A[:-1, :, :, 3] * x[:-1]
    y[:-1] += A[:-1, :, :, 3] * x[1:]
    return y


@pytest.mark.skipif(not os.path.exists(learned.WEIGHTS),
                    reason="trained weights not present")
def test_trained_network_gain_over_untrained_and_no_preconditioner():
    """What training gains, measured on the network alone. For a
    preconditioned step z from residual r, the exact line search removes
    (r.z)^2 / (z.A z) of the error's energy (A-norm squared). On held-out
    residuals of a 64^3 scene outside the training seeds, that energy per
    step, relative to the step without a preconditioner (z = r), must be
    larger for the trained network than for the same network untrained and
    than for no preconditioner. The multigrid V-cycle's z is printed for
    scale."""
    n = 64
    h = (1.0 / n,) * 3
    sc = scenes.sphere_union_scene(n, seed=9003)
    solver = jetgpu.FdmMgpcgSolver3(200, 6, 2, 2, 10, 2, 1e-6, 1.0, True)
    ps = jetgpu.GridFractionalSinglePhasePressureSolver3(solver)
    vel = jetgpu.FaceCenteredGrid3((n,) * 3, h, (0, 0, 0), sc["u"], sc["v"],
                                   sc["w"])
    g = lambda d: jetgpu.CellCenteredScalarGrid3((n,) * 3, h, (0, 0, 0), d)
    assert ps.solve(vel, 1 / 60, vel.clone(), g(sc["boundary_sdf"]), None,
                    g(sc["fluid_sdf"])) == 0
    A = ps.level(0, "A").reshape(n, n, n, 4)
    dev = torch.device("cuda", 0)
    N = n ** 3
    R = torch.empty((3, N), dtype=torch.float32, device=dev)
    Z = torch.empty((3, N), dtype=torch.float32, device=dev)
    cnt = C.c_uint(0)
    L = jetgpu.library()
    solver.check(L.jetgpu_harvest(solver.context(), 3, R.data_ptr(),
                                  Z.data_ptr(), C.byref(cnt)))
    rs = [R[k].cpu().numpy().astype(np.float64).reshape(n, n, n)
          for k in range(cnt.value)]

    def energy(r, z):
        return float(np.sum(r * z)) ** 2 / float(np.sum(z * _apply_rows(A, z)))

    gain = {"trained": [], "untrained": [], "multigrid": []}
    base = [energy(r, r) for r in rs]
    for name, params in (("trained", learned.load()),
                         ("untrained", learned.init_params(seed=0))):
        solver.load_network(learned.flatten(params))
        for k, r in enumerate(rs):
            z = torch.empty(N, dtype=torch.float32, device=dev)
            solver.check(L.jetgpu_net_apply(solver.context(), R[k].data_ptr(),
                                            z.data_ptr()))
            zz = z.cpu().numpy().astype(np.float64).reshape(n, n, n)
            gain[name].append(energy(r, zz) / base[k])
    for k, r in enumerate(rs):
        zz = Z[k].cpu().numpy().astype(np.float64).reshape(n, n, n)
        gain["multigrid"].append(energy(r, zz) / base[k])
    solver.close()
    tr, un, mg = (float(np.mean(gain[k]))
                  for k in ("trained", "untrained", "multigrid"))
    print(f"energy removed per step relative to no preconditioner: trained "
          f"{tr:.2f} untrained {un:.2f} multigrid {mg:.2f}")
    assert tr > 1.0 and tr > un
