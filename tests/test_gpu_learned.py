"""Learned preconditioner: the library's M r against the training-time
composition, training on the tensor-core kernels, and flexible PCG with the
trained network (GPU).

The preconditioner is z = V r + mask P^k net(R^k (r - A V r)): one multigrid
V-cycle, then the network's correction of the error the V-cycle leaves,
computed on level k of the hierarchy (jetgpu_net_level)."""
import os

import numpy as np
import pytest

import jetgpu
from jetgpu import learned, scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _solved(n, seed, levels=6):
    """A solver whose last system is the sphere-union scene of `seed`."""
    h = (1.0 / n,) * 3
    solver = jetgpu.FdmMgpcgSolver3(200, levels, 2, 2, 5, 2, 1e-6, 1.2, True)
    ps = jetgpu.GridFractionalSinglePhasePressureSolver3(solver)
    sc = scenes.sphere_union_scene(n, seed=seed)
    vel = jetgpu.FaceCenteredGrid3((n,) * 3, h, (0, 0, 0), sc["u"], sc["v"],
                                   sc["w"])
    g = lambda d: jetgpu.CellCenteredScalarGrid3((n,) * 3, h, (0, 0, 0), d)
    assert ps.solve(vel, 1 / 60, vel.clone(), g(sc["boundary_sdf"]), None,
                    g(sc["fluid_sdf"])) == 0
    return solver


@pytest.mark.parametrize("n", [32, 128])
def test_library_preconditioner_matches_training_composition(n):
    """jetgpu_learned_apply against the training code's composition of the
    same pieces (V-cycle, residual, masked restriction, network, masked
    prolongation) for an untrained network; k = 0 at 32^3 (the network on
    the finest level), k = 1 at 128^3."""
    solver = _solved(n, seed=7)
    params = learned.init_params(seed=1)
    # Scale the output layer up so that the network's share of z is not
    # negligible (the initial output layer starts near zero).
    params[-1] = (params[-1][0] * 100.0, params[-1][1])
    solver.load_network(learned.flatten(params))
    dev = torch.device("cuda", 0)
    k = learned.net_level(solver)
    assert k == (0 if n <= 64 else 1)
    A = learned.level0_rows(solver, n, dev)
    masks = learned.fluid_masks(solver, n, k, dev)
    r = learned.level0_rhs(solver, n, dev)
    z_lib = learned.learned_apply(solver, r.reshape(-1)).reshape(n, n, n)
    conv = learned.make_conv_fn()
    P = [(torch.tensor(w, device=dev), torch.tensor(b, device=dev))
         for w, b in params]
    with torch.no_grad():
        z0 = learned.vcycle_apply(solver, r)
        rho, rk = learned.coarse_residual(A, masks, r, z0, k)
        feat, rms = learned.net_input(solver, k, rk)
        y = learned.correction(conv, P, feat, rms, masks, k)
        # The network alone, through the C ABI, on the same level-k input.
        e_lib = torch.empty_like(rk)
        learned._sync()
        solver.check(jetgpu.library().jetgpu_net_apply(
            solver.context(), k, rk.contiguous().data_ptr(), e_lib.data_ptr()))
        e_py = learned.forward(conv, P, feat) * (rms / learned.NET_GAIN) * masks[k]
    assert float(y.abs().max()) > 0.05 * float(z0.abs().max())
    err_e = float((e_lib - e_py).abs().max() / e_py.abs().max())
    err_z = float((z_lib - (z0 + y)).abs().max() / (z0 + y).abs().max())
    print(f"n={n} k={k}: network {err_e:.2e}, preconditioner {err_z:.2e}")
    assert err_e < 2e-2
    assert err_z < 2e-2
    solver.close()


def test_training_on_tensor_core_kernels_reduces_loss():
    """A few optimiser steps on 32^3 scenes lower the correction loss (the
    change of the error's A-norm the correction makes, in steepest-descent
    steps) below zero: the network learns to remove error the V-cycle
    leaves."""
    params, hist = learned.train_stream(n=32, seeds=range(6), pairs=4,
                                        lr=1e-3, log=lambda *a: None)
    print("loss first/last:", hist[:3], hist[-3:])
    assert np.mean(hist[-4:]) < np.mean(hist[:2])
    assert np.mean(hist[-4:]) < 0.0
    assert len(learned.flatten(params)) == jetgpu.library().jetgpu_net_param_count()


def _fpcg_run(n, sc, pre, flat=None):
    h = (1.0 / n,) * 3
    s = jetgpu.FdmMgpcgSolver3(400, 6, 2, 2, 5, 2, 1e-6, 1.2, True,
                               preconditioner=pre, maxRefinements=8)
    if flat is not None:
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


@pytest.mark.skipif(not os.path.exists(learned.WEIGHTS),
                    reason="trained weights not present")
def test_learned_fpcg_converges_without_fallback():
    """Held-out 128^3 scene (a seed outside the training range): flexible PCG
    with the trained preconditioner reaches the 1e-6 relative residual by
    itself (no multigrid fallback), in no more iterations than multigrid
    PCG and far fewer than CG without a preconditioner."""
    n = 128
    sc = scenes.sphere_union_scene(n, seed=9001)
    flat = learned.flatten(learned.load())
    st_l, it_l, rel_l, fb = _fpcg_run(n, sc, "learned", flat)
    st_m, it_m, rel_m, _ = _fpcg_run(n, sc, "multigrid")
    st_n, it_n, rel_n, _ = _fpcg_run(n, sc, "none")
    print(f"iterations: learned {it_l} multigrid {it_m} none {it_n}")
    assert st_l == 0 and not fb and rel_l <= 1e-6
    assert it_l <= it_m
    assert it_l < it_n


@pytest.mark.skipif(not os.path.exists(learned.WEIGHTS),
                    reason="trained weights not present")
def test_trained_network_gain_over_the_vcycle():
    """What training gains, measured against the method without the
    network. A preconditioner step z from residual r leaves the error
    e - z, and removes G(z) = ||e||_A^2 - ||e - z||_A^2 = 2 z.r - z.A z of
    the error's energy (no solve needed). On held-out residuals of a 128^3
    scene outside the training seeds, the trained network's correction
    must remove more than the V-cycle alone, and more than the untrained
    network's correction does. The line-search energy (r.z)^2 / (z.A z) is
    printed beside it."""
    n = 128
    solver = _solved(n, seed=9003)
    dev = torch.device("cuda", 0)
    A = learned.level0_rows(solver, n, dev).double()
    R = torch.empty((3, n ** 3), dtype=torch.float32, device=dev)
    Z = torch.empty((3, n ** 3), dtype=torch.float32, device=dev)
    import ctypes as C
    cnt = C.c_uint(0)
    solver.check(jetgpu.library().jetgpu_harvest(
        solver.context(), 3, R.data_ptr(), Z.data_ptr(), C.byref(cnt)))
    rs = [R[i].reshape(n, n, n) for i in range(cnt.value)]

    def removed(r, z):
        r, z = r.double(), z.double()
        return float(2.0 * (z * r).sum() - (z * learned.apply_rows(A, z)).sum())

    gains, search = {}, {}
    for name, params in (("trained", learned.load()),
                         ("untrained", learned.init_params(seed=0))):
        solver.load_network(learned.flatten(params))
        g, s = [], []
        with torch.no_grad():
            for r in rs:
                z_v = learned.vcycle_apply(solver, r)
                z_l = learned.learned_apply(solver, r)
                g.append(removed(r, z_l) / removed(r, z_v))
                s.append(float(learned.step_energy(A, r.double(), z_l.double()) /
                               learned.step_energy(A, r.double(), z_v.double())))
        gains[name] = float(np.mean(g))
        search[name] = float(np.mean(s))
    solver.close()
    print(f"energy removed by the step, relative to the V-cycle alone: "
          f"trained {gains['trained']:.3f} untrained {gains['untrained']:.3f}; "
          f"with a line search: trained {search['trained']:.3f} untrained "
          f"{search['untrained']:.3f}")
    assert gains["trained"] > 1.0
    assert gains["trained"] > gains["untrained"]
