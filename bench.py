"""Benchmark: 256^3 FLIP pressure solve on one GB300 (replicas for N > 1).

Workload: the pressure system of the first sub-step of the 256^3 FLIP dam
break with a static solid sphere (water box [0,.3]x[0,.8]x[0,1], sphere
r=.15 at (.6,.2,.5), gravity for one 1/60 s step, closed walls; h = 1/256),
solved to a true relative residual of 1e-6 by
GridFractionalSinglePhasePressureSolver3 + MGPCG: weights, system build,
MGPCG and the pressure-gradient update — the whole projection per step.

Arms:
* ours (default): `value` = ms per pressure solve with inputs resident in
  HBM (device-pointer C ABI); `e2e` = the same through the host-pointer C ABI
  with pinned host buffers, called the way GridFluidSolver3 calls its
  pressure solver (the output holds the input's values; fluid_box_io, as
  the C++ adapter sets it): H2D of the SDFs and of the velocity faces
  around the fluid, D2H of the projected velocity faces, inside the timed
  region; the median of three batches of K solves.
* --impl reference: the reference's CPU algorithm (the oracle port, bit-exact
  with the reference; or the reference itself where it was compiled on this
  machine) on all host cores, each step one full reference pressure solve
  (about 10 s on 8 cores); the reference's MGPCG breaks down at 256^3 before
  1e-6, and the residual it reaches is reported.

Also in the line (same rules, not the headline): `flip_steps` — whole
FLIP frames resident on the GPU (transfers, particle SDF, boundary
conditions, gravity, pressure, advection under the reference's adaptive
sub-stepping) for the 256^3 dam break with the sphere (about 32M particles)
and the 64^3 dam break (60 frames); `smoke_512_pressure` — the projection of
the 512^3 smoke plume (all fluid, closed box); `blocked_pressure` — the
blocked solver (GridSinglePhasePressureSolver3) on the headline scene, with
one solve of the reference's CPU algorithm beside it.

Timing: W warm-up solves, then K solves bracketed by a barrier and
synchronize, timed with CUDA events on the library's own stream, max over
ranks. The working set (0.5 GB of FP64 inputs, 3+ GB of solver state) is
far larger than L2, so no flush is needed. Clocks are sampled during the
timed region: SM clock and clock-event reasons read through NVML every
5 ms (read-only queries), or nvidia-smi every 200 ms where NVML does not
load.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "fluid-engine-dev_gb300"))
sys.path.insert(0, REPO)

METRIC = ("256³ FLIP pressure-solve ms & steps/s at 1e-6 residual: "
          "learned vs plain MGPCG")
TOL = 1e-6


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", "--grid", dest="n", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-flip", action="store_true",
                    help="skip the whole-FLIP-frame measurements")
    ap.add_argument("--no-blocked", action="store_true",
                    help="skip the blocked pressure solver leg")
    ap.add_argument("--no-smoke", action="store_true",
                    help="skip the 512^3 smoke-plume projection")
    ap.add_argument("--flip-frames", type=int, default=30,
                    help="timed frames of the 256^3 FLIP dam break")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the accuracy block (pressure rel-L2 and "
                         "divergence against an FP64 answer)")
    ap.add_argument("--variants", default=",".join(VARIANTS),
                    help="comma-separated solver variants to run "
                         "(plain_mgpcg, mixed_mgpcg, learned_fpcg)")
    ap.add_argument("--conv-only", action="store_true",
                    help="time only the network's 128^3 convolutions (the "
                         "roofline_tensor block) and print it; for profiling")
    return ap.parse_args()


def dist_setup(args):
    """One process per GPU under torchrun; replicas (no collective on the
    data path, only a barrier and a max for the timing)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if args.impl == "ours" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        pg = dist
    return rank, world, local, pg


def barrier(pg, device=None):
    if pg is not None:
        if device is not None:
            pg.barrier(device_ids=[device])
        else:
            pg.barrier()


def max_over_ranks(pg, value: float, device=None) -> float:
    if pg is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64,
                     device=f"cuda:{device}" if device is not None else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class NvmlClocks:
    """SM clock and clock-event reasons read through NVML (the driver's
    libnvidia-ml, read-only queries) every few milliseconds from a thread,
    so that a timed region of well under a second still gets a dozen
    samples. Same result dictionary as Clocks; `ok` is False where NVML
    cannot be loaded."""

    # nvmlClocksEventReasons bits
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown",
               0x20: "sw_thermal_slowdown", 0x4: "sw_power_cap"}

    def __init__(self, gpu: int, period_s: float = 0.005):
        import ctypes
        import threading
        self.C, self.threading = ctypes, threading
        self.period = period_s
        self.ok = False
        self.rows = []
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                return
            h = ctypes.c_void_p()
            if nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(gpu),
                                                ctypes.byref(h)) != 0:
                return
            self.nv, self.h = nv, h
            self.reasons_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons",
                                      None) or nv.nvmlDeviceGetCurrentClocksThrottleReasons
            mx = ctypes.c_uint()
            if nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) != 0:
                return
            self.max_mhz = float(mx.value)
            self.ok = True
        except (OSError, AttributeError):
            self.ok = False

    def _sample(self):
        C = self.C
        mhz, rs = C.c_uint(), C.c_ulonglong()
        if (self.nv.nvmlDeviceGetClockInfo(self.h, 1, C.byref(mhz)) == 0 and
                self.reasons_fn(self.h, C.byref(rs)) == 0):
            self.rows.append((float(mhz.value), int(rs.value)))

    def start(self):
        self.rows, self.stop_ev = [], self.threading.Event()

        def run():
            while not self.stop_ev.is_set():
                self._sample()
                self.stop_ev.wait(self.period)

        self._sample()
        self.thread = self.threading.Thread(target=run, daemon=True)
        self.thread.start()

    def stop(self) -> dict:
        self.stop_ev.set()
        self.thread.join(timeout=5)
        self._sample()
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(r[0] for r in self.rows)
        reasons = sorted({name for _, bits in self.rows
                          for bit, name in self.REASONS.items() if bits & bit})
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": self.max_mhz,
                "reasons": reasons, "samples": len(self.rows),
                "source": "nvml"}


class Clocks:
    """nvidia-smi sampling during the timed region (NVML polling where the
    driver's library loads; nvidia-smi's 200 ms period otherwise)."""

    def __new__(cls, gpu: int):
        nv = NvmlClocks(gpu)
        if nv.ok:
            return nv
        return super().__new__(cls)

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,"
             "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if r[5 + i].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def workload(n: int):
    from jetgpu import scenes
    return scenes.flip_first_substep(n, box_hi=(0.3, 0.8, 1.0),
                                     sphere=((0.6, 0.2, 0.5), 0.15))


def solver_params(precision: str, preconditioner: str = "multigrid"):
    """GPU solver settings: FdmMgpcgSolver3(200, 6, 2, 2, 5, 2, 1e-6, 1.2,
    true). Two symmetric red-black SOR sweeps per level (omega 1.2) and a
    masked coarse residual give mesh-independent convergence (5-7
    iterations)."""
    return dict(numberOfCgIter=200, maxNumberOfLevels=6,
                numberOfRestrictionIter=2, numberOfCorrectionIter=2,
                numberOfCoarsestIter=5, numberOfFinalIter=2,
                maxTolerance=TOL, sorFactor=1.2, useRedBlackOrdering=True,
                precision=precision, preconditioner=preconditioner,
                maxRefinements=8)


# The solver variants the metric compares, all to the same 1e-6 relative
# true residual: plain MGPCG (FP32 Krylov and V-cycle, FP64-accurate
# reductions and refinement), the mixed-precision V-cycle (BF16 rows), and
# flexible PCG with the learned preconditioner (the mixed V-cycle plus the
# U-Net's coarse-level correction; when trained weights are present).
VARIANTS = {
    "plain_mgpcg": ("fp32", "multigrid"),
    "mixed_mgpcg": ("mixed", "multigrid"),
    "learned_fpcg": ("mixed", "learned"),
}


def peaks() -> dict:
    """Roofline denominators: the measured copy bandwidth and cuBLAS BF16
    burst throughput of the GB300s when MEASURED_PEAKS.json is
    present, else the fallback figures (6.8 TB/s, 1.9 PFLOP/s)."""
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return {"hbm_gbs": d.get("hbm_gbs"), "source": "measured",
                "bf16_tflops": d.get("bf16_tflops") or 1900.0,
                "tensor_source": "measured" if d.get("bf16_tflops")
                else "fallback"}
    return {"hbm_gbs": 6800.0, "source": "fallback", "bf16_tflops": 1900.0,
            "tensor_source": "fallback"}


def run_unet(local, n: int = 128, reps: int = 10):
    """Tensor-pipe roofline of the learned preconditioner's convolutions:
    the level-0 layer (3x3x3, 16 -> 16 channels, BF16, FP32 accumulation)
    at n^3 through jetgpu_conv3d, CUDA events over `reps` launches after
    warm-up; FLOP = 2 * 27 * C_in * C_out per cell."""
    import ctypes as C
    import torch
    import jetgpu
    L = jetgpu.library()
    dev = torch.device("cuda", local)
    out = {}
    for ci, co in ((16, 16), (48, 16)):
        g = torch.Generator(device=dev)
        g.manual_seed(0)
        x = (torch.randn((n, n, n, ci), generator=g, device=dev) * 0.1).to(
            torch.bfloat16)
        w = (torch.randn((27, co, ci), generator=g, device=dev) * 0.05).to(
            torch.bfloat16)
        b = torch.zeros(co, device=dev)
        y = torch.empty((n, n, n, co), dtype=torch.bfloat16, device=dev)
        err = torch.zeros(1, dtype=torch.int32, device=dev)
        res = (C.c_int * 3)(n, n, n)
        s = torch.cuda.current_stream(dev).cuda_stream

        def call():
            st = L.jetgpu_conv3d(s, x.data_ptr(), ci, w.data_ptr(),
                                 b.data_ptr(), co, res, 1, y.data_ptr(), None,
                                 err.data_ptr())
            if st != 0:
                raise RuntimeError(f"jetgpu_conv3d failed ({st})")

        for _ in range(3):
            call()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            call()
        e1.record()
        torch.cuda.synchronize()
        us = e0.elapsed_time(e1) / reps * 1e3
        flop = 2.0 * 27 * ci * co * n ** 3
        out[f"conv_{ci}_{co}_{n}"] = {"us": round(us, 1),
                                      "tflops": round(flop / us / 1e6, 1)}
    return out


def traffic_per_launch(kernel: str, variant: str, n: int):
    """DRAM bytes per launch of `kernel` in solver `variant` from the
    committed ncu summary (profiles/traffic.json), scaled by cells to this
    resolution; None when no capture covers the kernel."""
    path = os.path.join(REPO, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    rec = json.load(open(path)).get(kernel, {}).get(variant)
    if not rec:
        return None
    return rec["dram_bytes_per_launch"] * (n ** 3) / float(rec["cells"])


def run_ours(args, rank, world, local, pg):
    import numpy as np
    import torch
    import jetgpu

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.n
    h = 1.0 / n
    sc = workload(n)
    grid = jetgpu.Grid()
    grid.res[:] = (n, n, n)
    grid.spacing[:] = (h, h, h)
    grid.origin[:] = (0.0, 0.0, 0.0)

    # Device-resident inputs (the resident FLIP solver's layout: FP64 faces
    # and cell-centred SDF grids).
    d = {k: torch.from_numpy(np.ascontiguousarray(sc[k])).to(dev)
         for k in ("u", "v", "w", "boundary_sdf", "fluid_sdf")}
    out = {k: torch.empty_like(d[k]) for k in ("u", "v", "w")}
    p_out = torch.empty((n, n, n), dtype=torch.float64, device=dev)

    def field(t):
        f = jetgpu.ScalarField()
        f.kind = 1
        f.data = t.data_ptr()
        f.res[:] = (n, n, n)
        f.origin[:] = (0.5 * h,) * 3
        f.spacing[:] = (h, h, h)
        return f

    bsdf, fsdf = field(d["boundary_sdf"]), field(d["fluid_sdf"])
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def make_solver(name):
        prec, pre = VARIANTS[name]
        solver = jetgpu.FdmMgpcgSolver3(**solver_params(prec, pre),
                                        device=local)
        if pre == "learned":
            from jetgpu import learned
            if not os.path.exists(learned.WEIGHTS):
                solver.close()
                return None
            solver.load_network(learned.flatten(learned.load()))
        return solver

    def timed(solver, steps, warmup, clocks=None):
        """Device-API solves timed with CUDA events on the library stream."""
        stats = jetgpu.SolveStats()

        def solve_device():
            return jetgpu.solve_pressure_device(
                solver, grid, d["u"], d["v"], d["w"], bsdf, fsdf, out["u"],
                out["v"], out["w"], p_out, stats=stats)

        for _ in range(warmup):
            solve_device()
        stream = torch.cuda.ExternalStream(solver.stream(), device=dev)
        iters, rel = [], []
        barrier(pg, local)
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
        e0.record(stream)
        for _ in range(steps):
            solve_device()
            iters.append(stats.iterations)
            rel.append(stats.relative_residual)
        e1.record(stream)
        torch.cuda.synchronize()
        ck = clocks.stop() if clocks else None
        barrier(pg, local)
        ms = max_over_ranks(pg, e0.elapsed_time(e1) / steps, local)
        return dict(ms=ms, iters=iters, rel=rel, clocks=ck,
                    setup_ms=stats.setup_ms, solve_ms=stats.solve_ms,
                    fallback=stats.fallback_used, stream=stream,
                    solve=solve_device)

    variants = {}
    results = {}
    for name in args.variants.split(","):
        if name not in VARIANTS:
            raise SystemExit(f"unknown variant {name!r}")
        solver = make_solver(name)
        if solver is None:
            variants[name] = {"status": "skipped: no trained weights"}
            continue
        r = timed(solver, args.steps, args.warmup, Clocks(local))
        ok = max(r["rel"]) <= TOL
        variants[name] = {
            "ms_per_solve": round(r["ms"], 3),
            "steps_per_s": round(1000.0 / r["ms"], 2),
            "iterations_per_solve": r["iters"][-1],
            "relative_residual": max(r["rel"]),
            "reached_tolerance": ok,
            "setup_ms": round(r["setup_ms"], 3),
            "solve_ms": round(r["solve_ms"], 3),
        }
        if VARIANTS[name][1] == "learned":
            variants[name]["multigrid_fallback_used"] = bool(r["fallback"])
        results[name] = (solver, r, ok)
    # Headline: plain MGPCG, the method the metric measures the learned
    # variant against (the other variants are in `variants`); the fastest
    # variant that reached the tolerance if plain was not run.
    if "plain_mgpcg" in results and results["plain_mgpcg"][2]:
        head = "plain_mgpcg"
    else:
        head = min((k for k in results if results[k][2]),
                   key=lambda k: results[k][1]["ms"])
    solver, r, _ = results[head]
    for k, (s_, _, _) in results.items():
        if k != head:
            s_.close()
    ms, ck = r["ms"], r["clocks"]

    # Second pass of the same K solves with every launch bracketed by events
    # on the library stream: per-kernel durations and launch counts.
    solver.profile(True)
    for _ in range(args.steps):
        r["solve"]()
    prof = solver.profile_read()
    solver.profile(False)
    launches = sum(k["launches"] for k in prof)
    top = max(prof, key=lambda k: k["total_ms"])
    total_prof_ms = sum(k["total_ms"] for k in prof)
    pk = peaks()
    achieved = (top["bytes"] / top["launches"]) / (
        top["total_ms"] / top["launches"] * 1e-3) / 1e9
    traffic = traffic_per_launch(top["name"], head, n)
    roofline = {
        "kernel": top["name"], "bound": "hbm",
        "achieved": round(achieved, 1), "peak": pk["hbm_gbs"],
        "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 3),
        "peak_source": pk["source"],
        "algorithmic_bytes_per_launch": top["bytes"] / top["launches"],
        "avg_launch_us": round(top["total_ms"] / top["launches"] * 1e3, 2),
        "share": round(top["total_ms"] / total_prof_ms, 3),
        "traffic": traffic,
    }
    # Whole-solve roofline: algorithmic bytes of every launch / solve time.
    solve_bytes = sum(k["bytes"] for k in prof) / args.steps
    whole = solve_bytes / (ms * 1e-3) / 1e9

    # End-to-end through the host-pointer C ABI with pinned host buffers, the
    # way GridFluidSolver3::computePressure calls its pressure solver: the
    # output grid holds the input's values (the input is its clone), so the
    # solver moves only the velocity faces around the fluid cells
    # (fluid_box_io); the bytes moved are the solver's own count.
    solver.close()
    solver = jetgpu.FdmMgpcgSolver3(**solver_params(*VARIANTS[head]),
                                    device=local, fluidBoxIo=True)
    pin = {k: torch.from_numpy(np.ascontiguousarray(sc[k])).pin_memory()
           for k in ("u", "v", "w", "boundary_sdf", "fluid_sdf")}
    hout = {k: pin[k].clone().pin_memory() for k in ("u", "v", "w")}
    vel = jetgpu.FaceCenteredGrid3((n, n, n), (h, h, h), (0, 0, 0),
                                   pin["u"].numpy(), pin["v"].numpy(),
                                   pin["w"].numpy())
    outg = jetgpu.FaceCenteredGrid3((n, n, n), (h, h, h), (0, 0, 0),
                                    hout["u"].numpy(), hout["v"].numpy(),
                                    hout["w"].numpy())
    ps = jetgpu.GridFractionalSinglePhasePressureSolver3(solver)
    cg = lambda t: jetgpu.CellCenteredScalarGrid3((n, n, n), (h, h, h),
                                                  (0, 0, 0), t.numpy())
    bg, fg = cg(pin["boundary_sdf"]), cg(pin["fluid_sdf"])
    stream = torch.cuda.ExternalStream(solver.stream(), device=dev)
    for _ in range(max(1, args.warmup)):
        ps.solve(vel, 1 / 60, outg, bg, None, fg)
    # Three batches of K host-pointer solves; the median batch is reported
    # (all three are in the line), so that one slow batch on a shared host
    # does not stand for the whole run.
    batches = []
    for _ in range(3):
        barrier(pg, local)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            ps.solve(vel, 1 / 60, outg, bg, None, fg)
        e1.record(stream)
        torch.cuda.synchronize()
        batches.append(max_over_ranks(pg, e0.elapsed_time(e1) / args.steps,
                                      local))
    e2e_ms = sorted(batches)[1]
    h2d = int(ps.last_stats.h2d_bytes)
    d2h = int(ps.last_stats.d2h_bytes)
    solver.close()
    return dict(ms=ms, e2e_ms=e2e_ms, e2e_batches=batches, h2d=h2d, d2h=d2h,
                clocks=ck,
                iters=r["iters"], rel=r["rel"], roofline=roofline,
                launches=launches, whole_gbs=whole, solve_bytes=solve_bytes,
                profile=prof, setup_ms=r["setup_ms"], solve_ms=r["solve_ms"],
                peak=pk, head=head, variants=variants)


def residual_rows(A, x, b):
    """||b - A x|| / ||b|| for 7-point rows {center, right, up, front}
    ((nz,ny,nx,4) float64; the lower neighbours' couplings are the right/up/
    front entries of the cell before), in numpy."""
    import numpy as np
    r = b - A[..., 0] * x
    r[:, :, :-1] -= A[:, :, :-1, 1] * x[:, :, 1:]
    r[:, :, 1:] -= A[:, :, :-1, 1] * x[:, :, :-1]
    r[:, :-1, :] -= A[:, :-1, :, 2] * x[:, 1:, :]
    r[:, 1:, :] -= A[:, :-1, :, 2] * x[:, :-1, :]
    r[:-1] -= A[:-1, :, :, 3] * x[1:]
    r[1:] -= A[:-1, :, :, 3] * x[:-1]
    return float(np.linalg.norm(r) / np.linalg.norm(b))


def run_accuracy(args, local, names):
    """Per workload and solver variant, the error against an FP64 answer:
    the same projection in the FP64 mode solved to a relative true residual
    below 1e-12 (its residual recomputed here in numpy over the FP64 rows),
    then each variant at the 1e-6 tolerance: relative L2 of the pressure and
    the maximum over fluid cells of the cell-centre divergence
    (FaceCenteredGrid3::divergenceAtCellCenter) of the projected velocity,
    beside the FP64 answer's and their largest cell-wise difference. Host-
    pointer solves through the public API; not timed."""
    import numpy as np
    import jetgpu
    from jetgpu import scenes

    def div(u, v, w, h):
        return ((u[:, :, 1:] - u[:, :, :-1]) / h + (v[:, 1:, :] - v[:, :-1, :]) / h
                + (w[1:] - w[:-1]) / h)

    def solve(n, sc, prec, pre, tol, iters=200, refs=8):
        h = 1.0 / n
        prm = solver_params(prec, pre)
        prm.update(maxTolerance=tol, numberOfCgIter=iters, maxRefinements=refs)
        s = jetgpu.FdmMgpcgSolver3(**prm, device=local)
        if pre == "learned":
            from jetgpu import learned
            if not os.path.exists(learned.WEIGHTS):
                s.close()
                return None
            s.load_network(learned.flatten(learned.load()))
        ps = jetgpu.GridFractionalSinglePhasePressureSolver3(s)
        vel = jetgpu.FaceCenteredGrid3((n,) * 3, (h,) * 3, (0, 0, 0),
                                       sc["u"], sc["v"], sc["w"])
        out = vel.clone()
        g = lambda d: jetgpu.CellCenteredScalarGrid3((n,) * 3, (h,) * 3,
                                                     (0, 0, 0), d)
        ps.solve(vel, 1 / 60, out, g(sc["boundary_sdf"]), None,
                 g(sc["fluid_sdf"]))
        return ps, out

    result = {}
    work = [("headline_%d" % args.n, args.n, workload(args.n),
             [(k, VARIANTS[k]) for k in names]),
            ("sphere_union_128", 128, scenes.sphere_union_scene(128, seed=1),
             [("fp32", ("fp32", "multigrid")), ("fp64", ("fp64", "multigrid")),
              ("mixed", ("mixed", "multigrid"))])]
    for tag, n, sc, variants in work:
        ps64, out64 = solve(n, sc, "fp64", "multigrid", 1e-12, iters=400,
                            refs=20)
        p64 = ps64.pressure().copy()
        A = ps64.level(0, "A").reshape(n, n, n, 4)
        b = ps64.level(0, "b").reshape(n, n, n)
        fluid = ps64.level(0, "fluid").reshape(n, n, n) < 0
        d64 = div(out64.u, out64.v, out64.w, 1.0 / n)
        entry = {"fp64_answer": {
            "relative_residual": ps64.last_stats.relative_residual,
            "relative_residual_rechecked": residual_rows(A, p64, b),
            "iterations": ps64.last_stats.iterations,
            "max_div": float(np.abs(d64[fluid]).max())}}
        ps64.linearSystemSolver.close()
        for name, (prec, pre) in variants:
            r = solve(n, sc, prec, pre, TOL)
            if r is None:
                entry[name] = {"status": "skipped: no trained weights"}
                continue
            ps, out = r
            d = div(out.u, out.v, out.w, 1.0 / n)
            p = ps.pressure()
            entry[name] = {
                "p_rel_l2": float(np.linalg.norm(p - p64) / np.linalg.norm(p64)),
                "max_div": float(np.abs(d[fluid]).max()),
                "max_div_diff": float(np.abs(d - d64)[fluid].max()),
                "relative_residual": ps.last_stats.relative_residual,
                "iterations": ps.last_stats.iterations}
            ps.linearSystemSolver.close()
        result[tag] = entry
    return result


def run_flip(args, local, variant: str, frames: int, small: bool = True):
    """Whole FLIP frames on the GPU (jetgpu_flip_substep_device under the
    reference's adaptive sub-stepping): the 256^3 dam break with the static
    sphere obstacle (water box [0,.3]x[0,.8]x[0,1], 8 particles per cell
    from seed 2, sphere r = .15 at (.6,.2,.5)) for `frames` frames of 1/60 s
    after one warm-up frame, and the 64^3 dam break (box [0,.25]x[0,.75]x
    [0,1], seed 0, closed box) for 60 frames. CUDA events on the library
    stream; the particles never leave the device. The pressure projections
    of the timed frames are also timed one by one (SolveStats.setup_ms +
    solve_ms: CUDA events around the weights, system and MGPCG kernels of
    each solve) and averaged over the run's solves."""
    import numpy as np
    import torch
    import jetgpu
    from jetgpu import scenes
    dev = torch.device("cuda", local)
    out = {}
    legs = [("flip_256", args.n, (0.3, 0.8, 1.0), 2, True, frames, 1)]
    if small:
        legs.append(("flip_64_dam_break", 64, (0.25, 0.75, 1.0), 0, False,
                     60, 0))
    for tag, n, box, seed, sphere, nframes, warm in legs:
        prec, _ = VARIANTS[variant]
        ps = jetgpu.FdmMgpcgSolver3(**solver_params(prec, "multigrid"),
                                    device=local)
        h = 1.0 / n
        sim = jetgpu.FlipSolver3((n, n, n), h, (0, 0, 0), pressureSolver=ps,
                                 device=local)
        pos, _ = scenes.dam_break_particles(n, box, seed=seed)
        sim.setParticles(pos)
        if sphere:
            X, Y, Z = scenes.cell_centres(n)
            c, r = (0.6, 0.2, 0.5), 0.15
            sdf = np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 +
                          (Z - c[2]) ** 2) - r
            sim.setCollider(sdf, jetgpu.Collider.make(centre=c),
                            jetgpu.Sphere.make(r))
        for _ in range(warm):
            sim.update(1.0 / 60)
        kernels = None
        if tag == "flip_256":
            # Per-kernel-class split of one profiled frame (events around
            # every launch on the library stream), then the timed frames.
            ps.profile(True)
            s0 = sim.subSteps
            sim.update(1.0 / 60)
            prof = ps.profile_read()
            ps.profile(False)
            ns = max(sim.subSteps - s0, 1)
            kernels = {k["name"]: round(k["total_ms"] / ns, 3) for k in
                       sorted(prof, key=lambda k: -k["total_ms"])}
        stream = torch.cuda.ExternalStream(ps.stream(), device=dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        s0 = sim.subSteps
        p0, i0 = sim.pressureMs, sim.pressureIterations
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(nframes):
            sim.update(1.0 / 60)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        subs = sim.subSteps - s0
        out[tag] = {
            "grid": n, "particles": int(pos.shape[0]), "frames": nframes,
            "substeps": subs, "ms_per_frame": round(ms / nframes, 3),
            "ms_per_substep": round(ms / max(subs, 1), 3),
            "substeps_per_s": round(1000.0 * subs / ms, 2),
            "pressure_iterations_last": sim.lastStats.iterations,
            "pressure_ms_per_solve": round((sim.pressureMs - p0) / max(subs, 1), 3),
            "pressure_iterations_per_solve": round(
                (sim.pressureIterations - i0) / max(subs, 1), 2),
            "solver": variant, "collider": "sphere" if sphere else "none",
        }
        if kernels is not None:
            out[tag]["ms_per_substep_by_kernel_class"] = kernels
        del sim
        ps.close()
    return out


def run_smoke(args, local, variant: str, steps: int = 3, cpu: bool = False):
    """The projection of the 512^3 buoyant smoke plume (GridSmokeSolver3:
    all fluid, closed box; the source sphere r = .05 at (.5,.1,.5) pushing
    upward), one device-resident pressure solve per step to the same 1e-6
    relative true residual, after one warm-up solve: the headline variant
    (top-level fields) and, under `variants`, the others of `--variants`
    (the learned one when its weights are present)."""
    import torch
    import jetgpu
    n = 512
    h = 1.0 / n
    dev = torch.device("cuda", local)
    f64 = dict(dtype=torch.float64, device=dev)
    u = torch.zeros((n, n, n + 1), **f64)
    w = torch.zeros((n + 1, n, n), **f64)
    c = (torch.arange(n, **f64) + 0.5) * h
    yf = torch.arange(n + 1, **f64) * h
    r2 = ((c[None, None, :] - 0.5) ** 2 + (yf[None, :, None] - 0.1) ** 2 +
          (c[:, None, None] - 0.5) ** 2)
    v = (r2 < 0.05 ** 2).to(torch.float64)
    v[:, 0, :] = 0
    v[:, -1, :] = 0
    del r2
    out = [torch.empty_like(a) for a in (u, v, w)]
    grid = jetgpu.Grid()
    grid.res[:] = (n, n, n)
    grid.spacing[:] = (h, h, h)
    grid.origin[:] = (0, 0, 0)
    fb, ff = jetgpu.ScalarField(), jetgpu.ScalarField()
    fb.kind, fb.value = 0, jetgpu.kMaxD
    ff.kind, ff.value = 0, -jetgpu.kMaxD

    def timed(name):
        prec, pre = VARIANTS[name]
        solver = jetgpu.FdmMgpcgSolver3(**solver_params(prec, pre),
                                        device=local)
        if pre == "learned":
            from jetgpu import learned
            if not os.path.exists(learned.WEIGHTS):
                solver.close()
                return None
            solver.load_network(learned.flatten(learned.load()))
        stats = jetgpu.SolveStats()

        def solve():
            jetgpu.solve_pressure_device(solver, grid, u, v, w, fb, ff, *out,
                                         None, stats=stats)

        solve()
        stream = torch.cuda.ExternalStream(solver.stream(), device=dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            solve()
        e1.record(stream)
        torch.cuda.synchronize()
        r = {"ms_per_solve": round(e0.elapsed_time(e1) / steps, 3),
             "iterations_per_solve": stats.iterations,
             "relative_residual": stats.relative_residual,
             "setup_ms": round(stats.setup_ms, 3)}
        if pre == "learned":
            r["multigrid_fallback_used"] = bool(stats.fallback_used)
        solver.close()
        return r

    head = timed(variant)
    res = {"grid": n, "cells": n ** 3, "ms_per_solve": head["ms_per_solve"],
           "solves": steps, "iterations_per_solve": head["iterations_per_solve"],
           "relative_residual": head["relative_residual"],
           "setup_ms": head["setup_ms"], "solver": variant,
           "system": "all fluid, closed box (pure Neumann)"}
    others = {}
    for name in [x for x in args.variants.split(",") if x and x != variant]:
        r = timed(name)
        if r is not None:
            others[name] = r
    if others:
        res["variants"] = others
    if cpu and not args.no_cpu_baseline:
        res["cpu_reference"] = smoke_cpu_sample(n)
    return res


def smoke_cpu_sample(n: int, iterations: int = 2):
    """A bounded sample of the reference's CPU solve of the same 512^3
    smoke projection on all host cores: weights, system build and the first
    `iterations` MGPCG iterations of FdmMgpcgSolver3(., 5, 5, 5, 20, 20,
    1e-6, 1.5, true) (the whole solve takes minutes at this size)."""
    import numpy as np
    import oracle
    o, kind, threads = cpu_reference()
    h = 1.0 / n
    c = (np.arange(n) + 0.5) * h
    yf = np.arange(n + 1) * h
    v = ((c[None, None, :] - 0.5) ** 2 + (yf[None, :, None] - 0.1) ** 2 +
         (c[:, None, None] - 0.5) ** 2 < 0.05 ** 2).astype(np.float64)
    v[:, 0, :] = 0
    v[:, -1, :] = 0
    u = np.zeros((n, n, n + 1))
    w = np.zeros((n + 1, n, n))
    kmax = float(np.finfo(np.float64).max)
    prm = dict(REF_PARAMS, max_cg_iter=iterations)
    t = time.perf_counter()
    r = o.pressure_solve((n,) * 3, (h,) * 3, (0, 0, 0), u, v, w, kmax, -kmax,
                         oracle.MgParams(**prm))
    dt = time.perf_counter() - t
    return {"grid": n, "ms": round(dt * 1e3, 1), "cores": threads,
            "kind": kind, "iterations": r["iters"],
            "residual_norm": r["resid"],
            "sample": f"weights + system build + the first {iterations} "
                      f"MGPCG iterations of one {n}^3 reference solve "
                      "(FdmMgpcgSolver3(100,5,5,5,20,20,1e-6,1.5,true))"}


def run_blocked(args, local, variant: str, steps: int = 5, cpu: bool = True):
    """The blocked pressure solver (GridSinglePhasePressureSolver3) on the
    headline scene: device-resident solves to the same 1e-6 relative true
    residual, K timed after one warm-up, and (rank 0, no --no-cpu-baseline)
    one blocked solve of the reference's CPU algorithm on the host cores."""
    import numpy as np
    import torch
    import jetgpu
    n = args.n
    h = 1.0 / n
    dev = torch.device("cuda", local)
    sc = workload(n)
    prec, _ = VARIANTS[variant]
    solver = jetgpu.FdmMgpcgSolver3(**solver_params(prec, "multigrid"),
                                    device=local)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    u, v, w = T(sc["u"]), T(sc["v"]), T(sc["w"])
    bs, fs = T(sc["boundary_sdf"]), T(sc["fluid_sdf"])
    out = [torch.empty_like(a) for a in (u, v, w)]
    grid = jetgpu.Grid()
    grid.res[:] = (n, n, n)
    grid.spacing[:] = (h, h, h)
    grid.origin[:] = (0, 0, 0)

    def dfield(t):
        f = jetgpu.ScalarField()
        f.kind = 1
        f.data = t.data_ptr()
        f.res[:] = (n, n, n)
        f.origin[:] = (0.5 * h,) * 3
        f.spacing[:] = (h, h, h)
        return f

    fb, ff = dfield(bs), dfield(fs)
    stats = jetgpu.SolveStats()
    torch.cuda.synchronize()

    def solve():
        jetgpu.solve_pressure_blocked_device(solver, grid, u, v, w, fb, ff,
                                             *out, None, stats=stats)

    solve()
    stream = torch.cuda.ExternalStream(solver.stream(), device=dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        solve()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    res = {"grid": n, "ms_per_solve": round(ms, 3), "solves": steps,
           "iterations_per_solve": stats.iterations,
           "relative_residual": stats.relative_residual,
           "setup_ms": round(stats.setup_ms, 3), "solver": variant,
           "scene": "the headline 256^3 FLIP dam-break sub-step, cells "
                    "marked fluid/air/boundary at their centres"}
    solver.close()
    if cpu and not args.no_cpu_baseline:
        import oracle
        o, kind, threads = cpu_reference()
        m = max(n // 2, 8)  # a bounded sample: 1/8 of the cells
        sm = workload(m)
        t = time.perf_counter()
        r = o.blocked_pressure_solve((m,) * 3, (1.0 / m,) * 3, (0, 0, 0),
                                     sm["u"], sm["v"], sm["w"],
                                     sm["boundary_sdf"], sm["fluid_sdf"],
                                     oracle.MgParams(**REF_PARAMS))
        dt = time.perf_counter() - t
        res["cpu_reference"] = {
            "grid": m, "ms_per_solve": round(dt * 1e3, 1), "cores": threads,
            "kind": kind, "iterations": r["iters"],
            "final_residual_norm": r["resid"],
            "sample": f"one full {m}^3 blocked solve of the same scene with "
                      "the reference's FdmMgpcgSolver3(100,5,5,5,20,20,1e-6,"
                      "1.5,true) until its own stop"}
    return res


def cpu_reference():
    """The reference's CPU algorithm on this host: the compiled reference
    when it exists here, else the oracle port (bit-exact with it)."""
    import oracle
    kind = "port"
    o = None
    try:
        if os.path.exists(oracle.REF_SO):
            o = oracle.Oracle(oracle.REF_SO)
            kind = "reference"
    except OSError:
        o = None
    if o is None:
        o = oracle.port()
    threads = os.cpu_count() or 1
    o.set_threads(threads)
    return o, kind, threads


# The reference's MGPCG as the reference's configs install it
# (FdmMgpcgSolver3(100, L, 5, 5, 20, 20, tol, 1.5, true)).
REF_PARAMS = dict(max_cg_iter=100, max_levels=5, restrict_iter=5,
                  correct_iter=5, coarsest_iter=20, final_iter=20,
                  tolerance=TOL, sor=1.5, red_black=True)


def cpu_solve(o, n, sc):
    """One full reference pressure solve (weights, system, MGPCG to its own
    termination, gradient). Returns (seconds, iterations, true relative
    residual of the returned pressure)."""
    import numpy as np
    import oracle
    h = (1.0 / n,) * 3
    t = time.perf_counter()
    r = o.pressure_solve((n,) * 3, h, (0, 0, 0), sc["u"], sc["v"], sc["w"],
                         sc["boundary_sdf"], sc["fluid_sdf"],
                         oracle.MgParams(**REF_PARAMS))
    dt = time.perf_counter() - t
    A = o.level(0, "A", (n,) * 3)
    b = o.level(0, "b", (n,) * 3)
    res = o.residual(A, r["p"], b)
    return dt, r["iters"], float(np.linalg.norm(res) / np.linalg.norm(b))


def cpu_baseline(n: int, steps: int = 1, warmup: int = 0):
    """ms per reference pressure solve on all host cores. At 256^3 the
    reference's MGPCG stops after a few iterations when r.z turns
    non-positive (its V-cycle is not symmetric), so the solve it returns is
    far from 1e-6; the residual it reaches is reported beside the time."""
    sc = workload(n)
    o, kind, threads = cpu_reference()
    for _ in range(warmup):
        cpu_solve(o, n, sc)
    times, its, rel = [], None, None
    for _ in range(steps):
        dt, its, rel = cpu_solve(o, n, sc)
        times.append(dt * 1e3)
    value = sum(times) / len(times)
    sample = (f"full {n}^3 pressure solve with the reference's "
              f"FdmMgpcgSolver3(100,5,5,5,20,20,1e-6,1.5,true): {its} MGPCG "
              f"iterations until its own stop, true relative residual "
              f"{rel:.2e}; mean of {steps} solve(s)")
    return dict(value=value, unit="ms/solve", cores=threads, kind=kind,
                sample=sample, iterations=its, relative_residual=rel)


def run_reference(args, rank, world, pg):
    if rank != 0:
        return None
    cb = cpu_baseline(args.n, steps=args.steps, warmup=args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"],
        "unit": "ms/solve", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": cb["value"],
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded scene, no dataset)",
        "config": {"workload": f"{args.n}^3 FLIP dam break, first sub-step "
                               "pressure solve (sphere obstacle)",
                   "grid": args.n, "tolerance": TOL,
                   "solver": "FdmMgpcgSolver3(100,5,5,5,20,20,1e-6,1.5,true)"},
        "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind",
                                            "sample")},
        "reference_relative_residual": cb["relative_residual"],
        "reference_iterations": cb["iterations"],
        "e2e": {"value": cb["value"], "unit": "ms/solve",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def main():
    args = parse_args()
    rank, world, local, pg = dist_setup(args)
    if args.conv_only:
        if rank == 0:
            print(json.dumps(run_unet(local)), flush=True)
        return
    if args.impl == "reference":
        line = run_reference(args, rank, world, pg)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    r = run_ours(args, rank, world, local, pg)
    accuracy = None
    if not args.no_accuracy and rank == 0:
        accuracy = run_accuracy(args, local, r["variants"].keys())
    unet = run_unet(local) if rank == 0 else None
    flip = None
    if not args.no_flip:
        # The 256^3 dam break for 30 frames with each MGPCG variant (the
        # plain and the mixed-precision V-cycle), the 64^3 one for 60.
        flip = {}
        for name in ("plain_mgpcg", "mixed_mgpcg"):
            res = run_flip(args, local, name, frames=args.flip_frames,
                           small=name == r["head"])
            for tag, val in res.items():
                flip[tag if tag != "flip_256" else f"flip_256_{name}"] = val
    smoke = None
    if not args.no_smoke:
        smoke = run_smoke(args, local, r["head"], cpu=rank == 0 and world == 1)
    blocked = None
    if not args.no_blocked:
        blocked = run_blocked(args, local, r["head"],
                              cpu=rank == 0 and world == 1)
    cb = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(args.n, steps=1)
    if rank != 0:
        return
    iters = r["iters"]
    line = {
        "metric": METRIC, "value": round(r["ms"], 3), "unit": "ms/solve",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(r["ms"], 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "f32 (f64-accurate reductions/refinement)",
                  "mixed": "f32 Krylov, bf16 V-cycle rows (f64-accurate "
                           "reductions/refinement)"}[VARIANTS[r["head"]][0]],
        "data": "synthetic (seeded scene, no dataset)",
        "config": {
            "workload": f"{args.n}^3 FLIP dam break, first sub-step pressure "
                        "solve (weights + system + MGPCG + gradient), sphere "
                        "obstacle",
            "grid": args.n, "tolerance": TOL,
            "solver": r["head"] + ": MGPCG(200,6,2,2,5,2,1e-6,1.2,"
                      "red-black), masked symmetric V-cycle",
            "parallelism": f"replicas x{world}",
            "l2": "inputs and solver state >> L2 (no flush)",
            "roofline_timing": "per-launch CUDA events on the library stream "
                               "over a second pass of the K solves",
        },
        "variants": r["variants"],
        "iterations_per_solve": iters[-1] if iters else None,
        "relative_residual": max(r["rel"]) if r["rel"] else None,
        "steps_per_s": round(1000.0 / r["ms"], 2),
        "setup_ms": round(r["setup_ms"], 3),
        "solve_ms": round(r["solve_ms"], 3),
        "whole_solve_gbs": round(r["whole_gbs"], 1),
        "whole_solve_frac": round(r["whole_gbs"] / r["peak"]["hbm_gbs"], 3),
        "roofline": r["roofline"],
        "e2e": {"value": round(r["e2e_ms"], 3), "unit": "ms/solve",
                "batches_ms": [round(x, 3) for x in r["e2e_batches"]],
                "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"]},
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "kernels": [{"name": k["name"], "launches": k["launches"],
                     "ms": round(k["total_ms"], 3)} for k in
                    sorted(r["profile"], key=lambda k: -k["total_ms"])],
    }
    if accuracy is not None:
        line["accuracy"] = accuracy
    if unet is not None:
        pk = peaks()
        top = unet["conv_16_16_128"]
        line["roofline_tensor"] = {
            "kernel": "conv3d 3x3x3 16->16 (U-Net level 0) at 128^3",
            "bound": "tensor", "achieved": top["tflops"],
            "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
            "frac": round(top["tflops"] / pk["bf16_tflops"], 3),
            "peak_source": pk["tensor_source"], "layers": unet}
    if flip is not None:
        line["flip_steps"] = flip
    if smoke is not None:
        line["smoke_512_pressure"] = smoke
    if blocked is not None:
        line["blocked_pressure"] = blocked
    if cb is not None:
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores",
                                                   "kind", "sample")}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
