"""jetgpu — GB300-native pressure projection for the Jet fluid engine.

Host-side mirror of the reference's plug-in interface for this path, over the
C ABI of ``libjetgpu.so`` (``include/jetgpu.h``):

* :class:`GridFractionalSinglePhasePressureSolver3` — the drop-in
  ``GridPressureSolver3`` (include/jet/grid_pressure_solver3.h:29-75,
  include/jet/grid_fractional_single_phase_pressure_solver3.h:46-129):
  ``solve(input, dt, output, boundarySdf, boundaryVelocity, fluidSdf,
  useCompressed)``, ``pressure()``, ``linearSystemSolver``,
  ``suggestedBoundaryConditionSolver()``.
* :class:`FdmMgpcgSolver3` — the multigrid-preconditioned CG linear solver
  (include/jet/fdm_mgpcg_solver3.h:35-56) with ``solve(system)``,
  ``lastNumberOfIterations()``, ``lastResidual()``.
* :func:`transfer_from_particles_to_grids`,
  :func:`flip_transfer_from_grids_to_particles`,
  :func:`pic_transfer_from_grids_to_particles` — the FLIP/PIC transfers.

Every compute call runs the CUDA kernels of libjetgpu. There is no CPU
fallback: importing this package without the built library raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field as dc_field

import numpy as np

from . import _build

LIB_PATH = _build.LIB

# ---------------------------------------------------------------------------
# C structures (include/jetgpu.h)


class Config(C.Structure):
    _fields_ = [
        ("device", C.c_int),
        ("max_cg_iter", C.c_uint),
        ("max_levels", C.c_uint),
        ("restrict_iter", C.c_uint),
        ("correct_iter", C.c_uint),
        ("coarsest_iter", C.c_uint),
        ("final_iter", C.c_uint),
        ("tolerance", C.c_double),
        ("sor", C.c_double),
        ("red_black", C.c_int),
        ("precision", C.c_int),
        ("preconditioner", C.c_int),
        ("max_refinements", C.c_uint),
        ("ordered_p2g", C.c_int),
        ("fluid_box_io", C.c_int),
    ]


class ScalarField(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("value", C.c_double),
        ("data", C.c_void_p),
        ("res", C.c_int * 3),
        ("origin", C.c_double * 3),
        ("spacing", C.c_double * 3),
    ]


class Grid(C.Structure):
    _fields_ = [
        ("res", C.c_int * 3),
        ("spacing", C.c_double * 3),
        ("origin", C.c_double * 3),
    ]


class SolveStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_uint),
        ("refinements", C.c_uint),
        ("levels", C.c_uint),
        ("residual", C.c_double),
        ("relative_residual", C.c_double),
        ("b_norm", C.c_double),
        ("setup_ms", C.c_double),
        ("solve_ms", C.c_double),
        ("total_ms", C.c_double),
        ("fallback_used", C.c_int),
        ("h2d_bytes", C.c_ulonglong),
        ("d2h_bytes", C.c_ulonglong),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


STATUS = {0: "OK", 1: "NOT_CONVERGED", 2: "STALLED_FALLBACK_USED",
          3: "BAD_INPUT", 4: "CUDA_ERROR", 5: "OUT_OF_MEMORY",
          6: "NUMERICAL_ERROR", 7: "CAPACITY_EXCEEDED"}
PRECISION = {"fp32": 0, "fp64": 1, "mixed": 2, "bf16": 2}
PRECONDITIONER = {"multigrid": 0, "learned": 1, "none": 2}
SOLVED = (0, 1, 2)  # OK, NOT_CONVERGED (last iterate applied), fallback used

# Symbols include/jetgpu.h declares (checked by the CPU test suite).
EXPORTS = (
    "jetgpu_config_default", "jetgpu_create", "jetgpu_destroy",
    "jetgpu_last_error", "jetgpu_set_config", "jetgpu_solve_pressure",
    "jetgpu_solve_pressure_device", "jetgpu_solve_pressure_blocked",
    "jetgpu_solve_pressure_blocked_device", "jetgpu_mgpcg_solve_system",
    "jetgpu_p2g_device", "jetgpu_g2p_flip_device", "jetgpu_g2p_pic_device",
    "jetgpu_p2g", "jetgpu_g2p_flip", "jetgpu_g2p_pic", "jetgpu_get_level",
    "jetgpu_version", "jetgpu_get_stream", "jetgpu_profile",
    "jetgpu_profile_read", "jetgpu_p2g_device_noalloc", "jetgpu_conv3d",
    "jetgpu_conv3d_wgrad", "jetgpu_net_param_count", "jetgpu_load_unet",
    "jetgpu_harvest", "jetgpu_net_features", "jetgpu_net_apply",
    "jetgpu_constrain_velocity_device", "jetgpu_constrain_velocity",
    "jetgpu_constrain_velocity_blocked_device",
    "jetgpu_constrain_velocity_blocked",
    "jetgpu_extrapolate_to_region_device", "jetgpu_move_particles_device",
    "jetgpu_move_particles", "jetgpu_build_particle_sdf_device",
    "jetgpu_build_particle_sdf", "jetgpu_flip_params_default",
    "jetgpu_fluid_cfl_device", "jetgpu_flip_substep_device",
    "jetgpu_apic_p2g_device", "jetgpu_apic_g2p_device",
    "jetgpu_solve_pressure_collider", "jetgpu_vcycle_apply",
    "jetgpu_net_level", "jetgpu_learned_apply",
)

# closedDomainBoundaryFlag bits (include/jet/constants.h:312-335).
kDirectionLeft, kDirectionRight, kDirectionDown = 1, 2, 4
kDirectionUp, kDirectionBack, kDirectionFront = 8, 16, 32
kDirectionAll = 63


class Collider(C.Structure):
    """jetgpu_collider: a rigid collider's surface velocity
    linear + angular x (p - centre) and friction coefficient
    (RigidBodyCollider3, src/jet/rigid_body_collider3.cpp:25-28)."""
    _fields_ = [
        ("linear_velocity", C.c_double * 3),
        ("angular_velocity", C.c_double * 3),
        ("centre", C.c_double * 3),
        ("friction", C.c_double),
    ]

    @staticmethod
    def make(linear=(0, 0, 0), angular=(0, 0, 0), centre=(0, 0, 0),
             friction=0.0) -> "Collider":
        c = Collider()
        c.linear_velocity[:] = tuple(float(x) for x in linear)
        c.angular_velocity[:] = tuple(float(x) for x in angular)
        c.centre[:] = tuple(float(x) for x in centre)
        c.friction = float(friction)
        return c


class KernelStat(C.Structure):
    _fields_ = [
        ("name", C.c_char * 32),
        ("launches", C.c_uint),
        ("total_ms", C.c_double),
        ("bytes", C.c_double),
    ]


class JetGpuError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


_lib = None


def library() -> C.CDLL:
    """Loads libjetgpu.so (built by ``__graft_entry__.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is not built; run __graft_entry__.build() "
            "(the CUDA library is required, there is no CPU path)")
    L = C.CDLL(LIB_PATH)
    vp, dp, fp, up = C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p
    L.jetgpu_config_default.argtypes = [C.POINTER(Config)]
    L.jetgpu_config_default.restype = None
    L.jetgpu_create.argtypes = [C.POINTER(Config), C.POINTER(C.c_void_p)]
    L.jetgpu_create.restype = C.c_int
    L.jetgpu_destroy.argtypes = [vp]
    L.jetgpu_destroy.restype = None
    L.jetgpu_last_error.argtypes = [vp]
    L.jetgpu_last_error.restype = C.c_char_p
    L.jetgpu_set_config.argtypes = [vp, C.POINTER(Config)]
    L.jetgpu_set_config.restype = C.c_int
    solve_args = [vp, C.POINTER(Grid), dp, dp, dp, C.POINTER(ScalarField),
                  C.POINTER(ScalarField), dp, dp, dp, dp, dp, dp, dp,
                  C.POINTER(SolveStats)]
    L.jetgpu_solve_pressure.argtypes = solve_args
    L.jetgpu_solve_pressure.restype = C.c_int
    L.jetgpu_solve_pressure_device.argtypes = solve_args
    L.jetgpu_solve_pressure_device.restype = C.c_int
    L.jetgpu_solve_pressure_collider.argtypes = [
        vp, C.POINTER(Grid), dp, dp, dp, C.POINTER(ScalarField),
        C.POINTER(ScalarField), C.POINTER(Collider), dp, dp, dp, dp,
        C.POINTER(SolveStats)]
    L.jetgpu_solve_pressure_collider.restype = C.c_int
    blocked_args = [vp, C.POINTER(Grid), dp, dp, dp, C.POINTER(ScalarField),
                    C.POINTER(ScalarField), dp, dp, dp, dp,
                    C.POINTER(SolveStats)]
    L.jetgpu_solve_pressure_blocked.argtypes = blocked_args
    L.jetgpu_solve_pressure_blocked.restype = C.c_int
    L.jetgpu_solve_pressure_blocked_device.argtypes = blocked_args
    L.jetgpu_solve_pressure_blocked_device.restype = C.c_int
    L.jetgpu_mgpcg_solve_system.argtypes = [vp, C.POINTER(C.c_int), C.c_int,
                                            dp, dp, dp, C.POINTER(SolveStats)]
    L.jetgpu_mgpcg_solve_system.restype = C.c_int
    p2g_args = [vp, C.POINTER(Grid), C.c_long, dp, dp, dp, dp, dp, up, up, up,
                fp, fp, fp]
    L.jetgpu_p2g.argtypes = p2g_args
    L.jetgpu_p2g.restype = C.c_int
    L.jetgpu_p2g_device.argtypes = p2g_args
    L.jetgpu_p2g_device.restype = C.c_int
    L.jetgpu_p2g_device_noalloc.argtypes = p2g_args
    L.jetgpu_p2g_device_noalloc.restype = C.c_int
    flip_args = [vp, C.POINTER(Grid), C.c_long, dp, dp, dp, dp, dp, fp, fp, fp,
                 C.c_double]
    L.jetgpu_g2p_flip.argtypes = flip_args
    L.jetgpu_g2p_flip.restype = C.c_int
    L.jetgpu_g2p_flip_device.argtypes = flip_args
    L.jetgpu_g2p_flip_device.restype = C.c_int
    pic_args = [vp, C.POINTER(Grid), C.c_long, dp, dp, dp, dp, dp]
    L.jetgpu_g2p_pic.argtypes = pic_args
    L.jetgpu_g2p_pic.restype = C.c_int
    L.jetgpu_g2p_pic_device.argtypes = pic_args
    L.jetgpu_g2p_pic_device.restype = C.c_int
    bc_args = [vp, C.POINTER(Grid), vp, vp, vp, C.POINTER(ScalarField),
               C.POINTER(Collider), C.c_int, C.c_uint]
    L.jetgpu_constrain_velocity.argtypes = bc_args
    L.jetgpu_constrain_velocity.restype = C.c_int
    L.jetgpu_constrain_velocity_device.argtypes = bc_args
    L.jetgpu_constrain_velocity_device.restype = C.c_int
    L.jetgpu_constrain_velocity_blocked.argtypes = bc_args
    L.jetgpu_constrain_velocity_blocked.restype = C.c_int
    L.jetgpu_constrain_velocity_blocked_device.argtypes = bc_args
    L.jetgpu_constrain_velocity_blocked_device.restype = C.c_int
    L.jetgpu_extrapolate_to_region_device.argtypes = [
        vp, C.POINTER(C.c_int), vp, vp, C.c_uint]
    L.jetgpu_extrapolate_to_region_device.restype = C.c_int
    mp_args = [vp, C.POINTER(Grid), C.c_long, vp, vp, vp, vp, vp, C.c_double,
               C.c_double, C.c_int, C.POINTER(Collider), C.POINTER(Sphere)]
    L.jetgpu_move_particles.argtypes = mp_args
    L.jetgpu_move_particles.restype = C.c_int
    L.jetgpu_move_particles_device.argtypes = mp_args
    L.jetgpu_move_particles_device.restype = C.c_int
    sdf_args = [vp, C.POINTER(Grid), C.c_long, vp, C.POINTER(ScalarField),
                C.c_double, vp]
    L.jetgpu_build_particle_sdf.argtypes = sdf_args
    L.jetgpu_build_particle_sdf.restype = C.c_int
    L.jetgpu_build_particle_sdf_device.argtypes = sdf_args
    L.jetgpu_build_particle_sdf_device.restype = C.c_int
    L.jetgpu_apic_p2g_device.argtypes = [vp, C.POINTER(Grid), C.c_long, vp,
                                         vp, vp, vp, vp, vp, vp, vp, vp]
    L.jetgpu_apic_p2g_device.restype = C.c_int
    L.jetgpu_apic_g2p_device.argtypes = [vp, C.POINTER(Grid), C.c_long, vp,
                                         vp, vp, vp, vp, vp]
    L.jetgpu_apic_g2p_device.restype = C.c_int
    L.jetgpu_flip_params_default.argtypes = [C.POINTER(FlipParams)]
    L.jetgpu_flip_params_default.restype = None
    L.jetgpu_fluid_cfl_device.argtypes = [vp, C.POINTER(Grid), vp, vp, vp,
                                          C.c_double, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double)]
    L.jetgpu_fluid_cfl_device.restype = C.c_int
    L.jetgpu_flip_substep_device.argtypes = [
        vp, C.POINTER(Grid), C.c_long, vp, vp, vp, vp, vp, vp, vp,
        C.POINTER(ScalarField), C.POINTER(Collider), C.POINTER(Sphere),
        C.POINTER(FlipParams), C.c_double, C.POINTER(SolveStats)]
    L.jetgpu_flip_substep_device.restype = C.c_int
    L.jetgpu_get_level.argtypes = [vp, C.c_int, C.c_int, vp, C.c_size_t,
                                   C.POINTER(C.c_size_t)]
    L.jetgpu_get_level.restype = C.c_int
    L.jetgpu_version.argtypes = []
    L.jetgpu_version.restype = C.c_char_p
    L.jetgpu_conv3d.argtypes = [vp, vp, C.c_int, vp, vp, C.c_int,
                                C.POINTER(C.c_int), C.c_int, vp, vp, vp]
    L.jetgpu_conv3d.restype = C.c_int
    L.jetgpu_conv3d_wgrad.argtypes = [vp, vp, C.c_int, vp, C.c_int,
                                      C.POINTER(C.c_int), vp, vp]
    L.jetgpu_conv3d_wgrad.restype = C.c_int
    L.jetgpu_net_param_count.argtypes = []
    L.jetgpu_net_param_count.restype = C.c_size_t
    L.jetgpu_load_unet.argtypes = [vp, vp, C.c_size_t]
    L.jetgpu_load_unet.restype = C.c_int
    L.jetgpu_harvest.argtypes = [vp, C.c_uint, vp, vp, C.POINTER(C.c_uint)]
    L.jetgpu_harvest.restype = C.c_int
    L.jetgpu_net_level.argtypes = [vp]
    L.jetgpu_net_level.restype = C.c_uint
    L.jetgpu_net_features.argtypes = [vp, C.c_uint, vp, vp]
    L.jetgpu_net_features.restype = C.c_int
    L.jetgpu_net_apply.argtypes = [vp, C.c_uint, vp, vp]
    L.jetgpu_net_apply.restype = C.c_int
    L.jetgpu_learned_apply.argtypes = [vp, vp, vp]
    L.jetgpu_learned_apply.restype = C.c_int
    L.jetgpu_vcycle_apply.argtypes = [vp, vp, vp]
    L.jetgpu_vcycle_apply.restype = C.c_int
    L.jetgpu_get_stream.argtypes = [vp, C.POINTER(C.c_void_p)]
    L.jetgpu_get_stream.restype = C.c_int
    L.jetgpu_profile.argtypes = [vp, C.c_int]
    L.jetgpu_profile.restype = C.c_int
    L.jetgpu_profile_read.argtypes = [vp, C.POINTER(KernelStat), C.c_int,
                                      C.POINTER(C.c_int)]
    L.jetgpu_profile_read.restype = C.c_int
    _lib = L
    return L


def _p(a) -> int | None:
    """Address of a numpy array or torch tensor (None passes NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


# ---------------------------------------------------------------------------
# Host-side field types (mirroring the reference's argument types)


@dataclass
class FaceCenteredGrid3:
    """MAC velocity grid (src/jet/face_centered_grid3.cpp): numpy arrays
    u (nz,ny,nx+1), v (nz,ny+1,nx), w (nz+1,ny,nx), float64, i-fastest."""
    resolution: tuple
    gridSpacing: tuple = (1.0, 1.0, 1.0)
    origin: tuple = (0.0, 0.0, 0.0)
    u: np.ndarray = None
    v: np.ndarray = None
    w: np.ndarray = None

    def __post_init__(self):
        nx, ny, nz = self.resolution
        if np.isscalar(self.gridSpacing):
            self.gridSpacing = (float(self.gridSpacing),) * 3
        if self.u is None:
            self.u = np.zeros((nz, ny, nx + 1))
        if self.v is None:
            self.v = np.zeros((nz, ny + 1, nx))
        if self.w is None:
            self.w = np.zeros((nz + 1, ny, nx))

    def clone(self) -> "FaceCenteredGrid3":
        return FaceCenteredGrid3(self.resolution, self.gridSpacing,
                                 self.origin, self.u.copy(), self.v.copy(),
                                 self.w.copy())

    def c_grid(self) -> Grid:
        g = Grid()
        g.res[:] = tuple(int(r) for r in self.resolution)
        g.spacing[:] = tuple(float(h) for h in self.gridSpacing)
        g.origin[:] = tuple(float(o) for o in self.origin)
        return g


@dataclass
class ConstantScalarField3:
    value: float


@dataclass
class CellCenteredScalarGrid3:
    """Cell-centred scalar grid: data (nz,ny,nx) sampled trilinearly with the
    data origin at origin + h/2."""
    resolution: tuple
    gridSpacing: tuple
    origin: tuple
    data: np.ndarray

    def dataOrigin(self):
        return tuple(o + 0.5 * h for o, h in zip(self.origin, self.gridSpacing))


kMaxD = float(np.finfo(np.float64).max)


def _field(f, keep: list) -> ScalarField:
    s = ScalarField()
    if f is None:
        raise ValueError("field required")
    if np.isscalar(f):
        f = ConstantScalarField3(float(f))
    if isinstance(f, ConstantScalarField3):
        s.kind = 0
        s.value = float(f.value)
        return s
    if isinstance(f, CellCenteredScalarGrid3):
        data = f.data
        if isinstance(data, np.ndarray):
            data = np.ascontiguousarray(data, np.float64)
        keep.append(data)
        s.kind = 1
        s.data = _p(data)
        nz, ny, nx = data.shape
        s.res[:] = (nx, ny, nz)
        s.origin[:] = f.dataOrigin()
        s.spacing[:] = tuple(float(h) for h in f.gridSpacing)
        return s
    raise TypeError(f"unsupported field type {type(f).__name__}")


# ---------------------------------------------------------------------------
# Solvers


class FdmMgpcgSolver3:
    """GPU multigrid-preconditioned CG with the reference constructor's
    arguments (fdm_mgpcg_solver3.h:35-41). ``maxTolerance`` is the relative
    true residual ||b - Ax|| / ||b|| the solve reaches."""

    def __init__(self, numberOfCgIter=100, maxNumberOfLevels=6,
                 numberOfRestrictionIter=2, numberOfCorrectionIter=2,
                 numberOfCoarsestIter=5, numberOfFinalIter=2,
                 maxTolerance=1e-6, sorFactor=1.2, useRedBlackOrdering=True,
                 precision="fp32", device=0, maxRefinements=6,
                 preconditioner="multigrid", orderedP2G=True,
                 fluidBoxIo=False):
        if not useRedBlackOrdering:
            raise ValueError("the GPU smoother is red-black; the lexicographic "
                             "Gauss-Seidel sweep is serial by construction")
        self.config = Config()
        library().jetgpu_config_default(C.byref(self.config))
        cfg = self.config
        cfg.device = device
        cfg.max_cg_iter = numberOfCgIter
        cfg.max_levels = maxNumberOfLevels
        cfg.restrict_iter = numberOfRestrictionIter
        cfg.correct_iter = numberOfCorrectionIter
        cfg.coarsest_iter = numberOfCoarsestIter
        cfg.final_iter = numberOfFinalIter
        cfg.tolerance = maxTolerance
        cfg.sor = sorFactor
        cfg.red_black = 1
        cfg.precision = PRECISION[precision]
        cfg.preconditioner = PRECONDITIONER[preconditioner]
        cfg.max_refinements = maxRefinements
        # P2G in particle order (bit-exact with the reference) or by FP64
        # atomics (faster; rounding-level differences).
        cfg.ordered_p2g = 1 if orderedP2G else 0
        # Host-pointer solves move only the velocity faces around the fluid
        # (GridFluidSolver3's convention: the output holds the input's
        # values elsewhere).
        cfg.fluid_box_io = 1 if fluidBoxIo else 0
        self._ctx = None
        self.last_stats = SolveStats()

    # -- context ------------------------------------------------------------
    def context(self) -> C.c_void_p:
        if self._ctx is None:
            h = C.c_void_p()
            st = library().jetgpu_create(C.byref(self.config), C.byref(h))
            if st != 0:
                raise JetGpuError(st, "jetgpu_create failed")
            self._ctx = h
        return self._ctx

    def close(self):
        if self._ctx is not None:
            library().jetgpu_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_network(self, params: np.ndarray) -> None:
        """Uploads preconditioner-network parameters (flat FP32, the order
        of jetgpu_net_param_count) for preconditioner='learned'."""
        p = np.ascontiguousarray(params, np.float32).reshape(-1)
        self.check(library().jetgpu_load_unet(self.context(), _p(p), p.size))

    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        h = C.c_void_p()
        self.check(library().jetgpu_get_stream(self.context(), C.byref(h)))
        return h.value or 0

    def profile(self, enable: bool) -> None:
        self.check(library().jetgpu_profile(self.context(), int(enable)))

    def profile_read(self) -> list:
        arr = (KernelStat * 64)()
        cnt = C.c_int(0)
        self.check(library().jetgpu_profile_read(self.context(), arr, 64,
                                                 C.byref(cnt)))
        return [dict(name=arr[i].name.decode(), launches=arr[i].launches,
                     total_ms=arr[i].total_ms, bytes=arr[i].bytes)
                for i in range(min(cnt.value, 64))]

    def check(self, status: int, allow=(0,)) -> int:
        if status not in allow:
            msg = library().jetgpu_last_error(self._ctx)
            raise JetGpuError(status, msg.decode() if msg else "")
        return status

    # -- reference accessors ------------------------------------------------
    def maxNumberOfIterations(self) -> int:
        return self.config.max_cg_iter

    def lastNumberOfIterations(self) -> int:
        return self.last_stats.iterations

    def tolerance(self) -> float:
        return self.config.tolerance

    def lastResidual(self) -> float:
        return self.last_stats.relative_residual

    def solve(self, system) -> bool:
        """FdmMgpcgSolver3::solve(FdmMgLinearSystem3*): ``system`` has
        ``A`` (list of (nz,ny,nx,4) float64 rows per level, finest first),
        ``b`` (list; level 0 is read) and ``x`` (list; level 0 written)."""
        A0 = system.A[0]
        res0 = (C.c_int * 3)(A0.shape[2], A0.shape[1], A0.shape[0])
        A = np.ascontiguousarray(np.concatenate([a.reshape(-1) for a in system.A]))
        b = np.ascontiguousarray(system.b[0], np.float64)
        x = np.zeros(A0.shape[:3])
        st = library().jetgpu_mgpcg_solve_system(
            self.context(), res0, len(system.A), _p(A), _p(b), _p(x),
            C.byref(self.last_stats))
        self.check(st, allow=SOLVED)
        system.x[0][...] = x
        return st == 0


@dataclass
class FdmMgLinearSystem3:
    A: list = dc_field(default_factory=list)
    x: list = dc_field(default_factory=list)
    b: list = dc_field(default_factory=list)


class GridFractionalSinglePhasePressureSolver3:
    """Drop-in GPU GridPressureSolver3 (grid_pressure_solver3.h:58-64)."""

    def __init__(self, linearSystemSolver: FdmMgpcgSolver3 | None = None):
        self._solver = linearSystemSolver or FdmMgpcgSolver3()
        self._pressure = None
        self.last_stats = SolveStats()

    @property
    def linearSystemSolver(self) -> FdmMgpcgSolver3:
        return self._solver

    @linearSystemSolver.setter
    def linearSystemSolver(self, s: FdmMgpcgSolver3):
        if not isinstance(s, FdmMgpcgSolver3):
            raise TypeError("the GPU pressure solver takes an FdmMgpcgSolver3")
        self._solver = s

    def setLinearSystemSolver(self, s: FdmMgpcgSolver3):
        self.linearSystemSolver = s

    @staticmethod
    def suggestedBoundaryConditionSolver() -> str:
        # grid_fractional_single_phase_pressure_solver3.cpp:486-490
        return "GridFractionalBoundaryConditionSolver3"

    def pressure(self) -> np.ndarray:
        """The last solve's pressure ((nz, ny, nx)), read from the device on
        first use after the solve (the solve itself downloads none)."""
        if self._pressure is None and getattr(self, "_pshape", None):
            p = self._pressure_buffer(self._pshape)
            cnt = C.c_size_t(0)
            self._solver.check(library().jetgpu_get_level(
                self._solver.context(), 0, 6, _p(p), p.nbytes, C.byref(cnt)))
            self._pressure = p
        return self._pressure

    def solve(self, input: FaceCenteredGrid3, timeIntervalInSeconds: float,
              output: FaceCenteredGrid3,
              boundarySdf=ConstantScalarField3(kMaxD),
              boundaryVelocity=None,
              fluidSdf=ConstantScalarField3(-kMaxD),
              useCompressed: bool = False) -> int:
        """Projects ``input`` into ``output`` (host arrays). boundaryVelocity
        is None (static collider), a tuple of per-face normal components
        (solid_u, solid_v, solid_w), or a rigid collider's motion
        (``Collider``: RigidBodyCollider3::velocityAt evaluated on the GPU at
        every face). ``useCompressed`` selects the
        reference's CSR storage; the GPU system is matrix-row based either
        way, so it has no effect. Returns the C status (0 or NOT_CONVERGED)."""
        del timeIntervalInSeconds, useCompressed  # unused, as in the reference
        keep = []
        bs = _field(boundarySdf, keep)
        fs = _field(fluidSdf, keep)
        g = input.c_grid()
        u = np.ascontiguousarray(input.u, np.float64)
        v = np.ascontiguousarray(input.v, np.float64)
        w = np.ascontiguousarray(input.w, np.float64)
        su = sv = sw = None
        collider = None
        if isinstance(boundaryVelocity, Collider):
            collider = boundaryVelocity
        elif boundaryVelocity is not None:
            su, sv, sw = (None if a is None else np.ascontiguousarray(a, np.float64)
                          for a in boundaryVelocity)
        for a, ref in ((output.u, u), (output.v, v), (output.w, w)):
            if a.shape != ref.shape or a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError("output arrays must match the input layout")
        nx, ny, nz = input.resolution
        p = None  # the pressure stays on the device until pressure()
        solver = self._solver
        if collider is not None:
            st = library().jetgpu_solve_pressure_collider(
                solver.context(), C.byref(g), _p(u), _p(v), _p(w),
                C.byref(bs), C.byref(fs), C.byref(collider), _p(output.u),
                _p(output.v), _p(output.w), _p(p), C.byref(self.last_stats))
        else:
            st = library().jetgpu_solve_pressure(
                solver.context(), C.byref(g), _p(u), _p(v), _p(w),
                C.byref(bs), C.byref(fs), _p(su), _p(sv), _p(sw),
                _p(output.u), _p(output.v), _p(output.w), _p(p),
                C.byref(self.last_stats))
        solver.last_stats = self.last_stats
        solver.check(st, allow=SOLVED)
        self._pressure = None
        self._pshape = (nz, ny, nx)
        return st

    def _pressure_buffer(self, shape) -> np.ndarray:
        """The pressure output, kept across solves in page-locked memory when
        torch can provide it (the device-to-host copy then runs at full
        bandwidth; a fresh pageable array per solve costs page faults and a
        staged copy)."""
        buf = getattr(self, "_pbuf", None)
        if buf is None or buf.shape != tuple(shape):
            try:
                import torch
                t = torch.empty(tuple(shape), dtype=torch.float64).pin_memory()
                self._pbuf_owner = t
                buf = t.numpy()
            except Exception:  # no torch or no CUDA driver: pageable memory
                buf = np.empty(tuple(shape))
            self._pbuf = buf
        return buf

    def level(self, level: int, what: str) -> np.ndarray:
        """Internal weights/system of the last solve (for parity checks)."""
        solver = self._solver
        code = {"fluid": 0, "uw": 1, "vw": 2, "ww": 3, "A": 4, "b": 5}[what]
        cnt = C.c_size_t(0)
        L = library()
        # Query size first with a zero-capacity call.
        dummy = np.zeros(1, np.float64)
        L.jetgpu_get_level(solver.context(), level, code, _p(dummy), 0,
                           C.byref(cnt))
        n = cnt.value
        if what in ("fluid", "uw", "vw", "ww"):
            out = np.zeros(n, np.float32)
        elif what == "A":
            out = np.zeros(n * 4, np.float64)
        else:
            out = np.zeros(n, np.float64)
        st = L.jetgpu_get_level(solver.context(), level, code, _p(out),
                                out.nbytes, C.byref(cnt))
        solver.check(st)
        return out


class GridSinglePhasePressureSolver3(GridFractionalSinglePhasePressureSolver3):
    """Drop-in GPU GridSinglePhasePressureSolver3, the blocked solver
    (include/jet/grid_single_phase_pressure_solver3.h:30-118): cells are
    fluid, air or boundary by the SDFs at their centres and the system is the
    7-point Laplacian on those markers. The reference defaults to an
    FdmIccgSolver3 (grid_single_phase_pressure_solver3.cpp:173-175); this
    solver runs the GPU FdmMgpcgSolver3, whose multigrid levels get the
    reference's majority-vote coarse markers (:270-317)."""

    @staticmethod
    def suggestedBoundaryConditionSolver() -> str:
        # grid_single_phase_pressure_solver3.cpp:213-216
        return "GridBlockedBoundaryConditionSolver3"

    def solve(self, input: FaceCenteredGrid3, timeIntervalInSeconds: float,
              output: FaceCenteredGrid3,
              boundarySdf=ConstantScalarField3(kMaxD),
              boundaryVelocity=None,
              fluidSdf=ConstantScalarField3(-kMaxD),
              useCompressed: bool = False) -> int:
        """Projects ``input`` into ``output`` (host arrays). Like the
        reference, the boundary velocity is not used (:191) and
        ``useCompressed`` changes only the storage. Returns the C status."""
        del timeIntervalInSeconds, boundaryVelocity, useCompressed
        keep = []
        bs = _field(boundarySdf, keep)
        fs = _field(fluidSdf, keep)
        g = input.c_grid()
        u = np.ascontiguousarray(input.u, np.float64)
        v = np.ascontiguousarray(input.v, np.float64)
        w = np.ascontiguousarray(input.w, np.float64)
        for a, ref in ((output.u, u), (output.v, v), (output.w, w)):
            if a.shape != ref.shape or a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError("output arrays must match the input layout")
        nx, ny, nz = input.resolution
        p = None  # the pressure stays on the device until pressure()
        solver = self._solver
        st = library().jetgpu_solve_pressure_blocked(
            solver.context(), C.byref(g), _p(u), _p(v), _p(w), C.byref(bs),
            C.byref(fs), _p(output.u), _p(output.v), _p(output.w), _p(p),
            C.byref(self.last_stats))
        solver.last_stats = self.last_stats
        solver.check(st, allow=SOLVED)
        self._pressure = None
        self._pshape = (nz, ny, nx)
        return st


def solve_pressure_blocked_device(solver: FdmMgpcgSolver3, grid: Grid, u, v,
                                  w, boundary: ScalarField,
                                  fluid: ScalarField, out_u, out_v, out_w,
                                  out_p=None,
                                  stats: SolveStats | None = None) -> int:
    """Device-pointer form of the blocked solve (torch CUDA float64)."""
    stats = stats if stats is not None else SolveStats()
    st = library().jetgpu_solve_pressure_blocked_device(
        solver.context(), C.byref(grid), _p(u), _p(v), _p(w), C.byref(boundary),
        C.byref(fluid), _p(out_u), _p(out_v), _p(out_w), _p(out_p),
        C.byref(stats))
    solver.last_stats = stats
    return solver.check(st, allow=SOLVED)


def solve_pressure_device(solver: FdmMgpcgSolver3, grid: Grid, u, v, w,
                          boundary: ScalarField, fluid: ScalarField,
                          out_u, out_v, out_w, out_p=None, solid=(None, None, None),
                          stats: SolveStats | None = None) -> int:
    """Device-pointer form (torch CUDA float64 tensors)."""
    stats = stats if stats is not None else SolveStats()
    st = library().jetgpu_solve_pressure_device(
        solver.context(), C.byref(grid), _p(u), _p(v), _p(w), C.byref(boundary),
        C.byref(fluid), _p(solid[0]), _p(solid[1]), _p(solid[2]), _p(out_u),
        _p(out_v), _p(out_w), _p(out_p), C.byref(stats))
    solver.last_stats = stats
    return solver.check(st, allow=SOLVED)


# ---------------------------------------------------------------------------
# Particle transfers (host arrays)


def transfer_from_particles_to_grids(solver: FdmMgpcgSolver3,
                                     grid: FaceCenteredGrid3, positions,
                                     velocities, markers=True, snapshot=True):
    """PicSolver3::transferFromParticlesToGrids (+ FLIP snapshot).
    Fills grid.u/v/w; returns (markers, snapshots) lists."""
    pos = np.ascontiguousarray(positions, np.float64)
    vel = np.ascontiguousarray(velocities, np.float64)
    shapes = [grid.u.shape, grid.v.shape, grid.w.shape]
    marks = [np.zeros(s, np.uint8) for s in shapes] if markers else [None] * 3
    snaps = [np.zeros(s, np.float32) for s in shapes] if snapshot else [None] * 3
    g = grid.c_grid()
    st = library().jetgpu_p2g(solver.context(), C.byref(g), pos.shape[0],
                              _p(pos), _p(vel), _p(grid.u), _p(grid.v),
                              _p(grid.w), *[_p(m) for m in marks],
                              *[_p(s) for s in snaps])
    solver.check(st)
    return marks, snaps


def flip_transfer_from_grids_to_particles(solver: FdmMgpcgSolver3,
                                          grid: FaceCenteredGrid3, positions,
                                          velocities, snapshots,
                                          picBlendingFactor=0.0):
    """FlipSolver3::transferFromGridsToParticles. Updates ``velocities`` and
    turns ``snapshots`` into the float deltas, in place."""
    pos = np.ascontiguousarray(positions, np.float64)
    if not (velocities.dtype == np.float64 and velocities.flags.c_contiguous):
        raise ValueError("velocities must be C-contiguous float64")
    g = grid.c_grid()
    st = library().jetgpu_g2p_flip(solver.context(), C.byref(g), pos.shape[0],
                                   _p(pos), _p(velocities), _p(grid.u),
                                   _p(grid.v), _p(grid.w),
                                   *[_p(s) for s in snapshots],
                                   float(picBlendingFactor))
    solver.check(st)
    return velocities


def pic_transfer_from_grids_to_particles(solver: FdmMgpcgSolver3,
                                         grid: FaceCenteredGrid3, positions,
                                         velocities):
    """PicSolver3::transferFromGridsToParticles (in place)."""
    pos = np.ascontiguousarray(positions, np.float64)
    if not (velocities.dtype == np.float64 and velocities.flags.c_contiguous):
        raise ValueError("velocities must be C-contiguous float64")
    g = grid.c_grid()
    st = library().jetgpu_g2p_pic(solver.context(), C.byref(g), pos.shape[0],
                                  _p(pos), _p(velocities), _p(grid.u),
                                  _p(grid.v), _p(grid.w))
    solver.check(st)
    return velocities


class Sphere(C.Structure):
    """jetgpu_sphere: a Sphere3 collider surface under its Transform3
    (orientation matrix and inverse, row-major)."""
    _fields_ = [
        ("center", C.c_double * 3),
        ("radius", C.c_double),
        ("normal_flipped", C.c_int),
        ("orientation", C.c_double * 9),
        ("inverse_orientation", C.c_double * 9),
    ]

    @staticmethod
    def make(radius, center=(0, 0, 0), normal_flipped=False,
             orientation=None, inverse_orientation=None) -> "Sphere":
        s = Sphere()
        s.center[:] = tuple(float(x) for x in center)
        s.radius = float(radius)
        s.normal_flipped = int(bool(normal_flipped))
        eye = tuple(float(x) for x in np.eye(3).ravel())
        s.orientation[:] = eye if orientation is None else \
            tuple(float(x) for x in np.ravel(orientation))
        s.inverse_orientation[:] = eye if inverse_orientation is None else \
            tuple(float(x) for x in np.ravel(inverse_orientation))
        return s


def move_particles(solver: "FdmMgpcgSolver3", grid: FaceCenteredGrid3,
                   positions, velocities, dt: float, maxCfl: float = 5.0,
                   closed: int = kDirectionAll, collider: Collider = None,
                   sphere: Sphere = None):
    """PicSolver3::moveParticles (+ sphere collisions) in place on host
    arrays (C-contiguous float64, shape (n, 3))."""
    for a in (positions, velocities):
        if not (a.dtype == np.float64 and a.flags.c_contiguous):
            raise ValueError("positions/velocities must be C-contiguous float64")
    g = grid.c_grid()
    st = library().jetgpu_move_particles(
        solver.context(), C.byref(g), positions.shape[0], _p(positions),
        _p(velocities), _p(grid.u), _p(grid.v), _p(grid.w), float(dt),
        float(maxCfl), int(closed),
        C.byref(collider) if collider is not None else None,
        C.byref(sphere) if sphere is not None else None)
    solver.check(st)
    return positions, velocities


def move_particles_device(solver: "FdmMgpcgSolver3", grid: Grid, pos, vel, u,
                          v, w, dt: float, maxCfl: float = 5.0,
                          closed: int = kDirectionAll,
                          collider: Collider = None, sphere: Sphere = None):
    """jetgpu_move_particles_device on device tensors (in place)."""
    st = library().jetgpu_move_particles_device(
        solver.context(), C.byref(grid), pos.shape[0], _p(pos), _p(vel),
        _p(u), _p(v), _p(w), float(dt), float(maxCfl), int(closed),
        C.byref(collider) if collider is not None else None,
        C.byref(sphere) if sphere is not None else None)
    solver.check(st)


def build_signed_distance_field(solver: "FdmMgpcgSolver3",
                                grid: FaceCenteredGrid3, positions,
                                collider_sdf=None, maxCfl: float = 5.0):
    """PicSolver3::buildSignedDistanceField (+ extrapolation into the
    collider) from host particle positions (n, 3); returns the cell-centred
    liquid SDF (nz, ny, nx) the pressure solve takes."""
    pos = np.ascontiguousarray(positions, np.float64)
    nx, ny, nz = grid.resolution
    out = np.zeros((nz, ny, nx))
    keep = []
    f = _field(collider_sdf if collider_sdf is not None
               else ConstantScalarField3(kMaxD), keep)
    g = grid.c_grid()
    st = library().jetgpu_build_particle_sdf(
        solver.context(), C.byref(g), pos.shape[0], _p(pos), C.byref(f),
        float(maxCfl), _p(out))
    solver.check(st)
    return out


def build_signed_distance_field_device(solver: "FdmMgpcgSolver3", grid: Grid,
                                       pos, collider_sdf: ScalarField, out,
                                       maxCfl: float = 5.0):
    """jetgpu_build_particle_sdf_device on device tensors."""
    st = library().jetgpu_build_particle_sdf_device(
        solver.context(), C.byref(grid), pos.shape[0], _p(pos),
        C.byref(collider_sdf), float(maxCfl), _p(out))
    solver.check(st)


class FlipParams(C.Structure):
    """jetgpu_flip_params (GridFluidSolver3 / FlipSolver3 settings)."""
    _fields_ = [
        ("gravity", C.c_double * 3),
        ("max_cfl", C.c_double),
        ("closed_domain_flags", C.c_int),
        ("flip", C.c_int),
        ("pic_blending", C.c_double),
    ]


class FlipSolver3:
    """FlipSolver3 / PicSolver3 with particles and grid resident on the GPU
    (src/jet/flip_solver3.cpp, src/jet/pic_solver3.cpp).

    Particles are set with ``setParticles(positions, velocities)`` (host
    arrays (n, 3)); ``update(frameInterval)`` advances one frame with the
    reference's adaptive sub-stepping (PhysicsAnimation::onUpdate,
    src/jet/physics_animation.cpp:98-122): while time remains, take
    max(ceil(cfl / maxCfl), 1) equal sub-steps of the remaining time, each
    one ``jetgpu_flip_substep_device``. The pressure projection uses
    ``pressureSolver`` (an FdmMgpcgSolver3, which also owns the GPU
    context). Device state: positions, velocities, the face velocity u/v/w and
    the particle SDF, as torch tensors."""

    TRANSFERS = {"pic": 0, "flip": 1, "apic": 2}

    def __init__(self, resolution, gridSpacing, origin=(0.0, 0.0, 0.0),
                 pressureSolver: "FdmMgpcgSolver3 | None" = None,
                 flip: bool = True, device: int = 0,
                 transfer: str | None = None):
        import torch
        self._torch = torch
        self.solver = pressureSolver if pressureSolver is not None \
            else FdmMgpcgSolver3(device=device)
        self.dev = torch.device("cuda", device)
        nx, ny, nz = (int(r) for r in resolution)
        if np.isscalar(gridSpacing):
            gridSpacing = (float(gridSpacing),) * 3
        self.resolution = (nx, ny, nz)
        self.gridSpacing = tuple(float(h) for h in gridSpacing)
        self.origin = tuple(float(o) for o in origin)
        self.grid = Grid()
        self.grid.res[:] = self.resolution
        self.grid.spacing[:] = self.gridSpacing
        self.grid.origin[:] = self.origin
        f64 = dict(dtype=torch.float64, device=self.dev)
        self.u = torch.zeros((nz, ny, nx + 1), **f64)
        self.v = torch.zeros((nz, ny + 1, nx), **f64)
        self.w = torch.zeros((nz + 1, ny, nx), **f64)
        self.sdf = torch.zeros((nz, ny, nx), **f64)
        self.pos = torch.zeros((0, 3), **f64)
        self.vel = torch.zeros((0, 3), **f64)
        self.params = FlipParams()
        library().jetgpu_flip_params_default(C.byref(self.params))
        # transfer: "flip" (FlipSolver3), "pic" (PicSolver3) or "apic"
        # (ApicSolver3); `flip` chooses between the first two.
        if transfer is None:
            transfer = "flip" if flip else "pic"
        self.params.flip = self.TRANSFERS[transfer]
        self.affine = torch.zeros((0, 9), **f64)
        self._col_sdf = None
        self._collider = None
        self._sphere = None
        self.currentTimeInSeconds = 0.0
        self.subSteps = 0
        self.lastStats = SolveStats()
        # Sum over sub-steps of the pressure projection's device time
        # (weights, system and MGPCG solve: SolveStats.setup_ms + solve_ms,
        # CUDA events around those kernels) and iterations.
        self.pressureMs = 0.0
        self.pressureIterations = 0
        # The library works on its own stream; torch's uploads and reads of
        # these tensors are ordered against it explicitly.
        self._stream = torch.cuda.ExternalStream(self.solver.stream(),
                                                 device=self.dev)

    def _uploaded(self):
        """Orders torch's writes to the state before library work."""
        self._torch.cuda.current_stream(self.dev).synchronize()

    def synchronize(self):
        """Waits for the library's queued work on the state."""
        self._stream.synchronize()

    # -- settings (GridFluidSolver3 / FlipSolver3 accessors) ----------------
    def setGravity(self, g):
        self.params.gravity[:] = tuple(float(x) for x in g)

    def setMaxCfl(self, cfl: float):
        self.params.max_cfl = float(cfl)

    def setClosedDomainBoundaryFlag(self, flag: int):
        self.params.closed_domain_flags = int(flag)

    def setPicBlendingFactor(self, f: float):
        self.params.pic_blending = float(f)

    def setCollider(self, collider_sdf, collider: Collider = None,
                    sphere: Sphere = None):
        """The collider: its SDF on this grid's cell centres (what the
        reference's boundary solver builds from the surface; (nz,ny,nx)
        array), and optionally its motion and sphere surface for particle
        collisions."""
        self.synchronize()
        self._col_sdf = self._torch.as_tensor(
            np.ascontiguousarray(collider_sdf, np.float64), device=self.dev)
        self._collider = collider
        self._sphere = sphere
        self._uploaded()

    def setParticles(self, positions, velocities=None):
        pos = np.ascontiguousarray(positions, np.float64).reshape(-1, 3)
        vel = np.zeros_like(pos) if velocities is None else \
            np.ascontiguousarray(velocities, np.float64).reshape(-1, 3)
        self.synchronize()
        self.pos = self._torch.from_numpy(pos.copy()).to(self.dev)
        self.vel = self._torch.from_numpy(vel.copy()).to(self.dev)
        # APIC's affine matrices start at zero, as ApicSolver3's do once its
        # first G2P has run (apic_solver3.cpp:160-165).
        self.affine = self._torch.zeros((pos.shape[0], 9),
                                        dtype=self._torch.float64,
                                        device=self.dev)
        self._uploaded()

    def positions(self) -> np.ndarray:
        self.synchronize()
        return self.pos.cpu().numpy()

    def pressure(self) -> np.ndarray:
        """The last sub-step's pressure ((nz, ny, nx); the reference's
        GridFractionalSinglePhasePressureSolver3::pressure())."""
        self.synchronize()
        nx, ny, nz = self.resolution
        out = np.zeros(nx * ny * nz)
        cnt = C.c_size_t(0)
        self.solver.check(library().jetgpu_get_level(
            self.solver.context(), 0, 6, _p(out), out.nbytes, C.byref(cnt)))
        return out.reshape(nz, ny, nx)

    def velocities(self) -> np.ndarray:
        self.synchronize()
        return self.vel.cpu().numpy()

    # -- stepping ------------------------------------------------------------
    def _col_field(self) -> ScalarField:
        f = ScalarField()
        if self._col_sdf is None:
            f.kind = 0
            f.value = kMaxD
            return f
        f.kind = 1
        f.data = self._col_sdf.data_ptr()
        f.res[:] = self.resolution
        f.origin[:] = tuple(o + 0.5 * h for o, h in zip(self.origin,
                                                        self.gridSpacing))
        f.spacing[:] = self.gridSpacing
        return f

    def cfl(self, dt: float) -> float:
        out = C.c_double(0.0)
        g = (C.c_double * 3)(*self.params.gravity)
        st = library().jetgpu_fluid_cfl_device(
            self.solver.context(), C.byref(self.grid), _p(self.u), _p(self.v),
            _p(self.w), float(dt), g, C.byref(out))
        self.solver.check(st)
        return out.value

    def numberOfSubTimeSteps(self, dt: float) -> int:
        return int(max(np.ceil(self.cfl(dt) / self.params.max_cfl), 1.0))

    def advanceSubStep(self, dt: float):
        f = self._col_field()
        st = library().jetgpu_flip_substep_device(
            self.solver.context(), C.byref(self.grid), self.pos.shape[0],
            _p(self.pos), _p(self.vel),
            _p(self.affine) if self.params.flip == 2 else None,
            _p(self.u), _p(self.v), _p(self.w),
            _p(self.sdf), C.byref(f),
            C.byref(self._collider) if self._collider is not None else None,
            C.byref(self._sphere) if self._sphere is not None else None,
            C.byref(self.params), float(dt), C.byref(self.lastStats))
        self.solver.check(st, allow=SOLVED)
        self.subSteps += 1
        self.pressureMs += self.lastStats.setup_ms + self.lastStats.solve_ms
        self.pressureIterations += self.lastStats.iterations

    def update(self, frameInterval: float):
        """One frame (PhysicsAnimation::onUpdate's adaptive branch)."""
        remaining = float(frameInterval)
        eps = float(np.finfo(np.float64).eps)
        while remaining > eps:
            n = self.numberOfSubTimeSteps(remaining)
            dt = remaining / float(n)
            self.advanceSubStep(dt)
            remaining -= dt
            self.currentTimeInSeconds += dt
        self.synchronize()  # the reference's update() returns when done


def apic_transfer_from_particles_to_grids_device(solver: "FdmMgpcgSolver3",
                                                 grid: Grid, pos, vel, affine,
                                                 u, v, w, mu=None, mv=None,
                                                 mw=None):
    """ApicSolver3::transferFromParticlesToGrids on device tensors."""
    st = library().jetgpu_apic_p2g_device(
        solver.context(), C.byref(grid), pos.shape[0], _p(pos), _p(vel),
        _p(affine), _p(u), _p(v), _p(w), _p(mu), _p(mv), _p(mw))
    solver.check(st)


def apic_transfer_from_grids_to_particles_device(solver: "FdmMgpcgSolver3",
                                                 grid: Grid, pos, vel, affine,
                                                 u, v, w):
    """ApicSolver3::transferFromGridsToParticles on device tensors."""
    st = library().jetgpu_apic_g2p_device(
        solver.context(), C.byref(grid), pos.shape[0], _p(pos), _p(vel),
        _p(affine), _p(u), _p(v), _p(w))
    solver.check(st)


class GridFractionalBoundaryConditionSolver3:
    """Mirror of GridFractionalBoundaryConditionSolver3
    (src/jet/grid_fractional_boundary_condition_solver3.cpp) on the GPU.

    updateCollider(collider_sdf, collider) installs the collider: its SDF as
    a CellCenteredScalarGrid3 on the velocity grid (what colliderSdf() holds;
    None = no collider) and a ``Collider`` for its surface velocity and
    friction. constrainVelocity(velocity, extrapolationDepth) then matches the
    reference bit for bit. The GPU context is borrowed from ``owner`` (an
    FdmMgpcgSolver3), or a private one is created."""

    _entry = "jetgpu_constrain_velocity"

    def __init__(self, owner: "FdmMgpcgSolver3 | None" = None):
        self._owner = owner if owner is not None else FdmMgpcgSolver3()
        self._sdf = ConstantScalarField3(kMaxD)
        self._collider = None
        self._closed = kDirectionAll

    def updateCollider(self, collider_sdf=None, collider: Collider = None):
        self._sdf = collider_sdf if collider_sdf is not None \
            else ConstantScalarField3(kMaxD)
        self._collider = collider

    def colliderSdf(self):
        return self._sdf

    def setClosedDomainBoundaryFlag(self, flag: int):
        self._closed = int(flag)

    def closedDomainBoundaryFlag(self) -> int:
        return self._closed

    def constrainVelocity(self, velocity: FaceCenteredGrid3,
                          extrapolationDepth: int = 5):
        """In place on velocity.u/v/w (host arrays)."""
        for a in (velocity.u, velocity.v, velocity.w):
            if not (a.dtype == np.float64 and a.flags.c_contiguous):
                raise ValueError("velocity arrays must be C-contiguous float64")
        keep = []
        f = _field(self._sdf, keep)
        g = velocity.c_grid()
        col = C.byref(self._collider) if self._collider is not None else None
        st = getattr(library(), self._entry)(
            self._owner.context(), C.byref(g), _p(velocity.u), _p(velocity.v),
            _p(velocity.w), C.byref(f), col, self._closed,
            int(extrapolationDepth))
        self._owner.check(st)
        return velocity


class GridBlockedBoundaryConditionSolver3(GridFractionalBoundaryConditionSolver3):
    """Mirror of GridBlockedBoundaryConditionSolver3
    (src/jet/grid_blocked_boundary_condition_solver3.cpp), the solver the
    blocked pressure solver suggests: the fractional constraint, then the
    faces between collider cells (colliderSdf() < 0 at the cell) and the
    other cells take the collider velocity. Bit-identical to the reference."""

    _entry = "jetgpu_constrain_velocity_blocked"

    def marker(self, resolution) -> np.ndarray:
        """The reference's cell markers (:69-71): 0 collider, 1 fluid."""
        nx, ny, nz = resolution
        sdf = self._sdf
        if isinstance(sdf, CellCenteredScalarGrid3):
            return np.where(np.asarray(sdf.data) < 0, 0, 1).astype(np.int8)
        value = float(sdf.value)
        return np.full((nz, ny, nx), 0 if value < 0 else 1, np.int8)


def constrain_velocity_device(solver: "FdmMgpcgSolver3", grid: Grid, u, v, w,
                              collider_sdf: ScalarField,
                              collider: Collider = None,
                              closed: int = kDirectionAll, depth: int = 5,
                              blocked: bool = False):
    """jetgpu_constrain_velocity_device (or, with ``blocked``, the blocked
    solver's jetgpu_constrain_velocity_blocked_device) on device tensors (in
    place)."""
    col = C.byref(collider) if collider is not None else None
    fn = (library().jetgpu_constrain_velocity_blocked_device if blocked
          else library().jetgpu_constrain_velocity_device)
    st = fn(
        solver.context(), C.byref(grid), _p(u), _p(v), _p(w),
        C.byref(collider_sdf), col, int(closed), int(depth))
    solver.check(st)


def extrapolate_to_region_device(solver: "FdmMgpcgSolver3", data, valid,
                                 iterations: int):
    """extrapolateToRegion on a device tensor (nz,ny,nx) in place from the
    cells whose byte in ``valid`` (uint8 tensor, same shape) is non-zero."""
    nz, ny, nx = data.shape
    res = (C.c_int * 3)(nx, ny, nz)
    st = library().jetgpu_extrapolate_to_region_device(
        solver.context(), res, _p(data), _p(valid), int(iterations))
    solver.check(st)


def version() -> str:
    return library().jetgpu_version().decode()
