"""Oracle bindings — TEST INFRASTRUCTURE ONLY.

ctypes bindings for the two libraries that export ``oracle/oracle_api.h``:

* ``port()``: the CPU restatement of the Jet pressure projection written in
  this repository (``oracle/port/jet_port.cpp``), built by ``oracle/Makefile``.
  It is what the GPU tests compare against and the CPU baseline that
  ``bench.py`` times.
* ``reference()``: the Jet reference compiled from its own sources
  (``oracle/Makefile.ref`` + ``oracle/ref_harness.cpp``). It exists only where
  the reference sources are present; it pins the port.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may use this package. The product (``jetgpu``) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
PORT_SO = os.path.join(HERE, "_build", "liboracle_port.so")
REF_SO = os.path.join(HERE, "_ref", "libjet_ref_harness.so")
REF_SRC = "/root/reference"


class OrcField(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("value", C.c_double),
        ("data", C.POINTER(C.c_double)),
        ("res", C.c_int * 3),
        ("origin", C.c_double * 3),
        ("spacing", C.c_double * 3),
    ]


class OrcMgParams(C.Structure):
    _fields_ = [
        ("max_cg_iter", C.c_uint),
        ("max_levels", C.c_uint),
        ("restrict_iter", C.c_uint),
        ("correct_iter", C.c_uint),
        ("coarsest_iter", C.c_uint),
        ("final_iter", C.c_uint),
        ("tolerance", C.c_double),
        ("sor", C.c_double),
        ("red_black", C.c_int),
    ]


class OrcCollider(C.Structure):
    _fields_ = [
        ("lin", C.c_double * 3),
        ("ang", C.c_double * 3),
        ("centre", C.c_double * 3),
        ("friction", C.c_double),
    ]


class OrcSphere(C.Structure):
    _fields_ = [
        ("center", C.c_double * 3),
        ("radius", C.c_double),
        ("normal_flipped", C.c_int),
        ("orient", C.c_double * 9),
        ("inv_orient", C.c_double * 9),
        ("quat", C.c_double * 4),
    ]


class OrcGrid(C.Structure):
    _fields_ = [
        ("res", C.c_int * 3),
        ("spacing", C.c_double * 3),
        ("origin", C.c_double * 3),
    ]


_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_cp = C.POINTER(C.c_char)


def _ptr(a, t=_dp):
    if a is None:
        return None
    return a.ctypes.data_as(t)


def build_port(quiet: bool = True) -> str:
    """Compile the oracle port (seconds). Returns the library path."""
    subprocess.run(["make", "-s", "-f", "oracle/Makefile"], cwd=REPO,
                   check=True, capture_output=quiet)
    return PORT_SO


def build_reference(quiet: bool = True) -> str | None:
    """Compile the reference harness from the reference sources when they are
    present (about a minute with 8 cores). Returns the path or None."""
    if not os.path.isdir(os.path.join(REF_SRC, "src", "jet")):
        return REF_SO if os.path.exists(REF_SO) else None
    jobs = str(max(1, os.cpu_count() or 1))
    subprocess.run(["make", "-s", "-j", jobs, "-f", "oracle/Makefile.ref",
                    "REF=" + REF_SRC], cwd=REPO, check=True,
                   capture_output=quiet)
    return REF_SO


@dataclass
class MgParams:
    """FdmMgpcgSolver3 constructor arguments (fdm_mgpcg_solver3.h:35-41)."""
    max_cg_iter: int = 100
    max_levels: int = 5
    restrict_iter: int = 5
    correct_iter: int = 5
    coarsest_iter: int = 20
    final_iter: int = 20
    tolerance: float = 1e-9
    sor: float = 1.5
    red_black: bool = True

    def c(self) -> OrcMgParams:
        return OrcMgParams(self.max_cg_iter, self.max_levels,
                           self.restrict_iter, self.correct_iter,
                           self.coarsest_iter, self.final_iter,
                           self.tolerance, self.sor, int(self.red_black))


def field(value_or_grid, spacing=None, data_origin=None) -> tuple:
    """Builds an OrcField from a constant or a cell-centred grid (nz,ny,nx)."""
    f = OrcField()
    keep = None
    if np.isscalar(value_or_grid):
        f.kind = 0
        f.value = float(value_or_grid)
    else:
        g = np.ascontiguousarray(value_or_grid, dtype=np.float64)
        keep = g
        f.kind = 1
        f.data = _ptr(g)
        nz, ny, nx = g.shape
        f.res[:] = (nx, ny, nz)
        f.spacing[:] = tuple(spacing)
        f.origin[:] = tuple(data_origin)
    return f, keep


class Oracle:
    """One loaded oracle library (port or reference harness)."""

    def __init__(self, path: str):
        self.path = path
        L = C.CDLL(path)
        self.lib = L
        L.orc_pressure_solve.restype = C.c_int
        L.orc_pressure_solve.argtypes = [
            C.POINTER(OrcGrid), _dp, _dp, _dp, C.POINTER(OrcField),
            C.POINTER(OrcField), _dp, _dp, _dp, C.POINTER(OrcMgParams),
            _dp, _dp, _dp, _dp, C.POINTER(C.c_uint), _dp]
        L.orc_blocked_pressure_solve.restype = C.c_int
        L.orc_blocked_pressure_solve.argtypes = [
            C.POINTER(OrcGrid), _dp, _dp, _dp, C.POINTER(OrcField),
            C.POINTER(OrcField), C.POINTER(OrcMgParams),
            _dp, _dp, _dp, _dp, C.POINTER(C.c_uint), _dp]
        L.orc_blocked_get_level.restype = C.c_long
        L.orc_blocked_get_level.argtypes = [C.c_int, C.c_int, C.c_void_p]
        L.orc_level_count.restype = C.c_int
        L.orc_get_level.restype = C.c_long
        L.orc_get_level.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_size_t]
        L.orc_mgpcg_system.restype = C.c_int
        L.orc_mgpcg_system.argtypes = [C.POINTER(C.c_int), C.c_int, _dp, _dp,
                                       C.POINTER(OrcMgParams), _dp,
                                       C.POINTER(C.c_uint), _dp]
        L.orc_relax.restype = None
        L.orc_relax.argtypes = [C.POINTER(C.c_int), _dp, _dp, C.c_double,
                                C.c_int, C.c_int, _dp]
        L.orc_mg_restrict.argtypes = [C.POINTER(C.c_int), _dp, _dp]
        L.orc_mg_correct.argtypes = [C.POINTER(C.c_int), _dp, _dp]
        L.orc_residual.argtypes = [C.POINTER(C.c_int), _dp, _dp, _dp, _dp]
        L.orc_dot.restype = C.c_double
        L.orc_dot.argtypes = [C.c_long, _dp, _dp]
        L.orc_p2g.argtypes = [C.POINTER(OrcGrid), C.c_long, _dp, _dp, _dp,
                              _dp, _dp, _cp, _cp, _cp, _fp, _fp, _fp]
        L.orc_g2p_flip.argtypes = [C.POINTER(OrcGrid), C.c_long, _dp, _dp,
                                   _dp, _dp, _dp, _fp, _fp, _fp, C.c_double]
        L.orc_g2p_pic.argtypes = [C.POINTER(OrcGrid), C.c_long, _dp, _dp,
                                  _dp, _dp, _dp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_constrain_velocity.argtypes = [
            C.POINTER(OrcGrid), _dp, _dp, _dp, C.POINTER(OrcField),
            C.POINTER(OrcCollider), C.c_int, C.c_uint]
        L.orc_constrain_velocity_blocked.argtypes = \
            L.orc_constrain_velocity.argtypes
        L.orc_extrapolate.argtypes = [C.POINTER(C.c_int), _dp, _cp, C.c_uint]
        L.orc_move_particles.argtypes = [
            C.POINTER(OrcGrid), C.c_long, _dp, _dp, _dp, _dp, _dp, C.c_double,
            C.c_double, C.c_int, C.POINTER(OrcCollider), C.POINTER(OrcSphere)]
        L.orc_apic_p2g.argtypes = [C.POINTER(OrcGrid), C.c_long, _dp, _dp,
                                   _dp, _dp, _dp, _dp, _cp, _cp, _cp]
        L.orc_apic_g2p.argtypes = [C.POINTER(OrcGrid), C.c_long, _dp, _dp,
                                   _dp, _dp, _dp, _dp]
        L.orc_build_particle_sdf.argtypes = [
            C.POINTER(OrcGrid), C.c_long, _dp, C.POINTER(OrcField), C.c_double,
            _dp]
        if hasattr(L, "orc_flip_run"):
            L.orc_flip_run.argtypes = [
                C.POINTER(OrcGrid), C.c_long, _dp, _dp, C.c_int, C.c_double,
                C.c_double, C.c_int, _dp, C.c_int, C.POINTER(OrcMgParams)]
        if hasattr(L, "orc_flip_run_record"):
            L.orc_flip_run_record.argtypes = [
                C.POINTER(OrcGrid), C.c_long, _dp, _dp, C.c_int, C.c_double,
                C.c_double, C.c_int, _dp, C.c_int, C.POINTER(OrcMgParams),
                C.c_int, C.POINTER(C.c_int), _dp]
        if hasattr(L, "orc_flip_run_sphere"):
            L.orc_flip_run_sphere.argtypes = [
                C.POINTER(OrcGrid), C.c_long, _dp, _dp, C.c_int, C.c_double,
                C.c_double, C.c_int, _dp, C.c_int, C.POINTER(OrcMgParams),
                _dp, C.c_double, C.c_double]
        if hasattr(L, "orc_quaternion_matrices"):
            L.orc_quaternion_matrices.argtypes = [_dp, _dp, _dp]
        if hasattr(L, "orc_sphere_collider_sdf"):
            L.orc_sphere_collider_sdf.argtypes = [C.POINTER(OrcGrid), _dp,
                                                  C.c_double, _dp]

    def set_threads(self, n: int = 0) -> None:
        self.lib.orc_set_threads(int(n))

    def set_relative_stop(self, rel: float) -> None:
        """Port only: also stop on ||b-Ax||/||b|| <= rel (0 disables)."""
        f = self.lib.orc_set_relative_stop
        f.argtypes = [C.c_double]
        f(float(rel))

    # -- pressure projection ------------------------------------------------
    def pressure_solve(self, res, spacing, origin, u, v, w, boundary_sdf,
                       fluid_sdf, params: MgParams, solid=(None, None, None)):
        """GridFractionalSinglePhasePressureSolver3::solve + FdmMgpcgSolver3.

        u/v/w are (nz,ny,nx+1)/(nz,ny+1,nx)/(nz+1,ny,nx) float64 arrays.
        boundary_sdf / fluid_sdf are a constant or a cell-centred grid array
        on the velocity grid. Returns dict with u, v, w, p, iters, resid, ok.
        """
        g = OrcGrid()
        g.res[:] = tuple(res)
        g.spacing[:] = tuple(spacing)
        g.origin[:] = tuple(origin)
        data_origin = tuple(o + 0.5 * h for o, h in zip(origin, spacing))
        bf, bk = field(boundary_sdf, spacing, data_origin)
        ff, fk = field(fluid_sdf, spacing, data_origin)
        u = np.ascontiguousarray(u, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        w = np.ascontiguousarray(w, np.float64)
        su, sv, sw = (None if s is None else np.ascontiguousarray(s, np.float64)
                      for s in solid)
        ou, ov, ow = u.copy(), v.copy(), w.copy()
        nx, ny, nz = res
        p = np.zeros((nz, ny, nx))
        it = C.c_uint(0)
        rs = C.c_double(0)
        prm = params.c()
        ok = self.lib.orc_pressure_solve(
            C.byref(g), _ptr(u), _ptr(v), _ptr(w), C.byref(bf), C.byref(ff),
            _ptr(su), _ptr(sv), _ptr(sw), C.byref(prm), _ptr(ou), _ptr(ov),
            _ptr(ow), _ptr(p), C.byref(it), C.byref(rs))
        del bk, fk
        return dict(u=ou, v=ov, w=ow, p=p, iters=it.value, resid=rs.value,
                    ok=bool(ok))

    def blocked_pressure_solve(self, res, spacing, origin, u, v, w,
                               boundary_sdf, fluid_sdf, params: MgParams):
        """GridSinglePhasePressureSolver3::solve + FdmMgpcgSolver3 (the
        blocked solver); arguments and result as pressure_solve."""
        g = OrcGrid()
        g.res[:] = tuple(res)
        g.spacing[:] = tuple(spacing)
        g.origin[:] = tuple(origin)
        data_origin = tuple(o + 0.5 * h for o, h in zip(origin, spacing))
        bf, bk = field(boundary_sdf, spacing, data_origin)
        ff, fk = field(fluid_sdf, spacing, data_origin)
        u = np.ascontiguousarray(u, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        w = np.ascontiguousarray(w, np.float64)
        ou, ov, ow = u.copy(), v.copy(), w.copy()
        nx, ny, nz = res
        p = np.zeros((nz, ny, nx))
        it = C.c_uint(0)
        rs = C.c_double(0)
        prm = params.c()
        ok = self.lib.orc_blocked_pressure_solve(
            C.byref(g), _ptr(u), _ptr(v), _ptr(w), C.byref(bf), C.byref(ff),
            C.byref(prm), _ptr(ou), _ptr(ov), _ptr(ow), _ptr(p),
            C.byref(it), C.byref(rs))
        del bk, fk
        return dict(u=ou, v=ov, w=ow, p=p, iters=it.value, resid=rs.value,
                    ok=bool(ok))

    def blocked_level(self, level: int, what: str, res0):
        """State of the last blocked solve at `level`: "markers" (int8,
        0 fluid / 1 air / 2 boundary), "A" (cells x 4 doubles) or "b"."""
        nx, ny, nz = (r >> level for r in res0)
        code = {"markers": 0, "A": 4, "b": 5}[what]
        if what == "markers":
            out = np.zeros((nz, ny, nx), np.int8)
        elif what == "A":
            out = np.zeros((nz, ny, nx, 4))
        else:
            out = np.zeros((nz, ny, nx))
        n = self.lib.orc_blocked_get_level(level, code, out.ctypes.data)
        if n < 0:
            raise ValueError(f"no level {level}")
        return out

    def level_count(self) -> int:
        return self.lib.orc_level_count()

    def level(self, level: int, what: str, res0):
        """Internal state of the last pressure solve at `level`.
        what: fluid | uw | vw | ww | A | b."""
        nx, ny, nz = (r >> level for r in res0)
        shapes = {"fluid": (nz, ny, nx), "uw": (nz, ny, nx + 1),
                  "vw": (nz, ny + 1, nx), "ww": (nz + 1, ny, nx),
                  "A": (nz, ny, nx, 4), "b": (nz, ny, nx)}
        code = {"fluid": 0, "uw": 1, "vw": 2, "ww": 3, "A": 4, "b": 5}[what]
        dt = np.float32 if code < 4 else np.float64
        out = np.zeros(shapes[what], dt)
        n = self.lib.orc_get_level(level, code, out.ctypes.data_as(C.c_void_p),
                                   out.nbytes)
        if n == -2:
            raise ValueError(f"level {level} {what} does not fit {shapes[what]}"
                             f" (res0 must be the finest resolution)")
        if n < 0:
            raise IndexError(f"level {level} unavailable")
        return out

    # -- linear-system pieces ----------------------------------------------
    def mgpcg_system(self, A_levels, b_levels, params: MgParams):
        res0 = (A_levels[0].shape[2], A_levels[0].shape[1],
                A_levels[0].shape[0])
        A = np.ascontiguousarray(np.concatenate([a.reshape(-1) for a in A_levels]))
        b = np.ascontiguousarray(np.concatenate([x.reshape(-1) for x in b_levels]))
        x0 = np.zeros(A_levels[0].shape[:3])
        r = (C.c_int * 3)(*res0)
        it = C.c_uint(0)
        rs = C.c_double(0)
        prm = params.c()
        ok = self.lib.orc_mgpcg_system(r, len(A_levels), _ptr(A), _ptr(b),
                                       C.byref(prm), _ptr(x0), C.byref(it),
                                       C.byref(rs))
        return dict(x=x0, iters=it.value, resid=rs.value, ok=bool(ok))

    def relax(self, A, b, x, sor, red_black, sweeps):
        x = np.ascontiguousarray(x, np.float64).copy()
        r = (C.c_int * 3)(A.shape[2], A.shape[1], A.shape[0])
        self.lib.orc_relax(r, _ptr(np.ascontiguousarray(A)),
                           _ptr(np.ascontiguousarray(b)), sor, int(red_black),
                           sweeps, _ptr(x))
        return x

    def mg_restrict(self, finer):
        nz, ny, nx = finer.shape
        c = np.zeros((nz // 2, ny // 2, nx // 2))
        r = (C.c_int * 3)(nx // 2, ny // 2, nz // 2)
        self.lib.orc_mg_restrict(r, _ptr(np.ascontiguousarray(finer)), _ptr(c))
        return c

    def mg_correct(self, coarser, finer):
        nz, ny, nx = coarser.shape
        f = np.ascontiguousarray(finer, np.float64).copy()
        r = (C.c_int * 3)(nx, ny, nz)
        self.lib.orc_mg_correct(r, _ptr(np.ascontiguousarray(coarser)), _ptr(f))
        return f

    def residual(self, A, x, b):
        r = np.zeros(b.shape)
        res = (C.c_int * 3)(b.shape[2], b.shape[1], b.shape[0])
        self.lib.orc_residual(res, _ptr(np.ascontiguousarray(A)),
                              _ptr(np.ascontiguousarray(x)),
                              _ptr(np.ascontiguousarray(b)), _ptr(r))
        return r

    def dot(self, a, b) -> float:
        a = np.ascontiguousarray(a, np.float64).reshape(-1)
        b = np.ascontiguousarray(b, np.float64).reshape(-1)
        return self.lib.orc_dot(a.size, _ptr(a), _ptr(b))

    # -- particle transfers --------------------------------------------------
    def p2g(self, res, spacing, origin, pos, vel):
        g = OrcGrid()
        g.res[:] = tuple(res)
        g.spacing[:] = tuple(spacing)
        g.origin[:] = tuple(origin)
        nx, ny, nz = res
        shp = [(nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx)]
        grids = [np.zeros(s) for s in shp]
        marks = [np.zeros(s, np.int8) for s in shp]
        snaps = [np.zeros(s, np.float32) for s in shp]
        pos = np.ascontiguousarray(pos, np.float64)
        vel = np.ascontiguousarray(vel, np.float64)
        self.lib.orc_p2g(C.byref(g), pos.shape[0], _ptr(pos), _ptr(vel),
                         *[_ptr(a) for a in grids], *[_ptr(m, _cp) for m in marks],
                         *[_ptr(s, _fp) for s in snaps])
        return grids, marks, snaps

    def g2p_flip(self, res, spacing, origin, pos, vel, grids, snaps,
                 pic_blend=0.0):
        g = OrcGrid()
        g.res[:] = tuple(res)
        g.spacing[:] = tuple(spacing)
        g.origin[:] = tuple(origin)
        pos = np.ascontiguousarray(pos, np.float64)
        vel = np.ascontiguousarray(vel, np.float64).copy()
        grids = [np.ascontiguousarray(a, np.float64) for a in grids]
        snaps = [np.ascontiguousarray(s, np.float32).copy() for s in snaps]
        self.lib.orc_g2p_flip(C.byref(g), pos.shape[0], _ptr(pos), _ptr(vel),
                              *[_ptr(a) for a in grids],
                              *[_ptr(s, _fp) for s in snaps], pic_blend)
        return vel, snaps

    def g2p_pic(self, res, spacing, origin, pos, vel, grids):
        g = OrcGrid()
        g.res[:] = tuple(res)
        g.spacing[:] = tuple(spacing)
        g.origin[:] = tuple(origin)
        pos = np.ascontiguousarray(pos, np.float64)
        vel = np.ascontiguousarray(vel, np.float64).copy()
        grids = [np.ascontiguousarray(a, np.float64) for a in grids]
        self.lib.orc_g2p_pic(C.byref(g), pos.shape[0], _ptr(pos), _ptr(vel),
                             *[_ptr(a) for a in grids])
        return vel


    # -- boundary conditions ------------------------------------------------
    @staticmethod
    def _grid(res, spacing, origin) -> OrcGrid:
        g = OrcGrid()
        g.res[:] = tuple(res)
        g.spacing[:] = tuple(spacing)
        g.origin[:] = tuple(origin)
        return g

    def constrain_velocity(self, res, spacing, origin, u, v, w, collider_sdf,
                           collider=None, closed=63, depth=5, blocked=False):
        """GridFractionalBoundaryConditionSolver3::constrainVelocity (or, with
        `blocked`, GridBlockedBoundaryConditionSolver3's) on copies of u/v/w.
        collider_sdf: constant or cell-centred grid (nz,ny,nx).
        collider: dict(lin, ang, centre, friction) or None."""
        g = self._grid(res, spacing, origin)
        data_origin = tuple(o + 0.5 * h for o, h in zip(origin, spacing))
        f, keep = field(collider_sdf, spacing, data_origin)
        out = [np.ascontiguousarray(a, np.float64).copy() for a in (u, v, w)]
        col = self._collider(collider) if collider is not None else None
        fn = (self.lib.orc_constrain_velocity_blocked if blocked
              else self.lib.orc_constrain_velocity)
        fn(
            C.byref(g), *[_ptr(a) for a in out], C.byref(f),
            C.byref(col) if col is not None else None, int(closed), int(depth))
        del keep
        return out

    def extrapolate(self, data, valid, iterations):
        """extrapolateToRegion on a copy of data (nz,ny,nx) from valid cells."""
        d = np.ascontiguousarray(data, np.float64).copy()
        m = np.ascontiguousarray(valid, np.int8)
        r = (C.c_int * 3)(d.shape[2], d.shape[1], d.shape[0])
        self.lib.orc_extrapolate(r, _ptr(d), _ptr(m, _cp), int(iterations))
        return d

    def apic_p2g(self, res, spacing, origin, pos, vel, affine):
        """ApicSolver3::transferFromParticlesToGrids; affine (n, 9).
        Returns (grids, markers)."""
        g = self._grid(res, spacing, origin)
        nx, ny, nz = res
        shp = [(nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx)]
        grids = [np.zeros(s) for s in shp]
        marks = [np.zeros(s, np.int8) for s in shp]
        pos = np.ascontiguousarray(pos, np.float64)
        vel = np.ascontiguousarray(vel, np.float64)
        aff = np.ascontiguousarray(affine, np.float64)
        self.lib.orc_apic_p2g(C.byref(g), pos.shape[0], _ptr(pos), _ptr(vel),
                              _ptr(aff), *[_ptr(a) for a in grids],
                              *[_ptr(m, _cp) for m in marks])
        return grids, marks

    def apic_g2p(self, res, spacing, origin, pos, grids):
        """ApicSolver3::transferFromGridsToParticles; returns (vel, affine
        (n, 9))."""
        g = self._grid(res, spacing, origin)
        pos = np.ascontiguousarray(pos, np.float64)
        vel = np.zeros_like(pos)
        aff = np.zeros((pos.shape[0], 9))
        grids = [np.ascontiguousarray(a, np.float64) for a in grids]
        self.lib.orc_apic_g2p(C.byref(g), pos.shape[0], _ptr(pos), _ptr(vel),
                              _ptr(aff), *[_ptr(a) for a in grids])
        return vel, aff

    @staticmethod
    def _collider(c):
        col = OrcCollider()
        col.lin[:] = tuple(c.get("lin", (0, 0, 0)))
        col.ang[:] = tuple(c.get("ang", (0, 0, 0)))
        col.centre[:] = tuple(c.get("centre", (0, 0, 0)))
        col.friction = float(c.get("friction", 0.0))
        return col

    def quaternion_matrices(self, q):
        """Reference harness only: Transform3's orientation matrix and its
        inverse for quaternion q = (w, x, y, z), row-major."""
        o, i = np.zeros(9), np.zeros(9)
        self.lib.orc_quaternion_matrices(
            _ptr(np.ascontiguousarray(q, np.float64)), _ptr(o), _ptr(i))
        return o, i

    def move_particles(self, res, spacing, origin, pos, vel, grids, dt,
                       max_cfl=5.0, closed=63, collider=None, sphere=None):
        """PicSolver3::moveParticles (+ sphere collisions) on copies.
        sphere: dict(center, radius, normal_flipped, orient, inv_orient,
        quat)."""
        g = self._grid(res, spacing, origin)
        pos = np.ascontiguousarray(pos, np.float64).copy()
        vel = np.ascontiguousarray(vel, np.float64).copy()
        grids = [np.ascontiguousarray(a, np.float64) for a in grids]
        col = sph = None
        if collider is not None and sphere is not None:
            col = self._collider(collider)
            sph = OrcSphere()
            sph.center[:] = tuple(sphere.get("center", (0, 0, 0)))
            sph.radius = float(sphere["radius"])
            sph.normal_flipped = int(sphere.get("normal_flipped", 0))
            sph.orient[:] = tuple(sphere.get("orient", np.eye(3).ravel()))
            sph.inv_orient[:] = tuple(sphere.get("inv_orient", np.eye(3).ravel()))
            sph.quat[:] = tuple(sphere.get("quat", (1, 0, 0, 0)))
        self.lib.orc_move_particles(
            C.byref(g), pos.shape[0], _ptr(pos), _ptr(vel),
            *[_ptr(a) for a in grids], float(dt), float(max_cfl), int(closed),
            C.byref(col) if col is not None else None,
            C.byref(sph) if sph is not None else None)
        return pos, vel

    def build_particle_sdf(self, res, spacing, origin, pos, collider_sdf,
                           max_cfl=5.0):
        """PicSolver3::buildSignedDistanceField (+ extrapolation into the
        collider); returns the cell-centred SDF (nz,ny,nx)."""
        g = self._grid(res, spacing, origin)
        data_origin = tuple(o + 0.5 * h for o, h in zip(origin, spacing))
        f, keep = field(collider_sdf, spacing, data_origin)
        pos = np.ascontiguousarray(pos, np.float64)
        out = np.zeros((res[2], res[1], res[0]))
        self.lib.orc_build_particle_sdf(C.byref(g), pos.shape[0], _ptr(pos),
                                        C.byref(f), float(max_cfl), _ptr(out))
        del keep
        return out

    def flip_run(self, res, spacing, origin, pos, vel, frames, fps=60.0,
                 max_cfl=5.0, closed=63, gravity=(0.0, -9.8, 0.0), flip=True,
                 params: MgParams | None = None):
        """Reference harness only: FlipSolver3 / PicSolver3 for `frames`
        frames; returns the particles' (positions, velocities)."""
        g = self._grid(res, spacing, origin)
        pos = np.ascontiguousarray(pos, np.float64).copy()
        vel = np.ascontiguousarray(vel, np.float64).copy()
        prm = (params or MgParams()).c()
        gr = np.ascontiguousarray(gravity, np.float64)
        self.lib.orc_flip_run(C.byref(g), pos.shape[0], _ptr(pos), _ptr(vel),
                              int(frames), float(fps), float(max_cfl),
                              int(closed), _ptr(gr), int(flip),
                              C.byref(prm))
        return pos, vel

    def flip_run_sphere(self, res, spacing, origin, pos, vel, frames, centre,
                        radius, friction=0.0, fps=60.0, max_cfl=5.0,
                        closed=63, gravity=(0.0, -9.8, 0.0), flip=True,
                        params: MgParams | None = None):
        """Reference harness only: flip_run with a static sphere collider
        (radius `radius` at `centre`, friction coefficient `friction`)."""
        g = self._grid(res, spacing, origin)
        pos = np.ascontiguousarray(pos, np.float64).copy()
        vel = np.ascontiguousarray(vel, np.float64).copy()
        prm = (params or MgParams()).c()
        gr = np.ascontiguousarray(gravity, np.float64)
        cc = np.ascontiguousarray(centre, np.float64)
        self.lib.orc_flip_run_sphere(C.byref(g), pos.shape[0], _ptr(pos),
                                     _ptr(vel), int(frames), float(fps),
                                     float(max_cfl), int(closed), _ptr(gr),
                                     int(flip), C.byref(prm), _ptr(cc),
                                     float(radius), float(friction))
        return pos, vel

    def flip_run_record(self, res, spacing, origin, pos, vel, frames,
                        record_frames, fps=60.0, max_cfl=5.0, closed=63,
                        gravity=(0.0, -9.8, 0.0), flip=True,
                        params: MgParams | None = None):
        """flip_run that also returns the pressure solver's pressure() after
        each frame count in `record_frames` (ascending, 1..frames):
        (positions, velocities, pressures (len(record_frames), nz, ny,
        nx))."""
        g = self._grid(res, spacing, origin)
        pos = np.ascontiguousarray(pos, np.float64).copy()
        vel = np.ascontiguousarray(vel, np.float64).copy()
        prm = (params or MgParams()).c()
        gr = np.ascontiguousarray(gravity, np.float64)
        rec = (C.c_int * len(record_frames))(*record_frames)
        nx, ny, nz = res
        p = np.zeros((len(record_frames), nz, ny, nx))
        self.lib.orc_flip_run_record(C.byref(g), pos.shape[0], _ptr(pos),
                                     _ptr(vel), int(frames), float(fps),
                                     float(max_cfl), int(closed), _ptr(gr),
                                     int(flip), C.byref(prm),
                                     len(record_frames), rec, _ptr(p))
        return pos, vel, p

    def sphere_collider_sdf(self, res, spacing, origin, centre, radius):
        """Reference harness only: the collider SDF the reference builds for
        a sphere collider on this grid (cell-centred, (nz,ny,nx))."""
        g = self._grid(res, spacing, origin)
        out = np.zeros((res[2], res[1], res[0]))
        c = np.ascontiguousarray(centre, np.float64)
        self.lib.orc_sphere_collider_sdf(C.byref(g), _ptr(c), float(radius),
                                         _ptr(out))
        return out


_cache: dict = {}


def divergence_at_cell_center(u, v, w, spacing) -> np.ndarray:
    """FaceCenteredGrid3::divergenceAtCellCenter at every cell
    (src/jet/face_centered_grid3.cpp:137-151): (u(i+1)-u(i))/h.x +
    (v(j+1)-v(j))/h.y + (w(k+1)-w(k))/h.z, summed in that order. u, v, w are
    the (nz,ny,nx+1), (nz,ny+1,nx), (nz+1,ny,nx) face arrays; returns
    (nz,ny,nx)."""
    hx, hy, hz = spacing
    return ((u[:, :, 1:] - u[:, :, :-1]) / hx +
            (v[:, 1:, :] - v[:, :-1, :]) / hy +
            (w[1:, :, :] - w[:-1, :, :]) / hz)


def port() -> Oracle:
    if "port" not in _cache:
        if not os.path.exists(PORT_SO):
            build_port()
        _cache["port"] = Oracle(PORT_SO)
    return _cache["port"]


def reference() -> Oracle | None:
    """The compiled reference harness, or None where it cannot exist."""
    if "ref" not in _cache:
        path = REF_SO if os.path.exists(REF_SO) else build_reference()
        _cache["ref"] = Oracle(path) if path and os.path.exists(path) else None
    return _cache["ref"]
