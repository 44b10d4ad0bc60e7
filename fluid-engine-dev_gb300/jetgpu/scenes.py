"""Seeded synthetic scenes for the pressure-projection workloads.

The reference has no data files; its workloads are generated from
``std::mt19937(seed)`` with ``std::uniform_real_distribution<double>``. This
module reproduces that stream bit for bit in numpy (MT19937 state seeded by
the standard's initialisation recurrence; each double drawn from two 32-bit
outputs as (lo + hi * 2^32) / 2^64, the C++ standard's generate_canonical for
53 bits), so host code here and a C++ harness over the reference produce the
same inputs.

Scenes (h = 1/n, origin 0, unit cube):
* ``dam_break_particles`` — liquid box seeded with 8 jittered particles per
  cell whose centre lies inside the box (loop order k, j, i, sample; draws
  x, y, z per particle): 64^3 box [0,.25]x[0,.75]x[0,1] seed 0 (393,216
  particles); 256^3 box [0,.3]x[0,.8]x[0,1] seed 2 (32.3M particles).
* ``sphere_union_scene`` — 16 liquid spheres (centres U[.2,.8]^3, radii
  U[.05,.2], seed 1), a solid sphere r=.15 at (.5,.3,.5) and i.i.d. U[-1,1]
  face velocities drawn after the spheres (u, then v, then w, i-fastest).
* ``flip_first_substep`` — the state that enters the pressure solve on the
  first sub-step of a FLIP dam break at rest: fluid SDF of the liquid box at
  cell centres, gravity applied for one 1/60 s step on every v face, domain
  walls closed (normal velocity 0), a static solid sphere.
"""
from __future__ import annotations

import numpy as np


def _mt_key(seed: int) -> np.ndarray:
    key = np.zeros(624, np.uint32)
    key[0] = seed & 0xFFFFFFFF
    prev = int(key[0])
    for i in range(1, 624):
        prev = (1812433253 * (prev ^ (prev >> 30)) + i) & 0xFFFFFFFF
        key[i] = prev
    return key


class Mt19937Uniform:
    """std::mt19937 + std::uniform_real_distribution<double> stream."""

    def __init__(self, seed: int):
        self._bg = np.random.MT19937()
        self._bg.state = {"bit_generator": "MT19937",
                          "state": {"key": _mt_key(seed), "pos": 624}}

    def canonical(self, count: int) -> np.ndarray:
        raw = self._bg.random_raw(2 * count).astype(np.uint64) & 0xFFFFFFFF
        lo = raw[0::2].astype(np.float64)
        hi = raw[1::2].astype(np.float64)
        u = (lo + hi * 4294967296.0) / 18446744073709551616.0
        return np.where(u >= 1.0, np.nextafter(1.0, 0.0), u)

    def uniform(self, a: float, b: float, count: int) -> np.ndarray:
        return self.canonical(count) * (b - a) + a


def dam_break_particles(n: int, box_hi: tuple, seed: int, ppc: int = 8,
                        dtype=np.float64, chunk_cells: int = 1 << 20):
    """Particles jittered uniformly in every cell whose centre lies inside
    [0,box_hi]. Returns (positions (P,3), velocities (P,3) zeros)."""
    h = 1.0 / n
    cx = (np.arange(n) + 0.5) * h
    ni = int(np.count_nonzero(cx < box_hi[0]))
    nj = int(np.count_nonzero(cx < box_hi[1]))
    nk = int(np.count_nonzero(cx < box_hi[2]))
    P = nk * nj * ni * ppc
    pos = np.empty((P, 3), dtype)
    rng = Mt19937Uniform(seed)
    # Cell order k, j, i (i fastest), `ppc` particles per cell, x,y,z each.
    cells = nk * nj * ni
    done = 0
    for c0 in range(0, cells, chunk_cells):
        c1 = min(cells, c0 + chunk_cells)
        cnt = (c1 - c0) * ppc
        u = rng.canonical(3 * cnt).reshape(cnt, 3)
        cid = np.repeat(np.arange(c0, c1), ppc)
        i = cid % ni
        j = (cid // ni) % nj
        k = cid // (ni * nj)
        pos[done:done + cnt, 0] = (i + u[:, 0]) * h
        pos[done:done + cnt, 1] = (j + u[:, 1]) * h
        pos[done:done + cnt, 2] = (k + u[:, 2]) * h
        done += cnt
    return pos, np.zeros_like(pos)


def cell_centres(n: int):
    c = (np.arange(n) + 0.5) / n
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    return X, Y, Z


def sphere_union_scene(n: int = 128, seed: int = 1, spheres: int = 16):
    """Returns dict(u, v, w, fluid_sdf, boundary_sdf) (float64 arrays)."""
    rng = Mt19937Uniform(seed)
    cs, rs = [], []
    for _ in range(spheres):
        c = rng.uniform(0.2, 0.8, 3)
        r = rng.uniform(0.05, 0.2, 1)[0]
        cs.append(c)
        rs.append(r)
    X, Y, Z = cell_centres(n)
    fluid = np.full((n, n, n), np.inf)
    for c, r in zip(cs, rs):
        d = np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) - r
        np.minimum(fluid, d, out=fluid)
    walls = np.minimum.reduce([X, 1 - X, Y, 1 - Y, Z, 1 - Z])
    ball = np.sqrt((X - 0.5) ** 2 + (Y - 0.3) ** 2 + (Z - 0.5) ** 2) - 0.15
    solid = np.minimum(walls, ball)
    u = rng.uniform(-1.0, 1.0, (n + 1) * n * n).reshape(n, n, n + 1)
    v = rng.uniform(-1.0, 1.0, n * (n + 1) * n).reshape(n, n + 1, n)
    w = rng.uniform(-1.0, 1.0, n * n * (n + 1)).reshape(n + 1, n, n)
    return dict(u=u, v=v, w=w, fluid_sdf=fluid, boundary_sdf=solid,
                spheres=(np.array(cs), np.array(rs)))


def box_sdf(X, Y, Z, hi):
    """Signed distance to the liquid box [-inf,hi] (the domain walls are not
    liquid surfaces): negative inside."""
    dx, dy, dz = X - hi[0], Y - hi[1], Z - hi[2]
    outside = np.sqrt(np.maximum(dx, 0) ** 2 + np.maximum(dy, 0) ** 2 +
                      np.maximum(dz, 0) ** 2)
    inside = np.minimum(np.maximum(np.maximum(dx, dy), dz), 0.0)
    return outside + inside


def flip_first_substep(n: int = 256, box_hi=(0.3, 0.8, 1.0),
                       sphere=((0.6, 0.2, 0.5), 0.15), gravity=-9.8,
                       dt=1.0 / 60.0):
    """Pressure-solve input of the first sub-step of a FLIP dam break at rest
    (velocities zero before gravity): dict(u, v, w, fluid_sdf,
    boundary_sdf)."""
    X, Y, Z = cell_centres(n)
    fluid = box_sdf(X, Y, Z, box_hi)
    if box_hi[2] >= 1.0:
        # The box reaches the far wall: its surface there is not a liquid
        # surface either.
        fluid = box_sdf(X, Y, Z, (box_hi[0], box_hi[1], np.inf))
    c, r = sphere
    solid = np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) - r
    u = np.zeros((n, n, n + 1))
    v = np.full((n, n + 1, n), dt * gravity)
    w = np.zeros((n + 1, n, n))
    v[:, 0, :] = 0.0
    v[:, n, :] = 0.0
    return dict(u=u, v=v, w=w, fluid_sdf=fluid, boundary_sdf=solid)
