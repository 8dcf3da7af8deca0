"""Seeded synthetic particle scenes (tank, dam break, hydrostatic column, lattices).

The layout follows the reference's scene generators: fluid particles on a square
lattice ``(i*l0, j*l0)`` (Benchmark/DamBreak/generate_koshizukaoka1996.py:69-74),
a floor and two side walls made of layers of wall and dummy particles around the
tank (:76-149), and the domain starting at the outermost layer (:155-159).
Here the walls have ``wall_layers`` wall layers and ``dummy_layers`` dummy layers
(3 + 2 by default) and the corners are filled the same way.

Random numbers come from SplitMix64 (Steele, Lea, Flood 2014) so that every scene
is reproducible from its seed on any machine.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import _abi as abi

_MASK = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n outputs of SplitMix64 started at ``seed`` (uint64)."""
    with np.errstate(over="ignore"):
        k = np.arange(1, n + 1, dtype=np.uint64)
        zz = (np.uint64(seed) + k * np.uint64(0x9E3779B97F4A7C15)) & _MASK
        zz = ((zz ^ (zz >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _MASK
        zz = ((zz ^ (zz >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _MASK
        return zz ^ (zz >> np.uint64(31))


def uniform01(seed: int, n: int) -> np.ndarray:
    """n doubles in [0, 1) from the top 53 bits of SplitMix64."""
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclasses.dataclass
class Scene:
    """A particle set plus the domain and physical constants it was built for."""

    name: str
    type: np.ndarray
    x: np.ndarray
    z: np.ndarray
    u: np.ndarray
    w: np.ndarray
    p: np.ndarray
    n: np.ndarray
    l0: float
    min_x: float
    min_z: float
    max_x: float
    max_z: float
    meta: dict = dataclasses.field(default_factory=dict)

    @property
    def count(self) -> int:
        return int(self.type.shape[0])

    def counts(self) -> dict:
        return {
            "fluid": int(np.sum(self.type == abi.TYPE_FLUID)),
            "wall": int(np.sum(self.type == abi.TYPE_WALL)),
            "dummy": int(np.sum(self.type == abi.TYPE_DUMMY)),
        }

    def params(self, **kw) -> abi.MpsParams:
        base = dict(l0=self.l0, min_x=self.min_x, min_z=self.min_z, max_x=self.max_x,
                    max_z=self.max_z)
        base.update(self.meta.get("params", {}))
        base.update(kw)
        return abi.make_params(**base)

    def arrays(self):
        return (self.type, self.x, self.z, self.u, self.w, self.p, self.n)

    def copy(self) -> "Scene":
        return dataclasses.replace(self, type=self.type.copy(), x=self.x.copy(), z=self.z.copy(),
                                   u=self.u.copy(), w=self.w.copy(), p=self.p.copy(),
                                   n=self.n.copy(), meta=dict(self.meta))


def _make(name, t, x, z, l0, bounds, meta=None) -> Scene:
    n = len(t)
    return Scene(name=name, type=np.ascontiguousarray(t, dtype=np.int32),
                 x=np.ascontiguousarray(x, dtype=np.float64),
                 z=np.ascontiguousarray(z, dtype=np.float64),
                 u=np.zeros(n), w=np.zeros(n), p=np.zeros(n), n=np.zeros(n), l0=l0,
                 min_x=bounds[0], min_z=bounds[1], max_x=bounds[2], max_z=bounds[3],
                 meta=meta or {})


def tank(l0: float, water_cols: int, water_rows: int, tank_cols: int, tank_rows: int,
         wall_layers: int = 3, dummy_layers: int = 2, jitter: float = 0.0, seed: int = 0,
         name: str = "tank") -> Scene:
    """Water block in the left corner of an open tank.

    Fluid: ``water_cols x water_rows`` lattice points ``(i*l0, j*l0)``, column by
    column.  Boundary: every lattice point within ``wall_layers + dummy_layers``
    layers outside the tank interior ``[0, tank_cols) x [0, tank_rows)`` (floor,
    both side walls and the two lower corners); its layer is the Chebyshev distance
    to the interior, layers ``1..wall_layers`` are wall, the rest dummy.
    ``jitter`` (in units of l0) displaces fluid particles by seeded U(-jitter, jitter).
    """
    layers = wall_layers + dummy_layers
    ii, jj = np.meshgrid(np.arange(water_cols), np.arange(water_rows), indexing="ij")
    fx = ii.ravel() * l0
    fz = jj.ravel() * l0
    if jitter:
        rnd = uniform01(seed, 2 * fx.size)
        fx = fx + (2.0 * rnd[0::2] - 1.0) * jitter * l0
        fz = fz + (2.0 * rnd[1::2] - 1.0) * jitter * l0
    bi, bj = np.meshgrid(np.arange(-layers, tank_cols + layers), np.arange(-layers, tank_rows),
                         indexing="ij")
    bi = bi.ravel()
    bj = bj.ravel()
    dist_x = np.where(bi < 0, -bi, np.where(bi >= tank_cols, bi - tank_cols + 1, 0))
    dist_z = np.where(bj < 0, -bj, 0)
    layer = np.maximum(dist_x, dist_z)
    keep = layer > 0
    bi, bj, layer = bi[keep], bj[keep], layer[keep]
    btype = np.where(layer <= wall_layers, abi.TYPE_WALL, abi.TYPE_DUMMY)
    t = np.concatenate([np.full(fx.size, abi.TYPE_FLUID), btype])
    x = np.concatenate([fx, bi * l0])
    z = np.concatenate([fz, bj * l0])
    bounds = (-layers * l0, -layers * l0, (tank_cols + layers - 1) * l0, tank_rows * l0)
    return _make(name, t, x, z, l0, bounds,
                 {"water_cols": water_cols, "water_rows": water_rows, "tank_cols": tank_cols,
                  "tank_rows": tank_rows, "wall_layers": wall_layers,
                  "dummy_layers": dummy_layers, "jitter": jitter, "seed": seed})


def dam_break(l0: float, water_w: float = 0.2, water_h: float = 0.4, tank_w: float = 0.8,
              tank_h: float = 0.6, **kw) -> Scene:
    """Dam break: a ``water_w x water_h`` column in a ``tank_w x tank_h`` tank."""
    r = lambda v: int(round(v / l0))
    s = tank(l0, r(water_w), r(water_h), r(tank_w), r(tank_h), name="dam_break", **kw)
    s.meta.update(water_w=water_w, water_h=water_h, tank_w=tank_w, tank_h=tank_h)
    return s


def hydrostatic(l0: float = 2.5e-3, width: float = 1.0, depth: float = 0.5,
                tank_h: float = 0.6, jitter: float = 1e-4, seed: int = 20261203) -> Scene:
    """Water at rest filling a tank ``width`` wide to ``depth`` (seeded lattice jitter)."""
    r = lambda v: int(round(v / l0))
    s = tank(l0, r(width), r(depth), r(width), r(tank_h), jitter=jitter, seed=seed,
             name="hydrostatic")
    s.meta.update(width=width, depth=depth)
    return s


def lattice(nx: int, nz: int, l0: float, bounds, ptype: int = abi.TYPE_FLUID, u_fn=None,
            p_fn=None) -> Scene:
    """``nx x nz`` particles at ``(i*l0, j*l0)``, row by row (z outer, x inner),
    as the reference's unit tests lay them out."""
    jj, ii = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    x = ii.ravel().astype(np.float64) * l0
    z = jj.ravel().astype(np.float64) * l0
    s = _make("lattice", np.full(x.size, ptype), x, z, l0, bounds)
    if u_fn is not None:
        s.u, s.w = (np.ascontiguousarray(a, dtype=np.float64) for a in u_fn(x, z))
    if p_fn is not None:
        s.p = np.ascontiguousarray(p_fn(x, z), dtype=np.float64)
    return s


# ------------------------------------------------------ three-dimensional scenes
@dataclasses.dataclass
class Scene3:
    """A three-dimensional particle set (DIM3): positions (x, y, z), velocities (u, v, w)."""

    name: str
    type: np.ndarray
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    u: np.ndarray
    v: np.ndarray
    w: np.ndarray
    p: np.ndarray
    n: np.ndarray
    l0: float
    bounds: tuple  # (min_x, min_y, min_z, max_x, max_y, max_z)
    meta: dict = dataclasses.field(default_factory=dict)

    @property
    def count(self) -> int:
        return int(self.type.shape[0])

    def params(self, **kw) -> abi.MpsParams:
        b = self.bounds
        base = dict(l0=self.l0, min_x=b[0], min_y=b[1], min_z=b[2], max_x=b[3], max_y=b[4], max_z=b[5],
                    dim=3)
        base.update(self.meta.get("params", {}))
        base.update(kw)
        return abi.make_params(**base)

    def arrays3(self):
        return (self.type, self.x, self.y, self.z, self.u, self.v, self.w, self.p, self.n)

    def copy(self) -> "Scene3":
        return dataclasses.replace(self, **{k: getattr(self, k).copy() for k in
                                            ("type", "x", "y", "z", "u", "v", "w", "p", "n")},
                                   meta=dict(self.meta))


def tank3d(l0: float, water: tuple, tank: tuple, wall_layers: int = 1, dummy_layers: int = 2,
           jitter: float = 0.0, seed: int = 0, name: str = "tank3d") -> Scene3:
    """Water block ``water = (nx, ny, nz)`` lattice points in the corner of an open box
    ``tank = (nx, ny, nz)``: fluid at ``(i l0, j l0, k l0)``; boundary particles at every
    lattice point within ``wall_layers + dummy_layers`` layers outside the interior (floor
    and four side walls), layer = Chebyshev distance, the first ``wall_layers`` wall and
    the rest dummy.  ``jitter`` (units of l0) moves the fluid by seeded U(-jitter, jitter)."""
    layers = wall_layers + dummy_layers
    wi, wj, wk = np.meshgrid(*(np.arange(m) for m in water), indexing="ij")
    fx, fy, fz = (a.ravel() * l0 for a in (wi, wj, wk))
    if jitter:
        rnd = uniform01(seed, 3 * fx.size)
        fx = fx + (2.0 * rnd[0::3] - 1.0) * jitter * l0
        fy = fy + (2.0 * rnd[1::3] - 1.0) * jitter * l0
        fz = fz + (2.0 * rnd[2::3] - 1.0) * jitter * l0
    tx, ty, tz = tank
    bi, bj, bk = (a.ravel() for a in np.meshgrid(np.arange(-layers, tx + layers), np.arange(-layers, ty + layers),
                                                 np.arange(-layers, tz), indexing="ij"))
    out = lambda a, m: np.where(a < 0, -a, np.where(a >= m, a - m + 1, 0))
    layer = np.maximum(np.maximum(out(bi, tx), out(bj, ty)), np.where(bk < 0, -bk, 0))
    keep = layer > 0
    bi, bj, bk, layer = bi[keep], bj[keep], bk[keep], layer[keep]
    btype = np.where(layer <= wall_layers, abi.TYPE_WALL, abi.TYPE_DUMMY)
    t = np.concatenate([np.full(fx.size, abi.TYPE_FLUID), btype]).astype(np.int32)
    x = np.concatenate([fx, bi * l0])
    y = np.concatenate([fy, bj * l0])
    z = np.concatenate([fz, bk * l0])
    n = t.size
    bounds = (-layers * l0, -layers * l0, -layers * l0, (tx + layers - 1) * l0, (ty + layers - 1) * l0, tz * l0)
    return Scene3(name=name, type=t, x=x, y=y, z=z, u=np.zeros(n), v=np.zeros(n), w=np.zeros(n), p=np.zeros(n),
                  n=np.zeros(n), l0=l0, bounds=bounds,
                  meta={"water": tuple(water), "tank": tuple(tank), "wall_layers": wall_layers,
                        "dummy_layers": dummy_layers, "jitter": jitter, "seed": seed})


def dam_break3d(l0: float, water=(0.2, 0.1, 0.4), tank=(0.8, 0.1, 0.6), **kw) -> Scene3:
    """3D dam break: a ``water`` (x, y, z in m) column in the corner of a ``tank`` box."""
    r = lambda v: int(round(v / l0))
    s = tank3d(l0, tuple(r(a) for a in water), tuple(r(a) for a in tank), name="dam_break3d", **kw)
    s.meta.update(water_m=tuple(water), tank_m=tuple(tank))
    return s


# ----------------------------------------------------------------- workloads
PLAIN_PHYSICS = dict(rho=1000.0, nu=1e-6, g=9.8, surface_ratio=0.97, re_by_l0=2.1,
                     re_lap_by_l0=4.0, courant=0.1, flags=abi.PRESET_PLAIN)
# The workloads run the reference's stock method set (HS, HL, ECS, DS, SPP) with one
# radius, r_e = 4.0 l0, as the reference has one R_e; the PPE keeps its ~45 nonzeros per
# row.  Plain MPS with the midpoint gradient and no collision model diverges on these
# scenes (a CG failure or a cell overflow near step 500 of the l0 = 0.01 dam break,
# within ~30 steps at l0 = 5e-4), and so does the stock set with r_e = 2.1 l0 for the
# density and 4.0 l0 for the Laplacian (a cell overflow at step 140 of the hydrostatic
# tank and 235 of the 320k dam break); the oracle and the GPU fail alike.  The stock set
# at one radius runs the 2000 hydrostatic steps, the 500 dam-break steps and the 1000
# batched steps, and settles to the hydrostatic pressure.
STOCK_PHYSICS = dict(PLAIN_PHYSICS, flags=abi.PRESET_REFERENCE, re_by_l0=4.0, re_lap_by_l0=0.0)


def config_c0(physics: dict | None = None) -> Scene:
    """2D dam break: 0.2 x 0.4 m column at l0 = 0.01 m (800 fluid) in a 0.8 x 0.6 m
    tank with 3 wall + 2 dummy layers; dt = 5e-4, 1000 steps, CG to 1e-10."""
    s = dam_break(0.01)
    s.meta["params"] = dict(physics or STOCK_PHYSICS, eps=1e-10, max_dt=5e-4)
    s.meta.update(dt=5e-4, steps=1000)
    return s


def config_c0_plain() -> Scene:
    """The l0 = 0.01 dam break with plain MPS (standard source and Laplacian, surface
    flag n/n0 < 0.97): the reference's non-default preset, used for parity checks."""
    return config_c0(PLAIN_PHYSICS)


def config_c1() -> Scene:
    """Hydrostatic tank 1.0 m x 0.5 m at l0 = 2.5e-3 (80,000 fluid), dt = 1e-4."""
    s = hydrostatic()
    s.meta["params"] = dict(STOCK_PHYSICS, eps=1e-8, max_dt=1e-4)
    s.meta.update(dt=1e-4, steps=2000)
    return s


def config_c2() -> Scene:
    """320k dam break: 0.2 x 0.4 m column at l0 = 5e-4 m (320,000 fluid); dt = 2.5e-5 s
    keeps the l0 = 0.01 case's Courant number (dt scaled with l0)."""
    s = dam_break(5e-4)
    dt = 2.5e-5
    s.meta["params"] = dict(STOCK_PHYSICS, eps=1e-8, max_dt=dt)
    s.meta.update(dt=dt, steps=500)
    return s


def batch_scene(k: int, seed: int = 20261203, l0: float = 5e-3) -> Scene:
    """Scene k of the batched workload: width U[0.1,0.3] m, height U[0.2,0.5] m."""
    rnd = uniform01(seed + 7919 * k, 2)
    ww = 0.1 + 0.2 * rnd[0]
    hh = 0.2 + 0.3 * rnd[1]
    s = dam_break(l0, water_w=round(ww / l0) * l0, water_h=round(hh / l0) * l0)
    s.name = "batch_%d" % k
    s.meta["params"] = dict(STOCK_PHYSICS, eps=1e-8, max_dt=5e-4)
    s.meta.update(dt=5e-4, steps=1000)
    return s
