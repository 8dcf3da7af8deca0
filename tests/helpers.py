"""Shared helpers of the parity tests: paired GPU / oracle scenes and comparisons."""
from __future__ import annotations

import numpy as np

from openmps_gb300 import _abi as abi
from openmps_gb300 import scenes

FIELDS = ("x", "z", "u", "w", "p", "n")


def make_pair(scene, params, openmp=False):
    """The same particles in a GPU Computer and in the CPU oracle."""
    from openmps_gb300.computer import Computer
    from oracle.oracle import Oracle

    gpu = Computer(params)
    gpu.add_scene(scene)
    cpu = Oracle(params, openmp=openmp)
    cpu.add_scene(scene)
    return gpu, cpu


def copy_state(src_cpu, dst_gpu):
    """Copies particles and auxiliary arrays from the oracle into the GPU handle."""
    P = src_cpu.particles()
    dst_gpu.set_particles(P["type"], *[P[k] for k in FIELDS])
    A = src_cpu.aux()
    dst_gpu.set_aux(A["n_without_spp"], A["ecs"], A["ox"], A["oz"])


def assert_same_particles(gpu, cpu, fields=FIELDS, what=""):
    G = gpu.particles()
    C = cpu.particles()
    np.testing.assert_array_equal(G["type"], C["type"], err_msg="type " + what)
    for k in fields:
        np.testing.assert_array_equal(G[k], C[k], err_msg="%s %s" % (k, what))


def assert_same_neighbors(gpu, cpu, what=""):
    gc, gl = gpu.neighbors()
    cc, cl = cpu.neighbors()
    alive = cpu.particles()["type"] != abi.TYPE_DISABLED
    np.testing.assert_array_equal(gc[alive], cc[alive], err_msg="neighbour counts " + what)
    assert gl.size == cl.size, what
    np.testing.assert_array_equal(gl, cl, err_msg="neighbour lists " + what)


def assert_same_ppe(gpu, cpu, what=""):
    grp, gcol, gval, gb, gx = gpu.ppe()
    crp, ccol, cval, cb, cx = cpu.ppe()
    np.testing.assert_array_equal(grp, crp, err_msg="row_ptr " + what)
    np.testing.assert_array_equal(gcol, ccol, err_msg="columns " + what)
    np.testing.assert_array_equal(gval, cval, err_msg="values " + what)
    np.testing.assert_array_equal(gb, cb, err_msg="rhs " + what)
    np.testing.assert_array_equal(gx, cx, err_msg="initial guess " + what)


def rel_err(a, b, scale=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = np.max(np.abs(b)) if scale is None else scale
    if s == 0:
        return float(np.max(np.abs(a - b)))
    return float(np.max(np.abs(a - b)) / s)


# --------------------------------------------------------- small test scenes
def reference_tank(l0=0.008):
    """Stock-preset tank in the Sample.xml spirit (r_e = 2.4 l0, 1 wall + 3 dummy layers)."""
    s = scenes.dam_break(l0, water_w=19 * l0, water_h=37 * l0, tank_w=73 * l0, tank_h=45 * l0,
                         wall_layers=1, dummy_layers=3)
    s.meta["params"] = dict(re_by_l0=2.4, flags=abi.PRESET_REFERENCE, eps=1e-10, max_dt=5e-4,
                            rho=998.2, nu=1.004e-6, surface_ratio=0.97)
    s.meta["dt"] = 5e-4
    return s


def plain_tank(l0=0.01, ds=False):
    s = scenes.config_c0_plain() if l0 == 0.01 else scenes.dam_break(l0)
    s.meta.setdefault("params", dict(scenes.PLAIN_PHYSICS, eps=1e-10, max_dt=5e-4))
    if ds:
        s.meta["params"]["flags"] = abi.FLAG_DS
    s.meta["dt"] = 5e-4
    return s


def stock_tank():
    """The l0 = 0.01 dam break with the stock method set at one radius (the workload physics)."""
    return scenes.config_c0()


def stock_two_radii_tank():
    """The same dam break with the stock method set and two radii: r_e = 2.1 l0 for the
    density and gradient, 4.0 l0 for the Laplacian (the two-radius extension)."""
    return scenes.config_c0(dict(scenes.STOCK_PHYSICS, re_by_l0=2.1, re_lap_by_l0=4.0))


def jittered_tank(l0=0.01, jitter=0.05, seed=7, preset=abi.PRESET_PLAIN):
    """Hydrostatic-style tank with seeded lattice jitter (breaks lattice ties)."""
    s = scenes.tank(l0, 30, 20, 30, 30, jitter=jitter, seed=seed)
    params = dict(scenes.PLAIN_PHYSICS, eps=1e-10, max_dt=5e-4)
    params["flags"] = preset
    if preset == abi.PRESET_REFERENCE:
        params.update(re_by_l0=2.4, re_lap_by_l0=0.0)
    s.meta["params"] = params
    s.meta["dt"] = 5e-4
    return s


def far_tank(offset=(3071.37, -2047.13)):
    """The stock two-radius tank moved far from the origin: FP32 copies of its coordinates
    lose about 1e-4 m, so the FP32 range screen leaves many pairs to the FP64 test."""
    s = stock_tank()
    ox, oz = offset
    s.x = s.x + ox
    s.z = s.z + oz
    s.min_x += ox
    s.max_x += ox
    s.min_z += oz
    s.max_z += oz
    return s


def threshold_rings(l0=0.01, seed=5):
    """A fluid particle with rings of neighbours at distances within a few ulps to 1e-5
    (relative) of r_e, the Laplacian radius and the neighbour length, on both sides:
    every range test of the step meets pairs that only the FP64 comparison decides."""
    base = stock_two_radii_tank()
    prm = dict(base.meta["params"])
    re = prm.get("re_by_l0", 2.1) * l0
    rl = prm.get("re_lap_by_l0", 4.0) * l0
    nl = max(re, rl) * (1 + 2 * prm.get("courant", 0.1))
    rng = np.random.default_rng(seed)
    deltas = [-1e-5, -1e-7, -1e-9, -1e-12, -4e-16, 0.0, 4e-16, 1e-12, 1e-9, 1e-7, 1e-5]
    xc, zc = 0.3719, 0.2903
    xs, zs = [xc], [zc]
    for radius in (re, rl, nl):
        k = len(deltas) * 3
        for a in range(k):
            th = 2 * np.pi * (a + 0.5 * rng.random()) / k
            d = radius * (1 + deltas[a % len(deltas)])
            xs.append(xc + d * np.cos(th))
            zs.append(zc + d * np.sin(th))
    n = len(xs)
    t = np.full(n, abi.TYPE_FLUID, dtype=np.int32)
    u = rng.normal(size=n) * 0.05
    w = rng.normal(size=n) * 0.05
    s = scenes.Scene(name="threshold_rings", type=t, x=np.array(xs), z=np.array(zs), u=u, w=w,
                     p=np.zeros(n), n=np.zeros(n), l0=l0, min_x=0.0, min_z=0.0, max_x=0.8,
                     max_z=0.6)
    s.meta["params"] = prm
    s.meta["dt"] = base.meta.get("dt", 5e-4)
    return s
