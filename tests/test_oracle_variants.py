"""Analytic checks of the method variants on the oracle (CPU).

* GC (Computer.hpp:1457-1499): on an undisturbed lattice, sum_j W/r^2 dx dx^T over the
  neighbours of an interior particle is (n0 / D) I by symmetry, so C = (D / n0) I and
  the corrected gradient -dt n_i / (rho n0) sum (p_ij / r^2 W) C dx equals the plain one
  -dt / rho D / n0 sum (p_ij / r^2 W) dx scaled by n_i / n0 (in 2D and 3D);
* explicit pressure (Computer.hpp:1046-1067): p = c^2 (rho0 / n0 n - rho0) above rho0,
  restated in numpy on the oracle's densities.
"""
import numpy as np
import pytest

from openmps_gb300 import _abi as abi
from openmps_gb300 import scenes


def _lattice2(gc):
    s = scenes.lattice(21, 21, 0.01, (-0.05, -0.05, 0.25, 0.25))
    rng = np.random.default_rng(2)
    s.p = rng.uniform(100.0, 200.0, s.count)
    s.meta["params"] = dict(scenes.PLAIN_PHYSICS, re_by_l0=2.4, re_lap_by_l0=0.0, eps=1e-10, max_dt=1e-4,
                            flags=abi.FLAG_GC if gc else 0)
    return s


def _gradient_du2(gc):
    from oracle.oracle import Oracle

    s = _lattice2(gc)
    o = Oracle(s.params())
    o.add_scene(s)
    o.begin_step(1e-4)
    o.stage("search_neighbor")
    o.stage("density")
    before = o.particles()
    o.stage("pressure_gradient")
    after = o.particles()
    return s, before, after["u"] - before["u"], after["w"] - before["w"]


def test_gc_equals_plain_gradient_on_lattice_2d(oracle_lib):
    s, P, du_gc, dw_gc = _gradient_du2(True)
    _, _, du, dw = _gradient_du2(False)
    i, k = np.meshgrid(np.arange(21), np.arange(21), indexing="xy")
    inner = ((i.ravel() >= 4) & (i.ravel() <= 16) & (k.ravel() >= 4) & (k.ravel() <= 16))
    from oracle.oracle import Oracle
    n0 = Oracle(s.params()).environment().n0
    scale = P["n"][inner] / n0
    assert np.allclose(scale, 1.0, atol=1e-12)
    np.testing.assert_allclose(du_gc[inner], du[inner] * scale, rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(dw_gc[inner], dw[inner] * scale, rtol=1e-9, atol=1e-15)
    assert np.max(np.abs(du[inner])) > 0


def test_gc_equals_plain_gradient_on_lattice_3d(oracle_lib):
    from oracle.oracle import Oracle3

    def run(gc):
        s = scenes.tank3d(0.01, (12, 12, 12), (12, 12, 12), wall_layers=0, dummy_layers=0)
        s.bounds = (-0.05, -0.05, -0.05, 0.17, 0.17, 0.17)
        s.p = np.random.default_rng(3).uniform(100.0, 200.0, s.count)
        s.meta["params"] = dict(scenes.PLAIN_PHYSICS, re_by_l0=2.1, re_lap_by_l0=0.0, eps=1e-10, max_dt=1e-4,
                                flags=abi.FLAG_GC if gc else 0)
        o = Oracle3(s.params())
        o.add_scene(s)
        o.begin_step(1e-4)
        o.stage("search_neighbor")
        o.stage("density")
        before = o.particles()
        o.stage("pressure_gradient")
        after = o.particles()
        return o, before, np.stack([after[k] - before[k] for k in ("u", "v", "w")], axis=1)

    o, P, d_gc = run(True)
    _, _, d = run(False)
    idx = np.indices((12, 12, 12)).reshape(3, -1).T
    inner = np.all((idx >= 3) & (idx <= 8), axis=1)
    scale = P["n"][inner] / o.environment().n0
    assert np.allclose(scale, 1.0, atol=1e-12)
    np.testing.assert_allclose(d_gc[inner], d[inner] * scale[:, None], rtol=1e-9, atol=1e-15)


def test_explicit_pressure_formula(oracle_lib):
    from oracle.oracle import Oracle

    c = 25.0
    s = scenes.config_c0()
    s.meta["params"] = dict(s.meta["params"], flags=abi.PRESET_REFERENCE | abi.FLAG_PRESSURE_EXPLICIT,
                            sound_speed=c)
    o = Oracle(s.params())
    o.add_scene(s)
    env = o.environment()
    assert env.max_dt == min(5e-4, 0.1 * 0.01 / c)
    for _ in range(3):
        o.forward_time(env.max_dt)
    P = o.particles()
    rho0 = s.meta["params"]["rho"]
    rho = rho0 / env.n0 * P["n"]
    np.testing.assert_array_equal(P["p"], np.where(rho <= rho0, 0.0, c * c * (rho - rho0)))
