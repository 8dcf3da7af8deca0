"""Pins of the three-dimensional oracle (DIM3), which the reference's own tests do not
cover (its gtest cases are two-dimensional).

* n0 and lambda against an independent numpy evaluation of Environment.hpp:166-215;
* Detail::InvertMatrix<3> against numpy's inverse on symmetric and general matrices
  (the cofactor formula places each minor at its own index, Computer.hpp:396-418,
  which is the inverse for the symmetric matrices GC builds), and the identity branch;
* a scene one lattice layer thick in y: with dy = 0 the 27-cell search visits the
  populated cells in the 2D order, so its neighbour lists and densities must equal the
  2D oracle's on the same x-z particles bit for bit.
"""
import numpy as np
import pytest

from openmps_gb300 import _abi as abi
from openmps_gb300 import scenes


def _numpy_n0(re_by, l0):
    rng = int(np.ceil(re_by))
    n0 = lam = 0.0
    re = re_by * l0
    for i in range(-rng, rng):
        for j in range(-rng, rng):
            for k in range(-rng, rng):
                if i == j == k == 0:
                    continue
                r = np.sqrt(((0.0 + (i * l0) ** 2) + (j * l0) ** 2) + (k * l0) ** 2)
                if r < re:
                    w = re / r - 1
                    n0 += w
                    lam += r * r * w
    return n0, lam / n0


@pytest.mark.parametrize("re_by", [2.1, 2.4, 3.0])
def test_n0_lambda(oracle_lib, re_by):
    from oracle.oracle import Oracle3

    s = scenes.tank3d(0.01, (2, 2, 2), (4, 4, 4))
    o = Oracle3(s.params(re_by_l0=re_by))
    env = o.environment()
    n0, lam = _numpy_n0(re_by, 0.01)
    assert env.n0 == pytest.approx(n0, rel=1e-14)
    assert env.lambda_ == pytest.approx(lam, rel=1e-14)
    assert env.dim == 3 and env.grid_max_per_cell == (int(np.ceil(re_by * 1.2)) + 1) ** 3


def test_invert3(oracle_lib):
    from oracle.oracle import gc_invert3

    rng = np.random.default_rng(1)
    for _ in range(20):
        a = rng.normal(size=(3, 3))
        spd = a @ a.T + 0.5 * np.eye(3)
        np.testing.assert_allclose(gc_invert3(spd, 1.0).reshape(3, 3), np.linalg.inv(spd), rtol=1e-10, atol=1e-12)
    # diagonal and the zero-determinant branch
    np.testing.assert_allclose(gc_invert3(np.diag([1.0, 2.0, 4.0]), 1.0), np.diag([1.0, 0.5, 0.25]).ravel())
    np.testing.assert_array_equal(gc_invert3(np.zeros(9), 0.5), np.diag([0.5, 0.5, 0.5]).ravel())
    np.testing.assert_array_equal(gc_invert3(np.diag([1.0, 0.0, 3.0]), 2.0), np.diag([2.0, 2.0, 2.0]).ravel())


def single_layer_pair(l0=0.01):
    """The 2D dam break at l0 and the same particles as a 3D scene one layer thick."""
    s2 = scenes.tank(l0, 10, 16, 30, 24, wall_layers=1, dummy_layers=2, jitter=0.1, seed=3)
    n = s2.count
    s3 = scenes.Scene3(name="layer", type=s2.type.copy(), x=s2.x.copy(), y=np.zeros(n), z=s2.z.copy(),
                       u=np.zeros(n), v=np.zeros(n), w=np.zeros(n), p=np.zeros(n), n=np.zeros(n), l0=l0,
                       bounds=(s2.min_x, -l0, s2.min_z, s2.max_x, l0, s2.max_z))
    phys = dict(scenes.PLAIN_PHYSICS, re_lap_by_l0=0.0, eps=1e-10, max_dt=5e-4)
    s2.meta["params"] = dict(phys)
    s3.meta["params"] = dict(phys)
    return s2, s3


def test_single_layer_equals_2d(oracle_lib):
    from oracle.oracle import Oracle, Oracle3

    s2, s3 = single_layer_pair()
    o2 = Oracle(s2.params())
    o2.add_scene(s2)
    o3 = Oracle3(s3.params())
    o3.add_scene(s3)
    for o in (o2, o3):
        o.begin_step(5e-4)
        o.stage("search_neighbor")
        o.stage("density")
    c2, l2 = o2.neighbors()
    c3, l3 = o3.neighbors()
    np.testing.assert_array_equal(c3, c2)
    np.testing.assert_array_equal(l3, l2)
    np.testing.assert_array_equal(o3.particles()["n"], o2.particles()["n"])


def packed_cluster(l0=0.01, re_by=2.1):
    """27 particles in each of the 27 cells around a particle at a cell centre, all within
    NeighborLength of it: no cell holds more than maxPerCell (64) particles, but the
    centre's row needs 728 entries against the reference's 9 maxPerCell = 576."""
    nl = re_by * l0 * 1.2
    c = np.array([10.5, 10.5, 10.5]) * nl  # a cell centre with the domain origin at 0
    pts = []
    for d in np.ndindex(3, 3, 3):
        d = np.array(d) - 1
        for k in np.ndindex(3, 3, 3):
            k = np.array(k)
            off = np.where(d != 0, d * (0.52 + 0.02 * k), (k - 1) * 0.02)
            pts.append(c + nl * off)
    pts = np.array(pts)
    n = len(pts)
    s = scenes.Scene3(name="packed", type=np.zeros(n, dtype=np.int32), x=pts[:, 0].copy(), y=pts[:, 1].copy(),
                      z=pts[:, 2].copy(), u=np.zeros(n), v=np.zeros(n), w=np.zeros(n), p=np.zeros(n),
                      n=np.zeros(n), l0=l0, bounds=(0.0, 0.0, 0.0, 21 * nl, 21 * nl, 21 * nl))
    s.meta["params"] = dict(scenes.PLAIN_PHYSICS, re_by_l0=re_by, re_lap_by_l0=0.0, eps=1e-10, max_dt=5e-4)
    return s


def test_neighbor_row_overflow(oracle_lib):
    from oracle.oracle import Oracle3, OracleError

    s = packed_cluster()
    o = Oracle3(s.params())
    o.add_scene(s)
    o.begin_step(5e-4)
    with pytest.raises(OracleError) as e:
        o.stage("search_neighbor")
    assert e.value.code == abi.MPS_ERR_DEVICE_CHECK


def test_single_layer_ppe_against_2d(oracle_lib):
    # with the SPP method set (no surface test) the one-layer scene's PPE has the 2D
    # pattern, and its off-diagonal HL coefficients (5 - D) r_e / n0 / r^3 differ from the
    # 2D ones only by the factor (2 / n0_3D) / (3 / n0_2D)
    from oracle.oracle import Oracle, Oracle3

    s2, s3 = single_layer_pair()
    for s in (s2, s3):
        s.meta["params"]["flags"] = abi.PRESET_REFERENCE
    o2 = Oracle(s2.params())
    o2.add_scene(s2)
    o3 = Oracle3(s3.params())
    o3.add_scene(s3)
    for o in (o2, o3):
        o.begin_step(5e-4)
        for name in ("search_neighbor", "density", "error_correction", "explicit", "density", "set_ppe"):
            o.stage(name)
    rp2, col2, val2, _, _ = o2.ppe()
    rp3, col3, val3, _, _ = o3.ppe()
    np.testing.assert_array_equal(rp3, rp2)
    np.testing.assert_array_equal(col3, col2)
    rows = np.repeat(np.arange(rp2.size - 1), np.diff(rp2))
    off = col2 != rows
    ratio = (2.0 / o3.environment().n0) / (3.0 / o2.environment().n0)
    np.testing.assert_allclose(val3[off], val2[off] * ratio, rtol=1e-14)
