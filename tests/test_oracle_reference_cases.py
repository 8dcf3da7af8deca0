"""The reference's own unit-test cases, restated against the CPU oracle.

These pin the oracle to the reference: each case rebuilds the setup of a test in
src/OpenMps/test/ (lattice size, spacing, radius, analytic target, tolerance) and
runs it through the oracle's stage hooks, as the gtest fixtures call the private
stages of Computer through friend classes (src/OpenMps/Computer.hpp:437-460).
The reference's tests use the stock method set (MPS_HS, MPS_HL, MPS_ECS, MPS_DS,
MPS_SPP; src/OpenMps/defines.hpp), which is MPS_PRESET_REFERENCE here.
"""
import math

import numpy as np
import pytest

from openmps_gb300 import _abi as abi
from openmps_gb300 import scenes


def _oracle(params, scene=None):
    from oracle.oracle import Oracle

    o = Oracle(params)
    if scene is not None:
        o.add_scene(scene)
    return o


def _params(**kw):
    base = dict(max_dt=1.0 / 100, courant=0.1, g=9.8, rho=998.2, nu=1.004e-06, eps=1e-10,
                flags=abi.PRESET_REFERENCE)
    base.update(kw)
    return abi.make_params(**base)


# ------------------------------------------------- test_ComputerConstructor.cpp
def test_constructor_fields(oracle_lib):
    # test_ComputerConstructor.cpp:112-180: l0 = 1e-3, r_e = 2.4 l0, 7 x 9 lattice
    l0, re, courant, g = 0.001, 2.4, 0.1, 9.8
    prm = _params(l0=l0, re_by_l0=re, min_x=-0.004, min_z=-0.004, max_x=0.053, max_z=0.1)
    s = scenes.lattice(7, 9, l0, (-0.004, -0.004, 0.053, 0.1))
    o = _oracle(prm, s)
    env = o.environment()
    assert env.g == g and env.rho == 998.2 and env.nu == 1.004e-06
    assert env.l0 == l0 and env.re == re * l0
    assert (env.min_x, env.min_z, env.max_x, env.max_z) == (-0.004, -0.004, 0.053, 0.1)
    assert env.max_dt <= 1.0 / 100
    assert env.max_dt <= math.sqrt(2.0 * courant * l0 / g)
    assert env.max_dx >= courant * l0
    assert env.neighbor_length >= re * l0 * (1 + courant)
    P = o.particles()
    assert len(P["x"]) == 7 * 9
    assert np.all((P["x"] >= 0) & (P["x"] <= 6 * l0)) and np.all((P["z"] >= 0) & (P["z"] <= 8 * l0))


# ----------------------------------------------- test_ComputerNumberDensity.cpp
def _density_fixture():
    b = (-0.004, -0.004, 0.053, 0.1)
    prm = _params(l0=0.1, re_by_l0=2.1, min_x=b[0], min_z=b[1], max_x=b[2], max_z=b[3])
    return _oracle(prm, scenes.lattice(7, 7, 0.1, b))


def test_neighbor_symmetry_and_no_self(oracle_lib):
    # NeighborSymmetry :209-237, NeighborMyself :240-260
    o = _density_fixture()
    o.stage("search_neighbor")
    counts, lst = o.neighbors()
    rows = np.split(lst, np.cumsum(counts)[:-1])
    for i, row in enumerate(rows):
        assert i not in set(row.tolist())
        for j in row:
            assert i in set(rows[j].tolist())


def test_number_density_known_answer(oracle_lib):
    # NeighDensity :263-276: centre particle n = 6.539696962 (Koshizuka et al. 2014), 1e-5
    o = _density_fixture()
    o.stage("search_neighbor")
    o.stage("density")
    centre = (7 - 1) // 2 * (7 + 1)
    assert abs(o.particles()["n"][centre] - 6.539696962) < 1e-5
    assert abs(o.environment().n0 - 6.539696962) < 1e-9


@pytest.mark.parametrize("re,n0", [(2.1, 6.539696962), (2.4, 9.774726), (4.0, 35.609223)])
def test_reference_n0_values(oracle_lib, re, n0):
    # Environment.hpp:163-215 lattice sums at the radii used by the configs
    o = _oracle(_params(l0=0.01, re_by_l0=re, min_x=0, min_z=0, max_x=1, max_z=1))
    assert abs(o.environment().n0 - n0) < 1e-6


# ---------------------------------------------- test_ComputerImplicitForces.cpp
def _implicit_fixture(n, u_fn=None):
    # l0 = 1, r_e = 5, domain +-2 l0 num (:14-35); Dt = 0.01 set before the test (:85-86)
    prm = _params(l0=1.0, re_by_l0=5.0, min_x=-30.0, min_z=-30.0, max_x=30.0, max_z=30.0)
    o = _oracle(prm, scenes.lattice(n, n, 1.0, (-30, -30, 30, 30), u_fn=u_fn))
    o.begin_step(1.0 / 100)
    o.stage("search_neighbor")
    o.stage("density")
    o.stage("set_ppe")
    return o


def _dense(o):
    rp, col, val, b, _ = o.ppe()
    n = len(rp) - 1
    a = np.zeros((n, n))
    for i in range(n):
        a[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    return a, b


def test_ppe_matrix_symmetry(oracle_lib):
    # MatrixSymmetry :167-212 (6 x 6 lattice, 1e-3)
    a, _ = _dense(_implicit_fixture(6))
    assert math.sqrt(np.sum(np.tril(a - a.T, -1) ** 2)) < 1e-3


def test_ppe_diagonal_identity(oracle_lib):
    # MatrixDiagIdentity :216-258 (15 x 15, centre particle, 1e-3)
    a, _ = _dense(_implicit_fixture(15))
    c = (15 - 1) // 2 * (15 + 1)
    off = a[c].sum() - a[c, c]
    assert abs((a[c, c] - (-off)) / a[c, c]) < 1e-3


def test_ppe_zero_outside_neighbors(oracle_lib):
    # MatrixNeighborNonzero :262-320 (6 x 6)
    o = _implicit_fixture(6)
    a, _ = _dense(o)
    counts, lst = o.neighbors()
    rows = np.split(lst, np.cumsum(counts)[:-1])
    for i in range(36):
        outside = np.ones(36, dtype=bool)
        outside[rows[i]] = False
        outside[i] = False
        assert np.all(np.abs(a[i, outside]) < 1e-3)


def test_ppe_rhs_value(oracle_lib):
    # VectorValue :323-375: u = (x, -0.3 z), b = -rho/(dt n0) * (-div u * n), 10 % (wall margin 6)
    gx, gz = 1.0, -0.3
    o = _implicit_fixture(15, u_fn=lambda x, z: (gx * x, gz * z))
    _, b = _dense(o)
    env = o.environment()
    n = o.particles()["n"]
    for iz in range(6, 15 - 6):
        for ix in range(6, 15 - 6):
            i = ix + 15 * iz
            analy = -env.rho / (env.dt * env.n0) * (-(gx + gz) * n[i])
            assert abs((b[i] - analy) / analy) < 1e-1


def test_ppe_matrix_value(oracle_lib):
    # MatrixValue :378-455: HL coefficient (5 - D) r_e / n0 / r^3, 1e-3
    o = _implicit_fixture(15, u_fn=lambda x, z: (x, -0.3 * z))
    a, _ = _dense(o)
    env = o.environment()
    inner = [ix + 15 * iz for iz in range(6, 9) for ix in range(6, 9)]
    for i in inner:
        for j in inner:
            if i >= j or a[i, j] == 0.0:
                continue
            dx = (i % 15) - (j % 15)
            dz = (i // 15) - (j // 15)
            r = math.sqrt(dx * dx + dz * dz)
            analy = 3 * env.re / env.n0 / r ** 3
            assert abs((a[i, j] - analy) / a[i, j]) < 1e-3


# ------------------------------------------ test_ComputerConjugateGradient.cpp
def _csr(a):
    rp, col, val = [0], [], []
    for i in range(a.shape[0]):
        nz = np.nonzero(a[i])[0]
        col.extend(nz.tolist())
        val.extend(a[i, nz].tolist())
        rp.append(len(col))
    return np.array(rp), np.array(col), np.array(val)


def test_cg_identity(oracle_lib):
    # SolveIdentityMatrix :115-144 (eps 1e-7, 1e-3)
    from oracle.oracle import cg_solve_csr

    b = np.arange(10, dtype=np.float64)
    x, _, _, _, rc = cg_solve_csr(*_csr(np.eye(10)), b, np.zeros(10), 1e-7)
    assert rc == 0 and np.mean(np.abs(x - b)) < 1e-3


def test_cg_4x4(oracle_lib):
    # Solve4x4Matrix :146-183: symmetric indefinite, solution (2, 4, 6, 8)
    from oracle.oracle import cg_solve_csr

    a = np.array([[1, 1, 1, -1], [1, 1, -1, 1], [1, -1, 1, 1], [-1, 1, 1, 1]], dtype=np.float64)
    x, _, _, _, rc = cg_solve_csr(*_csr(a), 4.0 * np.array([1, 2, 3, 4.0]), np.zeros(4), 1e-7)
    assert rc == 0
    np.testing.assert_allclose(x, [2, 4, 6, 8], atol=1e-3)


def test_cg_1d_poisson(oracle_lib):
    # Solve1dODE :186-229: f'' = x, f(0) = 0, f(1) = 1 against the cubic solution
    from oracle.oracle import cg_solve_csr

    nx = 10
    dx = 1.0 / (nx + 1)
    dx2 = dx * dx
    A = np.zeros((nx, nx))
    rhs = np.zeros(nx)
    for j in range(1, nx - 1):
        A[j - 1, j] = 1.0 / dx2
        A[j, j] = -2.0 / dx2
        A[j + 1, j] = 1.0 / dx2
        rhs[j] = dx * (j + 1)
    A[0, 0] = -2.0 / dx2
    A[1, 0] = 1.0 / dx2
    A[nx - 1, nx - 1] = -2.0 / dx2
    A[nx - 2, nx - 1] = 1.0 / dx2
    rhs[0] = dx
    rhs[nx - 1] = -1.0 / dx2 + (1.0 - dx)
    x, _, _, _, rc = cg_solve_csr(*_csr(A), rhs, np.zeros(nx), 1e-7)
    xs = dx * (np.arange(nx) + 1)
    analy = xs ** 3 / 6.0 + (1.0 - 1.0 / 6.0) * xs
    assert rc == 0 and np.mean(np.abs((x - analy) / analy)) < 1e-3


def test_cg_reports_non_convergence(oracle_lib):
    # the reference throws after as many iterations as unknowns (Computer.hpp:1424-1428)
    from oracle.oracle import cg_solve_csr

    a = np.diag(np.arange(1, 51, dtype=np.float64))
    _, it, _, _, rc = cg_solve_csr(*_csr(a), np.ones(50), np.zeros(50), 1e-14, max_iters=3)
    assert rc == abi.MPS_ERR_CG_NOT_CONVERGED and it == 3


# --------------------------------------------- test_ComputerPressureGradient.cpp
@pytest.mark.parametrize("case", ["polynomial", "trigonometric"])
def test_pressure_gradient(oracle_lib, case):
    # GradValuePolynomial :117-185, GradValueTrignometric :188-254 (20 x 20, r_e 1.5, 5 %)
    re = 1.5
    if case == "polynomial":
        dl = re * 10.0
        gpx, gpz = 1.0 / dl ** 2, -1.0 / dl ** 2
        p_fn = lambda x, z: 0.5 * x * x * gpx + 1.0 / 3.0 * z ** 3 * gpz
        grad = lambda x, z: (gpx * x, gpz * z * z)
    else:
        k = 2.0 * math.pi / (10.0 * re)
        p_fn = lambda x, z: np.cos(k * x) - np.sin(k * z)
        grad = lambda x, z: (-np.sin(k * x) * k, -np.cos(k * z) * k)
    prm = _params(l0=1.0, re_by_l0=re, min_x=-50.0, min_z=-50.0, max_x=50.0, max_z=50.0)
    s = scenes.lattice(20, 20, 1.0, (-50, -50, 50, 50), p_fn=p_fn)
    o = _oracle(prm, s)
    o.begin_step(1.0 / 100)
    o.stage("search_neighbor")
    o.stage("density")
    o.stage("pressure_gradient")
    P = o.particles()
    env = o.environment()
    pref = -env.dt / env.rho
    for j in range(5, 15):
        for i in range(5, 15):
            idx = i + 20 * j
            gx, gz = grad(float(i), float(j))
            if case == "trigonometric":
                gx, gz = grad(P["x"][idx], P["z"][idx])
            assert abs((P["u"][idx] / pref - gx) / gx) < 0.05
            assert abs((P["w"][idx] / pref - gz) / gz) < 0.05
            assert abs(((P["x"][idx] - i) - pref * gx * env.dt) / (pref * gx * env.dt)) < 0.05
            assert abs(((P["z"][idx] - j) - pref * gz * env.dt) / (pref * gz * env.dt)) < 0.05


# ------------------------------------ test_ComputerNeighborDensityVariation.cpp
@pytest.mark.parametrize("case", ["linear", "polynomial"])
def test_density_variation(oracle_lib, case):
    # ValueTestLinear :114-163, ValueTestPolynomial :166-213 (35 x 35, r_e 5, margin 15, 10 %)
    if case == "linear":
        gx, gz = 1.0, -0.3
        u_fn = lambda x, z: (gx * x, gz * z)
        div = lambda x, z: gx + gz
    else:
        gx, gz = 1.0, -1.5
        u_fn = lambda x, z: (0.5 * gx * x * x, 1.0 / 3.0 * gz * z ** 3)
        div = lambda x, z: gx * x + gz * z * z
    prm = _params(l0=1.0, re_by_l0=5.0, g=0.0, min_x=-50.0, min_z=-50.0, max_x=50.0,
                  max_z=50.0)
    o = _oracle(prm, scenes.lattice(35, 35, 1.0, (-50, -50, 50, 50), u_fn=u_fn))
    o.begin_step(1.0 / 100)
    o.stage("search_neighbor")
    o.stage("density")
    speed = o.density_variation()
    n = o.particles()["n"]
    for j in range(15, 35 - 15):
        for i in range(15, 35 - 15):
            idx = i + 35 * j
            analy = -div(float(i), float(j))
            assert abs((speed[idx] / n[idx] - analy) / analy) < 0.10


# ------------------------------------------------------ test_ComputerMatrix.cpp
@pytest.mark.parametrize("m, inv", [
    # test_ComputerMatrix.cpp:19-33: diagonal
    ((1.0, 0.0, 0.0, 2.0), (1.0, 0.0, 0.0, 0.5)),
    # :35-49: anti-diagonal
    ((0.0, 1.0, 2.0, 0.0), (0.0, 0.5, 1.0, 0.0)),
    # :51-66: full, asymmetric
    ((1.0, 2.0, 3.0, 4.0), (-2.0, 1.0, 1.5, -0.5)),
])
def test_invert_matrix_known_answers(oracle_lib, m, inv):
    # the reference asserts the Frobenius distance is 0 with ASSERT_DOUBLE_EQ (4 ulps)
    from oracle.oracle import gc_invert

    got = gc_invert(m, 1.0)
    assert math.sqrt(float(np.sum((got - np.array(inv)) ** 2))) <= 4 * np.finfo(float).eps


def test_invert_matrix_singular_gives_scaled_identity(oracle_lib):
    # Detail::InvertMatrix<2> returns IdentityMatrix(val) when det == 0 (Computer.hpp:337-340)
    from oracle.oracle import gc_invert

    np.testing.assert_array_equal(gc_invert((1.0, 2.0, 2.0, 4.0), 0.25), [0.25, 0.0, 0.0, 0.25])
    np.testing.assert_array_equal(gc_invert((0.0, 0.0, 0.0, 0.0), 3.0), [3.0, 0.0, 0.0, 3.0])
