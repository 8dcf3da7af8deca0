"""PPE solvers on the GPU: the reference's CG known answers and the mixed solver.

The first three cases restate the reference's CG tests
(src/OpenMps/test/test_ComputerConjugateGradient.cpp:115-229, eps = 1e-7, checked
to 1e-3): an identity system, a 4 x 4 symmetric indefinite system with solution
(2, 4, 6, 8) and a 1-D Poisson problem against its cubic solution.
"""
import numpy as np
import pytest

from helpers import copy_state, make_pair, plain_tank, reference_tank, rel_err
from openmps_gb300 import _abi as abi
from openmps_gb300.computer import Computer

pytestmark = pytest.mark.gpu


def _dense_to_csr(a):
    rp, col, val = [0], [], []
    for i in range(a.shape[0]):
        for j in range(a.shape[1]):
            if a[i, j] != 0.0:
                col.append(j)
                val.append(a[i, j])
        rp.append(len(col))
    return np.array(rp), np.array(col), np.array(val)


@pytest.fixture(scope="module")
def solver_handle(gpu_lib):
    return Computer(abi.make_params())


@pytest.mark.parametrize("solver", [abi.SOLVER_CG64, abi.SOLVER_MIXED])
def test_identity(solver_handle, solver):
    n = 10
    rp, col, val = _dense_to_csr(np.eye(n))
    b = np.arange(n, dtype=np.float64)
    x, it, _ = solver_handle.cg_solve_csr(rp, col, val, b, np.zeros(n), 1e-7, solver=solver)
    assert np.mean(np.abs(x - b)) < 1e-3


def test_4x4_indefinite(solver_handle):
    a = np.array([[1, 1, 1, -1], [1, 1, -1, 1], [1, -1, 1, 1], [-1, 1, 1, 1]], dtype=np.float64)
    b = 4.0 * np.array([1, 2, 3, 4], dtype=np.float64)
    rp, col, val = _dense_to_csr(a)
    x, _, _ = solver_handle.cg_solve_csr(rp, col, val, b, np.zeros(4), 1e-7)
    np.testing.assert_allclose(x, [2, 4, 6, 8], atol=1e-3)


@pytest.mark.parametrize("solver", [abi.SOLVER_CG64, abi.SOLVER_MIXED])
def test_1d_poisson(solver_handle, solver):
    nx = 10
    dx = 1.0 / (nx + 1)
    dx2 = dx * dx
    a0, b1 = 0.0, 1.0
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
    rhs[0] = -1.0 / dx2 * a0 + dx
    rhs[nx - 1] = -1.0 / dx2 * b1 + (1.0 - dx)
    rp, col, val = _dense_to_csr(A)
    x, _, _ = solver_handle.cg_solve_csr(rp, col, val, rhs, np.zeros(nx), 1e-7, solver=solver)
    xs = dx * (np.arange(nx) + 1)
    analy = xs ** 3 / 6.0 + (b1 - a0 - 1.0 / 6.0) * xs + a0
    assert np.mean(np.abs((x - analy) / analy)) < 1e-3


def test_matches_oracle_cg_on_ppe(gpu_lib, oracle_lib):
    # the assembled PPE of a dam-break step solved by GPU CG64 and the oracle CG
    from oracle.oracle import cg_solve_csr

    s = plain_tank()
    gpu, cpu = make_pair(s, s.params(eps=1e-12))
    for _ in range(4):
        cpu.forward_time(s.meta["dt"])
    cpu.begin_step(s.meta["dt"])
    for st in ("search_neighbor", "density", "explicit", "density", "set_ppe"):
        cpu.stage(st)
    rp, col, val, b, x0 = cpu.ppe()
    xo, ito, _, _, rc = cg_solve_csr(rp, col, val, b, x0, 1e-12)
    assert rc == 0
    xg, itg, rel = gpu.cg_solve_csr(rp, col, val, b, x0, 1e-12)
    assert rel_err(xg, xo) < 1e-9
    assert abs(itg - ito) <= max(3, ito // 20)


@pytest.mark.parametrize("maker", [plain_tank, reference_tank])
def test_mixed_precision_step(gpu_lib, oracle_lib, maker):
    # FP32-inner CG with FP64 reliable updates reaches the FP64 solution
    s = maker()
    prm64 = s.params(eps=1e-13)
    gpu, cpu = make_pair(s, prm64)
    mixed = Computer(s.params(eps=1e-10, solver=abi.SOLVER_MIXED, criterion=abi.CRIT_RHS))
    mixed.add_scene(s)
    for k in range(4):
        cpu.forward_time(s.meta["dt"])
    copy_state(cpu, mixed)
    cpu.forward_time(s.meta["dt"])
    mixed.forward_time(s.meta["dt"])
    st = mixed.stats()
    assert st["cg_true_relres"] <= 1e-10
    assert st["cg_refinements"] >= 2
    err = rel_err(mixed.particles()["p"], cpu.particles()["p"])
    assert err < 1e-7, err
