"""The multigrid-preconditioned mixed-precision PPE solve (MPS_SOLVER_MIXED_MG).

The preconditioner changes the iteration, not the equation: a step solved with it
must reach the same pressure as the oracle's FP64 CG (the reference algorithm) at the
requested residual, with far fewer iterations, and fall back to the plain FP64 CG when
it is cut short.
"""
import numpy as np
import pytest

from helpers import copy_state, make_pair, plain_tank, reference_tank, rel_err, stock_tank
from openmps_gb300 import _abi as abi
from openmps_gb300 import scenes
from openmps_gb300.computer import Computer

pytestmark = pytest.mark.gpu


def _one_step(maker, **kw):
    s = maker()
    gpu, cpu = make_pair(s, s.params(eps=1e-13))
    mg = Computer(s.params(eps=1e-10, solver=abi.SOLVER_MIXED_MG, criterion=abi.CRIT_RHS, **kw))
    mg.add_scene(s)
    for _ in range(4):
        cpu.forward_time(s.meta["dt"])
    copy_state(cpu, mg)
    cpu.forward_time(s.meta["dt"])
    mg.forward_time(s.meta["dt"])
    return mg, cpu


@pytest.mark.parametrize("maker", [plain_tank, reference_tank, stock_tank])
def test_step_matches_fp64_cg(gpu_lib, oracle_lib, maker):
    mg, cpu = _one_step(maker)
    st = mg.stats()
    assert st["fallback"] == 0
    assert st["cg_true_relres"] <= 1e-10
    err = rel_err(mg.particles()["p"], cpu.particles()["p"])
    assert err < 1e-7, err
    # scenes this small have few cell levels: fewer iterations, not yet a large factor
    it64 = cpu.stats()["cg_iterations"]
    assert st["cg_iterations"] < it64, (st["cg_iterations"], it64)


def test_fallback_after_stall(gpu_lib, oracle_lib):
    # two preconditioned iterations cannot reach 1e-10: the FP64 CG finishes the solve
    mg, cpu = _one_step(stock_tank, max_cg_iters=2)
    st = mg.stats()
    assert st["fallback"] == 1
    assert st["cg_true_relres"] <= 1e-10
    assert rel_err(mg.particles()["p"], cpu.particles()["p"]) < 1e-7


def _run_launch(s, launch, steps=3):
    c = Computer(s.params(eps=1e-10, solver=abi.SOLVER_MIXED_MG, criterion=abi.CRIT_RHS, cg_launch=launch))
    c.add_scene(s)
    for _ in range(steps):
        c.forward_time(s.meta["dt"])
    return c.particles(), c.stats()


def test_host_launch_matches_graph(gpu_lib):
    # the host-driven loop runs the same per-phase kernels in the same order as the graph
    # of per-phase kernels: identical results
    s = stock_tank()
    a, sa = _run_launch(s, abi.CG_LAUNCH_GRAPH)
    b, sb = _run_launch(s, abi.CG_LAUNCH_HOST)
    for k in ("x", "z", "u", "w", "p"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert sa["cg_iterations"] == sb["cg_iterations"]


@pytest.mark.parametrize("maker", [stock_tank, reference_tank])
def test_persistent_kernel_matches_per_phase_kernels(gpu_lib, maker):
    # the persistent cooperative solve adds its dot products in another order: the same
    # solution to the solve tolerance, and no fallback
    s = maker()
    a, sa = _run_launch(s, abi.CG_LAUNCH_PERSISTENT)
    b, sb = _run_launch(s, abi.CG_LAUNCH_GRAPH)
    assert sa["fallback"] == 0 and sa["cg_true_relres"] <= 1e-10
    assert rel_err(a["p"], b["p"]) < 1e-7
    assert rel_err(a["x"], b["x"], scale=s.l0) < 1e-9
    assert abs(sa["cg_iterations"] - sb["cg_iterations"]) <= 2


def test_deterministic(gpu_lib):
    s = stock_tank()
    ps = []
    for _ in range(2):
        c = Computer(s.params(eps=1e-10, solver=abi.SOLVER_MIXED_MG, criterion=abi.CRIT_RHS))
        c.add_scene(s)
        for _ in range(3):
            c.forward_time(s.meta["dt"])
        ps.append(c.particles()["p"])
    np.testing.assert_array_equal(ps[0], ps[1])


def test_iterations_on_larger_dam_break(gpu_lib):
    # 20k-particle dam break: the same steps with CG64 and MIXED_MG agree, and the
    # preconditioned solve needs a small fraction of the iterations
    s = scenes.dam_break(2e-3)
    s.meta["params"] = dict(scenes.STOCK_PHYSICS, eps=1e-8, max_dt=1e-4)
    dt = 1e-4
    runs = {}
    for solver in (abi.SOLVER_CG64, abi.SOLVER_MIXED_MG):
        c = Computer(s.params(solver=solver, criterion=abi.CRIT_RHS, eps=1e-8))
        c.add_scene(s)
        its = []
        for _ in range(5):
            c.forward_time(dt)
            its.append(c.stats()["cg_iterations"])
            assert c.stats()["cg_true_relres"] <= 1e-8
        runs[solver] = (c.particles(), its)
    P64, it64 = runs[abi.SOLVER_CG64]
    Pmg, itmg = runs[abi.SOLVER_MIXED_MG]
    assert max(itmg) * 5 < min(it64), (itmg, it64)
    # both solve to |b - A x| <= 1e-8 |b|: after five steps the positions agree far below
    # l0; the pressures differ by a few 1e-5 of max |p| (measured 2.5e-5 at r_e = 4.0 l0)
    assert rel_err(Pmg["x"], P64["x"], scale=2e-3) < 1e-6
    assert rel_err(Pmg["p"], P64["p"]) < 1e-4


def test_deep_hierarchy_matches_fp64_cg(gpu_lib, oracle_lib):
    # The l0 = 0.01 dam break in a 40 m x 40 m domain: an 837 x 837 search grid (cells of
    # 4.8 l0), so 8 cell levels with the single-block bottom at level 5.  The cycle then
    # runs one level each way with the per-level kernels and three each way with the
    # fused sweeps (the workload's 320k dam break uses the fused sweeps alone).
    def deep():
        s = stock_tank()
        s.max_x = 40.0
        s.max_z = 40.0
        return s

    mg, cpu = _one_step(deep)
    st = mg.stats()
    assert mg.environment().grid_nx == 837 and mg.environment().grid_nz == 837
    assert st["fallback"] == 0
    assert st["cg_true_relres"] <= 1e-10
    err = rel_err(mg.particles()["p"], cpu.particles()["p"])
    print("deep hierarchy: %d iterations (FP64 CG %d), pressure rel err %.2e"
          % (st["cg_iterations"], cpu.stats()["cg_iterations"], err))
    assert err < 1e-7, err
