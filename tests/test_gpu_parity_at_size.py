"""Parity at the benchmark sizes, against the oracle.

The 320k-fluid dam break (340,050 particles, l0 = 5e-4 m, the headline workload) and
the 80k-fluid hydrostatic tank (84,450 particles, l0 = 2.5e-3 m) are advanced a few
steps by the OpenMP build of the oracle; the GPU then starts from that state.

* every stage of ForwardTime (src/OpenMps/Computer.hpp:1700-1742) bit for bit: the
  neighbour lists, number densities, ECS, explicit forces, SaveX, the PPE's row
  pointers, columns, values, right-hand side and initial guess
  (Computer.hpp:1145-1356), and, from the same pressure, the pressure gradient and DS;
* one whole step with both sides solving to eps = 1e-13: pressure within 1e-10 of
  max |p|, positions within 1e-12;
* the PPE solvers at the workload's tolerance (|b - A x| <= 1e-8 |b|) against the
  oracle's FP64 CG: each one's error against a 1e-14 oracle solution is stated, and
  must be no larger than a few times that of the oracle's own CG at 1e-8.
"""
import numpy as np
import pytest

from helpers import assert_same_neighbors, assert_same_particles, assert_same_ppe, rel_err
from openmps_gb300 import _abi as abi
from openmps_gb300 import scenes

pytestmark = pytest.mark.gpu

SIZES = {
    "c1_hydrostatic_84k": scenes.config_c1,
    "c2_dam_break_340k": scenes.config_c2,
}
WARM_STEPS = 2
P_TOL = 1e-10
X_TOL = 1e-12


@pytest.fixture(scope="module", params=sorted(SIZES))
def warmed(request, oracle_lib):
    """(name, scene, state after WARM_STEPS oracle steps)."""
    from oracle.oracle import Oracle

    s = SIZES[request.param]()
    cpu = Oracle(s.params(), openmp=True)
    cpu.add_scene(s)
    for _ in range(WARM_STEPS):
        cpu.forward_time(s.meta["dt"])
    return request.param, s, (cpu.particles(), cpu.aux())


def _pair(scene, state, params):
    from openmps_gb300.computer import Computer
    from oracle.oracle import Oracle

    P, A = state
    gpu = Computer(params)
    gpu.add_scene(scene)
    cpu = Oracle(params, openmp=True)
    cpu.add_scene(scene)
    for h in (gpu, cpu):
        h.set_particles(P["type"], P["x"], P["z"], P["u"], P["w"], P["p"], P["n"])
        h.set_aux(A["n_without_spp"], A["ecs"], A["ox"], A["oz"])
    return gpu, cpu


def _stages_to_ppe(h, dt, flags):
    h.begin_step(dt)
    h.stage("search_neighbor")
    h.stage("density")
    if flags & abi.FLAG_ECS:
        h.stage("error_correction")
    h.stage("explicit")
    h.stage("density")
    if flags & abi.FLAG_DS:
        h.stage("save_x")
    h.stage("set_ppe")


def test_stage_chain_at_size(gpu_lib, warmed):
    name, s, state = warmed
    prm = s.params(eps=1e-10)
    gpu, cpu = _pair(s, state, prm)
    dt = s.meta["dt"]
    flags = prm.flags
    for h in (gpu, cpu):
        h.begin_step(dt)
        h.stage("search_neighbor")
    assert_same_neighbors(gpu, cpu, name + " search")
    for h in (gpu, cpu):
        h.stage("density")
    assert_same_particles(gpu, cpu, what=name + " density")
    np.testing.assert_array_equal(gpu.aux()["n_without_spp"], cpu.aux()["n_without_spp"])
    np.testing.assert_array_equal(gpu.density_variation(), cpu.density_variation())
    if flags & abi.FLAG_ECS:
        for h in (gpu, cpu):
            h.stage("error_correction")
        np.testing.assert_array_equal(gpu.aux()["ecs"], cpu.aux()["ecs"])
    for h in (gpu, cpu):
        h.stage("explicit")
    assert_same_particles(gpu, cpu, what=name + " explicit")
    for h in (gpu, cpu):
        h.stage("density")
    assert_same_particles(gpu, cpu, what=name + " density 2")
    if flags & abi.FLAG_DS:
        for h in (gpu, cpu):
            h.stage("save_x")
        ga, ca = gpu.aux(), cpu.aux()
        np.testing.assert_array_equal(ga["ox"], ca["ox"])
        np.testing.assert_array_equal(ga["oz"], ca["oz"])
    for h in (gpu, cpu):
        h.stage("set_ppe")
    assert_same_ppe(gpu, cpu, name + " assembly")
    nnz = gpu.ppe()[1].size
    print("%s: %d particles, %d PPE nonzeros bit-identical" % (name, s.count, nnz))
    for h in (gpu, cpu):
        h.stage("solve_ppe")
        h.stage("assign_pressure")
    gp, cp = gpu.particles()["p"], cpu.particles()["p"]
    print("%s: pressure after both solves to eps 1e-10: rel err %.2e" % (name, rel_err(gp, cp)))
    assert rel_err(gp, cp) <= 1e-6
    cpu.set_particles(p=gp)
    for h in (gpu, cpu):
        h.stage("pressure_gradient")
    assert_same_particles(gpu, cpu, what=name + " pressure gradient")
    if flags & abi.FLAG_DS:
        for h in (gpu, cpu):
            h.stage("dynamic_stabilize")
        assert_same_particles(gpu, cpu, what=name + " dynamic stabilisation")


def test_step_at_size(gpu_lib, warmed):
    name, s, state = warmed
    gpu, cpu = _pair(s, state, s.params(eps=1e-13))
    dt = s.meta["dt"]
    gpu.forward_time(dt)
    cpu.forward_time(dt)
    G, C = gpu.particles(), cpu.particles()
    np.testing.assert_array_equal(G["type"], C["type"])
    ep = rel_err(G["p"], C["p"])
    ex = max(rel_err(G["x"], C["x"]), rel_err(G["z"], C["z"]))
    eu = max(rel_err(G["u"], C["u"]), rel_err(G["w"], C["w"]))
    print("%s: one step at eps 1e-13: CG iterations GPU %d / oracle %d; rel err p %.2e, x %.2e, "
          "u %.2e" % (name, gpu.stats()["cg_iterations"], cpu.stats()["cg_iterations"], ep, ex, eu))
    assert ep <= P_TOL, "%s: pressure rel err %.3e" % (name, ep)
    assert ex <= X_TOL, "%s: position rel err %.3e" % (name, ex)
    assert eu <= 1e-7, "%s: velocity rel err %.3e" % (name, eu)


def test_solvers_against_oracle_cg(gpu_lib, warmed):
    from openmps_gb300 import learned
    from openmps_gb300.computer import Computer
    from oracle.oracle import cg_solve_csr

    name, s, state = warmed
    dt = s.meta["dt"]
    gpu, _ = _pair(s, state, s.params())
    _stages_to_ppe(gpu, dt, gpu.params.flags)
    rp, col, val, b, x0 = gpu.ppe()
    x_ref, it_ref, _, _, rc = cg_solve_csr(rp, col, val, b, x0, 1e-14, abi.CRIT_RHS, openmp=True)
    assert rc == 0
    x_ora, it_ora, _, _, rc = cg_solve_csr(rp, col, val, b, x0, 1e-8, abi.CRIT_RHS, openmp=True)
    assert rc == 0
    scale = np.max(np.abs(x_ref))
    e_ora = float(np.max(np.abs(x_ora - x_ref)) / scale)
    lines = ["%s: oracle FP64 CG to 1e-8 |b|: %d iterations, error %.2e (reference solution: "
             "oracle CG to 1e-14 |b|, %d iterations)" % (name, it_ora, e_ora, it_ref)]
    blob = learned.load()
    for solver in (abi.SOLVER_CG64, abi.SOLVER_MIXED, abi.SOLVER_MIXED_MG, abi.SOLVER_LEARNED):
        c, _ = _pair(s, state, s.params(solver=solver, criterion=abi.CRIT_RHS, eps=1e-8))
        if solver == abi.SOLVER_LEARNED:
            c.learned_set_weights(blob)
        _stages_to_ppe(c, dt, c.params.flags)
        c.stage("solve_ppe")
        x = c.ppe()[4]
        st = c.stats()
        e = float(np.max(np.abs(x - x_ref)) / scale)
        lines.append("  %s: %d iterations, true relres %.2e, fallback %d, error %.2e"
                     % (abi.SOLVER_NAMES[solver], st["cg_iterations"], st["cg_true_relres"],
                        st["fallback"], e))
        assert st["cg_true_relres"] <= 1e-8
        assert e <= max(10 * e_ora, 1e-9), "%s: error %.3e vs oracle %.3e" % (solver, e, e_ora)
        del c
    print("\n".join(lines))
