"""Stage-by-stage parity of the GPU step against the oracle, from identical states.

Every per-particle stage (number density, ECS, explicit forces, PPE right-hand
side and matrix, pressure assignment, pressure gradient, dynamic stabilisation)
must reproduce the FP64 CPU path bit for bit: same neighbour order, same
expression order, no fused multiply-add.  The only stage that is not bit-exact
is the CG solve (its dot products reduce in a different order); to test the
stages after it, the GPU's pressure is handed to the oracle.
"""
import numpy as np
import pytest

from helpers import (assert_same_neighbors, assert_same_particles, assert_same_ppe, copy_state,
                     far_tank, jittered_tank, make_pair, plain_tank, reference_tank, stock_tank,
                     stock_two_radii_tank, threshold_rings)
from openmps_gb300 import _abi as abi

pytestmark = pytest.mark.gpu

CASES = {
    "reference_preset": lambda: reference_tank(),
    "plain_two_radii": lambda: plain_tank(),
    "plain_two_radii_ds": lambda: plain_tank(ds=True),
    "jittered_reference": lambda: jittered_tank(jitter=0.1, preset=abi.PRESET_REFERENCE),
    "jittered_plain": lambda: jittered_tank(jitter=0.1),
    "stock_one_radius": stock_tank,
    "stock_two_radii": stock_two_radii_tank,
    "stock_far_from_origin": far_tank,
}


def _advance_oracle(scene, cpu, steps):
    for _ in range(steps):
        cpu.forward_time(scene.meta["dt"])


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("warm_steps", [0, 3])
def test_stage_chain(gpu_lib, oracle_lib, case, warm_steps):
    s = CASES[case]()
    prm = s.params()
    gpu, cpu = make_pair(s, prm)
    _advance_oracle(s, cpu, warm_steps)
    copy_state(cpu, gpu)
    flags = prm.flags
    dt = s.meta["dt"]

    for h in (gpu, cpu):
        h.begin_step(dt)
    for h in (gpu, cpu):
        h.stage("search_neighbor")
    assert_same_neighbors(gpu, cpu, "search")

    for h in (gpu, cpu):
        h.stage("density")
    assert_same_particles(gpu, cpu, what="density")
    np.testing.assert_array_equal(gpu.aux()["n_without_spp"], cpu.aux()["n_without_spp"])

    np.testing.assert_array_equal(gpu.density_variation(), cpu.density_variation())

    if flags & abi.FLAG_ECS:
        for h in (gpu, cpu):
            h.stage("error_correction")
        np.testing.assert_array_equal(gpu.aux()["ecs"], cpu.aux()["ecs"])

    for h in (gpu, cpu):
        h.stage("explicit")
    assert_same_particles(gpu, cpu, what="explicit")

    for h in (gpu, cpu):
        h.stage("density")
    assert_same_particles(gpu, cpu, what="density 2")

    if flags & abi.FLAG_DS:
        for h in (gpu, cpu):
            h.stage("save_x")
        ga, ca = gpu.aux(), cpu.aux()
        np.testing.assert_array_equal(ga["ox"], ca["ox"])
        np.testing.assert_array_equal(ga["oz"], ca["oz"])

    for h in (gpu, cpu):
        h.stage("set_ppe")
    assert_same_ppe(gpu, cpu, "assembly")

    # solve on both (different reduction orders), then continue from the GPU pressure
    for h in (gpu, cpu):
        h.stage("solve_ppe")
    for h in (gpu, cpu):
        h.stage("assign_pressure")
    gp = gpu.particles()["p"]
    cp = cpu.particles()["p"]
    scale = max(np.max(np.abs(cp)), 1.0)
    assert np.max(np.abs(gp - cp)) <= 1e-6 * scale
    cpu.set_particles(p=gp)

    for h in (gpu, cpu):
        h.stage("pressure_gradient")
    assert_same_particles(gpu, cpu, what="pressure gradient")

    if flags & abi.FLAG_DS:
        for h in (gpu, cpu):
            h.stage("dynamic_stabilize")
        assert_same_particles(gpu, cpu, what="dynamic stabilisation")


def test_range_tests_at_thresholds(gpu_lib, oracle_lib):
    # pairs within 4e-16 .. 1e-5 (relative) of r_e, the Laplacian radius and the
    # neighbour length: the FP32 screen must leave each of them to the FP64 comparison
    s = threshold_rings()
    gpu, cpu = make_pair(s, s.params())
    dt = s.meta["dt"]
    for h in (gpu, cpu):
        h.begin_step(dt)
        h.stage("search_neighbor")
    assert_same_neighbors(gpu, cpu, "search")
    counts, _ = gpu.neighbors()
    assert counts[0] > 0 and counts[0] < s.count - 1  # the outer ring is split by the test
    for h in (gpu, cpu):
        h.stage("density")
    assert_same_particles(gpu, cpu, what="density")
    np.testing.assert_array_equal(gpu.density_variation(), cpu.density_variation())
    for h in (gpu, cpu):
        h.stage("error_correction")
    np.testing.assert_array_equal(gpu.aux()["ecs"], cpu.aux()["ecs"])
    for h in (gpu, cpu):
        h.stage("explicit")
    assert_same_particles(gpu, cpu, what="explicit")
    for h in (gpu, cpu):
        h.stage("density")
        h.stage("save_x")
        h.stage("set_ppe")
    assert_same_ppe(gpu, cpu, "assembly")
    # pressure gradient and stabilisation from the same pressure on both sides
    p = np.linspace(0.0, 50.0, s.count)
    gpu.set_particles(p=p)
    cpu.set_particles(p=p)
    for h in (gpu, cpu):
        h.stage("pressure_gradient")
    assert_same_particles(gpu, cpu, what="pressure gradient")
    for h in (gpu, cpu):
        h.stage("dynamic_stabilize")
    assert_same_particles(gpu, cpu, what="dynamic stabilisation")


def test_cfl_time_step(gpu_lib, oracle_lib):
    # ForwardTime() without dt: DetermineDt (Computer.hpp:759-777)
    s = jittered_tank()
    gpu, cpu = make_pair(s, s.params())
    rng = np.random.default_rng(3)
    u = rng.normal(size=s.count) * 0.3
    w = rng.normal(size=s.count) * 0.3
    gpu.set_particles(u=u, w=w)
    cpu.set_particles(u=u, w=w)
    expect = cpu.determine_dt()
    gpu.begin_step(-1.0)
    env = gpu.environment()
    assert env.dt == expect
    assert env.t == expect


@pytest.mark.parametrize("case", ["reference_preset", "plain_two_radii", "plain_two_radii_ds",
                                  "stock_one_radius", "stock_two_radii", "stock_far_from_origin"])
def test_step_equals_stage_chain(gpu_lib, oracle_lib, case):
    # mps_forward_time walks each neighbour row once for density, ECS and the explicit
    # accelerations together, and once for the second density and the PPE assembly
    # (SPP method set); the stage entry points run each stage separately.  The results
    # must be bit-identical (same terms, same order) through a whole step.
    s = CASES[case]()
    prm = s.params()
    flags = prm.flags
    a, cpu = make_pair(s, prm)
    b, _ = make_pair(s, prm)
    _advance_oracle(s, cpu, 2)
    copy_state(cpu, a)
    copy_state(cpu, b)
    dt = s.meta["dt"]
    a.forward_time(dt)
    b.begin_step(dt)
    names = ["search_neighbor", "density"]
    if flags & abi.FLAG_ECS:
        names.append("error_correction")
    names += ["explicit", "density"]
    if flags & abi.FLAG_DS:
        names.append("save_x")
    names += ["set_ppe", "solve_ppe", "assign_pressure", "pressure_gradient"]
    if flags & abi.FLAG_DS:
        names.append("dynamic_stabilize")
    for name in names:
        b.stage(name)
    A, B = a.particles(), b.particles()
    for k in ("type", "x", "z", "u", "w", "p", "n"):
        np.testing.assert_array_equal(A[k], B[k], err_msg="%s %s" % (case, k))
    xa, xb = a.aux(), b.aux()
    for k in ("n_without_spp", "ecs", "ox", "oz"):
        np.testing.assert_array_equal(xa[k], xb[k], err_msg="%s %s" % (case, k))
    # the PPE system each path assembled (the step fuses the second density into it
    # for the SPP method set)
    for ga, gb, what in zip(a.ppe(), b.ppe(), ("row_ptr", "columns", "values", "rhs", "guess")):
        np.testing.assert_array_equal(ga, gb, err_msg="%s %s" % (case, what))
