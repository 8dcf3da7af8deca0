"""Parity of the method variants: the GC corrective matrix (MPS_GC) and the explicit
pressure (PRESSURE_EXPLICIT), against the oracle.

* GC (Computer.hpp:1457-1499) changes only the pressure gradient: the stage must be
  bit-identical to the oracle's from the same state and pressure, with and without
  the SPP particle, on jittered rows, and on a row of particles whose corrective matrix
  is singular (the scaled-identity branch of InvertMatrix).
* The explicit pressure (Computer.hpp:1046-1067) removes the PPE, so a whole step is
  deterministic: free-running trajectories must match the oracle bit for bit, and so
  must a batch of scenes advanced by graph-replayed steps.
"""
import numpy as np
import pytest

from helpers import (assert_same_particles, copy_state, jittered_tank, make_pair, plain_tank,
                     reference_tank, rel_err, stock_tank, stock_two_radii_tank)
from openmps_gb300 import _abi as abi
from openmps_gb300 import scenes

pytestmark = pytest.mark.gpu

SOUND_SPEED = 27.5  # about ten times sqrt(2 g h) of the 0.37 m water columns


def _with_flags(scene, add):
    s = scene
    s.meta["params"] = dict(s.meta["params"])
    s.meta["params"]["flags"] = s.meta["params"].get("flags", 0) | add
    return s


def row_of_particles(l0=0.01, n=40):
    """One horizontal row of fluid particles: every dz is 0, so sum W/r^2 dx dx^T has a
    zero row and the GC matrix falls back to (D / n0) I (Computer.hpp:337-340)."""
    s = scenes.lattice(n, 1, l0, (-0.1, -0.1, n * l0 + 0.1, 0.2))
    s.meta["params"] = dict(scenes.STOCK_PHYSICS, eps=1e-10, max_dt=5e-4)
    s.meta["dt"] = 5e-4
    return s


GC_CASES = {
    "reference_preset": lambda: _with_flags(reference_tank(), abi.FLAG_GC),
    "plain_two_radii": lambda: _with_flags(plain_tank(), abi.FLAG_GC),
    "jittered_reference": lambda: _with_flags(jittered_tank(jitter=0.1, preset=abi.PRESET_REFERENCE),
                                              abi.FLAG_GC),
    "jittered_plain": lambda: _with_flags(jittered_tank(jitter=0.1), abi.FLAG_GC),
    "stock_one_radius": lambda: _with_flags(stock_tank(), abi.FLAG_GC),
    "stock_two_radii": lambda: _with_flags(stock_two_radii_tank(), abi.FLAG_GC),
}
GIVEN_PRESSURE_CASES = dict(GC_CASES, singular_row=lambda: _with_flags(row_of_particles(), abi.FLAG_GC))


@pytest.mark.parametrize("case", sorted(GIVEN_PRESSURE_CASES))
def test_gc_gradient_from_given_pressure(gpu_lib, oracle_lib, case):
    # the gradient stage alone on a seeded pressure field (no solve on either side)
    s = GIVEN_PRESSURE_CASES[case]()
    gpu, cpu = make_pair(s, s.params())
    rng = np.random.default_rng(3)
    cpu.set_particles(p=rng.uniform(0.0, 1000.0, s.count))
    copy_state(cpu, gpu)
    for h in (gpu, cpu):
        h.begin_step(s.meta["dt"])
    for name in ("search_neighbor", "density", "pressure_gradient"):
        for h in (gpu, cpu):
            h.stage(name)
        assert_same_particles(gpu, cpu, what="%s %s" % (name, case))


def _stages_to_pressure(gpu, cpu, prm, dt):
    """Runs both handles from begin_step to the assigned pressure, then hands the GPU's
    pressure to the oracle (the CG solves reduce in different orders)."""
    for h in (gpu, cpu):
        h.begin_step(dt)
    names = ["search_neighbor", "density"]
    if prm.flags & abi.FLAG_ECS:
        names.append("error_correction")
    names += ["explicit", "density"]
    if prm.flags & abi.FLAG_DS:
        names.append("save_x")
    names += ["set_ppe", "solve_ppe", "assign_pressure"]
    for name in names:
        for h in (gpu, cpu):
            h.stage(name)
    cpu.set_particles(p=gpu.particles()["p"])


@pytest.mark.parametrize("case", sorted(GC_CASES))
@pytest.mark.parametrize("warm_steps", [0, 2])
def test_gc_gradient_stage(gpu_lib, oracle_lib, case, warm_steps):
    s = GC_CASES[case]()
    prm = s.params()
    gpu, cpu = make_pair(s, prm)
    for _ in range(warm_steps):
        cpu.forward_time(s.meta["dt"])
    copy_state(cpu, gpu)
    _stages_to_pressure(gpu, cpu, prm, s.meta["dt"])
    for h in (gpu, cpu):
        h.stage("pressure_gradient")
    assert_same_particles(gpu, cpu, what="GC pressure gradient " + case)
    if prm.flags & abi.FLAG_DS:
        for h in (gpu, cpu):
            h.stage("dynamic_stabilize")
        assert_same_particles(gpu, cpu, what="dynamic stabilisation " + case)


def test_gc_changes_the_gradient(gpu_lib, oracle_lib):
    # the corrected and the plain gradient differ (the flag reaches the kernel)
    s = stock_tank()
    a, _ = make_pair(s, s.params())
    g = _with_flags(stock_tank(), abi.FLAG_GC)
    b, _ = make_pair(g, g.params())
    for h in (a, b):
        h.forward_time(s.meta["dt"])
    assert not np.array_equal(a.particles()["u"], b.particles()["u"])


@pytest.mark.parametrize("case", ["reference_preset", "stock_two_radii", "plain_two_radii"])
def test_gc_full_steps(gpu_lib, oracle_lib, case):
    # whole steps (the step's fused walks and cached weights) against the oracle, from
    # the same state each step; both solve the PPE tightly
    s = GC_CASES[case]()
    gpu, cpu = make_pair(s, s.params(eps=1e-13))
    for k in range(4):
        copy_state(cpu, gpu)
        gpu.forward_time(s.meta["dt"])
        cpu.forward_time(s.meta["dt"])
        G, C = gpu.particles(), cpu.particles()
        np.testing.assert_array_equal(G["type"], C["type"])
        assert rel_err(G["p"], C["p"]) <= 1e-10, (case, k)
        assert rel_err(G["x"], C["x"]) <= 1e-12, (case, k)
        assert rel_err(G["z"], C["z"]) <= 1e-12, (case, k)


# ------------------------------------------------------------- explicit pressure
def _explicit(scene, gc=False):
    s = _with_flags(scene, abi.FLAG_PRESSURE_EXPLICIT | (abi.FLAG_GC if gc else 0))
    s.meta["params"]["sound_speed"] = SOUND_SPEED
    s.meta["dt"] = 0.1 * s.l0 / SOUND_SPEED
    return s


EXPLICIT_CASES = {
    "stock_two_radii": lambda: _explicit(stock_tank()),
    "stock_two_radii_gc": lambda: _explicit(stock_tank(), gc=True),
    "reference_preset": lambda: _explicit(reference_tank()),
    "plain_two_radii": lambda: _explicit(plain_tank()),
    "plain_two_radii_ds": lambda: _explicit(plain_tank(ds=True)),
    "jittered_plain_gc": lambda: _explicit(jittered_tank(jitter=0.1), gc=True),
}


def _assert_bitwise(gpu, cpu, what):
    assert_same_particles(gpu, cpu, what=what)
    ga, ca = gpu.aux(), cpu.aux()
    for k in ("n_without_spp", "ecs", "ox", "oz"):
        np.testing.assert_array_equal(ga[k], ca[k], err_msg="%s %s" % (k, what))


@pytest.mark.parametrize("case", sorted(EXPLICIT_CASES))
def test_explicit_trajectory_bitwise(gpu_lib, oracle_lib, case):
    s = EXPLICIT_CASES[case]()
    gpu, cpu = make_pair(s, s.params())
    for k in range(12):
        gpu.forward_time(s.meta["dt"])
        cpu.forward_time(s.meta["dt"])
    _assert_bitwise(gpu, cpu, case)
    p = gpu.particles()["p"]
    assert np.all(p >= 0) and np.max(p) > 0
    st = gpu.stats()
    assert st["steps"] == 12 and st["cg_iterations"] == 0


def test_explicit_cfl_time_step(gpu_lib, oracle_lib):
    # MaxDt = min(maxDt, courant l0 / c) (Environment.hpp:135) and DetermineDt on top
    s = EXPLICIT_CASES["stock_two_radii"]()
    gpu, cpu = make_pair(s, s.params())
    env = gpu.environment()
    assert env.max_dt == min(s.meta["params"]["max_dt"], (0.1 * s.l0) / SOUND_SPEED)
    assert env.max_dt == cpu.environment().max_dt
    for _ in range(4):
        gpu.forward_time(None)
        cpu.forward_time(-1.0)
        assert gpu.environment().dt == cpu.environment().dt
    _assert_bitwise(gpu, cpu, "cfl")


def test_explicit_pressure_formula(gpu_lib, oracle_lib):
    # p = c^2 (rho0 / n0 n - rho0) where positive, for every particle, from the second
    # number density (restated here in numpy)
    s = EXPLICIT_CASES["plain_two_radii"]()
    gpu, _ = make_pair(s, s.params())
    for _ in range(3):
        gpu.forward_time(s.meta["dt"])
    P = gpu.particles()
    env = gpu.environment()
    rho0 = s.meta["params"]["rho"]
    rho = rho0 / env.n0 * P["n"]
    expect = np.where(rho <= rho0, 0.0, SOUND_SPEED * SOUND_SPEED * (rho - rho0))
    np.testing.assert_array_equal(P["p"], expect)


def test_explicit_stage_hooks(gpu_lib, oracle_lib):
    # the stage chain of an explicit step: no PPE entry points, the pressure stage
    # computes the explicit pressure; bit-identical to the oracle and to forward_time
    from openmps_gb300.computer import ComputerError

    s = EXPLICIT_CASES["stock_two_radii_gc"]()
    prm = s.params()
    gpu, cpu = make_pair(s, prm)
    step, _ = make_pair(s, prm)
    for _ in range(2):
        cpu.forward_time(s.meta["dt"])
    copy_state(cpu, gpu)
    copy_state(cpu, step)
    for h in (gpu, cpu):
        h.begin_step(s.meta["dt"])
    for name in ("search_neighbor", "density", "error_correction", "explicit", "density", "save_x",
                 "assign_pressure", "pressure_gradient", "dynamic_stabilize"):
        for h in (gpu, cpu):
            h.stage(name)
        assert_same_particles(gpu, cpu, what=name)
    step.forward_time(s.meta["dt"])
    assert_same_particles(step, gpu, what="forward_time")
    for name in ("set_ppe", "solve_ppe"):
        with pytest.raises(ComputerError) as e:
            gpu.stage(name)
        assert e.value.code == abi.MPS_ERR_STATE


def test_explicit_needs_sound_speed(gpu_lib):
    from openmps_gb300.computer import Computer, ComputerError

    s = stock_tank()
    with pytest.raises(ComputerError) as e:
        Computer(s.params(flags=abi.PRESET_REFERENCE | abi.FLAG_PRESSURE_EXPLICIT, sound_speed=0.0))
    assert e.value.code == abi.MPS_ERR_INVALID_ARGUMENT


def test_explicit_batch_matches_oracle(gpu_lib, oracle_lib):
    # a batch of uneven scenes with the explicit pressure: no solve, the stages alone,
    # captured and replayed as one graph; each scene bit-identical to its own oracle
    from openmps_gb300.computer import Batch
    from oracle.oracle import Oracle

    l0 = 5e-3
    sc = []
    for k in range(3):
        s = scenes.batch_scene(k, seed=11, l0=l0)
        s.meta["params"] = dict(scenes.STOCK_PHYSICS, max_dt=1.0, sound_speed=SOUND_SPEED,
                                flags=abi.PRESET_REFERENCE | abi.FLAG_PRESSURE_EXPLICIT | abi.FLAG_GC)
        sc.append(s)
    dt = 0.1 * l0 / SOUND_SPEED
    b = Batch(sc[0].params(), sc)
    b.forward(dt, 1)
    b.forward(dt, 3)
    for k, s in enumerate(sc):
        o = Oracle(s.params())
        o.add_scene(s)
        for _ in range(4):
            o.forward_time(dt)
        P, Q = b.scene(k), o.particles()
        for f in ("type", "x", "z", "u", "w", "p", "n"):
            np.testing.assert_array_equal(P[f], Q[f], err_msg="scene %d %s" % (k, f))


# ------------------------------------------------------------- central gravity
def _central(scene, dx, dz):
    """The scene moved by (dx, dz) around the origin, with the fluid particle nearest to it
    placed exactly at the origin (the c = 0 branch)."""
    s = scene
    s.x = s.x + dx
    s.z = s.z + dz
    s.min_x += dx
    s.max_x += dx
    s.min_z += dz
    s.max_z += dz
    fluid = np.flatnonzero(s.type == abi.TYPE_FLUID)
    k = fluid[np.argmin(s.x[fluid] ** 2 + s.z[fluid] ** 2)]
    s.x[k] = 0.0
    s.z[k] = 0.0
    s = _explicit(_with_flags(s, abi.FLAG_CENTRAL_GRAVITY))
    return s


def test_central_gravity_2d(gpu_lib, oracle_lib):
    # CENTRAL_GRAVITY (Computer.hpp:925-932, :981-988) through the step's fused walk and
    # through the stage hooks, both bit-identical to the oracle
    s = _central(stock_tank(), -0.1, -0.2)
    gpu, cpu = make_pair(s, s.params())
    hooks, _ = make_pair(s, s.params())
    for _ in range(6):
        gpu.forward_time(s.meta["dt"])
        cpu.forward_time(s.meta["dt"])
        hooks.begin_step(s.meta["dt"])
        for name in ("search_neighbor", "density", "error_correction", "explicit", "density", "save_x",
                     "assign_pressure", "pressure_gradient", "dynamic_stabilize"):
            hooks.stage(name)
    _assert_bitwise(gpu, cpu, "central gravity")
    assert_same_particles(hooks, cpu, what="central gravity, stage hooks")
    # gravity points to the origin: the fluid above it moves down, the fluid below it up
    P = gpu.particles()
    f = P["type"] == abi.TYPE_FLUID
    assert np.mean(P["w"][f & (P["z"] > 0.05)]) < 0 < np.mean(P["w"][f & (P["z"] < -0.05)])


def test_central_gravity_3d(gpu_lib, oracle_lib):
    from openmps_gb300.computer import Computer
    from oracle.oracle import Oracle3

    s = scenes.tank3d(0.01, (6, 5, 8), (14, 8, 12))
    off = (-0.03, -0.02, -0.04)
    s.x, s.y, s.z = s.x + off[0], s.y + off[1], s.z + off[2]
    b = s.bounds
    s.bounds = (b[0] + off[0], b[1] + off[1], b[2] + off[2], b[3] + off[0], b[4] + off[1], b[5] + off[2])
    fluid = np.flatnonzero(s.type == abi.TYPE_FLUID)
    k = fluid[np.argmin(s.x[fluid] ** 2 + s.y[fluid] ** 2 + s.z[fluid] ** 2)]
    s.x[k] = s.y[k] = s.z[k] = 0.0
    s.meta["params"] = dict(scenes.STOCK_PHYSICS, re_lap_by_l0=0.0, max_dt=1.0, sound_speed=SOUND_SPEED,
                            flags=abi.PRESET_REFERENCE | abi.FLAG_PRESSURE_EXPLICIT | abi.FLAG_CENTRAL_GRAVITY)
    prm = s.params()
    gpu = Computer(prm)
    gpu.add_particles3(*s.arrays3())
    cpu = Oracle3(prm)
    cpu.add_scene(s)
    dt = 0.1 * s.l0 / SOUND_SPEED
    for _ in range(6):
        gpu.forward_time(dt)
        cpu.forward_time(dt)
    G, C = gpu.particles3(), cpu.particles()
    for f in ("type", "x", "y", "z", "u", "v", "w", "p", "n"):
        np.testing.assert_array_equal(G[f], C[f], err_msg=f)
