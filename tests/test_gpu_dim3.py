"""Three-dimensional scenes (DIM3) on the GPU against the 3D oracle.

Same bar as the 2D stages: neighbour lists, every per-particle stage and the PPE system
bit-identical; the PPE solve within the solver tolerance (the pressure is handed from
the GPU to the oracle before the stages after it); whole steps within the step
tolerances; explicit-pressure trajectories bit for bit.  A scene one layer thick in y
must reproduce the 2D path's neighbour lists and densities.
"""
import numpy as np
import pytest

from helpers import rel_err
from openmps_gb300 import _abi as abi
from openmps_gb300 import scenes
from test_oracle_dim3 import single_layer_pair

pytestmark = pytest.mark.gpu

DT = 5e-4
FIELDS = ("x", "y", "z", "u", "v", "w", "p", "n")


def _scene(flags=abi.PRESET_REFERENCE, re_by=2.1, re_lap=0.0, jitter=0.0, **kw):
    s = scenes.tank3d(0.01, (6, 5, 8), (14, 8, 12), jitter=jitter, seed=11)
    s.meta["params"] = dict(scenes.PLAIN_PHYSICS, flags=flags, re_by_l0=re_by, re_lap_by_l0=re_lap, eps=1e-10,
                            max_dt=DT, **kw)
    return s


CASES = {
    "stock": lambda: _scene(),
    "plain": lambda: _scene(flags=abi.PRESET_PLAIN),
    "plain_ds": lambda: _scene(flags=abi.FLAG_DS),
    "stock_two_radii": lambda: _scene(re_lap=3.0),
    "jittered_reference_24": lambda: _scene(re_by=2.4, jitter=0.1),
    "jittered_plain_gc": lambda: _scene(flags=abi.FLAG_GC, jitter=0.1),
    "jittered_stock_gc": lambda: _scene(flags=abi.PRESET_REFERENCE | abi.FLAG_GC, jitter=0.1),
}


def _pair(s, **kw):
    from openmps_gb300.computer import Computer
    from oracle.oracle import Oracle3

    prm = s.params(**kw)
    gpu = Computer(prm)
    gpu.add_particles3(*s.arrays3())
    cpu = Oracle3(prm)
    cpu.add_scene(s)
    return gpu, cpu


def _copy(cpu, gpu):
    P = cpu.particles()
    gpu.set_particles3(P["type"], *[P[k] for k in FIELDS])
    A = cpu.aux()
    gpu.set_aux3(A["n_without_spp"], A["ecs"], A["ox"], A["oy"], A["oz"])


def _same(gpu, cpu, what):
    G, C = gpu.particles3(), cpu.particles()
    np.testing.assert_array_equal(G["type"], C["type"], err_msg=what)
    for k in FIELDS:
        np.testing.assert_array_equal(G[k], C[k], err_msg="%s %s" % (k, what))


def _same_aux(gpu, cpu, what):
    G, C = gpu.aux3(), cpu.aux()
    for k in G:
        np.testing.assert_array_equal(G[k], C[k], err_msg="%s %s" % (k, what))


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("warm", [0, 2])
def test_stage_chain(gpu_lib, oracle_lib, case, warm):
    s = CASES[case]()
    gpu, cpu = _pair(s)
    flags = s.params().flags
    for _ in range(warm):
        cpu.forward_time(DT)
    _copy(cpu, gpu)
    for h in (gpu, cpu):
        h.begin_step(DT)
    for h in (gpu, cpu):
        h.stage("search_neighbor")
    gc, gl = gpu.neighbors()
    cc, cl = cpu.neighbors()
    np.testing.assert_array_equal(gc, cc)
    np.testing.assert_array_equal(gl, cl)
    for h in (gpu, cpu):
        h.stage("density")
    _same(gpu, cpu, "density")
    _same_aux(gpu, cpu, "density")
    np.testing.assert_array_equal(gpu.density_variation(), cpu.density_variation())
    names = (["error_correction"] if flags & abi.FLAG_ECS else []) + ["explicit", "density"]
    names += ["save_x"] if flags & abi.FLAG_DS else []
    for name in names:
        for h in (gpu, cpu):
            h.stage(name)
        _same(gpu, cpu, name)
        _same_aux(gpu, cpu, name)
    for h in (gpu, cpu):
        h.stage("set_ppe")
    for a, b, what in zip(gpu.ppe(), cpu.ppe(), ("row_ptr", "columns", "values", "rhs", "guess")):
        np.testing.assert_array_equal(a, b, err_msg="PPE %s" % what)
    for name in ("solve_ppe", "assign_pressure"):
        for h in (gpu, cpu):
            h.stage(name)
    gp, cp = gpu.particles3()["p"], cpu.particles()["p"]
    assert np.max(np.abs(gp - cp)) <= 1e-6 * max(np.max(np.abs(cp)), 1.0)
    cpu.set_particles(p=gp)
    names = ["pressure_gradient"] + (["dynamic_stabilize"] if flags & abi.FLAG_DS else [])
    for name in names:
        for h in (gpu, cpu):
            h.stage(name)
        _same(gpu, cpu, name)


@pytest.mark.parametrize("case", ["stock", "plain", "stock_two_radii", "jittered_stock_gc"])
@pytest.mark.parametrize("solver", [abi.SOLVER_CG64, abi.SOLVER_MIXED])
def test_full_steps(gpu_lib, oracle_lib, case, solver):
    s = CASES[case]()
    gpu, cpu = _pair(s, eps=1e-13, solver=solver)
    for k in range(3):
        _copy(cpu, gpu)
        gpu.forward_time(DT)
        cpu.forward_time(DT)
        G, C = gpu.particles3(), cpu.particles()
        np.testing.assert_array_equal(G["type"], C["type"])
        assert rel_err(G["p"], C["p"]) <= 1e-10, (case, k)
        for f in ("x", "y", "z"):
            assert rel_err(G[f], C[f]) <= 1e-12, (case, k, f)
    assert gpu.stats()["cg_iterations"] > 0


@pytest.mark.parametrize("gc", [False, True])
def test_explicit_pressure_trajectory(gpu_lib, oracle_lib, gc):
    c = 20.0
    s = _scene(flags=abi.PRESET_REFERENCE | abi.FLAG_PRESSURE_EXPLICIT | (abi.FLAG_GC if gc else 0),
               sound_speed=c, jitter=0.05)
    gpu, cpu = _pair(s)
    dt = 0.1 * s.l0 / c
    for _ in range(8):
        gpu.forward_time(dt)
        cpu.forward_time(dt)
    _same(gpu, cpu, "explicit trajectory")
    _same_aux(gpu, cpu, "explicit trajectory")
    assert np.max(gpu.particles3()["p"]) > 0


def test_cfl_steps(gpu_lib, oracle_lib):
    s = _scene(jitter=0.1)
    gpu, cpu = _pair(s, eps=1e-13)
    for _ in range(3):
        _copy(cpu, gpu)
        gpu.forward_time(None)
        cpu.forward_time(-1.0)
        assert gpu.environment().dt == cpu.environment().dt
        assert gpu.environment().t == cpu.environment().t


def test_gc_gradient_from_given_pressure(gpu_lib, oracle_lib):
    s = _scene(flags=abi.PRESET_REFERENCE | abi.FLAG_GC, jitter=0.1)
    gpu, cpu = _pair(s)
    cpu.set_particles(p=np.random.default_rng(4).uniform(0.0, 500.0, s.count))
    _copy(cpu, gpu)
    for h in (gpu, cpu):
        h.begin_step(DT)
    for name in ("search_neighbor", "density", "pressure_gradient"):
        for h in (gpu, cpu):
            h.stage(name)
        _same(gpu, cpu, name)


def test_single_layer_equals_2d_path(gpu_lib, oracle_lib):
    from openmps_gb300.computer import Computer

    s2, s3 = single_layer_pair()
    g2 = Computer(s2.params())
    g2.add_scene(s2)
    g3 = Computer(s3.params())
    g3.add_particles3(*s3.arrays3())
    for g in (g2, g3):
        g.begin_step(DT)
        g.stage("search_neighbor")
        g.stage("density")
    c2, l2 = g2.neighbors()
    c3, l3 = g3.neighbors()
    np.testing.assert_array_equal(c3, c2)
    np.testing.assert_array_equal(l3, l2)
    np.testing.assert_array_equal(g3.particles3()["n"], g2.particles()["n"])


def test_environment_and_errors(gpu_lib, oracle_lib):
    from openmps_gb300.computer import Batch, Computer, ComputerError

    s = _scene()
    gpu, cpu = _pair(s)
    e, f = gpu.environment(), cpu.environment()
    for k in ("n0", "lambda_", "max_dt", "neighbor_length", "grid_nx", "grid_ny", "grid_nz", "grid_max_per_cell",
              "dim"):
        assert getattr(e, k) == getattr(f, k), k
    with pytest.raises(ComputerError) as err:
        gpu.particles()  # the 2D call on a 3D handle
    assert err.value.code == abi.MPS_ERR_STATE
    with pytest.raises(ComputerError) as err:
        Computer(s.params(solver=abi.SOLVER_MIXED_MG))
    assert err.value.code == abi.MPS_ERR_NOT_SUPPORTED
    with pytest.raises(ComputerError) as err:  # switching an existing 3D handle
        gpu.set_solver(abi.SOLVER_LEARNED, abi.CRIT_RHS, 1e-8)
    assert err.value.code == abi.MPS_ERR_NOT_SUPPORTED
    assert gpu.lib.mps_learned_collect(gpu.h, 1) == abi.MPS_ERR_NOT_SUPPORTED
    with pytest.raises(ComputerError) as err:
        Batch(s.params(), [scenes.batch_scene(0)])
    assert err.value.code == abi.MPS_ERR_NOT_SUPPORTED


# ------------------------------------------------------------------ failures
def test_cell_overflow_and_recovery(gpu_lib, oracle_lib):
    from openmps_gb300.computer import ComputerError
    from oracle.oracle import OracleError

    s = _scene()
    bad = s.copy()
    bad.x[:80] = 0.021  # 80 particles in one cell (maxPerCell is 64 at r_e = 2.1 l0)
    bad.y[:80] = 0.021
    bad.z[:80] = 0.021 + np.arange(80) * 1e-6
    gpu, cpu = _pair(bad)
    with pytest.raises(ComputerError) as e:
        gpu.forward_time(DT)
    assert e.value.code == abi.MPS_ERR_CELL_OVERFLOW
    with pytest.raises(OracleError) as e:
        cpu.forward_time(DT)
    assert e.value.code == abi.MPS_ERR_CELL_OVERFLOW
    gpu.set_particles3(*s.arrays3())  # the handle stays usable
    gpu.forward_time(DT)


def test_out_of_domain_disabled(gpu_lib, oracle_lib):
    s = _scene()
    s.y[3] = 5.0  # beyond maxY: Grid::Store fails, the particle is disabled (Computer.hpp:710-715)
    s.x[4] = -7.0
    gpu, cpu = _pair(s, eps=1e-13)
    gpu.forward_time(DT)
    cpu.forward_time(DT)
    G, C = gpu.particles3(), cpu.particles()
    assert G["type"][3] == abi.TYPE_DISABLED and G["type"][4] == abi.TYPE_DISABLED
    np.testing.assert_array_equal(G["type"], C["type"])
    assert gpu.stats()["disabled"] == 2


def test_neighbor_row_overflow_is_an_error(gpu_lib):
    from openmps_gb300.computer import Computer, ComputerError
    from test_oracle_dim3 import packed_cluster

    s = packed_cluster()
    gpu = Computer(s.params())
    gpu.add_particles3(*s.arrays3())
    gpu.begin_step(DT)
    with pytest.raises(ComputerError) as e:
        gpu.stage("search_neighbor")
    assert e.value.code == abi.MPS_ERR_DEVICE_CHECK


def test_cg_not_converged(gpu_lib):
    from openmps_gb300.computer import Computer, ComputerError

    s = _scene()
    c = Computer(s.params(max_cg_iters=2, eps=1e-12))
    c.add_particles3(*s.arrays3())
    with pytest.raises(ComputerError) as e:
        c.forward_time(DT)
    assert e.value.code == abi.MPS_ERR_CG_NOT_CONVERGED
    assert np.all(c.particles3()["p"] == 0.0)
