"""The reference's own input states as test cases (tests/golden/, written by
make_reference_fixtures.py from Benchmark/Sample/Sample.xml and src/OpenMps/particles.csv).

* the oracle reads the sample's environment as the reference does: n0 at r_e = 2.4 l0
  is 9.774726 (Environment.hpp:163-215), and the particles the sample places beyond maxX
  stay inside the grid's margin cells (Grid.hpp:137-150), so none is disabled;
* the driver reads an input in the sample's layout, minY = maxY = 0 included, as 2D;
* on the GPU, every stage of a step from these states is bit-identical to the oracle.
"""
import os
import subprocess

import numpy as np
import pytest

from helpers import assert_same_neighbors, assert_same_particles, assert_same_ppe, copy_state, make_pair
from openmps_gb300 import _abi as abi
from openmps_gb300 import build, scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def sample_scene():
    """Sample.xml: its environment, its particles, the stock method set."""
    d = _load("reference_sample.npz")
    env = {str(k): float(v) for k, v in zip(d["env_keys"], d["env_values"])}
    g = lambda k: env["environment." + k]
    n = d["x"].size
    s = scenes.Scene(name="reference_sample", type=d["Type"].astype(np.int32), x=d["x"].copy(), z=d["z"].copy(),
                     u=d["u"].copy(), w=d["w"].copy(), p=d["p"].copy(), n=d["n"].copy(), l0=g("l_0"),
                     min_x=g("minX"), min_z=g("minZ"), max_x=g("maxX"), max_z=g("maxZ"))
    assert n == 1323
    s.meta["params"] = dict(max_dt=env["condition.outputInterval"] / g("minStepCountPerOutput"), courant=g("courant"),
                            g=g("g"), rho=g("rho"), nu=g("nu"), surface_ratio=g("surfaceRatio"),
                            re_by_l0=g("r_eByl_0"), re_lap_by_l0=0.0, eps=env["condition.eps"],
                            flags=abi.PRESET_REFERENCE)
    s.meta["dt"] = s.meta["params"]["max_dt"]
    s.meta["env"] = env
    return s


def particles_csv_scene():
    """src/OpenMps/particles.csv (l0 = 0.001 m) in a domain spanning its particles, with
    the sample's constants."""
    d = _load("reference_particles_csv.npz")
    s = scenes.Scene(name="reference_particles_csv", type=d["Type"].astype(np.int32), x=d["x"].copy(),
                     z=d["z"].copy(), u=d["u"].copy(), w=d["w"].copy(), p=d["p"].copy(), n=d["n"].copy(), l0=0.001,
                     min_x=-0.004, min_z=-0.004, max_x=0.104, max_z=0.2)
    assert s.count == 8016
    s.meta["params"] = dict(max_dt=1e-4, courant=0.1, g=9.8, rho=998.2, nu=1.004e-6, surface_ratio=0.97,
                            re_by_l0=2.4, re_lap_by_l0=0.0, eps=1e-10, flags=abi.PRESET_REFERENCE)
    s.meta["dt"] = 1e-4
    return s


def test_sample_environment_and_steps(oracle_lib):
    from oracle.oracle import Oracle

    s = sample_scene()
    o = Oracle(s.params())
    o.add_scene(s)
    assert o.environment().n0 == pytest.approx(9.774726, abs=5e-7)
    assert np.max(s.x) > s.max_x  # particles beyond maxX, inside the margin cells
    for _ in range(2):
        o.forward_time(s.meta["dt"])
    P = o.particles()
    assert np.all(P["type"] != abi.TYPE_DISABLED)
    assert np.all(np.isfinite(P["p"])) and np.max(P["p"]) > 0


def test_driver_reads_sample_layout_as_2d(tmp_path):
    from test_driver import write_case

    build.build()
    s = sample_scene()
    env = s.meta["env"]
    xml = tmp_path / "sample.xml"
    write_case(xml, s, end=env["condition.endTime"], interval=env["condition.outputInterval"],
               eps=env["condition.eps"], steps_per_output=int(env["environment.minStepCountPerOutput"]),
               extra='    <minY value="-0.000" />\n    <maxY value=" 0.000" />\n    <c value="1.5" />\n')
    out = subprocess.run([build.DRIVER, str(xml), "--parse-only"], capture_output=True, text=True, cwd=tmp_path)
    assert out.returncode == 0, out.stderr
    assert "1323 particles" in out.stdout
    kv = dict(item.split("=", 1) for item in out.stdout.strip().splitlines()[-1].split()
              if "=" in item and not item.startswith(("min=", "max=")))
    assert int(kv["dim"]) == 2
    assert float(kv["maxDt"]) == 0.005 / 10


CASES = {"sample_xml": sample_scene, "particles_csv": particles_csv_scene}


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("warm", [0, 2])
def test_stage_chain_from_reference_states(gpu_lib, oracle_lib, case, warm):
    s = CASES[case]()
    prm = s.params()
    gpu, cpu = make_pair(s, prm)
    dt = s.meta["dt"]
    for _ in range(warm):
        cpu.forward_time(dt)
    copy_state(cpu, gpu)
    for h in (gpu, cpu):
        h.begin_step(dt)
    for h in (gpu, cpu):
        h.stage("search_neighbor")
    assert_same_neighbors(gpu, cpu, case)
    for name in ("density", "error_correction", "explicit", "density", "save_x"):
        for h in (gpu, cpu):
            h.stage(name)
        assert_same_particles(gpu, cpu, what="%s %s" % (case, name))
    for h in (gpu, cpu):
        h.stage("set_ppe")
    assert_same_ppe(gpu, cpu, case)
    for name in ("solve_ppe", "assign_pressure"):
        for h in (gpu, cpu):
            h.stage(name)
    cpu.set_particles(p=gpu.particles()["p"])
    for name in ("pressure_gradient", "dynamic_stabilize"):
        for h in (gpu, cpu):
            h.stage(name)
        assert_same_particles(gpu, cpu, what="%s %s" % (case, name))
