"""Moving walls: the positionWall targets of the non-fluid particles (Computer.hpp:995-1020),
set before each step through mps_set_wall_positions(3), against the oracle.

Each step moves the right-hand wall and dummy layers of the tank by a prescribed
displacement; the explicit step puts every non-fluid particle at its target and gives
it the velocity (target - position) / dt.  With the explicit pressure the whole step is
deterministic, so the trajectories must match the oracle bit for bit, in 2D and in 3D.
"""
import numpy as np
import pytest

from helpers import make_pair, stock_tank
from openmps_gb300 import _abi as abi
from openmps_gb300 import scenes

pytestmark = pytest.mark.gpu

C = 27.5


def _targets(x0, moving, t, amplitude):
    """Wall targets at time t: the moving particles displaced by amplitude sin(40 t)."""
    return np.where(moving, x0 + amplitude * np.sin(40.0 * t), x0)


def test_moving_walls_2d(gpu_lib, oracle_lib):
    s = stock_tank()
    s.meta["params"] = dict(s.meta["params"], sound_speed=C,
                            flags=abi.PRESET_REFERENCE | abi.FLAG_PRESSURE_EXPLICIT)
    dt = 0.1 * s.l0 / C
    gpu, cpu = make_pair(s, s.params())
    moving = (s.type != abi.TYPE_FLUID) & (s.x > 0.5)
    for k in range(8):
        wx = _targets(s.x, moving, (k + 1) * dt, 2e-3)
        for h in (gpu, cpu):
            h.set_wall_positions(wx, s.z)
            h.forward_time(dt)
        G, P = gpu.particles(), cpu.particles()
        for f in ("type", "x", "z", "u", "w", "p", "n"):
            np.testing.assert_array_equal(G[f], P[f], err_msg="step %d %s" % (k, f))
        np.testing.assert_array_equal(G["x"][moving], wx[moving])
    assert np.max(np.abs(G["u"][moving])) > 0  # the walls carry the prescribed velocity


def test_moving_walls_3d(gpu_lib, oracle_lib):
    from openmps_gb300.computer import Computer
    from oracle.oracle import Oracle3

    s = scenes.tank3d(0.01, (6, 5, 8), (14, 8, 12))
    s.meta["params"] = dict(scenes.STOCK_PHYSICS, re_lap_by_l0=0.0, max_dt=1.0, sound_speed=C,
                            flags=abi.PRESET_REFERENCE | abi.FLAG_PRESSURE_EXPLICIT)
    dt = 0.1 * s.l0 / C
    prm = s.params()
    gpu = Computer(prm)
    gpu.add_scene(s)
    cpu = Oracle3(prm)
    cpu.add_scene(s)
    moving = (s.type != abi.TYPE_FLUID) & (s.y > 0.07)  # the back wall moves along y
    for k in range(8):
        wy = _targets(s.y, moving, (k + 1) * dt, 2e-3)
        gpu.set_wall_positions3(s.x, wy, s.z)
        cpu.set_wall_positions(s.x, wy, s.z)
        gpu.forward_time(dt)
        cpu.forward_time(dt)
        G, P = gpu.particles3(), cpu.particles()
        for f in ("type", "x", "y", "z", "u", "v", "w", "p", "n"):
            np.testing.assert_array_equal(G[f], P[f], err_msg="step %d %s" % (k, f))
        np.testing.assert_array_equal(G["y"][moving], wy[moving])
    assert np.max(np.abs(G["v"][moving])) > 0
