"""Failure paths of the GPU step (made on the host; nothing faults the GPU).

* A cell holding more than maxPerCell particles is the reference's
  "Too many particle in a block" (src/OpenMps/Grid.hpp:314-318).
* A CG that cannot reach its tolerance within the iteration limit is the reference's
  "Conjugate Gradient method couldn't solve ..." (src/OpenMps/Computer.hpp:1424-1428).
The handle stays usable after either error.
"""
import numpy as np
import pytest

from helpers import jittered_tank, plain_tank
from openmps_gb300 import _abi as abi
from openmps_gb300.computer import Computer, ComputerError

pytestmark = pytest.mark.gpu


def test_cell_overflow(gpu_lib):
    s = jittered_tank()
    s.x[:50] = 0.05  # 50 particles in one cell (maxPerCell is 36 at r_lap = 4 l0)
    s.z[:50] = 0.05 + np.arange(50) * 1e-6
    c = Computer(s.params())
    c.add_scene(s)
    with pytest.raises(ComputerError) as e:
        c.forward_time(5e-4)
    assert e.value.code == abi.MPS_ERR_CELL_OVERFLOW
    # fix the state and keep going on the same handle
    fresh = jittered_tank()
    c.set_particles(fresh.type, fresh.x, fresh.z, fresh.u, fresh.w, fresh.p, fresh.n)
    c.forward_time(5e-4)


def test_cg_not_converged(gpu_lib):
    s = plain_tank()
    c = Computer(s.params(max_cg_iters=2, eps=1e-12))
    c.add_scene(s)
    with pytest.raises(ComputerError) as e:
        c.forward_time(5e-4)
    assert e.value.code == abi.MPS_ERR_CG_NOT_CONVERGED
    # the pressure was not assigned and positions not corrected by the gradient
    P = c.particles()
    assert np.all(P["p"] == 0.0)


def test_invalid_arguments(gpu_lib):
    with pytest.raises(ComputerError):
        Computer(abi.make_params(l0=0.0))
    c = Computer(abi.make_params())
    with pytest.raises(ComputerError):
        c.forward_time(1e-3)  # no particles yet
    with pytest.raises(ComputerError):
        c.add_particles(np.array([7]), np.zeros(1), np.zeros(1))  # bad type
