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


def _wait_limit_case(solver, launch):
    from helpers import stock_tank
    from openmps_gb300 import learned

    s = stock_tank()
    c = Computer(s.params(eps=1e-10, solver=solver, criterion=abi.CRIT_RHS, cg_launch=launch))
    if solver == abi.SOLVER_LEARNED:
        c.learned_set_weights(learned.load())
    c.add_scene(s)
    c.forward_time(s.meta["dt"])  # one ordinary step first
    return s, c


@pytest.mark.parametrize("which", ["mma", "barrier"])
def test_bounded_wait_runs_out(gpu_lib, which):
    # A wait bound of 0 cycles makes every tensor-core completion wait (learned solve) or
    # every grid-barrier wait that is not already released (persistent solve) give up at
    # its first check.  The kernel records the timeout and returns (the tensor-core
    # kernel first waits, bounded, for the MMAs it issued, then frees TMEM); the step
    # completes without the part that waited and the call reports MPS_ERR_TIMEOUT.
    # With the default bounds restored the same handle steps normally.
    if which == "mma":
        s, c = _wait_limit_case(abi.SOLVER_LEARNED, abi.CG_LAUNCH_GRAPH)
        c.set_wait_limits(mma_clocks=0)
    else:
        s, c = _wait_limit_case(abi.SOLVER_MIXED_MG, abi.CG_LAUNCH_PERSISTENT)
        c.set_wait_limits(barrier_clocks=0)
    t0 = c.environment().t
    with pytest.raises(ComputerError) as e:
        c.forward_time(s.meta["dt"])
    assert e.value.code == abi.MPS_ERR_TIMEOUT, e.value
    st = c.stats()
    # the step finished: time advanced and the FP64 true residual meets the tolerance
    assert c.environment().t > t0
    assert st["cg_true_relres"] <= 1e-10
    if which == "barrier":
        assert st["fallback"] == 1
    P = c.particles()
    assert all(np.all(np.isfinite(P[k])) for k in ("x", "z", "u", "w", "p"))
    c.set_wait_limits()
    for _ in range(2):
        c.forward_time(s.meta["dt"])
    st = c.stats()
    assert st["fallback"] == 0 and st["cg_true_relres"] <= 1e-10
