"""Neighbour search on the GPU against the oracle: bit-exact lists, same order.

The reference builds each list by walking the nine cells around a particle in a
fixed order and each cell in insertion (ascending index) order
(src/OpenMps/Computer.hpp:698-756, src/OpenMps/Grid.hpp:276-559).  The GPU list
must be identical element for element, including which particles end up
disabled because they left the domain.
"""
import numpy as np
import pytest

from helpers import (assert_same_neighbors, far_tank, jittered_tank, make_pair, plain_tank,
                     reference_tank, threshold_rings)
from openmps_gb300 import _abi as abi
from openmps_gb300 import scenes

pytestmark = pytest.mark.gpu


def _search_both(gpu, cpu):
    gpu.stage("search_neighbor")
    cpu.stage("search_neighbor")
    np.testing.assert_array_equal(gpu.particles()["type"], cpu.particles()["type"])
    assert_same_neighbors(gpu, cpu)


def test_unit_lattice(gpu_lib, oracle_lib):
    # the reference's number-density fixture: 7 x 7 lattice, l0 = 0.1, r_e = 2.1 l0
    b = (-0.004, -0.004, 0.053, 0.1)
    s = scenes.lattice(7, 7, 0.1, b)
    prm = abi.make_params(l0=0.1, re_by_l0=2.1, min_x=b[0], min_z=b[1], max_x=b[2], max_z=b[3],
                          max_dt=0.01)
    gpu, cpu = make_pair(s, prm)
    _search_both(gpu, cpu)
    counts, _ = gpu.neighbors()
    assert counts.reshape(7, 7)[3, 3] == 20


@pytest.mark.parametrize("maker", [plain_tank, reference_tank, jittered_tank, far_tank, threshold_rings])
def test_tanks(gpu_lib, oracle_lib, maker):
    s = maker()
    gpu, cpu = make_pair(s, s.params())
    _search_both(gpu, cpu)


def test_after_oracle_steps(gpu_lib, oracle_lib):
    # a moved (non-lattice) state: run the oracle, hand its state to the GPU
    from helpers import copy_state

    s = jittered_tank(jitter=0.2, seed=11)
    gpu, cpu = make_pair(s, s.params())
    for _ in range(5):
        cpu.forward_time(s.meta["dt"])
    copy_state(cpu, gpu)
    _search_both(gpu, cpu)


def test_out_of_domain_particles_are_disabled(gpu_lib, oracle_lib):
    s = jittered_tank()
    # push a few fluid particles out of the grid (beyond the +2 guard cells) and one to NaN
    s.x[0] = s.max_x + 10.0
    s.z[1] = s.min_z - 10.0
    s.x[2] = np.nan
    s.type[3] = abi.TYPE_DISABLED
    gpu, cpu = make_pair(s, s.params())
    _search_both(gpu, cpu)
    t = gpu.particles()["type"]
    assert (t[:4] == abi.TYPE_DISABLED).all()
    assert gpu.stats()["disabled"] == 4


def test_empty_cells_and_single_particle(gpu_lib, oracle_lib):
    # ragged input: one fluid particle alone in a large domain
    s = scenes.lattice(1, 1, 0.01, (-0.1, -0.1, 0.1, 0.1))
    prm = abi.make_params(l0=0.01, re_by_l0=2.1, min_x=-0.1, min_z=-0.1, max_x=0.1, max_z=0.1)
    gpu, cpu = make_pair(s, prm)
    _search_both(gpu, cpu)
    assert gpu.neighbors()[0][0] == 0


def test_config_c2_full_size(gpu_lib, oracle_lib):
    # the 340k-particle 320k-fluid dam break: bit-exact at full size
    s = scenes.config_c2()
    gpu, cpu = make_pair(s, s.params())
    _search_both(gpu, cpu)
    st = gpu.stats()
    assert st["disabled"] == 0
