"""Seeded scene generators: reproducible layouts with the documented particle counts."""
import numpy as np

from openmps_gb300 import _abi as abi
from openmps_gb300 import scenes


def test_splitmix64_vector():
    # SplitMix64 from state 0 (Steele, Lea & Flood 2014): published first outputs
    out = scenes.splitmix64(0, 3)
    assert [int(v) for v in out] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]
    u = scenes.uniform01(20261203, 1000)
    assert u.min() >= 0.0 and u.max() < 1.0 and abs(u.mean() - 0.5) < 0.05


def test_dam_break_counts():
    c0 = scenes.config_c0()
    assert c0.counts() == {"fluid": 800, "wall": 618, "dummy": 432}
    c2 = scenes.config_c2()
    assert c2.counts()["fluid"] == 320000 and c2.count == 340050
    assert c2.params().flags == abi.PRESET_REFERENCE
    # one radius, 4.0 l0: the Laplacian radius of the workload (about 45 PPE nonzeros a row)
    assert c2.params().re_by_l0 == 4.0 and c2.params().re_lap_by_l0 == 0.0


def test_hydrostatic_jitter_is_seeded():
    a = scenes.hydrostatic(l0=0.01, width=0.2, depth=0.1)
    b = scenes.hydrostatic(l0=0.01, width=0.2, depth=0.1)
    np.testing.assert_array_equal(a.x, b.x)
    fluid = a.type == abi.TYPE_FLUID
    dev = np.abs(a.x[fluid] / 0.01 - np.round(a.x[fluid] / 0.01))
    assert 0 < dev.max() <= 1e-4


def test_batch_scenes_ranges():
    for k in range(16):
        s = scenes.batch_scene(k)
        f = s.counts()["fluid"]
        assert 800 <= f <= 6000, f
        assert s.meta["water_w"] <= 0.3 + 1e-9 and s.meta["water_h"] <= 0.5 + 1e-9
