"""Batched scenes (mps_batch_*): independent uneven dam breaks advanced together.

Each scene of a batch must behave as its own single-scene Computer: identical neighbour
lists after the search (bit for bit, up to the row offset of the scene), the same
pressure and motion as the single-scene multigrid solver (both solve the PPE to the
same residual), every scene converged, and graph-replayed steps identical to eager ones.
"""
import numpy as np
import pytest

from helpers import rel_err
from openmps_gb300 import _abi as abi
from openmps_gb300 import scenes
from openmps_gb300.computer import Batch, Computer

pytestmark = pytest.mark.gpu

L0 = 5e-3
DT = L0 / 20.0


def batch_scenes(n, seed=20261203):
    out = []
    for k in range(n):
        s = scenes.batch_scene(k, seed=seed, l0=L0)
        s.meta["params"] = dict(scenes.STOCK_PHYSICS, eps=1e-8, max_dt=DT)
        out.append(s)
    return out


def params(s):
    return s.params(solver=abi.SOLVER_MIXED_MG, criterion=abi.CRIT_RHS, eps=1e-8)


def test_batch_matches_single_scenes(gpu_lib):
    sc = batch_scenes(5)
    assert len({s.count for s in sc}) > 1  # uneven
    b = Batch(params(sc[0]), sc)
    singles = []
    for s in sc:
        c = Computer(params(s))
        c.add_scene(s)
        singles.append(c)
    b.forward(DT, 1)
    # neighbour lists of step 1: bit-identical per scene
    bc, bl = b.neighbors()
    row0 = 0
    offs = []
    for k, (s, c) in enumerate(zip(sc, singles)):
        c.forward_time(DT)
        cc, cl = c.neighbors()
        pad = (s.count + 31) // 32 * 32
        start = int(np.sum(bc[:row0]))
        got = bl[start:start + int(np.sum(bc[row0:row0 + s.count]))] - row0
        np.testing.assert_array_equal(bc[row0:row0 + s.count], cc, err_msg="counts scene %d" % k)
        np.testing.assert_array_equal(got, cl, err_msg="lists scene %d" % k)
        offs.append(row0)
        row0 += pad
    for _ in range(4):
        b.forward(DT, 1)
        for c in singles:
            c.forward_time(DT)
    for k, (s, c) in enumerate(zip(sc, singles)):
        st = b.scene_stats(k)
        assert st["converged"] == 1 and st["true_relres"] <= 1e-8, st
        assert st["fallback"] == 0
        P, Q = b.scene(k), c.particles()
        np.testing.assert_array_equal(P["type"], Q["type"])
        assert rel_err(P["p"], Q["p"]) < 1e-5, k
        assert rel_err(P["x"], Q["x"], scale=L0) < 1e-6, k
        assert rel_err(P["z"], Q["z"], scale=L0) < 1e-6, k


def test_graph_replay_equals_eager_steps(gpu_lib):
    sc = batch_scenes(3, seed=5)
    a = Batch(params(sc[0]), sc)
    g = Batch(params(sc[0]), sc)
    for _ in range(4):
        a.forward(DT, 1)
    g.forward(DT, 4)
    assert a.stats()["steps"] == g.stats()["steps"] == 4
    for k in range(len(sc)):
        A, G = a.scene(k), g.scene(k)
        for key in ("x", "z", "u", "w", "p", "n"):
            np.testing.assert_array_equal(A[key], G[key], err_msg="%s scene %d" % (key, k))


def test_autotuner_reports_candidates(gpu_lib):
    sc = batch_scenes(6, seed=9)
    b = Batch(params(sc[0]), sc)
    b.forward(DT, 2)
    t = b.tuning()
    assert t["threads"] in (128, 256, 512, 1024)
    assert t["order"] in (0, 1)
    ms = [c["ms"] for c in t["candidates"]]
    assert len(ms) >= 4 and all(m > 0 for m in ms)
    best = min(t["candidates"], key=lambda c: c["ms"])
    assert (best["threads"], best["order"]) == (t["threads"], t["order"])


def test_batch_rejects_single_scene_calls(gpu_lib):
    sc = batch_scenes(2)
    b = Batch(params(sc[0]), sc)
    with pytest.raises(Exception):
        b.forward_time(DT)
    with pytest.raises(Exception):
        b.forward(-1.0, 1)


def test_batch_matches_oracle(gpu_lib, oracle_lib):
    # each scene of a batch against the oracle run as its own Computer: bit-identical
    # neighbour lists after the first search, and after five steps the same pressure and
    # motion as the oracle's FP64 CG to the same residual
    from oracle.oracle import Oracle

    sc = batch_scenes(4, seed=31)
    b = Batch(params(sc[0]), sc)
    cpus = []
    for s in sc:
        o = Oracle(s.params(criterion=abi.CRIT_RHS, eps=1e-8))
        o.add_scene(s)
        cpus.append(o)
    b.forward(DT, 1)
    bc, bl = b.neighbors()
    row0 = 0
    for k, (s, o) in enumerate(zip(sc, cpus)):
        o.forward_time(DT)
        cc, cl = o.neighbors()
        start = int(np.sum(bc[:row0]))
        got = bl[start:start + int(np.sum(bc[row0:row0 + s.count]))] - row0
        np.testing.assert_array_equal(bc[row0:row0 + s.count], cc, err_msg="counts scene %d" % k)
        np.testing.assert_array_equal(got, cl, err_msg="lists scene %d" % k)
        row0 += (s.count + 31) // 32 * 32
    for _ in range(4):
        b.forward(DT, 1)
        for o in cpus:
            o.forward_time(DT)
    for k, (s, o) in enumerate(zip(sc, cpus)):
        P, Q = b.scene(k), o.particles()
        np.testing.assert_array_equal(P["type"], Q["type"])
        ep = rel_err(P["p"], Q["p"])
        ex = max(rel_err(P["x"], Q["x"], scale=L0), rel_err(P["z"], Q["z"], scale=L0))
        print("batch scene %d (%d particles) vs oracle after 5 steps: p %.2e, x %.2e l0" % (k, s.count, ep, ex))
        assert ep < 1e-5 and ex < 1e-6, k
