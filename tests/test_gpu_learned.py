"""The learned PPE warm start and preconditioner scale on the GPU.

* the FP32 training kernels' loss and gradient equal the numpy FP64 oracle's;
* tensor-core inference (BF16 operands, FP32 accumulation) equals the oracle run with
  the same BF16 roundings;
* training on samples the FP64 CG generates lowers the loss;
* the learned solve reaches the requested residual (the FP64 true residual judges it)
  without the FP64 fallback, matches the plain solution, and its iteration count is
  compared with the same solve driven by a zero network.
"""
import numpy as np
import pytest

from helpers import rel_err
from oracle import mlp
from openmps_gb300 import _abi as abi
from openmps_gb300 import learned, scenes
from openmps_gb300.computer import Computer, mlp_infer, mlp_loss_grad, mlp_train

pytestmark = pytest.mark.gpu


def _random_case(seed, n):
    rng = np.random.default_rng(seed)
    mu = rng.standard_normal(16) * 0.2
    sd = 0.5 + rng.random(16)
    blob = mlp.init_blob(mu, sd, seed=seed)
    samples = np.concatenate([mu + sd * rng.standard_normal((n, 16)), rng.standard_normal((n, 2))], axis=1)
    return blob, samples.astype(np.float32)


@pytest.mark.parametrize("n", [1, 63, 64, 1000, 5003])
def test_gradient_matches_oracle(gpu_lib, n):
    blob, samples = _random_case(11 + n, n)
    loss, grad = mlp_loss_grad(blob, samples)
    loss_o, grad_o = mlp.loss_grad(blob.astype(np.float64), samples.astype(np.float64))
    assert abs(loss - loss_o) <= 1e-5 * abs(loss_o)
    assert np.all(grad[:32] == 0.0)
    err = np.linalg.norm(grad - grad_o) / np.linalg.norm(grad_o)
    assert err < 1e-4, err


@pytest.mark.parametrize("n", [1, 127, 128, 129, 20000])
def test_tensor_core_inference_matches_oracle(gpu_lib, n):
    blob, samples = _random_case(7 + n, n)
    feats = samples[:, :16]
    out = mlp_infer(blob, feats)
    ref = mlp.forward(blob, feats.astype(np.float64), bf16_path=True)
    scale = max(np.max(np.abs(ref)), 1e-3)
    # same BF16 roundings, FP32 accumulation in a different order: rare one-ulp flips of
    # a BF16 activation bound the difference
    assert np.max(np.abs(out - ref)) <= 2e-2 * scale, np.max(np.abs(out - ref))
    assert np.mean(np.abs(out - ref)) <= 1e-3 * scale
    full = mlp.forward(blob, feats.astype(np.float64))
    assert np.max(np.abs(out - full)) <= 5e-2 * max(np.max(np.abs(full)), 1e-3)


def test_training_lowers_loss(gpu_lib):
    rng = np.random.default_rng(1)
    x = rng.standard_normal((6000, 16)).astype(np.float32)
    y = np.tanh(x[:, 0] - 0.5 * x[:, 3]) + 0.1 * x[:, 7]
    g = y / (1.0 + 0.2 * np.tanh(x[:, 5]))  # reachable: s = 1 + 0.2 tanh(x5)
    samples = np.concatenate([x, y[:, None], g[:, None]], axis=1).astype(np.float32)
    blob = learned.init_weights(samples, seed=2)
    l0, _ = mlp_loss_grad(blob, samples)
    trained, losses = mlp_train(blob, samples, epochs=15, batch=512, lr=3e-3, seed=4)
    l1, _ = mlp_loss_grad(trained, samples)
    assert losses[-1] < losses[0]
    assert l1 < 0.3 * l0, (l0, l1)
    # deterministic: same seed, same weights
    again, _ = mlp_train(blob, samples, epochs=15, batch=512, lr=3e-3, seed=4)
    np.testing.assert_array_equal(trained, again)


@pytest.fixture(scope="module")
def small_weights(gpu_lib):
    data = learned.collect(n_scenes=6, target=30000, steps=24, every=4, seed=77)
    assert data.shape[0] > 10000 and np.all(np.isfinite(data))
    blob, losses = learned.train(data, epochs=12, batch=2048, lr=2e-3, seed=5)
    assert losses[-1] < losses[0]
    return blob


def _dam(seed_k):
    s = learned.training_scene(seed_k, seed=991)
    return s


def zero_network():
    """The network with zero output: s = 1 and the warm start one preconditioned step."""
    blob = np.zeros(abi.MLP_BLOB_FLOATS, dtype=np.float32)
    blob[16:32] = 1.0
    return blob


def _run(s, solver, blob=None, steps=12):
    c = Computer(s.params(solver=solver, criterion=abi.CRIT_RHS, eps=1e-8))
    if blob is not None:
        c.learned_set_weights(blob)
    c.add_scene(s)
    its = []
    for _ in range(steps):
        c.forward_time(s.meta["dt"])
        st = c.stats()
        assert st["cg_true_relres"] <= 1e-8
        assert st["fallback"] == 0
        its.append(st["cg_iterations"])
    return c.particles(), np.array(its)


def test_learned_solve_matches_plain_cg(small_weights):
    s = _dam(3)
    P64, it64 = _run(s, abi.SOLVER_CG64)
    Pmg, itmg = _run(s, abi.SOLVER_MIXED_MG)
    Pl, itl = _run(s, abi.SOLVER_LEARNED, small_weights)
    Pz, itz = _run(s, abi.SOLVER_LEARNED, zero_network())
    for P in (Pmg, Pl, Pz):
        assert rel_err(P["p"], P64["p"]) < 1e-5
        assert rel_err(P["x"], P64["x"], scale=s.l0) < 1e-6
    # what the trained network gains over the same solve without it (zero network)
    print("iterations over %d steps: CG64 %d, MIXED_MG %d, zero network %d, trained network %d"
          % (len(it64), it64.sum(), itmg.sum(), itz.sum(), itl.sum()))
    assert itz.sum() <= itmg.sum()
    assert itl.sum() <= 1.05 * itz.sum()
    assert itl.sum() * 2 < it64.sum()


def test_learned_requires_weights(gpu_lib):
    s = _dam(0)
    c = Computer(s.params(solver=abi.SOLVER_LEARNED, criterion=abi.CRIT_RHS, eps=1e-8))
    c.add_scene(s)
    with pytest.raises(Exception) as e:
        c.forward_time(s.meta["dt"])
    assert getattr(e.value, "code", None) == abi.MPS_ERR_STATE


def test_collected_samples_are_consistent(gpu_lib):
    # y is the error the coarse correction misses, in units of sigma: solving from
    # x0 + c + sigma y gives the solution, so the samples are exact on the solved step
    s = _dam(1)
    c = Computer(s.params(solver=abi.SOLVER_CG64, criterion=abi.CRIT_RHS, eps=1e-12))
    c.add_scene(s)
    for _ in range(3):
        c.forward_time(s.meta["dt"])
    c.learned_collect(True)
    c.forward_time(s.meta["dt"])
    smp, act = c.learned_samples()
    assert act.sum() > 0.5 * s.count
    a = smp[act != 0]
    assert np.all(np.isfinite(a))
    # the Jacobi feature (8, in units of sigma) has unit RMS over the active rows
    assert abs(np.sqrt(np.mean(a[:, 8].astype(np.float64) ** 2)) - 1.0) < 1e-3
    np.testing.assert_allclose(a[:, 17], a[:, 8], rtol=1e-6, atol=1e-7)
