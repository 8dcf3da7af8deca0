"""Training data, training and weights of the learned PPE warm start / preconditioner scale.

The network (16 -> 64 -> 64 -> 64 -> 2, GELU) is trained on (state, pressure) pairs
that the plain FP64 CG (``MPS_SOLVER_CG64``) produces on seeded dam breaks whose column
widths and heights are drawn like the batched workload (width U[0.1, 0.3] m, height
U[0.2, 0.5] m, l0 = 5 mm).  Every step of a collecting handle yields one sample per
PPE row: the features of the step before the solve and, from the converged solution,
the part of the error the first coarse-grid correction misses.  Training runs on the
GPU (``mps_mlp_train``: FP32 forward/backward kernels, Adam); inference in the solver
runs on the tensor cores.

``python -m openmps_gb300.learned --out openmps_gb300/data/learned_mlp.npz`` regenerates
the shipped weights (seeded; about a minute on one GB300).
"""
from __future__ import annotations

import argparse
import os

import numpy as np

from . import _abi as abi
from . import scenes
from .computer import Computer, mlp_train

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "data", "learned_mlp.npz")

# dt scaled with l0 like the 320k workload (l0 / dt = 20 m/s)
def scene_dt(l0: float) -> float:
    return l0 / 20.0


def training_scene(k: int, seed: int) -> scenes.Scene:
    s = scenes.batch_scene(k, seed=seed)
    dt = scene_dt(s.l0)
    s.meta["params"] = dict(scenes.STOCK_PHYSICS, eps=1e-10, max_dt=dt)
    s.meta["dt"] = dt
    return s


def collect(n_scenes: int = 64, target: int = 200_000, steps: int = 60, every: int = 4,
            seed: int = 20261203, device: int = 0, verbose: bool = False) -> np.ndarray:
    """(target, 18) samples from `n_scenes` seeded dam breaks solved by the FP64 CG."""
    rng = np.random.default_rng(seed)
    per_scene = -(-target // n_scenes)
    out = []
    for k in range(n_scenes):
        s = training_scene(k, seed)
        c = Computer(s.params(solver=abi.SOLVER_CG64, criterion=abi.CRIT_RHS, eps=1e-10), device)
        c.add_scene(s)
        rows = []
        for step in range(steps):
            take = step % every == every - 1
            c.learned_collect(take)
            c.forward_time(s.meta["dt"])
            if take:
                smp, act = c.learned_samples()
                rows.append(smp[act != 0])
        c.close()
        pool = np.concatenate(rows) if rows else np.zeros((0, abi.MLP_SAMPLE_FLOATS), np.float32)
        pool = pool[np.all(np.isfinite(pool), axis=1)]
        if pool.shape[0] > per_scene:
            pool = pool[rng.choice(pool.shape[0], per_scene, replace=False)]
        out.append(pool)
        if verbose:
            print("scene %d: %d particles, %d samples" % (k, s.count, pool.shape[0]), flush=True)
    data = np.concatenate(out)
    return data[:target].astype(np.float32)


def feature_stats(samples: np.ndarray):
    x = samples[:, :16].astype(np.float64)
    mu = x.mean(axis=0)
    sd = np.maximum(x.std(axis=0), 1e-3)
    return mu, sd


def init_weights(samples: np.ndarray, seed: int = 0) -> np.ndarray:
    """Seeded He initialisation with the feature standardisation of `samples`."""
    mu, sd = feature_stats(samples)
    rng = np.random.default_rng(seed)
    blob = np.zeros(abi.MLP_BLOB_FLOATS, dtype=np.float32)
    blob[0:16] = mu
    blob[16:32] = sd
    at = 32
    for fo, fi, small in ((64, 16, False), (64, 64, False), (64, 64, False), (2, 64, True)):
        w = rng.standard_normal((fo, fi)) * np.sqrt(2.0 / fi) * (0.1 if small else 1.0)
        blob[at:at + fo * fi] = w.ravel()
        at += fo * fi + fo  # biases stay zero
    assert at == abi.MLP_BLOB_FLOATS
    return blob


def train(samples: np.ndarray, epochs: int = 30, batch: int = 4096, lr: float = 1e-3,
          seed: int = 0, device: int = 0):
    """GPU training from a seeded initialisation; returns (blob, per-epoch mean loss)."""
    blob = init_weights(samples, seed)
    return mlp_train(blob, samples, epochs=epochs, batch=batch, lr=lr, seed=seed, device=device)


def save(blob, path: str = WEIGHTS, **meta):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, blob=np.asarray(blob, dtype=np.float32), **meta)


def load(path: str = WEIGHTS) -> np.ndarray:
    with np.load(path) as d:
        blob = d["blob"].astype(np.float32)
    if blob.size != abi.MLP_BLOB_FLOATS:
        raise ValueError("%s: expected %d weights, found %d" % (path, abi.MLP_BLOB_FLOATS, blob.size))
    return blob


def main():
    ap = argparse.ArgumentParser(description="collect samples and train the learned-solve network")
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--scenes", type=int, default=64)
    ap.add_argument("--samples", type=int, default=200_000)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--seed", type=int, default=20261203)
    args = ap.parse_args()
    data = collect(args.scenes, args.samples, seed=args.seed, verbose=True)
    blob, losses = train(data, epochs=args.epochs, seed=args.seed & 0xffff)
    print("samples %d, loss per epoch %s" % (data.shape[0], np.array2string(losses, precision=4)))
    save(blob, args.out, losses=losses, samples=data.shape[0], scenes=args.scenes, seed=args.seed)


if __name__ == "__main__":
    main()
