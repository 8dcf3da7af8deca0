"""CPU checks of the learned-solve network's oracle (numpy FP64) and its layout."""
import os
import re

import numpy as np

from oracle import mlp
from openmps_gb300 import _abi as abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_layout_matches_header():
    hdr = open(os.path.join(ROOT, "include", "mps.h")).read()
    blob = int(re.search(r"#define MPS_MLP_BLOB_FLOATS (\d+)", hdr).group(1))
    sample = int(re.search(r"#define MPS_MLP_SAMPLE_FLOATS (\d+)", hdr).group(1))
    assert blob == mlp.BLOB_FLOATS == abi.MLP_BLOB_FLOATS
    assert sample == abi.MLP_SAMPLE_FLOATS == 18


def test_oracle_gradient_finite_differences():
    rng = np.random.default_rng(3)
    blob = mlp.init_blob(rng.standard_normal(16) * 0.1, 0.5 + rng.random(16), seed=5).astype(np.float64)
    samples = rng.standard_normal((40, 18))
    _, grad = mlp.loss_grad(blob, samples)
    h = 1e-6
    for idx in (32, 700, 1100, 3000, 5300, 9200, 9500, 9568, 9569):
        bp = blob.copy(); bp[idx] += h
        bm = blob.copy(); bm[idx] -= h
        fd = (mlp.loss_grad(bp, samples)[0] - mlp.loss_grad(bm, samples)[0]) / (2 * h)
        assert abs(fd - grad[idx]) <= 1e-6 + 1e-5 * abs(fd), (idx, fd, grad[idx])


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -3.14159, 65504.0, 1e-30], dtype=np.float32)
    r = mlp.bf16(x)
    # representable values stay, ties go to the even mantissa, others to the nearest
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625
    assert abs(r[3] + 3.140625) < 1e-12
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8)
