"""The FP64 CPU restatement of the selector MLP (the checker of the GPU
kernels) against central finite differences, and the parameter layout."""
import numpy as np

from oracle import mlp_ref as R


def test_param_count_matches_header():
    import re
    import os
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "blis_gb300.h")).read()
    n = int(re.search(r"#define GB_MLP_NPARAMS (\d+)", hdr).group(1))
    assert n == R.NPARAMS


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = R.init(1)
    x = rng.normal(size=(7, R.NIN))
    y = rng.normal(size=(7, R.NOUT))
    mask = (rng.uniform(size=(7, R.NOUT)) < 0.7).astype(np.float64)
    norm = mask.sum()
    _, g = R.loss_grad(p, x, y, mask, norm)
    idx = rng.choice(R.NPARAMS, 200, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (R.loss_grad(p + e, x, y, mask, norm)[0] - R.loss_grad(p - e, x, y, mask, norm)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd)


def test_adam_step_reduces_loss():
    rng = np.random.default_rng(2)
    p = R.init(3)
    x = rng.normal(size=(64, R.NIN))
    y = rng.normal(size=(64, R.NOUT)) * 0.1
    mask = np.ones((64, R.NOUT))
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    l0, _ = R.loss_grad(p, x, y, mask, mask.sum())
    for step in range(1, 51):
        _, g = R.loss_grad(p, x, y, mask, mask.sum())
        p, m, v = R.adam(p, g, m, v, 1e-3, 0.9, 0.999, 1e-8, 0.0, step)
    l1, _ = R.loss_grad(p, x, y, mask, mask.sum())
    assert l1 < 0.5 * l0
