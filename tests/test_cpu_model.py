"""The cost model's CPU restatement (oracle) checked against finite
differences, and the committed trained parameters' shape (no GPU)."""
import numpy as np
import pytest

import colo
import oracle


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1, (n, colo.MODEL_FEATURES)).astype(np.float32)
    x[:, 0] = rng.integers(2, 9, n) / 8.0
    t = rng.normal(2, 1, n).astype(np.float32)
    return x, t


def test_exact_gradient_matches_finite_differences():
    p = colo.init_model(3)
    p[32 * 64:32 * 64 + 64] = 0.1     # non-zero biases so that most units are active
    x, t = _data(6, 11)
    g, loss = oracle.mlp_grad(p, x, t, bf16=False)
    rng = np.random.default_rng(5)
    idx = np.concatenate([rng.choice(24 * 64, 40, replace=False),                   # W1 (real input rows)
                          32 * 64 + rng.choice(64, 8, replace=False),               # b1
                          32 * 64 + 64 + rng.choice(64 * 64, 40, replace=False),    # W2
                          np.arange(colo.MODEL_PARAMS - 65, colo.MODEL_PARAMS)])    # W3, b3
    h = 1e-3
    for i in idx:
        pp = p.astype(np.float64)
        for sgn, store in ((1, "hi"), (-1, "lo")):
            q = pp.copy()
            q[i] += sgn * h
            # exact mode: the oracle computes in double from float32 parameters, so perturb by a
            # float32-representable step and use the exact difference that results
            q32 = q.astype(np.float32)
            if store == "hi":
                lhi = oracle.mlp_grad(q32, x, t, bf16=False)[1]
                dhi = float(q32[i]) - float(p[i])
            else:
                llo = oracle.mlp_grad(q32, x, t, bf16=False)[1]
                dlo = float(p[i]) - float(q32[i])
        fd = (lhi - llo) / (dhi + dlo)
        assert abs(fd - g[i]) <= 2e-3 * max(1.0, abs(g[i])) + 1e-5, (i, fd, g[i])


def test_padding_rows_have_no_gradient():
    p = colo.init_model(0)
    x, t = _data(32, 1)
    g, _ = oracle.mlp_grad(p, x, t, bf16=True)
    assert np.all(g[24 * 64:32 * 64] == 0)


def test_bf16_forward_is_close_to_exact():
    p = colo.init_model(2)
    x, _ = _data(256, 4)
    ye = oracle.mlp_forward(p, x, bf16=False)
    yb = oracle.mlp_forward(p, x, bf16=True)
    assert np.max(np.abs(ye - yb)) < 0.05 * max(1.0, np.max(np.abs(ye)))


def test_committed_model_has_the_right_shape():
    p = colo.load_model()
    assert p.shape == (colo.MODEL_PARAMS,) and np.all(np.isfinite(p))
    assert np.all(p[24 * 64:32 * 64] == 0)
