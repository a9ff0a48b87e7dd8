"""The CPU restatement of the learned path's network (oracle/mlp.py), the
yardstick of the tensor-core training kernels: its float64 gradient against
central finite differences of its own loss (the error estimate's target
|y - t| held constant, as the kernels hold it), and its BF16 emulation
against float64."""

from __future__ import annotations

import numpy as np

from oracle import mlp as M


def _case(n=24, seed=0):
    rng = np.random.default_rng(seed)
    p = rng.normal(0.0, 0.3, M.NPARAMS)
    x = rng.uniform(-1, 1, (n, M.IN))
    y = rng.uniform(0, 1, (n, 3))
    return p, x, y


def test_layout():
    assert M.NPARAMS == 64 * 42 + 64 + 2 * (64 * 64 + 64) + 4 * 64 + 4 == 11332
    p = np.arange(M.NPARAMS, dtype=np.float64)
    w = M.unpack(p)
    assert w["W4"].shape == (4, 64) and w["b4"].shape == (4,)
    assert np.array_equal(M.pack(w), p)


def test_gradient_matches_finite_differences():
    p, x, y = _case()
    out, loss, g = M.forward_backward(p, x, y)
    assert out.shape == (24, 4)
    err0 = np.sqrt(((out[:, :3] - y) ** 2).sum(1))

    def loss_at(q):
        o = M.forward_backward(q, x)[0]
        return ((o[:, :3] - y) ** 2).sum() / (3 * len(x)) + M.CONF_WEIGHT * ((o[:, 3] - err0) ** 2).sum() / len(x)

    assert abs(loss_at(p) - loss) < 1e-12
    rng = np.random.default_rng(1)
    # every block, including the error estimate's row of W4 and its bias
    idx = np.concatenate([rng.choice(M.NPARAMS, 40, replace=False), [11072 + 3 * 64 + 5, 11331]])
    eps = 1e-6
    for i in idx:
        e = np.zeros(M.NPARAMS)
        e[i] = eps
        fd = (loss_at(p + e) - loss_at(p - e)) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_error_estimate_gradient_stays_out_of_the_irradiance_outputs():
    """Only W4's fourth row and b4[3] see the estimate's term directly: with
    the irradiance exact (y = network output), their gradients are the whole
    of W4/b4's gradient."""
    p, x, _ = _case(seed=2)
    y = M.forward_backward(p, x)[0][:, :3]
    _, _, g = M.forward_backward(p, x, y)
    w4 = g[11072:11328].reshape(4, 64)
    assert np.abs(w4[:3]).max() == 0.0 and np.abs(g[11328:11331]).max() == 0.0
    assert np.abs(w4[3]).max() > 0.0


def test_bf16_emulation_close_to_float64():
    p, x, y = _case(n=200, seed=3)
    o64, l64, g64 = M.forward_backward(p, x, y)
    oe, le, ge = M.forward_backward(p, x, y, emulate_bf16=True)
    assert np.linalg.norm(oe - o64) / np.linalg.norm(o64) < 2e-2
    assert abs(le - l64) / l64 < 5e-2
    assert float(ge @ g64 / (np.linalg.norm(ge) * np.linalg.norm(g64))) > 0.99
