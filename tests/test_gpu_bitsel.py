"""GPU parity of the bit selector's MLP kernels against the NumPy oracle.

Forward, loss, gradient and Adam are FP32 on the GPU (fixed-order sums) and
float64 in the oracle; the tolerances below are FP32 rounding bounds for these
sizes (64-wide layers, a few hundred rows)."""
import numpy as np
import pytest

import mlp_oracle as mo
import sagb

pytestmark = pytest.mark.gpu

NIN, HID, NOUT = sagb.NUM_FEATURES, 64, 21


@pytest.fixture(scope="module")
def ctx():
    c = sagb.Context(0)
    yield c
    c.close()


def _data(n, seed=3):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, NIN)).astype(np.float32) * 3 + 1
    T = rng.standard_normal((n, NOUT)).astype(np.float32)
    M = (rng.random((n, NOUT)) > 0.25).astype(np.float32)
    return X, T, M


def test_init_matches_oracle(ctx):
    net = sagb.Mlp(ctx, NIN, HID, NOUT, seed=42)
    np.testing.assert_array_equal(net.params(), mo.init_params(NIN, HID, NOUT, 42).astype(np.float32))
    net.close()


def test_forward_and_gradient(ctx):
    X, T, M = _data(300)
    mu, sd = X.mean(0), X.std(0) + 0.1
    net = sagb.Mlp(ctx, NIN, HID, NOUT, seed=7)
    net.set_norm(mu, sd)
    p = net.params().astype(np.float64)
    y_ref, _ = mo.forward(p, X.astype(np.float64), NIN, HID, NOUT, mu.astype(np.float64), sd.astype(np.float64))
    y = net.predict(X)
    assert np.abs(y - y_ref).max() <= 1e-4 * max(1.0, np.abs(y_ref).max())
    loss, g = net.gradient(X, T, M)
    l_ref, g_ref = mo.loss_grad(p, X.astype(np.float64), T.astype(np.float64), M.astype(np.float64), NIN, HID,
                                NOUT, mu.astype(np.float64), sd.astype(np.float64))
    assert loss == pytest.approx(l_ref, rel=1e-4)
    assert np.abs(g - g_ref).max() <= 2e-4 * np.abs(g_ref).max()
    net.close()


def test_training_matches_oracle_and_is_reproducible(ctx):
    X, T, M = _data(200, seed=5)
    mu, sd = X.mean(0), X.std(0) + 0.1
    runs = []
    for _ in range(2):
        net = sagb.Mlp(ctx, NIN, HID, NOUT, seed=11)
        net.set_norm(mu, sd)
        p0 = net.params().astype(np.float64)
        hist = net.train(X, T, M, epochs=4, batch=32, lr=1e-3, seed=9)
        runs.append((net.params(), hist))
        net.close()
    np.testing.assert_array_equal(runs[0][0], runs[1][0])  # fixed-order kernels: bitwise reproducible
    p_ref, h_ref = mo.train(p0, X.astype(np.float64), T.astype(np.float64), M.astype(np.float64), NIN, HID, NOUT,
                            epochs=4, batch=32, lr=1e-3, seed=9, mu=mu.astype(np.float64),
                            sd=sd.astype(np.float64))
    np.testing.assert_allclose(runs[0][1], h_ref, rtol=2e-3)
    # Adam normalises each step, so FP32 differences stay at the lr * eps level
    assert np.abs(runs[0][0] - p_ref).max() <= 2e-4


def test_select_bits_is_argmin(ctx):
    net = sagb.Mlp(ctx, NIN, HID, NOUT, seed=1)
    X, _, _ = _data(5)
    Y = net.predict(X)
    for i in range(5):
        assert net.select_bits(X[i], 8) == 8 + int(np.argmin(Y[i]))
    net.close()
