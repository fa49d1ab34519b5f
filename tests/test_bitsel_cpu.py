"""Learned bit selector on the host: the MLP oracle and the matrix features.

The oracle (oracle/mlp_oracle.py) is pinned by central finite differences in
float64, since the reference has no learned component to compare with.  The
features are host computations over the integer setup."""
import numpy as np
import pytest

import bitsel
import mlp_oracle as mo
import sagb


def _toy(n=37, nin=20, hid=64, nout=21, seed=1):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, nin))
    T = rng.standard_normal((n, nout))
    M = (rng.random((n, nout)) > 0.2).astype(np.float64)
    p = mo.init_params(nin, hid, nout, seed) + 0.01 * rng.standard_normal(
        sum(int(np.prod(s)) for _, s in mo.shapes(nin, hid, nout)))
    return X, T, M, p


def test_oracle_gradient_matches_finite_differences():
    nin, hid, nout = 6, 8, 5
    X, T, M, p = _toy(n=11, nin=nin, hid=hid, nout=nout)
    loss, g = mo.loss_grad(p, X, T, M, nin, hid, nout)
    rng = np.random.default_rng(0)
    h = 1e-6
    for i in rng.choice(p.size, 60, replace=False):
        e = np.zeros_like(p)
        e[i] = h
        lp, _ = mo.loss_grad(p + e, X, T, M, nin, hid, nout)
        lm, _ = mo.loss_grad(p - e, X, T, M, nin, hid, nout)
        assert abs((lp - lm) / (2 * h) - g[i]) <= 1e-6 * max(1.0, abs(g[i])), i


def test_oracle_normalisation_and_mask():
    nin, hid, nout = 4, 8, 3
    X, T, M, p = _toy(n=9, nin=nin, hid=hid, nout=nout)
    mu, sd = X.mean(0), X.std(0) + 0.5
    y1, _ = mo.forward(p, X, nin, hid, nout, mu, sd)
    y2, _ = mo.forward(p, (X - mu) / sd, nin, hid, nout)
    np.testing.assert_allclose(y1, y2, rtol=1e-12)
    # a masked-out target does not change the loss or the gradient
    T2 = T.copy()
    T2[M == 0] += 100.0
    l1, g1 = mo.loss_grad(p, X, T, M, nin, hid, nout)
    l2, g2 = mo.loss_grad(p, X, T2, M, nin, hid, nout)
    assert l1 == pytest.approx(l2, rel=1e-12)
    np.testing.assert_allclose(g1, g2, rtol=1e-12, atol=1e-15)


def test_oracle_training_reduces_loss():
    nin, hid, nout = 5, 16, 4
    rng = np.random.default_rng(2)
    X = rng.standard_normal((64, nin))
    W = rng.standard_normal((nout, nin))
    T = np.tanh(X @ W.T)
    M = np.ones_like(T)
    p0 = mo.init_params(nin, hid, nout, 7)
    p, hist = mo.train(p0, X, T, M, nin, hid, nout, epochs=30, batch=16, lr=3e-3, seed=5)
    assert hist[-1] < 0.3 * hist[0]


def test_features_of_a_setup():
    A = sagb.HostCsr.generate(sagb.GEN_POISSON3D, 14)
    xs, b = A.rhs(1)
    A.lmax1_scaling(b)
    r, c, v = A.arrays()
    s = sagb.Setup(sagb.INT, r, c, v)
    for ratio in (0.5, 3.7, 1000.0):
        f = sagb.setup_features(s, ratio)
        assert f.shape == (sagb.NUM_FEATURES,) and np.isfinite(f).all()
        assert f[0] == pytest.approx(np.log2(len(r) - 1))
        assert f[1] == pytest.approx(c.size / (len(r) - 1), rel=1e-6)
        assert f[3] == s.depth
        q = ratio
        rule = 29 if q < 1 else 31 - (int(np.ceil(np.log2(int(q) + 1))) + 1)
        assert f[7] == rule
        assert f[10] == pytest.approx(0.0, abs=1e-7)  # symmetric operator
    # convection makes the operator nonsymmetric
    B = sagb.HostCsr.generate(sagb.GEN_CONVDIFF3D, 10, 50.0)
    xs, b = B.rhs(1)
    B.lmax1_scaling(b)
    rb, cb, vb = B.arrays()
    f = sagb.setup_features(sagb.Setup(sagb.INT, rb, cb, vb), 1.0)
    assert f[10] > 0.01
    # a floating-point setup has no integer operators to describe
    with pytest.raises(sagb.SagbError):
        sagb.setup_features(sagb.Setup(sagb.F64, r, c, v), 1.0)


def test_trained_selector_gains_on_heldout_sweeps():
    """The committed network, evaluated by the oracle's forward pass on the
    held-out 20 % of the GPU sweep dataset, against the reference's rule with
    the overflow fallback (a failing F redone with one bit less: the first F at
    or below the rule's that converges, its failed attempts not charged, which
    favours the rule).  The selector must need fewer iterations overall, a
    fifth fewer on the anisotropic systems (where the rule's F = 29 converges
    slowly), pick no failing F, and never cost much more than the rule."""
    import json
    import os
    d = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "sc23-ad_gb300", "data")
    z = np.load(os.path.join(d, "bitsel_mlp.npz"))
    ds = np.load(os.path.join(d, "bitsel_dataset.npz"))
    X, meta = ds["X"].astype(np.float64), json.loads(str(ds["meta"]))
    nin, hid, nout, f_lo = int(z["n_in"]), int(z["hidden"]), int(z["n_out"]), int(z["f_lo"])
    ntr = int(round(0.8 * len(X)))
    # the selector clamps features to the training range before the forward pass
    np.testing.assert_array_equal(z["x_lo"], X[:ntr].min(0))
    np.testing.assert_array_equal(z["x_hi"], X[:ntr].max(0))
    Xh = np.clip(X[ntr:], z["x_lo"].astype(np.float64), z["x_hi"].astype(np.float64))
    Y, _ = mo.forward(z["params"].astype(np.float64), Xh, nin, hid, nout, z["mu"].astype(np.float64),
                      z["sd"].astype(np.float64))
    sel_it = rule_it = sel_an = rule_an = 0
    fails_sel = 0
    for k, y in enumerate(Y):
        m = meta[ntr + k]
        sw = {q["bit"]: q for q in m["sweep"]}
        rule = m["rule"]
        f = f_lo + int(np.argmin(y))
        if y[rule - f_lo] - y[f - f_lo] < bitsel.MARGIN:  # the selector's margin
            f = rule
        r_it = next((sw[g]["iters"] for g in range(rule, f_lo - 1, -1) if sw[g]["converged"]), 120)
        if sw[f]["converged"]:
            s_it = sw[f]["iters"]
        else:
            fails_sel += 1
            s_it = 120 + r_it
        assert s_it <= 1.5 * r_it + 4, (m["spec"], f, s_it, rule, r_it)
        sel_it += s_it
        rule_it += r_it
        if m["spec"][0] == sagb.GEN_ANISO2D:
            sel_an += s_it
            rule_an += r_it
    assert fails_sel == 0
    assert sel_it < rule_it, (sel_it, rule_it)
    assert sel_an < 0.8 * rule_an, (sel_an, rule_an)
