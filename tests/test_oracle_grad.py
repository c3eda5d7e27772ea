"""Finite-difference checks (float64, eps 1e-6) of the oracle's analytic
gradients: compositing (ray_utils.py:408-551), the NeRF MLP
(model.py:334-394) and the proposal network. No GPU."""
import numpy as np


def test_composite_backward_fd(oracle):
    rng = np.random.default_rng(0)
    R, S = 3, 9
    t = np.sort(rng.uniform(2, 6, (R, S)), 1)
    sig = rng.exponential(1.0, R * S)
    rgb = rng.random((R * S, 3))
    G = rng.normal(size=(R, 3))
    gw = rng.normal(size=(R, S))

    def L(s, c):
        out = oracle.post_process_model_output(c, s.reshape(-1, 1), t, True)
        return np.sum(out["pred_rgb"] * G) + np.sum(out["weights"] * gw)

    ds, dc = oracle.composite_backward(sig, t, rgb, G, gw, True)
    for i in range(sig.size):
        a, b = sig.copy(), sig.copy()
        a[i] += 1e-6
        b[i] -= 1e-6
        assert abs((L(a, rgb) - L(b, rgb)) / 2e-6 - ds[i]) < 1e-7
    for i in range(rgb.size):
        a, b = rgb.copy().reshape(-1), rgb.copy().reshape(-1)
        a[i] += 1e-6
        b[i] -= 1e-6
        fd = (L(sig, a.reshape(-1, 3)) - L(sig, b.reshape(-1, 3))) / 2e-6
        assert abs(fd - dc.reshape(-1)[i]) < 1e-7


def test_proposal_weights_backward_fd(oracle):
    rng = np.random.default_rng(5)
    R, S = 2, 8
    t = np.sort(rng.uniform(2, 6, (R, S)), 1)
    sig = rng.exponential(1.0, R * S)
    gw = rng.normal(size=(R, S))
    ds, _ = oracle.composite_backward(sig, t, np.zeros((R * S, 3)), None, gw, False, last_delta=None)
    for i in range(R * S):
        a, b = sig.copy(), sig.copy()
        a[i] += 1e-6
        b[i] -= 1e-6
        fd = (np.sum(gw * oracle.proposal_weights(a, t)) - np.sum(gw * oracle.proposal_weights(b, t))) / 2e-6
        assert abs(fd - ds[i]) < 1e-7


def test_mlp_backward_fd(oracle):
    rng = np.random.default_rng(1)
    p = oracle.glorot_params(3, np.float64)
    for k in p:
        p[k] = (p[k][0], rng.uniform(-0.1, 0.1, p[k][1].shape))
    x = rng.uniform(-2, 2, (6, 3))
    d = rng.normal(size=(6, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    dr, ds = rng.normal(size=(6, 3)), rng.normal(size=(6,))
    g = oracle.mlp_backward(p, x, d, dr, ds)

    def f(q):
        r, s = oracle.mlp_forward(q, x, d, np.float64)
        return np.sum(r * dr) + np.sum(s[:, 0] * ds)

    for name in ("dense_0", "dense_4", "dense_5", "dense_7", "sigma", "dense_8", "dense_9", "rgb"):
        W, b = p[name]
        for _ in range(4):
            i = tuple(rng.integers(0, s) for s in W.shape)
            q = dict(p)
            Wp, Wm = W.copy(), W.copy()
            Wp[i] += 1e-6
            Wm[i] -= 1e-6
            q[name] = (Wp, b)
            a = f(q)
            q[name] = (Wm, b)
            assert abs((a - f(q)) / 2e-6 - g[name][0][i]) < 1e-6
        j = rng.integers(0, b.size)
        bp, bm = b.copy(), b.copy()
        bp[j] += 1e-6
        bm[j] -= 1e-6
        q = dict(p)
        q[name] = (W, bp)
        a = f(q)
        q[name] = (W, bm)
        assert abs((a - f(q)) / 2e-6 - g[name][1][j]) < 1e-6


def test_proposal_backward_fd(oracle):
    rng = np.random.default_rng(2)
    blob = rng.normal(scale=0.3, size=6785)
    x = rng.uniform(-2, 2, (5, 3))
    dsg = rng.normal(size=5)
    g = oracle.prop_backward(blob, x, dsg)
    for i in rng.choice(6785, 40, replace=False):
        a, b = blob.copy(), blob.copy()
        a[i] += 1e-6
        b[i] -= 1e-6
        fd = (np.sum(dsg * oracle.prop_forward(a, x, np.float64))
              - np.sum(dsg * oracle.prop_forward(b, x, np.float64))) / 2e-6
        assert abs(fd - g[i]) < 1e-6 * max(1.0, abs(g[i]))


def test_apply_adam_first_step(oracle):
    var, m, v = np.ones(4), np.zeros(4), np.zeros(4)
    g = np.array([1.0, -2.0, 0.5, 0.0])
    var2, m2, v2 = oracle.apply_adam(var, m, v, g, 1, 1e-3)
    # first step: m = 0.1 g, v = 0.001 g^2, lr_t = lr sqrt(0.001)/0.1 -> step ~ lr sign(g)
    np.testing.assert_allclose(var2[:3], 1 - 1e-3 * np.sign(g[:3]), atol=1e-8)
    assert var2[3] == 1.0


def test_lr_schedule(oracle):
    assert oracle.lr_schedule(0) == 5e-4
    assert abs(oracle.lr_schedule(500000) - 5e-5) < 1e-15
