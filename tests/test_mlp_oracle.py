"""CPU checks of the learned-radial-basis oracle (no GPU): the hand-derived
backpropagation against finite differences, the BF16 rounding, and the
Hernquist-Ostriker prior (SciPy Gegenbauer vs the recurrence the kernels use)."""
import os

import numpy as np

from tests.conftest import GOLDEN


def _params(seed=0, nout=12):
    from exptool_gb300.basis.learned import init_params
    return init_params(1, nout, seed)[0].astype(np.float64)


def test_backprop_matches_finite_differences():
    from oracle import mlp
    rng = np.random.default_rng(0)
    nout = 12
    p = _params(nout=nout)
    t = rng.uniform(-1, 1, 16)
    T = rng.normal(size=(16, mlp.NOP))
    loss, g = mlp.loss_and_grad(p, t, T, nout, emulate=False)
    # a sample of coordinates from every block
    idx = np.concatenate([rng.choice(np.arange(a, b), 6, replace=False) for a, b in
                          ((mlp.W1, mlp.B1), (mlp.B1, mlp.W2), (mlp.W2, mlp.B2), (mlp.B2, mlp.W3), (mlp.W3, mlp.B3),
                           (mlp.B3, mlp.W4), (mlp.W4, mlp.W4 + nout * mlp.HID), (mlp.B4, mlp.B4 + nout))])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp.loss_and_grad(pp, t, T, nout, emulate=False)[0] - mlp.loss_and_grad(pm, t, T, nout, emulate=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (i, fd, g[i])
    # padded outputs carry no gradient
    assert np.all(g[mlp.W4 + nout * mlp.HID:mlp.B4] == 0) and np.all(g[mlp.B4 + nout:] == 0)


def test_emulated_gradient_close_to_exact():
    from oracle import mlp
    rng = np.random.default_rng(1)
    nout = 12
    p = _params(seed=1, nout=nout)
    t = rng.uniform(-1, 1, 256)
    T = rng.normal(size=(256, mlp.NOP))
    _, g = mlp.loss_and_grad(p, t, T, nout, emulate=False)
    _, ge = mlp.loss_and_grad(p, t, T, nout, emulate=True)
    assert np.linalg.norm(ge - g) <= 3e-2 * np.linalg.norm(g)


def test_bf16_rounding():
    from oracle.mlp import bf16
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.140625, 1e-30, 65504.0], dtype=np.float32)
    y = bf16(x)
    # 1 + 2^-8 is a tie -> even (1.0); 1 + 3*2^-9 rounds up to 1 + 2^-7
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == np.float32(1.0 + 2 ** -7)
    assert y[3] == np.float32(-3.140625)
    assert np.all(np.abs(y - x) <= np.abs(x) * 2 ** -8)


def test_prior_recurrence_matches_scipy():
    from exptool_gb300.basis.learned import ho_radial_np
    from oracle.mlp import ho_radial
    u = np.exp(np.linspace(np.log(1e-3), np.log(100.0), 400))
    for l in range(8):
        a, da = ho_radial_np(u, l, 24)
        b, db = ho_radial(u, l, 24)
        assert np.allclose(a, b, rtol=1e-10, atol=1e-12 * np.max(np.abs(b)))
        assert np.allclose(da, db, rtol=1e-9, atol=1e-11 * np.max(np.abs(db)))
    # u dHO/du against a centred difference in ln u
    h = 1e-6
    a, da = ho_radial_np(u, 3, 10)
    fd = (ho_radial_np(u * np.exp(h), 3, 10)[0] - ho_radial_np(u * np.exp(-h), 3, 10)[0]) / (2 * h)
    assert np.allclose(da, fd, rtol=1e-5, atol=1e-8 * np.max(np.abs(fd)))


def test_oracle_labels_vanish_for_exact_prior():
    """Labels are (table - s HO)/sig: with s fitted, residuals are small next to
    the functions themselves on the golden Hernquist table."""
    from oracle import mlp
    from oracle.sl import load_table
    from exptool_gb300.basis.learned import ho_radial_np
    tab = load_table(os.path.join(GOLDEN, "sl_c2.cache"), os.path.join(GOLDEN, "sl_c2.model"))
    K = tab["nmax"]
    L = tab["lmax"] + 1
    r = np.exp(tab["xi"])
    phi = tab["p0"][None, None, :] * tab["ef"][:, :K, :] / np.sqrt(tab["ev"][:, :K, None])
    s = np.zeros((L, K))
    for l in range(L):
        ho, _ = ho_radial_np(r, l, K)
        s[l] = np.sum(phi[l] * ho.T, axis=1) / np.sum(ho.T ** 2, axis=1)
    sig = np.ones((L, 2 * K))
    rr = np.exp(np.random.default_rng(2).uniform(np.log(1e-3), np.log(100.0), 300))
    t, T = mlp.labels(rr, tab, K, 1.0, s, sig, 0.0, 1.0 / 7.0)
    pot, force = mlp.table_radial(rr, tab, K)
    assert T.shape == (L, 300, 64) and np.all(T[:, :, 2 * K:] == 0)
    # l = 1..4, n = 0: the prior captures the function to a small residual
    for l in range(1, L):
        assert np.max(np.abs(T[l, :, 0])) < 0.05 * np.max(np.abs(pot[:, l, 0]))
