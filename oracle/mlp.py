"""Oracle: the learned radial basis (per-l networks over an SL table).

TEST INFRASTRUCTURE.  The network has no counterpart in the reference; this
module restates its mathematics in NumPy FP64 so the GPU training and
inference kernels can be checked:

* ``forward`` / ``backward``: the network 1 -> 128 -> 128 -> 128 -> 64
  (SiLU) and its hand-derived backpropagation for the MSE loss over the
  first ``nout`` outputs.  ``emulate=True`` rounds to BF16 at exactly the
  points where the GPU stores BF16 (weights W2, W3, W4; activations H1..H3;
  the output gradient and the hidden-layer gradients fed to the products),
  so GPU and oracle differ only by FP32 accumulation order.  ``emulate=False``
  is the exact FP64 network, checked against finite differences.
* ``adam``: Kingma & Ba (2015) with bias correction.
* ``ho_radial`` / ``labels``: Hernquist-Ostriker prior and the training
  targets built from the table interpolation of ``oracle.sl`` (which follows
  ``spheresl.get_halo_dens_pot_force``, ``spheresl.py:106-160``).
* ``learned_all_eval``: potential and gradient from the network + prior in
  the ``spheresl.all_eval`` formulation (``spheresl.py:987-1102``).
"""
from __future__ import annotations

import numpy as np
from scipy.special import eval_gegenbauer

from . import sl as osl

HID = 128
NOP = 64
W1, B1 = 0, HID
W2 = B1 + HID
B2 = W2 + HID * HID
W3 = B2 + HID
B3 = W3 + HID * HID
W4 = B3 + HID
B4 = W4 + NOP * HID
SIZE = B4 + NOP


def unpack(p):
    """Views (w1, b1, W2, b2, W3, b3, W4, b4) of one network's parameter block."""
    return (p[W1:B1], p[B1:W2], p[W2:B2].reshape(HID, HID), p[B2:W3], p[W3:B3].reshape(HID, HID), p[B3:W4],
            p[W4:B4].reshape(NOP, HID), p[B4:SIZE])


def bf16(x):
    """Round float values to bfloat16 (round to nearest even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32)


def sigmoid(z):
    return 0.5 + 0.5 * np.tanh(0.5 * z)


def silu(z):
    return z * sigmoid(z)


def dsilu(z):
    s = sigmoid(z)
    return s * (1.0 + z * (1.0 - s))


def _q(x, emulate):
    return bf16(x).astype(np.float64) if emulate else np.asarray(x, dtype=np.float64)


def forward(p, t, emulate=True):
    """Outputs (B, 64) of one network at inputs t (B,), and the saved values."""
    w1, b1, w2, b2, w3, b3, w4, b4 = (np.asarray(a, dtype=np.float64) for a in unpack(np.asarray(p)))
    W2q, W3q, W4q = (_q(w, emulate) for w in (w2, w3, w4))
    t = np.asarray(t, dtype=np.float64)
    z1 = t[:, None] * w1[None, :] + b1[None, :]
    if emulate:
        z1 = z1.astype(np.float32).astype(np.float64)
    h1 = _q(silu(z1), emulate)
    z2 = h1 @ W2q.T + b2
    h2 = _q(silu(z2), emulate)
    z3 = h2 @ W3q.T + b3
    h3 = _q(silu(z3), emulate)
    y = h3 @ W4q.T + b4
    return y, dict(t=t, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3, h3=h3, W2q=W2q, W3q=W3q, W4q=W4q)


def loss_and_grad(p, t, T, nout, emulate=True):
    """MSE over the first nout outputs and its gradient (SIZE,) for one network."""
    y, c = forward(p, t, emulate)
    B = y.shape[0]
    r = np.zeros_like(y)
    r[:, :nout] = y[:, :nout] - np.asarray(T, dtype=np.float64)[:, :nout]
    loss = float(np.sum(r[:, :nout] ** 2) / (B * nout))
    dY = 2.0 * r / (B * nout)
    if emulate:
        dY = dY.astype(np.float32).astype(np.float64)
    dYq = _q(dY, emulate)
    g = np.zeros(SIZE)
    g[W4:B4] = (dYq.T @ c["h3"]).ravel()
    g[B4:SIZE] = dY.sum(axis=0)
    dZ3 = (dYq @ c["W4q"]) * dsilu(c["z3"])
    dZ3q = _q(dZ3, emulate)
    g[W3:B3] = (dZ3q.T @ c["h2"]).ravel()
    g[B3:W4] = dZ3.sum(axis=0)
    dZ2 = (dZ3q @ c["W3q"]) * dsilu(c["z2"])
    dZ2q = _q(dZ2, emulate)
    g[W2:B2] = (dZ2q.T @ c["h1"]).ravel()
    g[B2:W3] = dZ2.sum(axis=0)
    dZ1 = (dZ2q @ c["W2q"]) * dsilu(c["z1"])
    g[W1:B1] = dZ1.T @ c["t"]
    g[B1:W2] = dZ1.sum(axis=0)
    g[W4 + nout * HID:B4] = 0.0
    g[B4 + nout:SIZE] = 0.0
    return loss, g


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (returns new p, m, v)."""
    m = b1 * m + (1.0 - b1) * g
    v = b2 * v + (1.0 - b2) * g * g
    c1 = 1.0 - b1 ** step
    c2 = 1.0 - b2 ** step
    return p - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v


# ---------------------------------------------------------------- prior and labels
def ho_radial(u, l, K):
    """Hernquist-Ostriker HO_nl(u) = -u^l/(1+u)^(2l+1) C_n^(2l+3/2)(xi) and
    u dHO_nl/du for n < K; returns two (N, K) arrays."""
    u = np.atleast_1d(np.asarray(u, dtype=np.float64))
    xi = (u - 1.0) / (u + 1.0)
    a = 2 * l + 1.5
    pre = u ** l / (1.0 + u) ** (2 * l + 1)
    g1 = l - (2 * l + 1) * u / (1.0 + u)
    g2 = 2.0 * u / (1.0 + u) ** 2
    ho = np.empty((u.size, K))
    uho = np.empty((u.size, K))
    for n in range(K):
        c = eval_gegenbauer(n, a, xi)
        dc = 2.0 * a * eval_gegenbauer(n - 1, a + 1.0, xi) if n > 0 else np.zeros_like(xi)
        ho[:, n] = -pre * c
        uho[:, n] = -pre * (g1 * c + g2 * dc)
    return ho, uho


def table_radial(r, table, K):
    """Table interpolation of phi_nl and dphi_nl/dr: two (N, lmax+1, K) arrays."""
    _, force, pot = osl.halo_dens_force_pot(np.atleast_1d(r), table["lmax"], K, table["ev"], table["ef"], table["xi"],
                                            table["d0"], table["p0"], table["cmap"], table["scale"], table["rmin"],
                                            table["rmax"])
    return pot, force


def labels(r, table, K, a_prior, s, sig, c0, c1):
    """(t, T) with T of shape (lmax+1, N, 64), as xt_mlp_labels computes."""
    r = np.atleast_1d(np.asarray(r, dtype=np.float64))
    rc = np.clip(r, table["rmin"], table["rmax"])
    t = np.clip((np.log(rc) - c0) * c1, -1.0, 1.0)
    pot, force = table_radial(rc, table, K)
    L = table["lmax"] + 1
    T = np.zeros((L, r.size, NOP))
    for l in range(L):
        ho, uho = ho_radial(rc / a_prior, l, K)
        T[l, :, :K] = (pot[:, l, :] - s[l] * ho) / sig[l, :K]
        T[l, :, K:2 * K] = (rc[:, None] * force[:, l, :] - s[l] * uho) / sig[l, K:]
    return t, T


def learned_all_eval(params, r, costh, phi, expcoef, table, K, a_prior, s, sig, c0, c1, coef_scale=1.0):
    """Potential and gradient of the learned expansion (networks with BF16
    emulation + prior), all_eval formulation: (pot0 + pot1, potr, pott, potp)."""
    r = np.atleast_1d(np.asarray(r, dtype=np.float64))
    costh = np.atleast_1d(np.asarray(costh, dtype=np.float64))
    phi = np.atleast_1d(np.asarray(phi, dtype=np.float64))
    lmax = table["lmax"]
    rc = np.clip(r, table["rmin"], table["rmax"])
    t = np.clip((np.log(rc) - c0) * c1, -1.0, 1.0)
    ec = coef_scale * np.asarray(expcoef)[:, :K]
    potd = np.empty((r.size, lmax + 1, K))
    dpot = np.empty((r.size, lmax + 1, K))
    for l in range(lmax + 1):
        y, _ = forward(params[l], t, emulate=True)
        ho, uho = ho_radial(rc / a_prior, l, K)
        potd[:, l] = s[l] * ho + sig[l, :K] * y[:, :K]
        dpot[:, l] = (s[l] * uho + sig[l, K:2 * K] * y[:, K:2 * K]) / rc[:, None]
    legs, dlegs = osl.dlegendre_R(lmax, costh)
    fact = osl.factorial_return(lmax)
    pot0 = fact[0, 0] * np.sum(ec[0] * potd[:, 0], axis=1)
    potr = fact[0, 0] * np.sum(ec[0] * dpot[:, 0], axis=1)
    pot1 = np.zeros(r.size)
    pott = np.zeros(r.size)
    potp = np.zeros(r.size)
    for l, m, row in osl._rows(lmax):
        if l == 0:
            continue
        f = fact[l, m]
        if m == 0:
            pv = np.sum(ec[row] * potd[:, l], axis=1)
            dv = np.sum(ec[row] * dpot[:, l], axis=1)
            pot1 += f * legs[l, m] * pv
            potr += f * legs[l, m] * dv
            pott += f * dlegs[l, m] * pv
        else:
            pc, ps = np.sum(ec[row] * potd[:, l], axis=1), np.sum(ec[row + 1] * potd[:, l], axis=1)
            dc, ds = np.sum(ec[row] * dpot[:, l], axis=1), np.sum(ec[row + 1] * dpot[:, l], axis=1)
            cm, sm = np.cos(m * phi), np.sin(m * phi)
            pot1 += f * legs[l, m] * (pc * cm + ps * sm)
            potr += f * legs[l, m] * (dc * cm + ds * sm)
            pott += f * dlegs[l, m] * (pc * cm + ps * sm)
            potp += f * legs[l, m] * m * (-pc * sm + ps * cm)
    return pot0 + pot1, potr, pott, potp
