"""Radial / vertical table maps with the interface of
``exptool/basis/compatibility.py`` (host-side helpers for table set-up; the
kernels use their own device copies in csrc/xt_common.cuh)."""
from __future__ import annotations

import numpy as np


def r_to_xi(r, cmap, scale):
    """compatibility.py:16-49: cmap 1 (r/s-1)/(r/s+1), cmap 2 log r, else r; r < 0 -> 0."""
    r = np.asarray(r, dtype=np.float64)
    scalar = r.ndim == 0
    r = np.atleast_1d(r)
    with np.errstate(divide="ignore", invalid="ignore"):
        if cmap == 1:
            out = (r / scale - 1.0) / (r / scale + 1.0)
        elif cmap == 2:
            out = np.log(r)
        else:
            out = r.copy()
    out[r < 0.0] = 0.0
    return np.squeeze(out) if scalar else out


def xi_to_r(xi, cmap, scale):
    """compatibility.py:54-62."""
    if cmap == 1:
        return (1.0 + xi) / (1.0 - xi) * scale
    if cmap == 2:
        return np.exp(xi)
    return xi


def d_xi_to_r(xi, cmap, scale):
    """compatibility.py:65-80."""
    if cmap == 1:
        return 0.5 * (1.0 - xi) * (1.0 - xi) / scale
    if cmap == 2:
        return np.exp(-xi)
    return 1.0


def z_to_y(z, hscale):
    """compatibility.py:83-91: z/(|z|+1e-8) asinh(|z/h|)."""
    return (z / (np.abs(z) + 1.0e-8)) * np.arcsinh(np.abs(z / hscale))


def y_to_z(y, hscale):
    """compatibility.py:94-101."""
    return hscale * np.sinh(y)
