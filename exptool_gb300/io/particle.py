"""Particle containers with the interface of ``exptool/io/particle.py``.

``holder`` is the attribute container (``.xpos .ypos .zpos .mass`` ...,
particle.py:142-157); ``ParticleData`` provides the ``.data`` dict of
``particle.Input`` (keys x y z vx vy vz m potE) for in-memory arrays.  The
snapshot readers are ``psp_io.Input`` and ``spl_io.Input``.
"""
from __future__ import annotations

import numpy as np


class holder(object):
    """All the PSP-style quantities (particle.py:142-157)."""
    filename = None
    comp = None
    nbodies = None
    time = None
    xpos = None
    ypos = None
    zpos = None
    xvel = None
    yvel = None
    zvel = None
    mass = None
    pote = None
    id = None


class ParticleData(object):
    """In-memory stand-in for ``particle.Input``: ``.data`` dict plus the holder
    attributes, ``.time``, ``.filename`` and ``.comp``."""

    def __init__(self, x, y, z, m, vx=None, vy=None, vz=None, time=0.0, filename="", comp=""):
        n = np.asarray(x).size
        zeros = np.zeros(n)
        self.data = {"x": np.asarray(x, dtype=np.float64), "y": np.asarray(y, dtype=np.float64),
                     "z": np.asarray(z, dtype=np.float64), "m": np.asarray(m, dtype=np.float64),
                     "vx": zeros if vx is None else np.asarray(vx), "vy": zeros if vy is None else np.asarray(vy),
                     "vz": zeros if vz is None else np.asarray(vz), "potE": zeros}
        self.xpos, self.ypos, self.zpos, self.mass = self.data["x"], self.data["y"], self.data["z"], self.data["m"]
        self.time = time
        self.filename = filename
        self.comp = comp


def positions(P, allow_device=False):
    """(x, y, z, m) float64 arrays of a holder-like or ``.data``-like container.
    With allow_device, columns that are CUDA tensors (a snapshot read with
    ``device=True``) are returned as float64 CUDA tensors instead."""
    if hasattr(P, "data") and isinstance(getattr(P, "data"), dict) and "x" in P.data:
        cols = [P.data[k] for k in ("x", "y", "z", "m")]
    else:
        cols = [P.xpos, P.ypos, P.zpos, P.mass]
    if allow_device and all(getattr(c, "is_cuda", False) for c in cols):
        import torch
        return tuple(c.to(torch.float64).contiguous() for c in cols)
    return tuple(np.asarray(c.cpu() if hasattr(c, "cpu") else c, dtype=np.float64) for c in cols)
