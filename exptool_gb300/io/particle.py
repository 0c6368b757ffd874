"""Particle containers with the interface of ``exptool/io/particle.py``.

``Input`` reads one component of an EXP snapshot, choosing the SPL or PSP
reader from the file name (particle.py:17-106); ``holder`` is the attribute
container (``.xpos .ypos .zpos .mass`` ..., particle.py:142-157);
``ParticleData`` provides the ``.data`` dict of ``particle.Input`` (keys x y z
vx vy vz m potE) for in-memory arrays.
"""
from __future__ import annotations

import numpy as np


class Input:
    """particle.Input (particle.py:66-106): ``SPL.`` in the file name selects
    ``spl_io.Input``, every other name ``psp_io.Input`` (the reference's
    ``elif 'OUT.':`` tests a non-empty string, so it never reaches its
    'unknown' branch).  Exposes ``.header .filename .time``; with a component,
    ``.comp`` and either ``.data`` or, with ``legacy=True``, the holder
    attributes (``.id`` when the component is indexed).  ``device=True``
    leaves the columns on the GPU as float64 CUDA tensors (no counterpart in
    the reference)."""

    def __init__(self, filename, comp=None, legacy=False, verbose=0, device=False):
        from . import psp_io, spl_io
        self.style = "SPL" if "SPL." in filename else "OUT"
        reader = spl_io.Input if self.style == "SPL" else psp_io.Input
        I = reader(filename, comp=comp, verbose=verbose, device=device)
        self.header = I.header
        self.filename = I.filename
        self.time = I.time
        if I.comp is None:
            return
        if legacy:
            d = I.data
            self.mass, self.xpos, self.ypos, self.zpos = d["m"], d["x"], d["y"], d["z"]
            self.xvel, self.yvel, self.zvel, self.pote = d["vx"], d["vy"], d["vz"], d["potE"]
            from .snapshot import _indexing
            if _indexing(I.header[I.comp]):
                self.id = d["id"]
        else:
            self.data = I.data
        self.comp = I.comp


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
