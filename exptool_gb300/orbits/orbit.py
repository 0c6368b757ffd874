"""Orbit container with the interface of ``exptool/orbits/orbit.py``.

``Orbits`` is the dict returned by ``leapfrog_integrate`` (keys T X Y Z VX VY
VZ P TX TY VTX VTY [FX FY FZ]); frequency analysis is in
``exptool_gb300.orbits.frequencies``.  Snapshot orbit mapping and plotting are
outside this package.
"""
from __future__ import annotations


class Orbits(dict):
    """Orbit dictionary (orbit.py:50)."""

    def __init__(self):
        pass

    def polar_coordinates(self):
        """orbit.py:212-226: adds Rp, Phi (and Phib from TX, TY when present)."""
        import numpy as np
        self["Rp"] = np.power(self["X"] * self["X"] + self["Y"] * self["Y"], 0.5)
        self["Phi"] = np.arctan2(self["Y"], self["X"])
        if "TX" in self and "TY" in self:
            self["Phib"] = np.arctan2(self["TY"], self["TX"])

    def compute_quantities(self):
        """orbit.py:198-209: adds E = v^2 + P (the reference omits the 1/2) and LZ."""
        v2 = self["VX"] * self["VX"] + self["VY"] * self["VY"] + self["VZ"] * self["VZ"]
        self["E"] = v2 + self["P"]
        self["LZ"] = self["X"] * self["VY"] - self["Y"] * self["VX"]
