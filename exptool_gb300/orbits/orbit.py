"""Orbit container with the interface of ``exptool/orbits/orbit.py``.

``Orbits`` is the dict returned by ``leapfrog_integrate`` (keys T X Y Z VX VY
VZ P TX TY VTX VTY [FX FY FZ]); snapshot orbit mapping and plotting are
outside this package.
"""
from __future__ import annotations


class Orbits(dict):
    """Orbit dictionary (orbit.py:50)."""

    def __init__(self):
        pass

    def compute_quantities(self):
        """orbit.py:198-209: adds E = v^2 + P (the reference omits the 1/2) and LZ."""
        v2 = self["VX"] * self["VX"] + self["VY"] * self["VY"] + self["VZ"] * self["VZ"]
        self["E"] = v2 + self["P"]
        self["LZ"] = self["X"] * self["VY"] - self["Y"] * self["VX"]
