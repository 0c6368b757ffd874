"""Coefficient time series straight from EXP snapshot files: each file's
component is read into page-locked memory, de-interleaved on the GPU and
accumulated there, while a background thread reads the next file into a
second page-locked buffer.  Coefficients stay on the device until one copy at
the end.  (The reference computes one snapshot per call,
spheresl.compute_coefficients / eof.compute_coefficients, reading each file
through psp_io / spl_io.)
"""
from __future__ import annotations

import threading

import numpy as np
import torch

from . import snapshot


class _Reader(threading.Thread):
    """Reads one file's component records into a page-locked buffer (the
    file reads release the GIL, so this overlaps the GPU work of the previous
    file)."""

    def __init__(self, path, comp, kind, buf):
        super().__init__(daemon=True)
        self.path, self.comp, self.kind, self.buf = path, comp, kind, buf
        self.error = None

    def run(self):
        try:
            with open(self.path, "rb") as f:
                if self.kind == "psp":
                    self.time, fl, heads = snapshot.read_psp_header(f)
                    subs = None
                else:
                    self.time, fl, heads, subs = snapshot.read_spl_header(f)
            if self.comp not in heads:
                raise IOError(f"{self.path}: no component {self.comp!r}")
            head = heads[self.comp]
            rec, cols = snapshot.record_layout(fl, snapshot._indexing(head), head["nint_attr"],
                                               head["nfloat_attr"])
            self.rec, self.cols = rec, [c for c in cols if c[0] in ("x", "y", "z", "m")]
            if self.kind == "psp":
                n = int(head["nbodies"])
                self.buf = snapshot._grow(self.buf, n * rec)
                snapshot._read_into(self.path, int(head["data_start"]), self.buf, 0, n * rec)
            else:
                indir = self.path.split("SPL")[0]
                counts = []
                for name in subs[self.comp]:
                    with open(indir + name, "rb") as g:
                        counts.append(snapshot._u32(g, 1)[0])
                n = int(sum(counts))
                self.buf = snapshot._grow(self.buf, n * rec)
                at = 0
                for name, c in zip(subs[self.comp], counts):
                    snapshot._read_into(indir + name, 4, self.buf, at, c * rec)
                    at += c * rec
            self.n = n
        except Exception as e:          # reported on join
            self.error = e


def coefficient_series(files, comp, accumulate, reader="psp"):
    """times and the list of device coefficient tensors ``accumulate(x, y, z, m)``
    returns for each file (x, y, z, m float64 CUDA tensors)."""
    if reader not in ("psp", "spl"):
        raise ValueError("reader must be 'psp' or 'spl'")
    files = list(files)
    times, coefs = [], []
    bufs = [None, None]
    nxt = None
    if files:
        nxt = _Reader(files[0], comp, reader, bufs[0])
        nxt.start()
    for i in range(len(files)):
        cur = nxt
        cur.join()
        if cur.error is not None:
            raise cur.error
        bufs[i % 2] = cur.buf
        if i + 1 < len(files):
            nxt = _Reader(files[i + 1], comp, reader, bufs[(i + 1) % 2])
            nxt.start()
        cols = snapshot.columns(cur.buf, cur.n, cur.rec, cur.cols, device=True)
        times.append(cur.time)
        coefs.append(accumulate(cols["x"], cols["y"], cols["z"], cols["m"]))
    return np.array(times, dtype=np.float64), coefs


def stack_to_host(coefs):
    from .. import device as dev
    if not coefs:
        return np.zeros(0)
    return dev.to_host(torch.stack(coefs))
