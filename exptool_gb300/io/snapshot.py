"""EXP particle snapshots (PSP ``OUT.*`` and split ``SPL.*`` files) read into
page-locked memory and de-interleaved on the GPU.

Layout (the reference's readers, exptool/io/psp_io.py:102-230 and
spl_io.py:108-270):

* primary header: time (f8), total bodies (u32), component count (u32);
  the u32 at byte 16 equal to 2915019716 marks single-precision particles;
* PSP component header: [2 u32 when single precision] nbodies, nint_attr,
  nfloat_attr, info-string length (u32 each), then the YAML info string, then
  the component's packed records;
* SPL component header: 7 u32 (2 leading words, nprocs, nbodies, nint_attr,
  nfloat_attr, info length), the info string, then nprocs 1024-byte
  NUL-padded sub-file names; each sub-file holds its body count (u32) and its
  records from byte 4;
* record: [id i8 when parameters.indexing] m x y z vx vy vz potE (f4 or f8),
  nint_attr i4, nfloat_attr (f4 or f8), packed.

Records are read straight into page-locked host memory; one kernel
(xt_records_to_columns) reads them over the host link and writes the columns
either to the device (``device=True``: float columns as float64 tensors, the
form the basis pipelines take) or to page-locked host arrays with the file's
types (the reference's ``.data``).
"""
from __future__ import annotations

import ctypes
import os
import struct

import numpy as np
import torch

from .. import _lib
from .. import device as dev
from . import yaml_lite

FLOAT_MAGIC = 2915019716
_BASE = ["m", "x", "y", "z", "vx", "vy", "vz", "potE"]


def record_layout(float_len, indexing, nint, nfloat):
    """(record bytes, [(name, byte offset, file kind)]) with kind one of
    'i8', 'f4', 'f8', 'i4' (psp_io.py:199-217)."""
    fk = "f4" if float_len == 4 else "f8"
    cols, off = [], 0
    if indexing:
        cols.append(("id", 0, "i8"))
        off = 8
    for name in _BASE:
        cols.append((name, off, fk))
        off += float_len
    for i in range(int(nint)):
        cols.append((f"i_attr{i}", off, "i4"))
        off += 4
    for i in range(int(nfloat)):
        cols.append((f"f_attr{i}", off, fk))
        off += float_len
    return off, cols


def _indexing(head):
    """parameters.indexing of a component info dict (psp_io.py:166-169)."""
    try:
        return bool(head["parameters"]["indexing"])
    except (KeyError, TypeError):
        return head.get("indexing") == "true"


def _u32(f, n):
    b = f.read(4 * n)
    if len(b) != 4 * n:
        raise IOError("truncated snapshot header")
    return struct.unpack(f"<{n}I", b)


def read_psp_header(f):
    """Primary and component headers of a PSP file (psp_io.py:102-193):
    (time, float_len, {name: header dict with nbodies, nint_attr, nfloat_attr,
    data_start, data_end})."""
    f.seek(16)
    (cmagic,) = _u32(f, 1)
    float_len = 4 if cmagic == FLOAT_MAGIC else 8
    f.seek(0)
    (time,) = struct.unpack("<d", f.read(8))
    _ntot, ncomp = _u32(f, 2)
    headers = {}
    pos = 16
    for _ in range(ncomp):
        f.seek(pos)
        if float_len == 4:
            _a, _b, nbodies, nint, nfloat, ninfo = _u32(f, 6)
        else:
            nbodies, nint, nfloat, ninfo = _u32(f, 4)
        head = yaml_lite.load(f.read(ninfo).split(b"\x00")[0].decode())
        start = f.tell()
        rec, _ = record_layout(float_len, _indexing(head), nint, nfloat)
        head["nint_attr"], head["nfloat_attr"], head["nbodies"] = nint, nfloat, nbodies
        head["data_start"], head["data_end"] = start, start + nbodies * rec
        headers[head["name"]] = head
        pos = start + nbodies * rec
    return time, float_len, headers


def read_spl_header(f):
    """Primary and component headers of an SPL file (spl_io.py:108-170):
    (time, float_len, {name: header dict}, {name: [sub-file names]})."""
    f.seek(16)
    (cmagic,) = _u32(f, 1)
    float_len = 4 if cmagic == FLOAT_MAGIC else 8
    f.seek(0)
    (time,) = struct.unpack("<d", f.read(8))
    _ntot, ncomp = _u32(f, 2)
    headers, subfiles = {}, {}
    pos = 16
    for _ in range(ncomp):
        f.seek(pos)
        _a, _b, nprocs, nbodies, nint, nfloat, ninfo = _u32(f, 7)
        head = yaml_lite.load(f.read(ninfo).split(b"\x00")[0].decode())
        head["nint_attr"], head["nfloat_attr"] = nint, nfloat
        names = []
        for _p in range(nprocs):
            names.append(f.read(1024).split(b"\x00")[0].decode())
        headers[head["name"]] = head
        subfiles[head["name"]] = names
        pos = pos + 4 * 7 + ninfo + nprocs * 1024
    return time, float_len, headers, subfiles


def _pinned_bytes(nbytes):
    return torch.empty(max(int(nbytes), 16), dtype=torch.uint8, pin_memory=True)


def _grow(buf, nbytes):
    """`buf` if it holds nbytes, else a new page-locked buffer."""
    return buf if buf is not None and buf.numel() >= nbytes else _pinned_bytes(nbytes)


def _read_into(path, offset, buf, at, nbytes):
    """nbytes of `path` from `offset` into buf[at:at+nbytes] (one read)."""
    view = memoryview(buf.numpy())[at:at + nbytes]
    with open(path, "rb", buffering=0) as f:
        f.seek(offset)
        got = 0
        while got < nbytes:
            k = f.readinto(view[got:])
            if not k:
                raise IOError(f"{path}: truncated particle data")
            got += k


def columns(records, n, rec_bytes, cols, device=False):
    """De-interleave n records held in `records` (a page-locked uint8 tensor or
    a CUDA tensor) into a dict of columns: CUDA tensors (float columns as
    float64) when device, else page-locked NumPy arrays of the file's types."""
    if n == 0:
        empty = {"i8": np.int64, "i4": np.int32, "f4": np.float32, "f8": np.float64}
        return {name: (torch.empty(0, dtype=torch.float64 if k[0] == "f" else torch.int64, device=dev.device())
                       if device else np.empty(0, dtype=empty[k])) for name, _o, k in cols}
    kind_dev = {"i8": (_lib.XT_COL_I64, torch.int64), "i4": (_lib.XT_COL_I32, torch.int32),
                "f4": (_lib.XT_COL_F32_TO_F64, torch.float64), "f8": (_lib.XT_COL_F64, torch.float64)}
    kind_host = {"i8": (_lib.XT_COL_I64, torch.int64), "i4": (_lib.XT_COL_I32, torch.int32),
                 "f4": (_lib.XT_COL_F32, torch.float32), "f8": (_lib.XT_COL_F64, torch.float64)}
    kinds = kind_dev if device else kind_host
    outs = []
    for _name, _off, k in cols:
        code, dt = kinds[k]
        outs.append(torch.empty(n, dtype=dt, device=dev.device()) if device else
                    torch.empty(n, dtype=dt, pin_memory=True))
    lib = _lib.load()
    offs = (ctypes.c_int * len(cols))(*[o for _n, o, _k in cols])
    codes = (ctypes.c_int * len(cols))(*[kinds[k][0] for _n, _o, k in cols])
    pp, keep = _lib.ptr_array([t.data_ptr() for t in outs])
    _lib.check(lib.xt_records_to_columns(ctypes.c_void_p(records.data_ptr()), int(n), int(rec_bytes), len(cols),
                                         offs, codes, pp, dev.stream_ptr()), "xt_records_to_columns")
    torch.cuda.current_stream().synchronize()
    return {name: (t if device else t.numpy()) for (name, _o, _k), t in zip(cols, outs)}


def load_psp_component(path, head, float_len, device=False):
    rec, cols = record_layout(float_len, _indexing(head), head["nint_attr"], head["nfloat_attr"])
    n = int(head["nbodies"])
    buf = _pinned_bytes(n * rec)
    _read_into(path, int(head["data_start"]), buf, 0, n * rec)
    return columns(buf, n, rec, cols, device)


def load_spl_component(main_path, head, float_len, subfiles, device=False):
    """All sub-files of one component, concatenated in sub-file order
    (spl_io.py:183-204)."""
    rec, cols = record_layout(float_len, _indexing(head), head["nint_attr"], head["nfloat_attr"])
    indir = main_path.split("SPL")[0]
    counts = []
    for name in subfiles:
        with open(indir + name, "rb") as f:
            counts.append(_u32(f, 1)[0])
    n = int(sum(counts))
    buf = _pinned_bytes(n * rec)
    at = 0
    for name, c in zip(subfiles, counts):
        _read_into(indir + name, 4, buf, at, c * rec)
        at += c * rec
    return columns(buf, n, rec, cols, device)


# ------------------------------------------------------------------ writers
def _info_bytes(name, indexing, extra=None):
    lines = [f"name: {name}", "parameters:", f"  indexing: {'true' if indexing else 'false'}"]
    for k, v in (extra or {}).items():
        lines.append(f"{k}: {v}")
    return ("\n".join(lines) + "\n").encode()


def _records(comp, float_len, indexing):
    n = len(comp["m"])
    nint = len([k for k in comp if k.startswith("i_attr")])
    nfloat = len([k for k in comp if k.startswith("f_attr")])
    rec, cols = record_layout(float_len, indexing, nint, nfloat)
    np_kind = {"i8": "<i8", "i4": "<i4", "f4": "<f4", "f8": "<f8"}
    dt = np.dtype({"names": [c[0] for c in cols], "formats": [np_kind[c[2]] for c in cols],
                   "offsets": [c[1] for c in cols], "itemsize": rec})
    a = np.zeros(n, dtype=dt)
    for name, _o, _k in cols:
        a[name] = comp[name] if name in comp else 0
    return a, nint, nfloat


def write_psp(path, time, comps, float_len=8, indexing=False):
    """Write a PSP file readable by psp_io.Input: `comps` maps component name
    to a dict of columns (m x y z vx vy vz potE, optional id, i_attr*,
    f_attr*)."""
    with open(path, "wb") as f:
        f.write(struct.pack("<dII", time, sum(len(c["m"]) for c in comps.values()), len(comps)))
        for name, comp in comps.items():
            a, nint, nfloat = _records(comp, float_len, indexing)
            info = _info_bytes(name, indexing)
            if float_len == 4:
                f.write(struct.pack("<6I", FLOAT_MAGIC, 4, len(a), nint, nfloat, len(info)))
            else:
                f.write(struct.pack("<4I", len(a), nint, nfloat, len(info)))
            f.write(info)
            f.write(a.tobytes())


def write_spl(path, time, comps, nsub=2, float_len=8, indexing=False):
    """Write an SPL main file and its sub-files (`path` + component index +
    sub-file index, in the same directory) readable by spl_io.Input."""
    base = os.path.basename(path)
    folder = os.path.dirname(path)
    with open(path, "wb") as f:
        f.write(struct.pack("<dII", time, sum(len(c["m"]) for c in comps.values()), len(comps)))
        for ci, (name, comp) in enumerate(comps.items()):
            a, nint, nfloat = _records(comp, float_len, indexing)
            info = _info_bytes(name, indexing)
            f.write(struct.pack("<7I", FLOAT_MAGIC if float_len == 4 else 0, float_len, nsub, len(a), nint, nfloat,
                                len(info)))
            f.write(info)
            parts = np.array_split(np.arange(len(a)), nsub)
            for si, idx in enumerate(parts):
                sub = f"{base}_{ci}-{si}"
                with open(os.path.join(folder, sub), "wb") as g:
                    g.write(struct.pack("<I", len(idx)))
                    g.write(a[idx].tobytes())
                f.write(sub.encode().ljust(1024, b"\x00"))
