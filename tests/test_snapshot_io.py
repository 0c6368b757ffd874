"""Snapshot readers on the CPU: the YAML subset, header parsing and the
record layout, against the reference's own psp_io / spl_io outputs
(tests/golden/snapshots.npz, made by tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

SNAP = os.path.join(GOLDEN, "snap")
FILES = {"OUT.f4idx": "psp", "OUT.f8": "psp", "SPL.f4": "spl", "SPL.f8idx": "spl"}


def _golden():
    return np.load(os.path.join(GOLDEN, "snapshots.npz"))


def test_yaml_subset():
    from exptool_gb300.io import yaml_lite as y
    doc = """name: star   # comment
parameters:
  indexing: true
  EJ: 2
  lst: [1, 2.5, ~]
force:
  id: cylinder
  parameters: {acyl: 0.01, hcyl: 1e-3, 'q': "a # b", flag: Off}
seq:
  - 1
  - {a: .5}
  - key: val
    other: 3
"""
    d = y.load(doc)
    assert d["name"] == "star"
    assert d["parameters"] == {"indexing": True, "EJ": 2, "lst": [1, 2.5, None]}
    # YAML 1.1 resolution: no decimal point -> string; Off -> false
    assert d["force"]["parameters"] == {"acyl": 0.01, "hcyl": "1e-3", "q": "a # b", "flag": False}
    assert d["seq"] == [1, {"a": 0.5}, {"key": "val", "other": 3}]
    assert y.load("a: 010\nb: 0x1f\nc: -.inf\nd: Yes\ne: yEs\n") == {"a": 8, "b": 31, "c": float("-inf"),
                                                                      "d": True, "e": "yEs"}


@pytest.mark.parametrize("fname", list(FILES))
def test_headers_match_reference(fname):
    from exptool_gb300.io import snapshot
    g = _golden()
    ref = json.loads(str(g[f"{fname}/header"]))
    with open(os.path.join(SNAP, fname), "rb") as f:
        if FILES[fname] == "psp":
            time, _fl, head = snapshot.read_psp_header(f)
            assert time == 1.25
        else:
            time, _fl, head, subs = snapshot.read_spl_header(f)
            assert time == 2.5
            assert all(len(v) == 3 for v in subs.values())
    assert json.loads(json.dumps(head, sort_keys=True)) == ref


@pytest.mark.parametrize("fname", list(FILES))
def test_record_layout_matches_reference(fname):
    """The layout the GPU de-interleave uses, applied on the CPU as a
    structured view of the raw bytes, reproduces the reference's columns."""
    from exptool_gb300.io import snapshot
    g = _golden()
    path = os.path.join(SNAP, fname)
    with open(path, "rb") as f:
        hdr = snapshot.read_psp_header(f) if FILES[fname] == "psp" else snapshot.read_spl_header(f)
    fl, heads = hdr[1], hdr[2]
    kinds = {"i8": "<i8", "i4": "<i4", "f4": "<f4", "f8": "<f8"}
    for cname, head in heads.items():
        rec, cols = snapshot.record_layout(fl, snapshot._indexing(head), head["nint_attr"], head["nfloat_attr"])
        dt = np.dtype({"names": [c[0] for c in cols], "formats": [kinds[c[2]] for c in cols],
                       "offsets": [c[1] for c in cols], "itemsize": rec})
        if FILES[fname] == "psp":
            raw = np.fromfile(path, dtype=np.uint8)[head["data_start"]:head["data_end"]]
        else:
            parts = []
            for sub in hdr[3][cname]:
                b = np.fromfile(os.path.join(SNAP, sub), dtype=np.uint8)
                n = int(b[:4].view("<u4")[0])
                parts.append(b[4:4 + n * rec])
            raw = np.concatenate(parts)
        a = raw.view(dt)
        for name, _o, _k in cols:
            want = g[f"{fname}/{cname}/{name}"]
            assert a[name].dtype == want.dtype.newbyteorder("<")
            assert np.array_equal(a[name], want), (fname, cname, name)
