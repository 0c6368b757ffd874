"""Autotuner for launch shapes of the batched kernels.

Each tunable operation lists candidate configurations; ``tune`` times every
feasible candidate on the caller's own inputs (CUDA events, after one
warm-up), keeps the fastest and caches it in a JSON file keyed by the
operation, its problem parameters and the GPU name, so later runs reuse it.
Cache file: $XT_AUTOTUNE_CACHE or ~/.cache/exptool_gb300/autotune.json.
"""
from __future__ import annotations

import json
import os
import threading

import torch

from ._lib import XTError

_lock = threading.Lock()


def cache_path() -> str:
    p = os.environ.get("XT_AUTOTUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "exptool_gb300", "autotune.json")


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(d):
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + f".tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


def key(op: str, **params) -> str:
    gpu = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    return op + "|" + "|".join(f"{k}={params[k]}" for k in sorted(params)) + "|" + gpu


def lookup(k: str):
    with _lock:
        return _load().get(k)


def tune(k: str, candidates, run, reps: int = 3, force: bool = False):
    """Return (best_config, timings_ms).  ``run(cfg)`` launches one call."""
    if not force:
        hit = lookup(k)
        if hit is not None:
            return hit["best"], hit.get("ms", {})
    timings = {}
    for cfg in candidates:
        try:
            run(cfg)
            torch.cuda.synchronize()
        except XTError:
            continue                      # infeasible launch shape on this GPU
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            run(cfg)
        e1.record()
        torch.cuda.synchronize()
        timings[json.dumps(cfg)] = e0.elapsed_time(e1) / reps
    if not timings:
        raise RuntimeError(f"autotune {k}: no feasible candidate")
    best = json.loads(min(timings, key=timings.get))
    with _lock:
        d = _load()
        d[k] = {"best": best, "ms": timings}
        _store(d)
    return best, timings


def sph_batched_config(table, xyzm, offsets, force=False, sample_snaps=32):
    """Chunk size and CTA size of xt_sph_accumulate_batched for this table,
    tuned on (up to) the first ``sample_snaps`` snapshots of the batch."""
    import numpy as np
    offs = np.asarray(offsets, dtype=np.int64)
    ns = min(len(offs) - 1, sample_snaps)
    sub_offs = offs[:ns + 1]
    sub = xyzm[:int(sub_offs[-1])]
    k = key("sph_batched_v2", lmax=table.lmax, nmax=table.nmax, numr=table.numr)
    cands = [{"chunk": c, "threads": t} for c in (32768, 65536, 131072, 262144) for t in (256, 512, 768, 1024)]
    return tune(k, cands, lambda cfg: table.accumulate_batched(sub, sub_offs, chunk=cfg["chunk"],
                                                               threads=cfg["threads"]), force=force)


def sph_batched_tc_config(table, xyzm, offsets, force=False, sample_snaps=32):
    """Work-item size (particles), operand stages, CTAs per SM and threads per
    particle of xt_sph_accumulate_batched_tc for this table, tuned on (up to)
    the first ``sample_snaps`` snapshots of the batch.  The MMA tile is fixed
    by the table: M = 128 radial nodes, N = (lmax+1)^2 rows padded to 16,
    K = 128 particles per stage (48 KB of shared memory per stage at lmax 6).
    Candidates: chunks of 8k, 16k and 32k particles x 1 to 3 stages x one or
    two threads per particle x the full residency at that shape and one CTA
    per SM fewer."""
    import numpy as np
    offs = np.asarray(offsets, dtype=np.int64)
    ns = min(len(offs) - 1, sample_snaps)
    sub_offs = offs[:ns + 1]
    sub = xyzm[:int(sub_offs[-1])]
    k = key("sph_batched_tc_v4", lmax=table.lmax, nmax=table.nmax, numr=table.numr)
    cands = []
    for sp in (1, 2):
        for st in (1, 2, 3):
            res = table.batched_tc_residency(st, sp)
            for cp in sorted({res, max(1, res - 1)}):
                for c in (8192, 16384, 32768):
                    cands.append({"chunk": c, "stages": st, "ctas_per_sm": cp, "threads_per_particle": sp})
    ws = {}

    def run(cfg):
        need = table.batched_tc_workspace(sub_offs, cfg["chunk"])
        if ws.get("n", 0) < need:
            ws["t"] = torch.empty(need, dtype=torch.uint8, device=xyzm.device)
            ws["n"] = need
        table.accumulate_batched_tc(sub, sub_offs, chunk=cfg["chunk"], stages=cfg["stages"],
                                    ctas_per_sm=cfg["ctas_per_sm"], threads_per_particle=cfg["threads_per_particle"],
                                    workspace=ws["t"])

    return tune(k, cands, run, force=force)
