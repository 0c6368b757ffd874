"""Device-side objects: uploaded SL / EOF tables and the calls on them.

``SphTable`` and ``CylTable`` own a C-ABI table handle; their methods take and
return torch CUDA tensors and launch on the current torch stream.  Table
handles are cached by file identity (path, size, mtime) or by the identity
and a content fingerprint of the NumPy arrays they were built from, so the
reference-style APIs that pass tables on every call upload them once.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import threading

import numpy as np
import torch

from . import _lib

_F = {"f64": _lib.XT_F64, "f32": _lib.XT_F32, _lib.XT_F64: _lib.XT_F64, _lib.XT_F32: _lib.XT_F32}


def precision_code(p) -> int:
    try:
        return _F[p]
    except KeyError:
        raise ValueError(f"precision must be 'f64' or 'f32', got {p!r}") from None


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("exptool_gb300 needs a CUDA device (GB300, sm_103a); none is available")
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def to_dev(a, dtype=torch.float64) -> torch.Tensor:
    """numpy / tensor -> contiguous CUDA tensor of ``dtype``."""
    if isinstance(a, torch.Tensor):
        t = a.to(device=device(), dtype=dtype)
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64))).to(device(), dtype=dtype)
    return t.contiguous()


def to_dev_async(a) -> torch.Tensor:
    """numpy float64 -> CUDA float64 tensor, enqueued on the current stream
    without waiting when the source is in pinned memory (the caller keeps the
    source alive until the stream has passed the copy); pageable sources are
    copied synchronously by torch."""
    t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64)))
    return t.to(device(), non_blocking=True)


def host_access(a: np.ndarray) -> int:
    """How kernels can reach a NumPy array's buffer (``_lib.XT_PTR_*``)."""
    return int(_lib.load().xt_pointer_access(ctypes.c_void_p(a.ctypes.data)))


def kernel_input(a):
    """A float64 particle array in the form the kernels read: a CUDA tensor
    stays on the device; a contiguous array in page-locked host memory is
    passed in place (the kernels read it over the host link, so the transfer
    overlaps their work); anything else is copied to the device first."""
    if isinstance(a, torch.Tensor) and a.is_cuda:
        return a.to(torch.float64).contiguous()
    a = np.asarray(a, dtype=np.float64)
    if a.size and a.flags.c_contiguous and host_access(a) == _lib.XT_PTR_PINNED:
        return a
    return to_dev_async(a)


def pinned_empty(n: int, count: int) -> list:
    """``count`` float64 arrays of length n in page-locked host memory (torch's
    caching host allocator), as torch tensors the kernels can write directly."""
    return [torch.empty(n, dtype=torch.float64, pin_memory=True) for _ in range(count)]


def _addr(a) -> int:
    """Address of a tensor's, an array's or a raw address's data."""
    if isinstance(a, int):
        return a
    if isinstance(a, torch.Tensor):
        return a.data_ptr()
    return a.ctypes.data


def copy_and_sync(pairs):
    """Copy each (destination address, source address, bytes) on the current
    stream with one library call, then wait for the stream."""
    lib = _lib.load()
    k = len(pairs)
    dst = (ctypes.c_void_p * k)(*[p[0] for p in pairs])
    src = (ctypes.c_void_p * k)(*[p[1] for p in pairs])
    nb = (ctypes.c_size_t * k)(*[p[2] for p in pairs])
    st = stream_ptr()
    _lib.check(lib.xt_copy_async(k, dst, src, nb, st), "xt_copy_async")
    _lib.check(lib.xt_stream_sync(st), "xt_stream_sync")


def to_host_many(ts) -> list:
    """Several device tensors -> NumPy arrays in pinned host memory: all
    copies enqueued on the current stream, one synchronisation (None entries
    stay None)."""
    hs = [None if t is None else torch.empty(t.shape, dtype=t.dtype, pin_memory=True) for t in ts]
    for h, t in zip(hs, ts):
        if t is not None:
            h.copy_(t, non_blocking=True)
    torch.cuda.current_stream().synchronize()
    return [None if h is None else h.numpy() for h in hs]


_fetch_scratch = threading.local()
_coef_block = threading.local()


def fetch_many(ts) -> list:
    """Small device tensors (coefficients) -> NumPy arrays of their own: one
    library copy each into a per-thread page-locked scratch block, one wait,
    then a host copy out of the block.  Cheaper per call than fresh
    page-locked tensors from torch for a few kilobytes."""
    ts = [t.contiguous() for t in ts]
    nbs = [t.numel() * t.element_size() for t in ts]
    offs = np.cumsum([0] + [(nb + 255) & ~255 for nb in nbs]).tolist()
    buf = pinned_scratch(offs[-1])
    base = buf.data_ptr()
    copy_and_sync([(base + o, t.data_ptr(), nb) for o, t, nb in zip(offs, ts, nbs) if nb])
    hb = buf.numpy()
    return [hb[o:o + nb].view(_NP_DTYPE[t.dtype]).reshape(tuple(t.shape)).copy() for o, t, nb in zip(offs, ts, nbs)]


def pinned_scratch(nbytes: int) -> torch.Tensor:
    """This thread's page-locked scratch block (uint8, at least nbytes), kept
    between calls; its contents are valid until the thread's next use."""
    buf = getattr(_fetch_scratch, "v", None)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 1 << 16), dtype=torch.uint8, pin_memory=True)
        _fetch_scratch.v = buf
    return buf


_NP_DTYPE = {torch.float64: np.float64, torch.float32: np.float32, torch.int32: np.int32, torch.int64: np.int64}


def to_host(t: torch.Tensor) -> np.ndarray:
    """Device tensor -> NumPy array in pinned host memory (torch's caching
    host allocator), so the device-to-host copy is a direct DMA; the array
    owns its buffer."""
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t)
    return h.numpy()


def dptr(t) -> int:
    return 0 if t is None else t.data_ptr()


def fingerprint(*arrays) -> str:
    """Cheap content fingerprint of numpy arrays (shape, dtype and a hash of a
    bounded strided sample plus the full bytes of small arrays)."""
    h = hashlib.blake2b(digest_size=16)
    for a in arrays:
        a = np.asarray(a)
        h.update(str((a.shape, a.dtype.str)).encode())
        flat = a.reshape(-1)
        if flat.size <= 1 << 17:
            h.update(np.ascontiguousarray(flat).tobytes())
        else:
            step = max(1, flat.size // (1 << 16))
            h.update(np.ascontiguousarray(flat[::step]).tobytes())
            h.update(np.ascontiguousarray(flat[-64:]).tobytes())
    return h.hexdigest()


def file_key(path: str):
    st = os.stat(path)
    return (os.path.abspath(path), st.st_size, st.st_mtime_ns)


class _Cache:
    def __init__(self, limit=8):
        self._d = {}
        self._lock = threading.Lock()
        self._limit = limit

    def get(self, key, make):
        with self._lock:
            if key in self._d:
                v = self._d.pop(key)
                self._d[key] = v
                return v
        v = make()
        with self._lock:
            self._d[key] = v
            while len(self._d) > self._limit:
                self._d.pop(next(iter(self._d)))
        return v


TABLES = _Cache()


class SphTable:
    """Uploaded spherical SL basis (halo_methods.read_cached_table + init_table)."""

    def __init__(self, lmax, nmax, numr, cmap, rmin, rmax, scale, xi, p0, d0, ev, ef):
        device()
        lib = _lib.load()
        self.lmax, self.nmax, self.numr, self.cmap = int(lmax), int(nmax), int(numr), int(cmap)
        self.rmin, self.rmax, self.scale = float(rmin), float(rmax), float(scale)
        self.xi = np.ascontiguousarray(xi, dtype=np.float64)
        self.xi_min = float(np.min(self.xi))
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (xi, p0, d0, ev, ef)]
        if arrs[0].size != self.numr or arrs[3].shape != (self.lmax + 1, self.nmax) or \
                arrs[4].shape != (self.lmax + 1, self.nmax, self.numr):
            raise ValueError("SL table arrays do not match lmax/nmax/numr")
        self.p0, self.d0, self.ev, self.ef = arrs[1], arrs[2], arrs[3], arrs[4]
        h = _lib.c_vp()
        _lib.check(lib.xt_sph_table_create(self.lmax, self.nmax, self.numr, self.cmap, self.rmin, self.rmax,
                                           self.scale, *[a.ctypes.data for a in arrs], _lib.ctypes.byref(h)),
                   "xt_sph_table_create")
        self.handle = h.value
        self._lib = lib
        self.field_cache = _Cache(limit=8)

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self._lib.xt_sph_table_destroy(self.handle)
        except Exception:
            pass

    @property
    def nrow(self):
        return (self.lmax + 1) ** 2

    def accumulate(self, x, y, z, m, no_odd=False, precision="f64", workspace=None):
        n = int(x.numel())
        out = torch.empty((self.nrow, self.nmax), dtype=torch.float64, device=x.device)
        need = self._lib.xt_sph_accumulate_workspace(self.handle)
        ws = workspace if workspace is not None else torch.empty(need, dtype=torch.uint8, device=x.device)
        _lib.check(self._lib.xt_sph_accumulate(self.handle, dptr(x), dptr(y), dptr(z), dptr(m), n, int(bool(no_odd)),
                                               precision_code(precision), dptr(out), dptr(ws), ws.numel(),
                                               stream_ptr()), "xt_sph_accumulate")
        return out

    def accumulate_batched(self, xyzm, offsets, no_odd=False, chunk=262144, threads=512, workspace=None):
        """Coefficients of many snapshots in one persistent launch.  xyzm: (N, 4)
        float32 CUDA tensor; offsets: host int64 array (nsnap+1).  Returns a
        (nsnap, (lmax+1)^2, nmax) float64 tensor."""
        offs = np.ascontiguousarray(np.asarray(offsets, dtype=np.int64))
        nsnap = offs.size - 1
        if xyzm.dtype != torch.float32 or xyzm.dim() != 2 or xyzm.shape[1] != 4 or not xyzm.is_contiguous():
            raise ValueError("xyzm must be a contiguous (N, 4) float32 CUDA tensor")
        out = torch.empty((nsnap, self.nrow, self.nmax), dtype=torch.float64, device=xyzm.device)
        need = self._lib.xt_sph_batched_workspace(self.handle, nsnap, int(offs[-1]), int(chunk))
        ws = workspace if (workspace is not None and workspace.numel() >= need) else \
            torch.empty(need, dtype=torch.uint8, device=xyzm.device)
        _lib.check(self._lib.xt_sph_accumulate_batched(self.handle, dptr(xyzm), offs.ctypes.data, nsnap,
                                                       int(bool(no_odd)), int(chunk), int(threads), dptr(out),
                                                       dptr(ws), ws.numel(), stream_ptr()),
                   "xt_sph_accumulate_batched")
        return out

    def accumulate_batched_tc(self, xyzm, offsets, no_odd=False, chunk=16384, stages=2, ctas_per_sm=0,
                              threads_per_particle=1, workspace=None):
        """Coefficients of many snapshots on the tensor cores: particles
        counting-sorted by (snapshot, radial window), then per window a BF16
        tcgen05 product of the interpolation weights and the angular basis
        values with FP32 accumulation, FP64 sums of the window partials and an
        FP64 contraction.  Arguments as for accumulate_batched; ``chunk`` is
        the most particles of one work item, ``stages`` the operand buffers per
        CTA (1 to 3), ``ctas_per_sm`` the CTAs of the persistent launch per SM
        (0: as many as are resident), ``threads_per_particle`` 1 or 2 (the
        angular rows split by the parity of m).  Returns a (nsnap,
        (lmax+1)^2, nmax) float64 tensor."""
        offs = np.ascontiguousarray(np.asarray(offsets, dtype=np.int64))
        nsnap = offs.size - 1
        if xyzm.dtype != torch.float32 or xyzm.dim() != 2 or xyzm.shape[1] != 4 or not xyzm.is_contiguous():
            raise ValueError("xyzm must be a contiguous (N, 4) float32 CUDA tensor")
        out = torch.empty((nsnap, self.nrow, self.nmax), dtype=torch.float64, device=xyzm.device)
        need = self._lib.xt_sph_batched_tc_workspace(self.handle, nsnap, offs.ctypes.data, int(chunk))
        if need == 0:
            raise ValueError("bad batched arguments (offsets, chunk)")
        ws = workspace if (workspace is not None and workspace.numel() >= need) else \
            torch.empty(need, dtype=torch.uint8, device=xyzm.device)
        _lib.check(self._lib.xt_sph_accumulate_batched_tc(self.handle, dptr(xyzm), offs.ctypes.data, nsnap,
                                                          int(bool(no_odd)), int(chunk), int(stages),
                                                          int(ctas_per_sm), int(threads_per_particle), dptr(out),
                                                          dptr(ws), ws.numel(), stream_ptr()),
                   "xt_sph_accumulate_batched_tc")
        return out

    def batched_tc_residency(self, stages, threads_per_particle=1):
        """CTAs of the tensor-core accumulation resident per SM at this
        pipeline depth and split (the largest useful ``ctas_per_sm``)."""
        v = ctypes.c_int(0)
        _lib.check(self._lib.xt_sph_batched_tc_residency(self.handle, int(stages), int(threads_per_particle),
                                                         ctypes.byref(v)),
                   "xt_sph_batched_tc_residency")
        return int(v.value)

    def batched_tc_workspace(self, offsets, chunk=16384):
        offs = np.ascontiguousarray(np.asarray(offsets, dtype=np.int64))
        return int(self._lib.xt_sph_batched_tc_workspace(self.handle, offs.size - 1, offs.ctypes.data, int(chunk)))

    def prepare(self, expcoef, coef_scale=1.0, lmax_use=-1, nmax_use=-1, precision="f64"):
        pc = precision_code(precision)
        nbytes = self._lib.xt_sph_field_bytes(self.handle, pc)
        field = torch.empty(nbytes, dtype=torch.uint8, device=device())
        ec = to_dev(expcoef)
        if ec.shape != (self.nrow, self.nmax):
            raise ValueError(f"expcoef shape {tuple(ec.shape)} != {(self.nrow, self.nmax)}")
        _lib.check(self._lib.xt_sph_prepare(self.handle, dptr(ec), float(coef_scale), int(lmax_use), int(nmax_use), pc,
                                            dptr(field), nbytes, stream_ptr()), "xt_sph_prepare")
        return SphField(self, field, pc, lmax_use if 0 <= lmax_use <= self.lmax else self.lmax)

    def eval_points(self, field, a, b, c, mode, coord_mode, L1=-1000, L2=1000, no_odd=False, lmax_use=-1,
                    trig_l=False, want=None):
        n = int(a.numel())
        outs = [torch.empty(n, dtype=torch.float64, device=a.device) if (want is None or want[k]) else None
                for k in range(8)]
        pp, keep = _lib.ptr_array([dptr(t) for t in outs])
        _lib.check(self._lib.xt_sph_eval_points(self.handle, dptr(field.buf), field.precision, coord_mode, dptr(a),
                                                dptr(b), dptr(c), n, mode, int(L1), int(L2), int(bool(no_odd)),
                                                int(lmax_use), int(bool(trig_l)), pp, stream_ptr()),
                   "xt_sph_eval_points")
        return outs


class SphField:
    """Coefficient-contracted radial field of a SphTable."""

    def __init__(self, table, buf, precision, lmax_use):
        self.table, self.buf, self.precision, self.lmax_use = table, buf, precision, lmax_use


class CylTable:
    """Uploaded EOF basis (eof.parse_eof + eof_params + set_table_params)."""

    def __init__(self, mmax, norder, numx, numy, cmap, dens, XMIN, dX, YMIN, dY, ascale, hscale, potC, rforceC,
                 zforceC, densC, potS, rforceS, zforceS, densS):
        device()
        lib = _lib.load()
        self.mmax, self.norder, self.numx, self.numy = int(mmax), int(norder), int(numx), int(numy)
        self.cmap, self.dens = int(cmap), int(bool(dens))
        self.XMIN, self.dX, self.YMIN, self.dY = float(XMIN), float(dX), float(YMIN), float(dY)
        self.ascale, self.hscale = float(ascale), float(hscale)
        shape = (self.mmax + 1, self.norder, self.numx + 1, self.numy + 1)
        arrs = []
        for a in (potC, rforceC, zforceC, densC if self.dens else None, potS, rforceS, zforceS,
                  densS if self.dens else None):
            if a is None:
                arrs.append(None)
                continue
            a = np.ascontiguousarray(np.asarray(a, dtype=np.float64)[:shape[0], :shape[1]])
            if a.shape != shape:
                raise ValueError(f"EOF table shape {a.shape} != {shape}")
            arrs.append(a)
        ptrs = [a.ctypes.data if a is not None else None for a in arrs]
        h = _lib.c_vp()
        _lib.check(lib.xt_cyl_table_create(self.mmax, self.norder, self.numx, self.numy, self.cmap, self.dens,
                                           self.XMIN, self.dX, self.YMIN, self.dY, self.ascale, self.hscale, *ptrs,
                                           _lib.ctypes.byref(h)), "xt_cyl_table_create")
        self.handle = h.value
        self._lib = lib
        self.field_cache = _Cache(limit=8)
        self._fused_bufs = threading.local()
        self._sorted_ws = threading.local()

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self._lib.xt_cyl_table_destroy(self.handle)
        except Exception:
            pass

    def accumulate(self, x, y, z, m, precision="f64", workspace=None):
        n = int(x.numel())
        cos = torch.empty((self.mmax + 1, self.norder), dtype=torch.float64, device=x.device)
        sin = torch.empty_like(cos)
        need = self._lib.xt_cyl_accumulate_workspace(self.handle)
        ws = workspace if workspace is not None else torch.empty(need, dtype=torch.uint8, device=x.device)
        _lib.check(self._lib.xt_cyl_accumulate(self.handle, dptr(x), dptr(y), dptr(z), dptr(m), n,
                                               precision_code(precision), dptr(cos), dptr(sin), dptr(ws), ws.numel(),
                                               stream_ptr()), "xt_cyl_accumulate")
        return cos, sin

    def accumulate_eval(self, x, y, z, m, precision="f64", m1=0, m2=1000, workspace=None, nan_to_origin=True,
                        outs=None, coef=None):
        """Fused accumulate + accumulated_eval_particles at the same particles:
        returns cos, sin, [p0, p, fr, fp, fz, R].  x, y, z, m are CUDA tensors
        or contiguous float64 NumPy arrays the device addresses (see
        ``kernel_input``); ``outs`` optionally gives the six result arrays
        (CUDA tensors or page-locked host tensors, written in place) and
        ``coef`` a (2, mmax+1, norder) device tensor for cos and sin."""
        n = int(x.numel()) if isinstance(x, torch.Tensor) else int(np.asarray(x).size)
        pc = precision_code(precision)
        if coef is None:
            coef = torch.empty((2, self.mmax + 1, self.norder), dtype=torch.float64, device=device())
        cos, sin = coef[0], coef[1]
        if outs is None:
            outs = [torch.empty(n, dtype=torch.float64, device=device()) for _ in range(6)]
        need = self._lib.xt_cyl_accumulate_eval_workspace(self.handle, n, pc)
        ws = workspace if (workspace is not None and workspace.numel() >= need) else \
            torch.empty(need, dtype=torch.uint8, device=device())

        def ptr(a):
            return a.data_ptr() if isinstance(a, torch.Tensor) else a.ctypes.data

        pp, keep = _lib.ptr_array([ptr(t) for t in outs])
        _lib.check(self._lib.xt_cyl_accumulate_eval(self.handle, ptr(x), ptr(y), ptr(z), ptr(m), n, pc, int(m1),
                                                    int(m2), int(bool(nan_to_origin)), dptr(cos), dptr(sin), pp,
                                                    dptr(ws), ws.numel(), stream_ptr()), "xt_cyl_accumulate_eval")
        return cos, sin, outs

    def active_blocks(self, workspace, n, precision="f64"):
        """(listed, total) node blocks of the last fused call made on
        ``workspace`` for n particles: the blocks the contraction and the
        field stage read (those touching a cell with particles).  Synchronises
        the device."""
        a, t = ctypes.c_int(0), ctypes.c_int(0)
        _lib.check(self._lib.xt_cyl_active_blocks(self.handle, dptr(workspace), int(n), precision_code(precision),
                                                  ctypes.byref(a), ctypes.byref(t)), "xt_cyl_active_blocks")
        return a.value, t.value

    def accumulate_eval_blocks(self, x, y, z, m, precision="f64", m1=0, m2=1000, nan_to_origin=True, r_out=None,
                               res_out=None):
        """accumulate_eval into per-thread buffers kept for the last particle
        count and precision: returns the (2, mmax+1, norder) coefficient block
        (cos, sin) and the (5, n) block of p0, p, fr, fp, fz.  The next call on
        this thread with the same size overwrites both, so callers copy them
        out first.  R goes to ``r_out`` (a length-n float64 tensor or a raw
        address, device or page-locked host memory; the binning kernel writes
        it directly).  With ``res_out`` (the address of 5 n page-locked
        float64) p0 p fr fp fz go there instead, each part of the particles
        copied out while the next is evaluated, and the second value returned
        is None; the copies are complete when the stream's work is.  The call's
        C arguments are kept with the buffers, so a repeated call only sets the
        particle and result addresses."""
        n = int(x.numel()) if isinstance(x, torch.Tensor) else int(np.asarray(x).size)
        pc = precision_code(precision)
        key = (n, pc)
        b = getattr(self._fused_bufs, "v", None)
        if b is None or b[0] != key:
            need = self._lib.xt_cyl_accumulate_eval_workspace(self.handle, n, pc)
            ws = torch.empty(need, dtype=torch.uint8, device=device())
            coef = torch.empty((2, self.mmax + 1, self.norder), dtype=torch.float64, device=device())
            res = torch.empty((6, n), dtype=torch.float64, device=device())
            outs = (ctypes.c_void_p * 6)(*[res.data_ptr() + 8 * n * k for k in range(6)])
            b = (key, ws, coef, res, outs)
            self._fused_bufs.v = b
        _, ws, coef, res, outs = b
        for k in range(5):
            outs[k] = (res_out + 8 * n * k) if res_out is not None else res.data_ptr() + 8 * n * k
        outs[5] = _addr(r_out) if r_out is not None else res.data_ptr() + 40 * n
        cos_p = coef.data_ptr()
        _lib.check(self._lib.xt_cyl_accumulate_eval(self.handle, _addr(x), _addr(y), _addr(z), _addr(m), n, pc,
                                                    int(m1), int(m2), int(bool(nan_to_origin)), cos_p,
                                                    cos_p + 8 * (self.mmax + 1) * self.norder, outs, ws.data_ptr(),
                                                    ws.numel(), stream_ptr()), "xt_cyl_accumulate_eval")
        return coef, (None if res_out is not None else res[:5])

    def sorted_ok(self):
        """Whether the table fits the sorted pipeline (mmax <= 8, norder <= 24,
        numx * numy <= 2^20 cells)."""
        return self.mmax <= 8 and self.norder <= 24 and self.numx * self.numy <= (1 << 20)

    def _sorted_workspace(self, n, pc):
        """Per-thread device workspace of the sorted calls, grown as needed."""
        need = self._lib.xt_cyl_accumulate_eval_workspace(self.handle, n, pc)
        ws = getattr(self._sorted_ws, "v", None)
        if ws is None or ws.numel() < need:
            ws = torch.empty(need, dtype=torch.uint8, device=device())
            self._sorted_ws.v = ws
        return ws

    def accumulate_sorted(self, x, y, z, m, precision="f64", nan_to_origin=True, host=False):
        """Coefficients through the sorted pipeline (binning, counting sort by
        cell, run-accumulated deposit, contraction): a (2, mmax+1, norder)
        device tensor of cos and sin, or with ``host`` a NumPy array of its
        own (the last kernel writes the coefficients into a per-thread
        page-locked block, then one wait).  x, y, z, m as for accumulate_eval."""
        n = int(x.numel()) if isinstance(x, torch.Tensor) else int(np.asarray(x).size)
        pc = precision_code(precision)
        ws = self._sorted_workspace(n, pc)
        nc = (self.mmax + 1) * self.norder
        if host:
            coef = None
            base = pinned_scratch(16 * nc).data_ptr()
        else:
            coef = torch.empty((2, self.mmax + 1, self.norder), dtype=torch.float64, device=device())
            base = coef.data_ptr()
        _lib.check(self._lib.xt_cyl_accumulate_sorted(self.handle, _addr(x), _addr(y), _addr(z), _addr(m), n, pc,
                                                      int(bool(nan_to_origin)), base, base + 8 * nc,
                                                      ws.data_ptr(), ws.numel(), stream_ptr()),
                   "xt_cyl_accumulate_sorted")
        if not host:
            return coef
        copy_and_sync([])
        return pinned_scratch(16 * nc).numpy()[:16 * nc].view(np.float64).reshape(2, self.mmax + 1,
                                                                                 self.norder).copy()

    def eval_sorted(self, x, y, z, cos, sin, precision="f64", m1=0, m2=1000, r_out=None, res_out=None):
        """accumulated_eval_particles (no density) through the sorted pipeline
        from coefficients cos, sin ((mmax+1, norder) float64, device tensors or
        page-locked host arrays the kernels read in place): a (6, n)
        device tensor of p0, p, fr, fp, fz, R in particle order.  With
        ``r_out`` (a length-n float64 tensor or a raw address, device or
        page-locked host memory) R is written there by the binning kernel
        instead of into row 5.  With ``res_out`` (the address of 5 n
        page-locked float64) p0 p fr fp fz go there, one part of the particles
        (3/8, then 5/8) at a time behind the evaluation, and None is returned;
        they are complete when the stream's work is."""
        n = int(x.numel()) if isinstance(x, torch.Tensor) else int(np.asarray(x).size)
        pc = precision_code(precision)
        ws = self._sorted_workspace(n, pc)
        res = None
        if res_out is None:
            res = torch.empty((6, n), dtype=torch.float64, device=device())
            outs = (ctypes.c_void_p * 6)(*[res.data_ptr() + 8 * n * k for k in range(6)])
        else:
            outs = (ctypes.c_void_p * 6)(*[res_out + 8 * n * k for k in range(5)], None)
        if r_out is not None:
            outs[5] = _addr(r_out)
        _lib.check(self._lib.xt_cyl_eval_sorted(self.handle, _addr(x), _addr(y), _addr(z), n, pc, int(m1), int(m2),
                                                _addr(cos), _addr(sin), outs, ws.data_ptr(), ws.numel(), stream_ptr()),
                   "xt_cyl_eval_sorted")
        return res

    def prepare(self, cos, sin, mmax_use=-1, nmax_use=-1, density=False, precision="f64"):
        pc = precision_code(precision)
        nbytes = self._lib.xt_cyl_field_bytes(self.handle, int(bool(density)), pc)
        field = torch.empty(nbytes, dtype=torch.uint8, device=device())
        c = to_dev(np.asarray(cos, dtype=np.float64) if not isinstance(cos, torch.Tensor) else cos)
        s = to_dev(np.asarray(sin, dtype=np.float64) if not isinstance(sin, torch.Tensor) else sin)
        c = pad2(c, self.mmax + 1, self.norder)
        s = pad2(s, self.mmax + 1, self.norder)
        _lib.check(self._lib.xt_cyl_prepare(self.handle, dptr(c), dptr(s), int(mmax_use), int(nmax_use),
                                            int(bool(density)), pc, dptr(field), nbytes, stream_ptr()),
                   "xt_cyl_prepare")
        return CylField(self, field, pc, bool(density))

    def eval_points(self, field, a, b, c, mode, coord_mode, m1=0, m2=1000, mmax_use=-1, no_odd=False,
                    perturb=False, want=None):
        n = int(a.numel())
        outs = [torch.empty(n, dtype=torch.float64, device=a.device) if (want is None or want[k]) else None
                for k in range(8)]
        pp, keep = _lib.ptr_array([dptr(t) for t in outs])
        _lib.check(self._lib.xt_cyl_eval_points(self.handle, dptr(field.buf), field.precision, int(field.density),
                                                coord_mode, dptr(a), dptr(b), dptr(c), n, mode, int(m1), int(m2),
                                                int(mmax_use), int(bool(no_odd)), int(bool(perturb)), pp,
                                                stream_ptr()), "xt_cyl_eval_points")
        return outs


def coef_pair(cos, sin, rows, cols):
    """Coefficients (cos, sin) zero-padded or cropped to (rows, cols) float64,
    in the form the sorted evaluation reads them: CUDA tensors stay on the
    device; host arrays are written into this thread's page-locked
    coefficient block and read there in place by the kernels over the host
    link (no copy).  The block is rewritten by the thread's next call, so the
    caller waits for the kernels first."""
    if isinstance(cos, torch.Tensor) or isinstance(sin, torch.Tensor):
        return pad2(to_dev(cos), rows, cols), pad2(to_dev(sin), rows, cols)
    nb = 2 * rows * cols * 8
    buf = getattr(_coef_block, "v", None)
    if buf is None or buf.numel() < nb:
        buf = torch.empty(max(nb, 1 << 16), dtype=torch.uint8, pin_memory=True)
        _coef_block.v = buf
    hn = buf.numpy()[:nb].view(np.float64).reshape(2, rows, cols)
    hn[...] = 0.0
    for k, a in enumerate((cos, sin)):
        a = np.asarray(a, dtype=np.float64)
        r, c = min(rows, a.shape[0]), min(cols, a.shape[1])
        hn[k, :r, :c] = a[:r, :c]
    return hn[0], hn[1]


def pad2(t, rows, cols):
    """Zero-pad / crop a (r, c) coefficient tensor to (rows, cols)."""
    if t.shape == (rows, cols):
        return t.contiguous()
    out = torch.zeros((rows, cols), dtype=t.dtype, device=t.device)
    r, c = min(rows, t.shape[0]), min(cols, t.shape[1])
    out[:r, :c] = t[:r, :c]
    return out


class CylField:
    def __init__(self, table, buf, precision, density):
        self.table, self.buf, self.precision, self.density = table, buf, precision, density


def cyl_field_engine(engine):
    """Kernel of the cylindrical field stage for later calls: 0 automatic
    (the bulk-copy pipeline where it fits), 1 the pipeline, 2 row loads."""
    _lib.check(_lib.load().xt_cyl_field_engine(int(engine)), "xt_cyl_field_engine")


def cyl_status():
    """Raise XTError if a cylindrical field launch reported a bulk-copy wait
    that timed out; synchronises the device."""
    _lib.check(_lib.load().xt_cyl_status(), "xt_cyl_status")


def batched_tc_status():
    """Raise XTError if a batched tensor-core launch reported an error (an
    MMA wait that timed out, or a particle outside its sorted window);
    synchronises the device."""
    _lib.check(_lib.load().xt_sph_batched_tc_status(), "xt_sph_batched_tc_status")


def fields_forces(sph_field, cyl_field, x, y, z, rotpos=None, rotpos_scalar=0.0, halo_l=-1, disk_m=-1,
                  no_odd=False, trig_l=True, precision=None):
    """Fields.return_forces_cart at the points (x, y, z): 8 output tensors."""
    lib = _lib.load()
    pc = sph_field.precision if precision is None else precision_code(precision)
    if sph_field.precision != pc or cyl_field.precision != pc:
        raise ValueError("both fields must be prepared at the requested precision")
    n = int(x.numel())
    outs = [torch.empty(n, dtype=torch.float64, device=x.device) for _ in range(8)]
    pp, keep = _lib.ptr_array([dptr(t) for t in outs])
    _lib.check(lib.xt_fields_forces(sph_field.table.handle, dptr(sph_field.buf), cyl_field.table.handle,
                                    dptr(cyl_field.buf), pc, int(halo_l), int(disk_m), int(bool(no_odd)),
                                    int(bool(trig_l)), dptr(x), dptr(y), dptr(z), dptr(rotpos),
                                    float(rotpos_scalar), n, pp, stream_ptr()), "xt_fields_forces")
    return outs


STATE_SLOTS = ("x", "y", "z", "vx", "vy", "vz", "fx", "fy", "fz", "pot", "r2m1", "r2m2", "aps", "nstep", "e0",
               "edev")


def orbit_sort_workspace(cyl_field, n):
    return int(_lib.load().xt_orbit_sort_workspace(cyl_field.table.handle, int(n)))


def orbit_sort(cyl_field, state_in, state_out, order_in, order_out, workspace):
    """Counting sort of the orbits of ``state_in`` (16 x n float64) by disc
    table cell into ``state_out``, carrying the original indices
    (xt_orbit_sort)."""
    n = int(state_in.shape[1])
    _lib.check(_lib.load().xt_orbit_sort(cyl_field.table.handle, dptr(state_in), dptr(state_out), n, dptr(order_in),
                                         dptr(order_out), dptr(workspace), workspace.numel(), stream_ptr()),
               "xt_orbit_sort")


def orbit_unsort(state_in, state_out, order):
    """Orbit q of ``state_in`` to column order[q] of ``state_out``."""
    _lib.check(_lib.load().xt_orbit_unsort(dptr(state_in), dptr(state_out), int(state_in.shape[1]), dptr(order),
                                           stream_ptr()), "xt_orbit_unsort")


def leapfrog(sph_field, cyl_field, state, step0, nsteps, nint, dt, rotc=0.0, apse=False, ap_max=1000, traj=None,
             halo_l=-1, disk_m=-1, no_odd=False, trig_l=True, dts=None):
    """Advance orbit ensemble ``state`` (16 x n float64 tensor) in place;
    ``dts`` (n float64 CUDA tensor) gives each orbit its own step."""
    lib = _lib.load()
    n = int(state.shape[1])
    pp, keep = _lib.ptr_array([state[k].data_ptr() for k in range(len(STATE_SLOTS))])
    _lib.check(lib.xt_leapfrog(sph_field.table.handle, dptr(sph_field.buf), cyl_field.table.handle,
                               dptr(cyl_field.buf), sph_field.precision, int(halo_l), int(disk_m), int(bool(no_odd)),
                               int(bool(trig_l)), pp, n, int(step0), int(nsteps), int(nint), float(dt), float(rotc),
                               int(bool(apse)), int(ap_max), dptr(traj), dptr(dts), stream_ptr()), "xt_leapfrog")
