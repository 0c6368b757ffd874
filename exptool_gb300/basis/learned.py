"""Learned radial basis for the spherical SL expansion.

One network per harmonic l maps log r to all K radial functions phi_nl and
their radial derivatives at once (layers 1 -> 128 -> 128 -> 128 -> 2K, SiLU,
BF16 weights, FP32 accumulation).  The networks learn the residual of the
method's own table functions (the table interpolation of
``spheresl.get_halo_dens_pot_force``, spheresl.py:106-160) over the analytic
Hernquist-Ostriker functions, which are the SL eigenfunctions of an
untruncated Hernquist background:

    phi_nl(r)      = s_nl HO_nl(r/a) + sig_nl      Y_n(t)
    r dphi_nl/dr   = s_nl u HO'_nl   + sig'_nl     Y_{K+n}(t),   t = normalised ln r

Training, labels and inference run in this package's CUDA library
(``xt_mlp_*``, ``xt_learned_*``): the GPU labels radii from the uploaded
tables, trains with its own forward/backward/Adam kernels, and evaluates
forces with the coefficient contraction folded into the last layer.  Table
interpolation is both the error reference and the fallback: ``calibrate`` measures the
median relative force error of the network path against FP64 table
interpolation in equal bands of ln r and keeps the table (FP32
interpolation) in every band that misses the bar.
"""
from __future__ import annotations

import math
import time

import numpy as np
import torch

from .. import _lib
from .. import device as dev

HID = 128


def _layout():
    W1, B1 = 0, HID
    W2 = B1 + HID
    B2 = W2 + HID * HID
    W3 = B2 + HID
    B3 = W3 + HID * HID
    W4 = B3 + HID
    B4 = W4 + 64 * HID
    return dict(W1=W1, B1=B1, W2=W2, B2=B2, W3=W3, B3=B3, W4=W4, B4=B4, SIZE=B4 + 64)


LAYOUT = _layout()


def init_params(L, nout, seed=0):
    """Initial parameters (L, SIZE) float32.  Layer 1 places the SiLU kinks
    uniformly in t in [-1, 1] with slopes |w| in [2, 24]; hidden and output
    layers use U(-1/sqrt(128), 1/sqrt(128))."""
    rng = np.random.default_rng(seed)
    lay = LAYOUT
    p = np.zeros((L, lay["SIZE"]), dtype=np.float32)
    bound = 1.0 / math.sqrt(HID)
    for l in range(L):
        w = rng.uniform(2.0, 24.0, HID) * rng.choice([-1.0, 1.0], HID)
        tk = rng.uniform(-1.0, 1.0, HID)
        p[l, lay["W1"]:lay["B1"]] = w
        p[l, lay["B1"]:lay["W2"]] = -w * tk
        for a, b in (("W2", "B2"), ("W3", "B3")):
            p[l, lay[a]:lay[b]] = rng.uniform(-bound, bound, HID * HID)
        for a, b, n in (("B2", "W3", HID), ("B3", "W4", HID)):
            p[l, lay[a]:lay[b]] = rng.uniform(-bound, bound, n)
        w4 = rng.uniform(-bound, bound, (64, HID))
        w4[nout:] = 0.0
        p[l, lay["W4"]:lay["B4"]] = w4.ravel()
    return p


def ho_radial_np(u, l, K):
    """Hernquist-Ostriker functions HO_nl(u) and u dHO_nl/du (N, K), FP64, by
    the Gegenbauer recurrences (host side: prior fit)."""
    u = np.atleast_1d(np.asarray(u, dtype=np.float64))
    xi = (u - 1.0) / (u + 1.0)
    a = 2 * l + 1.5
    pre = u ** l / (1.0 + u) ** (2 * l + 1)
    g1 = l - (2 * l + 1) * u / (1.0 + u)
    g2 = 2.0 * u / (1.0 + u) ** 2
    C = np.zeros((K, u.size))
    D = np.zeros((max(K - 1, 1), u.size))     # C^(a+1)_k
    for n in range(K):
        if n == 0:
            C[n] = 1.0
        elif n == 1:
            C[n] = 2.0 * a * xi
        else:
            C[n] = (2.0 * (n + a - 1.0) * xi * C[n - 1] - (n + 2.0 * a - 2.0) * C[n - 2]) / n
    for k in range(K - 1):
        if k == 0:
            D[k] = 1.0
        elif k == 1:
            D[k] = 2.0 * (a + 1.0) * xi
        else:
            D[k] = (2.0 * (k + a) * xi * D[k - 1] - (k + 2.0 * a) * D[k - 2]) / k
    dC = np.zeros_like(C)
    for n in range(1, K):
        dC[n] = 2.0 * a * D[n - 1]
    return (-pre * C).T, (-pre * (g1 * C + g2 * dC)).T


class LearnedRadialBasis:
    """Per-l networks over the radial functions of an uploaded SL table.

    table: ``device.SphTable`` (cmap 2, lmax <= 7).  K: radial orders
    learned (default the table's nmax, <= 32).  a_prior: Hernquist scale of
    the prior.  nbands: equal ln r bands of the fallback decision."""

    def __init__(self, table, K=None, a_prior=1.0, nbands=12, seed=0):
        if table.cmap != 2:
            raise ValueError("the learned radial basis needs a logarithmic (cmap 2) SL table")
        if table.lmax > 7:
            raise ValueError("the learned radial basis supports lmax <= 7")
        self.table = table
        self.L = table.lmax + 1
        self.K = int(K if K is not None else table.nmax)
        if not 1 <= self.K <= min(table.nmax, 32):
            raise ValueError("K must be in [1, min(nmax, 32)]")
        self.a_prior = float(a_prior)
        self.nbands = int(nbands)
        self.lnr0, self.lnr1 = math.log(table.rmin), math.log(table.rmax)
        self.c0 = 0.5 * (self.lnr0 + self.lnr1)
        self.c1 = 2.0 / (self.lnr1 - self.lnr0)
        self._lib = _lib.load()
        self.psize = self._lib.xt_mlp_param_size()
        self.s = self._fit_prior()
        self.sig = np.ones((self.L, 2 * self.K))
        p = init_params(self.L, 2 * self.K, seed)
        h = _lib.c_vp()
        dev.device()
        _lib.check(self._lib.xt_mlp_create(self.L, 2 * self.K, p.ctypes.data, _lib.ctypes.byref(h)), "xt_mlp_create")
        self.handle = h.value
        self.band_use = np.zeros(self.nbands, dtype=np.int32)
        self.engine = "tc"
        self.history = []
        self.report = None
        self._prep_key = None

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self._lib.xt_mlp_destroy(self.handle)
        except Exception:
            pass

    # ------------------------------------------------------------ prior
    def node_radial(self):
        """Table radial functions at the nodes: phi (L, K, numr) = p0 ef/sqrt(ev), radii (numr,)."""
        t = self.table
        r = np.exp(t.xi)
        phi = t.p0[None, None, :] * t.ef[:, :self.K, :] / np.sqrt(t.ev[:, :self.K, None])
        return phi, r

    def _fit_prior(self):
        """Least-squares scale s_nl of HO_nl onto the table's phi_nl at the nodes."""
        phi, r = self.node_radial()
        s = np.zeros((self.L, self.K))
        for l in range(self.L):
            ho, _ = ho_radial_np(r / self.a_prior, l, self.K)
            for n in range(self.K):
                h = ho[:, n]
                s[l, n] = float(np.dot(phi[l, n], h) / np.dot(h, h))
        return s

    # ------------------------------------------------------------ data
    def labels(self, r):
        """(t, T) on the device for radii r (device FP64 tensor); T (L, N, 64)."""
        n = int(r.numel())
        t = torch.empty(n, dtype=torch.float32, device=r.device)
        T = torch.empty((self.L, n, 64), dtype=torch.float32, device=r.device)
        s = dev.to_dev(self.s)
        sig = dev.to_dev(self.sig)
        _lib.check(self._lib.xt_mlp_labels(self.table.handle, self.K, dev.dptr(r), n, self.a_prior, dev.dptr(s),
                                           dev.dptr(sig), self.c0, self.c1, dev.dptr(t), dev.dptr(T), n * 64,
                                           dev.stream_ptr()), "xt_mlp_labels")
        return t, T

    def sample_radii(self, n, seed):
        """n log-uniform radii over the table range (NumPy PCG64 seed)."""
        rng = np.random.default_rng(seed)
        return np.exp(rng.uniform(self.lnr0, self.lnr1, n))

    def fit_scales(self, n=65536, seed=1):
        """Target scales sig = max |residual| per (l, output) on a probe set."""
        self.sig = np.ones((self.L, 2 * self.K))
        _, T = self.labels(dev.to_dev(self.sample_radii(n, seed)))
        m = dev.to_host(T[:, :, :2 * self.K].abs().amax(dim=1)).astype(np.float64)
        self.sig = np.maximum(m, 1e-300)
        return self.sig

    # ------------------------------------------------------------ training
    def params(self, which=0):
        out = np.empty((self.L, self.psize), dtype=np.float32)
        _lib.check(self._lib.xt_mlp_get(self.handle, int(which), out.ctypes.data), "xt_mlp_get")
        return out

    def set_params(self, p, step=0):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _lib.check(self._lib.xt_mlp_set_params(self.handle, p.ctypes.data, int(step)), "xt_mlp_set_params")
        self._prep_key = None

    def forward(self, t):
        """Network outputs (L, B, 64) at inputs t (device float32, B % 64 == 0)."""
        B = int(t.numel())
        Y = torch.empty((self.L, B, 64), dtype=torch.float32, device=t.device)
        ws = torch.empty(self._lib.xt_mlp_workspace(self.handle, B), dtype=torch.uint8, device=t.device)
        _lib.check(self._lib.xt_mlp_forward(self.handle, dev.dptr(t), B, dev.dptr(Y), dev.dptr(ws), ws.numel(),
                                            dev.stream_ptr()), "xt_mlp_forward")
        return Y

    def train_step(self, t, T, ldT, B, lr, update=True, workspace=None, loss=None):
        """One step on t[:B] (device pointer offset allowed through views) and
        targets T (per-network stride ldT floats)."""
        ws = workspace if workspace is not None else \
            torch.empty(self._lib.xt_mlp_workspace(self.handle, B), dtype=torch.uint8, device=t.device)
        loss = loss if loss is not None else torch.zeros(self.L, dtype=torch.float64, device=t.device)
        _lib.check(self._lib.xt_mlp_train_step(self.handle, dev.dptr(t), dev.dptr(T), int(ldT), int(B), float(lr),
                                               int(bool(update)), dev.dptr(loss), dev.dptr(ws), ws.numel(),
                                               dev.stream_ptr()), "xt_mlp_train_step")
        self._prep_key = None
        return loss

    def train(self, n_train=1_000_000, seed=4, batch=8192, steps=20000, lr=1e-3, lr_final=1e-5, log_every=1000,
              time_limit=None):
        """Adam at rate lr (cosine decay to lr_final) on n_train log-uniform
        radii labelled by the tables.  Returns the wall time (s)."""
        if self.sig is None or np.all(self.sig == 1.0):
            self.fit_scales()
        r = dev.to_dev(self.sample_radii(n_train, seed))
        t, T = self.labels(r)
        del r
        nb = n_train // batch
        if nb < 1:
            raise ValueError("n_train smaller than one batch")
        ws = torch.empty(self._lib.xt_mlp_workspace(self.handle, batch), dtype=torch.uint8, device=t.device)
        loss = torch.zeros(self.L, dtype=torch.float64, device=t.device)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        done = 0
        for step in range(steps):
            b0 = (step % nb) * batch
            frac = step / max(steps - 1, 1)
            rate = lr_final + 0.5 * (lr - lr_final) * (1.0 + math.cos(math.pi * frac))
            self.train_step(t[b0:b0 + batch], T[:, b0:b0 + batch, :], n_train * 64, batch, rate, True, ws, loss)
            done = step + 1
            if log_every and (step % log_every == 0 or step == steps - 1):
                self.history.append((step, rate, dev.to_host(loss).tolist()))
            if time_limit is not None and step % 100 == 99:
                torch.cuda.synchronize()
                if time.perf_counter() - t0 > time_limit:
                    break
        torch.cuda.synchronize()
        self.steps_done = done
        self.train_seconds = time.perf_counter() - t0
        _lib.check(self._lib.xt_learned_status(), "learned network training")   # tensor-core GEMM waits
        return self.train_seconds

    # ------------------------------------------------------------ inference
    def prepare(self, expcoef, coef_scale=1.0):
        """Fold one coefficient set into the networks and upload the FP32
        table field of the fallback."""
        ec = dev.to_dev(expcoef)
        key = (dev.fingerprint(dev.to_host(ec)), float(coef_scale))
        if self._prep_key == key:
            return
        nbytes = self._lib.xt_learned_prep_bytes(self.handle, self.K)
        self._prep = torch.empty(nbytes, dtype=torch.uint8, device=ec.device)
        self._s_dev = dev.to_dev(self.s)
        self._sig_dev = dev.to_dev(self.sig)
        _lib.check(self._lib.xt_learned_prepare(self.table.handle, self.handle, self.K, dev.dptr(ec), float(coef_scale),
                                                dev.dptr(self._s_dev), dev.dptr(self._sig_dev), dev.dptr(self._prep),
                                                nbytes, dev.stream_ptr()), "xt_learned_prepare")
        self._field32 = self.table.prepare(ec, coef_scale, -1, -1, "f32")
        self._prep_key = key

    ENGINES = {"mma": 0, "tc": 1}

    def radial_pass(self, xyzw, engine="tc", band_use=None):
        """The network pass alone: (N, rstride) float32 folded network sums
        (rows of points outside network bands are left unset)."""
        bu = np.ascontiguousarray(np.ones(self.nbands) if band_use is None else band_use, dtype=np.int32)
        n = int(xyzw.shape[0])
        rs = (2 * self.L * self.L + 3) // 4 * 4
        R = torch.zeros((n, rs), dtype=torch.float32, device=xyzw.device)
        _lib.check(self._lib.xt_learned_radial_pass(self.table.handle, self.handle, dev.dptr(self._prep), self.K,
                                                    self.a_prior, self.c0, self.c1, bu.ctypes.data, self.nbands,
                                                    dev.dptr(xyzw), n,
                                                    self.ENGINES[engine], dev.dptr(R), dev.stream_ptr()),
                   "xt_learned_radial_pass")
        return R

    def status(self):
        """Raise if a tensor-memory network pass gave up waiting for its MMAs."""
        _lib.check(self._lib.xt_learned_status(), "learned network pass")

    def eval(self, xyzw, band_use=None, no_odd=False, out=None, workspace=None, engine=None):
        """float4 (pot, dpot/dr, dpot/dcos(theta), dpot/dphi) per point of xyzw
        ((N, 4) float32 CUDA tensor), all_eval formulation.  band_use: per band
        1 = network, 0 = table (default: the calibrated choice)."""
        if self._prep_key is None:
            raise RuntimeError("call prepare(expcoef) first")
        if xyzw.dtype != torch.float32 or xyzw.dim() != 2 or xyzw.shape[1] != 4 or not xyzw.is_contiguous():
            raise ValueError("xyzw must be a contiguous (N, 4) float32 CUDA tensor")
        n = int(xyzw.shape[0])
        bu = np.ascontiguousarray(self.band_use if band_use is None else band_use, dtype=np.int32)
        if bu.size != self.nbands:
            raise ValueError(f"band_use needs {self.nbands} entries")
        out = out if out is not None else torch.empty((n, 4), dtype=torch.float32, device=xyzw.device)
        need = self._lib.xt_learned_eval_workspace(self.table.handle, n)
        ws = workspace if (workspace is not None and workspace.numel() >= need) else \
            torch.empty(max(need, 1), dtype=torch.uint8, device=xyzw.device)
        _lib.check(self._lib.xt_learned_eval(self.table.handle, dev.dptr(self._field32.buf), self.handle,
                                             dev.dptr(self._prep), self.K, self.a_prior, self.c0, self.c1,
                                             bu.ctypes.data, self.nbands, dev.dptr(xyzw), n, int(bool(no_odd)),
                                             self.ENGINES[engine or self.engine], dev.dptr(out), dev.dptr(ws),
                                             ws.numel(), dev.stream_ptr()),
                   "xt_learned_eval")
        return out

    # ------------------------------------------------------------ judging
    def band_of(self, r):
        rc = np.clip(r, self.table.rmin, self.table.rmax)
        b = ((np.log(rc) - self.lnr0) * (self.nbands / (self.lnr1 - self.lnr0))).astype(np.int64)
        return np.clip(b, 0, self.nbands - 1)

    @staticmethod
    def grad_components(res, r, costh):
        """Physical gradient components (d/dr, (1/r) d/dtheta, 1/(r sin) d/dphi)."""
        pot, potr, pott, potp = res
        sin = np.sqrt(np.maximum(1.0 - costh * costh, 1e-300))
        return np.stack([potr, -sin * pott / r, potp / (r * sin)], axis=1)

    def calibrate(self, expcoef, xyz, bar=1e-5, coef_scale=1.0):
        """Per band: median relative force error of the network path and of
        FP32 table interpolation against FP64 table interpolation at points
        xyz ((N, 3) float64); bands whose network median exceeds `bar` use the
        table.  Returns the report dict."""
        xyz = np.asarray(xyz, dtype=np.float64)
        x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
        r = np.sqrt(x * x + y * y + z * z)
        costh = np.where(r > 0, z / np.where(r > 0, r, 1.0), 0.0)
        phi = np.arctan2(y, x)
        self.prepare(expcoef, coef_scale)
        f64 = self.table.prepare(dev.to_dev(expcoef), coef_scale, -1, -1, "f64")
        outs = self.table.eval_points(f64, dev.to_dev(r), dev.to_dev(costh), dev.to_dev(phi), _lib.XT_SPH_ALL_EVAL,
                                      _lib.XT_COORD_SPH)
        den0, den1, pot0, pot1, potr, pott, potp = (dev.to_host(o) for o in outs[:7])
        ref = (pot0 + pot1, potr, pott, potp)
        xyzw = torch.zeros((r.size, 4), dtype=torch.float32)
        xyzw[:, :3] = torch.from_numpy(xyz.astype(np.float32))
        xyzw = xyzw.to(dev.device())
        net = dev.to_host(self.eval(xyzw, band_use=np.ones(self.nbands, np.int32))).astype(np.float64).T
        tab = dev.to_host(self.eval(xyzw, band_use=np.zeros(self.nbands, np.int32))).astype(np.float64).T
        g_ref = self.grad_components(ref, r, costh)
        nref = np.linalg.norm(g_ref, axis=1)
        e_net = np.linalg.norm(self.grad_components(net, r, costh) - g_ref, axis=1) / nref
        e_tab = np.linalg.norm(self.grad_components(tab, r, costh) - g_ref, axis=1) / nref
        pe_net = np.abs(net[0] - ref[0]) / np.abs(ref[0])
        pe_tab = np.abs(tab[0] - ref[0]) / np.abs(ref[0])
        band = self.band_of(r)
        rows = []
        use = np.zeros(self.nbands, dtype=np.int32)
        for b in range(self.nbands):
            sel = band == b
            cnt = int(sel.sum())
            if cnt == 0:
                rows.append(dict(band=b, count=0))
                continue
            mn, mt = float(np.median(e_net[sel])), float(np.median(e_tab[sel]))
            use[b] = int(mn <= bar)
            lo = math.exp(self.lnr0 + b * (self.lnr1 - self.lnr0) / self.nbands)
            hi = math.exp(self.lnr0 + (b + 1) * (self.lnr1 - self.lnr0) / self.nbands)
            rows.append(dict(band=b, r_lo=lo, r_hi=hi, count=cnt, net_median=mn, table32_median=mt,
                             net_p99=float(np.quantile(e_net[sel], 0.99)), net_pot_median=float(np.median(pe_net[sel])),
                             table32_pot_median=float(np.median(pe_tab[sel])), use_net=bool(use[b])))
        self.band_use = use
        hyb = np.where(use[band] != 0, e_net, e_tab)
        self.report = dict(bar=bar, bands=rows, net_median=float(np.median(e_net)),
                           table32_median=float(np.median(e_tab)), hybrid_median=float(np.median(hyb)),
                           hybrid_max=float(np.max(hyb)), net_bands=int(use.sum()),
                           net_fraction=float(np.mean(use[band] != 0)))
        return self.report

    # ------------------------------------------------------------ persistence
    def save(self, path):
        np.savez(path, params=self.params(), s=self.s, sig=self.sig, band_use=self.band_use, K=self.K,
                 a_prior=self.a_prior, nbands=self.nbands, c0=self.c0, c1=self.c1)

    def load(self, path):
        d = np.load(path)
        if int(d["K"]) != self.K or d["params"].shape != (self.L, self.psize):
            raise ValueError("saved networks do not match this table / K")
        self.s, self.sig = d["s"], d["sig"]
        self.band_use = d["band_use"].astype(np.int32)
        self.a_prior = float(d["a_prior"])
        self.set_params(d["params"])

    def memory_bytes(self):
        """Device bytes the evaluation reads: BF16 networks vs the FP32 table field."""
        return dict(network_bf16=int(self.L * (2 * HID * HID + 64 * HID) * 2 + self.L * 5 * HID * 4),
                    table_f32_field=int(self.table.numr * self.table.nrow * 2 * 4),
                    table_f64_radial=int(self.L * self.K * self.table.numr * 8 * 2))
