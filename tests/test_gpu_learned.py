"""GPU checks of the learned radial basis against the NumPy oracle: labels,
gradients of the hand-written backward kernels, Adam, training progress, and
the two-pass force evaluation (network + prior, and the table fallback)."""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _basis(K=None, seed=0):
    from exptool_gb300.basis import learned, spheresl
    table = spheresl.table_from_files(os.path.join(GOLDEN, "sl_c2.cache"), os.path.join(GOLDEN, "sl_c2.model"))
    return learned.LearnedRadialBasis(table, K=K, nbands=8, seed=seed)


def _otable():
    from oracle.sl import load_table
    return load_table(os.path.join(GOLDEN, "sl_c2.cache"), os.path.join(GOLDEN, "sl_c2.model"))


def test_labels_match_oracle():
    from exptool_gb300 import device as dev
    from oracle import mlp
    lb = _basis()
    lb.fit_scales(n=4096)
    r = np.exp(np.random.default_rng(3).uniform(np.log(5e-4), np.log(150.0), 512))   # includes clamped radii
    t, T = lb.labels(dev.to_dev(r))
    to, To = mlp.labels(r, _otable(), lb.K, lb.a_prior, lb.s, lb.sig, lb.c0, lb.c1)
    assert np.allclose(dev.to_host(t), to, rtol=0, atol=2e-7)
    Tg = dev.to_host(T).astype(np.float64)
    # FP32 storage of FP64 labels
    assert np.max(np.abs(Tg - To)) <= 2e-6 * max(1.0, np.max(np.abs(To)))


def _batch(lb, B, seed):
    from exptool_gb300 import device as dev
    r = lb.sample_radii(B, seed)
    t, T = lb.labels(dev.to_dev(r))
    return t, T


def test_gradients_match_oracle():
    from exptool_gb300 import device as dev
    from oracle import mlp
    lb = _basis(seed=5)
    lb.fit_scales(n=4096)
    B = 256
    t, T = _batch(lb, B, 7)
    p0 = lb.params().astype(np.float64)
    loss = lb.train_step(t, T, B * 64, B, 1e-3, update=False)
    g = lb.params(which=1).astype(np.float64)
    th, Th = dev.to_host(t), dev.to_host(T).astype(np.float64)
    lg = dev.to_host(loss)
    blocks = [(mlp.W1, mlp.B1), (mlp.B1, mlp.W2), (mlp.W2, mlp.B2), (mlp.B2, mlp.W3), (mlp.W3, mlp.B3),
              (mlp.B3, mlp.W4), (mlp.W4, mlp.B4), (mlp.B4, mlp.SIZE)]
    for l in range(lb.L):
        lo, go = mlp.loss_and_grad(p0[l], th, Th[l], 2 * lb.K, emulate=True)
        _, gx = mlp.loss_and_grad(p0[l], th, Th[l], 2 * lb.K, emulate=False)
        assert abs(lg[l] - lo) <= 1e-3 * lo
        for a, b in blocks:
            # same BF16 rounding points: FP32 accumulation order and the
            # hardware tanh are the only differences
            assert np.linalg.norm(g[l, a:b] - go[a:b]) <= 1e-2 * np.linalg.norm(go[a:b]) + 1e-12, (l, a)
            # and the BF16 network's gradient tracks the exact FP64 gradient
            assert np.linalg.norm(g[l, a:b] - gx[a:b]) <= 6e-2 * np.linalg.norm(gx[a:b]) + 1e-12, (l, a)


def test_adam_update_matches_oracle():
    from oracle import mlp
    lb = _basis(seed=6)
    lb.fit_scales(n=4096)
    B = 128
    t, T = _batch(lb, B, 8)
    p0 = lb.params().astype(np.float64)
    lb.train_step(t, T, B * 64, B, 1e-3, update=True)
    g = lb.params(which=1).astype(np.float64)
    p1 = lb.params().astype(np.float64)
    pe, _, _ = mlp.adam(p0, g, np.zeros_like(g), np.zeros_like(g), 1, 1e-3)
    nout = 2 * lb.K
    for l in range(lb.L):
        pe[l, mlp.W4 + nout * mlp.HID:mlp.B4] = 0
        pe[l, mlp.B4 + nout:] = 0
    assert np.max(np.abs(p1 - pe)) <= 2e-6 * max(1.0, np.max(np.abs(pe)))


def test_training_reduces_loss_and_forward_matches_oracle():
    from exptool_gb300 import device as dev
    from oracle import mlp
    lb = _basis(seed=2)
    lb.fit_scales(n=8192)
    lb.train(n_train=65536, seed=4, batch=2048, steps=600, lr=1e-3, lr_final=1e-4, log_every=100)
    first = np.array(lb.history[0][2])
    last = np.array(lb.history[-1][2])
    assert np.all(last < 0.1 * first), (first, last)
    # forward kernel == oracle forward with BF16 emulation
    t = dev.to_dev(np.linspace(-1, 1, 256), dtype=__import__("torch").float32)
    Y = dev.to_host(lb.forward(t)).astype(np.float64)
    p = lb.params().astype(np.float64)
    # Training uses split-K atomics, so the trained weights differ from run to
    # run; an activation that lands next to a BF16 rounding boundary can round
    # the other way (FP32 accumulation order, hardware tanh) and the flip is
    # amplified through the three SiLU layers at a few outputs.  Bounds: the
    # bulk of the outputs to 1e-3, the 99th percentile to 1e-2 and the worst
    # output to 5e-2 of the largest output.
    for l in range(lb.L):
        yo, _ = mlp.forward(p[l], dev.to_host(t), emulate=True)
        d = np.abs(Y[l] - yo)
        scale = np.max(np.abs(yo)) + 1e-6
        assert np.median(d) <= 1e-3 * scale, (l, np.median(d) / scale)
        assert np.quantile(d, 0.99) <= 1e-2 * scale, (l, np.quantile(d, 0.99) / scale)
        assert np.max(d) <= 5e-2 * scale, (l, np.max(d) / scale)


def test_learned_eval_matches_oracle_and_fallback_matches_table():
    import torch
    from exptool_gb300 import device as dev
    from exptool_gb300.tables.samplers import hernquist_sample
    from oracle import mlp
    from oracle.sl import all_eval, compute_coefficients_solitary
    lb = _basis(seed=3)
    lb.fit_scales(n=8192)
    lb.train(n_train=65536, seed=4, batch=2048, steps=300, lr=1e-3, lr_final=1e-4, log_every=0)
    tab = _otable()
    x, y, z, m = hernquist_sample(20000, seed=11)
    ec = compute_coefficients_solitary(x, y, z, m, tab)
    px, py, pz, _ = hernquist_sample(2000, seed=12)
    xyzw = torch.zeros((px.size, 4), dtype=torch.float32)
    xyzw[:, 0], xyzw[:, 1], xyzw[:, 2] = (torch.from_numpy(a.astype(np.float32)) for a in (px, py, pz))
    xyzw = xyzw.to(dev.device())
    lb.prepare(ec)
    net = dev.to_host(lb.eval(xyzw, band_use=np.ones(lb.nbands, np.int32))).astype(np.float64)
    tabf = dev.to_host(lb.eval(xyzw, band_use=np.zeros(lb.nbands, np.int32))).astype(np.float64)
    # evaluate the oracle at the FP32-rounded positions the kernels saw
    xf, yf, zf = (a.astype(np.float32).astype(np.float64) for a in (px, py, pz))
    r = np.sqrt(xf * xf + yf * yf + zf * zf)
    costh, phi = zf / r, np.arctan2(yf, xf)
    ref_net = np.stack(mlp.learned_all_eval(lb.params(), r, costh, phi, ec, tab, lb.K, lb.a_prior, lb.s, lb.sig,
                                            lb.c0, lb.c1), axis=1)
    _, _, pot0, pot1, potr, pott, potp = all_eval(r, costh, phi, ec, tab)
    ref_tab = np.stack([pot0 + pot1, potr, pott, potp], axis=1)

    def grad(v):
        return lb.grad_components(v.T, r, costh)

    def ferr(a, b):
        return np.linalg.norm(grad(a) - grad(b), axis=1) / np.linalg.norm(grad(b), axis=1)

    # network path: FP32 arithmetic, folded last layer, hardware tanh
    e = ferr(net, ref_net)
    assert np.median(e) <= 2e-5 and np.quantile(e, 0.99) <= 5e-4, (np.median(e), np.quantile(e, 0.99))
    assert np.median(np.abs(net[:, 0] - ref_net[:, 0]) / np.abs(ref_net[:, 0])) <= 2e-5
    # table fallback: FP32 interpolation of the contracted field
    e = ferr(tabf, ref_tab)
    assert np.median(e) <= 5e-6 and np.quantile(e, 0.99) <= 1e-4, (np.median(e), np.quantile(e, 0.99))
    # calibration keeps the table wherever the network misses the bar
    rep = lb.calibrate(ec, np.stack([px, py, pz], axis=1), bar=1e-5)
    assert rep["hybrid_median"] <= 1e-5
    for row in rep["bands"]:
        if row.get("count", 0) and row["use_net"]:
            assert row["net_median"] <= 1e-5


def test_tensor_memory_pass_matches_mma_pass():
    """The two network-pass engines (tcgen05 with the prior folded into its
    epilogue; mma.sync with the prior in the second pass) give the same
    potential and forces: same BF16 operands and rounding points, different
    accumulation order inside the tensor cores."""
    import torch
    from exptool_gb300 import device as dev
    from exptool_gb300.tables.samplers import hernquist_sample
    from oracle.sl import compute_coefficients_solitary
    lb = _basis(seed=4)
    lb.fit_scales(n=4096)
    lb.train(n_train=16384, seed=4, batch=2048, steps=50, lr=1e-3, lr_final=1e-4, log_every=0)
    tab = _otable()
    x, y, z, m = hernquist_sample(5000, seed=13)
    lb.prepare(compute_coefficients_solitary(x, y, z, m, tab))
    ones = np.ones(lb.nbands, np.int32)
    for n in (300, 4096 + 77):
        px, py, pz, _ = hernquist_sample(n, seed=14)
        xyzw = torch.zeros((n, 4), dtype=torch.float32)
        xyzw[:, 0], xyzw[:, 1], xyzw[:, 2] = (torch.from_numpy(a.astype(np.float32)) for a in (px, py, pz))
        xyzw = xyzw.to(dev.device())
        out_a = dev.to_host(lb.eval(xyzw, band_use=ones, engine="mma")).astype(np.float64)
        out_b = dev.to_host(lb.eval(xyzw, band_use=ones, engine="tc")).astype(np.float64)
        lb.status()
        r = np.sqrt(px * px + py * py + pz * pz)
        costh = pz / r
        ga = lb.grad_components(out_a.T, r, costh)
        gb = lb.grad_components(out_b.T, r, costh)
        e = np.linalg.norm(ga - gb, axis=1) / np.linalg.norm(ga, axis=1)
        assert np.median(e) <= 1e-5 and np.max(e) <= 1e-3, (np.median(e), np.max(e))
        pe = np.abs(out_a[:, 0] - out_b[:, 0]) / np.abs(out_a[:, 0])
        assert np.median(pe) <= 1e-6 and np.max(pe) <= 1e-4, (np.median(pe), np.max(pe))


def test_trained_network_gains_over_prior_alone(tmp_path):
    """What the trained network adds, on the Hernquist SL basis the learned
    path targets (lmax 6, nmax 20, 2000-point table, cmap 2): median relative
    force error against FP64 table interpolation of the learned basis (prior +
    trained residual network) against the same basis with the network's output
    layer zeroed, i.e. the Hernquist-Ostriker prior fitted by least squares
    alone, both through the same GPU evaluation.  Also the memory read at
    evaluation."""
    import torch
    from exptool_gb300 import device as dev
    from exptool_gb300.basis import learned, spheresl
    from exptool_gb300.tables.samplers import hernquist_sample
    from exptool_gb300.tables.sl_solver import make_hernquist_sl
    from oracle import mlp
    from oracle.sl import all_eval, compute_coefficients_solitary, load_table
    make_hernquist_sl(str(tmp_path), lmax=6, nmax=20, numr=2000, rmin=1e-3, rmax=100.0, cmap=2, scale=1.0, tag="t")
    cache, model = str(tmp_path / "SLGridSph.cache.t"), str(tmp_path / "SLGridSph.model.t")
    lb = learned.LearnedRadialBasis(spheresl.table_from_files(cache, model), nbands=12, seed=0)
    lb.fit_scales()
    lb.train(n_train=1_000_000, seed=4, batch=8192, steps=12000, lr=1e-3, lr_final=1e-5, log_every=0)
    tab = load_table(cache, model)
    x, y, z, m = hernquist_sample(50000, seed=11)
    ec = compute_coefficients_solitary(x, y, z, m, tab)
    px, py, pz, _ = hernquist_sample(20000, seed=12)
    xyzw = torch.zeros((px.size, 4), dtype=torch.float32)
    xyzw[:, 0], xyzw[:, 1], xyzw[:, 2] = (torch.from_numpy(a.astype(np.float32)) for a in (px, py, pz))
    xyzw = xyzw.to(dev.device())
    xf, yf, zf = (a.astype(np.float32).astype(np.float64) for a in (px, py, pz))
    r = np.sqrt(xf * xf + yf * yf + zf * zf)
    costh, phi = zf / r, np.arctan2(yf, xf)
    _, _, pot0, pot1, potr, pott, potp = all_eval(r, costh, phi, ec, tab)
    ref = np.stack([pot0 + pot1, potr, pott, potp], axis=1)
    ones = np.ones(lb.nbands, np.int32)

    def med_err(out):
        g, gr = lb.grad_components(out.T, r, costh), lb.grad_components(ref.T, r, costh)
        return float(np.median(np.linalg.norm(g - gr, axis=1) / np.linalg.norm(gr, axis=1)))

    lb.prepare(ec)
    e_net = med_err(dev.to_host(lb.eval(xyzw, band_use=ones)).astype(np.float64))
    p = lb.params()
    p[:, mlp.W4:mlp.SIZE] = 0.0          # output layer and bias: the residual network contributes nothing
    lb.set_params(p)
    lb.prepare(ec)
    e_prior = med_err(dev.to_host(lb.eval(xyzw, band_use=ones)).astype(np.float64))
    print(f"median force error: prior alone {e_prior:.2e}, prior + trained network {e_net:.2e}")
    # measured: prior alone 5.0e-4, with the network 2.8e-5 (coefficients from 5e4 particles; the
    # absolute 1e-5 bar is judged per radius band by calibrate on the full workload)
    assert e_net <= 0.1 * e_prior, (e_net, e_prior)
    mem = lb.memory_bytes()
    assert mem["network_bf16"] < mem["table_f64_radial"]
