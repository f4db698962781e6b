"""The learned warm start of the fitter: features, network kernels, training,
and what the trained network gains over the plain fitter.

Gradients of the hand-written forward/backward kernels are checked against
the numpy oracle (oracle/mlp.py, FP64) at FP32 tolerance. The gain test runs
the plain fitter (every permutation from the whole parameter box, as the
reference) and the warm-started one on the same fields and compares the
differential-evolution work and the leave-one-out kriging error of the
chosen variograms.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import mlp as omlp  # noqa: E402


def test_features_match_oracle():
    from spinterps_gb300.warmstart import step_features
    rng = np.random.default_rng(1)
    pts = []
    for n in (50, 333, 800):
        x, y = rng.uniform(0, 1e5, n), rng.uniform(0, 2e5, n)
        pts.append((x, y, rng.gamma(0.8, 2.0, n)))
    f = step_features(pts, [0, 1, 2])
    for k, (x, y, z) in enumerate(pts):
        ref = omlp.features(x, y, z)
        assert np.allclose(f[k], ref, rtol=2e-6, atol=1e-7), (k, np.abs(f[k] - ref).max())


def test_mlp_loss_and_gradient_match_oracle():
    from spinterps_gb300.warmstart import WarmStartMLP
    m = WarmStartMLP(seed=3)
    rng = np.random.default_rng(4)
    B = 64
    X = rng.normal(size=(B, 20)).astype(np.float32)
    cls = rng.integers(0, m.n_class, B).astype(np.int32)
    yp = rng.normal(size=(B, 3)).astype(np.float32)
    mask = (rng.uniform(size=(B, 3)) < 0.7).astype(np.float32)
    dev = torch.device("cuda")
    loss, grad = m.loss_grad(torch.as_tensor(X, device=dev), torch.as_tensor(cls, device=dev),
                             torch.as_tensor(yp, device=dev), torch.as_tensor(mask, device=dev),
                             wp=0.7)
    ref_loss, ref_grad = omlp.loss_grad(m.params.cpu().numpy().astype(np.float64), X, cls, yp,
                                        mask, 0.7, m.dims, m.n_class)
    assert abs(float(loss.sum()) - ref_loss) <= 1e-5 * max(1.0, abs(ref_loss))
    g = grad.cpu().numpy()
    assert np.abs(g - ref_grad).max() <= 1e-4 * np.abs(ref_grad).max()
    # forward outputs too
    O = m.forward(X * m.sd + m.mu)
    _, _, ref_O = omlp.forward(m.params.cpu().numpy().astype(np.float64), X, m.dims)
    assert np.abs(O - ref_O).max() <= 1e-4 * np.abs(ref_O).max()


def test_training_reduces_loss():
    from spinterps_gb300.warmstart import WarmStartMLP
    rng = np.random.default_rng(5)
    n = 1024
    X = rng.normal(size=(n, 20)).astype(np.float32)
    Wc = rng.normal(size=(20, 5))
    cls = np.argmax(X @ Wc, 1).astype(np.int32)
    yp = np.tanh(X[:, :3]).astype(np.float32)
    mask = np.ones((n, 3), dtype=np.float32)
    m = WarmStartMLP(seed=6)
    hist = m.train(X, cls, yp, mask, epochs=40, batch=128, lr=3e-3)
    assert hist[-1] < 0.3 * hist[0], hist[::10]
    acc = np.mean(np.argmax(m.forward(X)[:, :5], 1) == cls)
    assert acc > 0.9


def _fields_as_table(pts):
    xs = np.concatenate([p[0] for p in pts])
    ys = np.concatenate([p[1] for p in pts])
    data = np.full((len(pts), xs.size), np.nan)
    o = 0
    for k, (x, _, z) in enumerate(pts):
        data[k, o:o + x.size] = z
        o += x.size
    return xs, ys, data


def test_trained_warm_start_gain():
    """The trained network makes the fitter do at least 5x less DE work on
    fields it has not seen, and the variograms it leads to krige as well:
    leave-one-out RMSE within 1% of the plain fit's on average."""
    from spinterps_gb300 import fitvgs, steps, warmstart
    from spinterps_gb300.train_warmstart import synth_points
    mlp = warmstart.WarmStartMLP.load()
    pts, _ = synth_points(24, seed=987654, n_lo=300, n_hi=700)
    plain, dp = fitvgs.fit_steps(None, None, None, emp=fitvgs.Empirical(
        None, None, None, points=pts).run(), seed=1, return_details=True)
    warm, dw = warmstart.warm_fit_steps(None, None, None, mlp, points=pts, seed=1)
    assert dw["_de_member_evals"] * 5 <= dp["_de_member_evals"], (
        dw["_de_member_evals"], dp["_de_member_evals"])
    xs, ys, data = _fields_as_table(pts)
    _, r_plain = steps.krige_loo(xs, ys, data, [s[-1] for s in plain])
    _, r_warm = steps.krige_loo(xs, ys, data, [s[-1] for s in warm])
    ok = np.isfinite(r_plain) & np.isfinite(r_warm)
    assert ok.sum() >= 20
    assert r_warm[ok].mean() <= 1.01 * r_plain[ok].mean(), (r_warm[ok].mean(),
                                                             r_plain[ok].mean())


def test_refine_matches_dense_search():
    """spi_vg_refine against a dense CPU search of the same profile (4000
    log-ranges, closed-form clipped sill, the oracle's objective): the GPU
    result is at least as good, its reported objective is the oracle's at
    its parameters, and its noise is bin_noise of the bins."""
    import ctypes
    from spinterps_gb300 import _native as nat
    from spinterps_gb300 import fitvgs, warmstart
    from spinterps_gb300.steps import _ptr, _stream
    from spinterps_gb300.train_warmstart import synth_points
    from oracle import fitter
    pts, _ = synth_points(3, seed=77, n_lo=300, n_hi=500)
    emp = fitvgs.Empirical(None, None, None, points=pts).run()
    perms = [("Sph",), ("Exp",), ("Nug", "Sph"), ("Nug", "Exp"), ("Nug",)]
    probs, r0, keys = [], [], []
    for k in range(emp.S):
        for o in perms:
            p = fitvgs.DeProblem()
            p.step, p.n_comp = k, len(o)
            for c, name in enumerate(o):
                p.code[c] = fitvgs.CODES[name]
            p.fixed_first = 1 if len(o) > 1 else 0
            p.var2 = float(emp.var2[k])
            probs.append(p)
            r0.append(20e3)
            keys.append((k, o))
    raw = bytes((fitvgs.DeProblem * len(probs))(*probs))
    dev = torch.device("cuda")
    d_prob = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(dev)
    d_r0 = torch.as_tensor(np.array(r0), device=dev)
    P = len(probs)
    x = torch.empty((P, 4), dtype=torch.float64, device=dev)
    f = torch.empty(P, dtype=torch.float64, device=dev)
    nz = torch.empty(P, dtype=torch.float64, device=dev)
    nat.call("spi_vg_refine", P, _ptr(d_prob), _ptr(emp.d_bin_off), _ptr(emp.n_bins),
             _ptr(emp.bin_h), _ptr(emp.bin_g), _ptr(d_r0), 4.0, _ptr(x), _ptr(f), _ptr(nz),
             _stream())
    x, f, nz = x.cpu().numpy(), f.cpu().numpy(), nz.cpu().numpy()
    for q, (k, o) in enumerate(keys):
        h, g, _ = emp.bins(k)
        var2 = float(emp.var2[k])
        assert abs(nz[q] - warmstart.bin_noise(g)) <= 1e-12 * warmstart.bin_noise(g)
        names = list(o)
        xo = x[q, :2 * len(o)]
        assert abs(f[q] - fitter.objective(xo, names, h, g)) <= 1e-9 * max(f[q], 1e-300)
        if o == ("Nug",):
            best = fitter.objective(np.array([h[0], np.clip(g.mean(), 1e-5, var2)]), names, h, g)
        else:
            best = np.inf
            base = g[0] if len(o) > 1 else 0.0
            for r in np.exp(np.linspace(np.log(max(5e3, h[0])), np.log(80e3), 4000)):
                rho = np.asarray(fitter.MODELS[o[-1]](h, (r, 1.0)), dtype=np.float64)
                y = g - base
                sl = np.clip(np.dot(rho, y) / np.dot(rho, rho), 1e-5, var2)
                arg = (np.array([h[0], g[0], r, sl]) if len(o) > 1 else np.array([r, sl]))
                best = min(best, fitter.objective(arg, names, h, g))
        assert f[q] <= best * (1 + 1e-6) + 1e-12, (k, o, f[q], best)
