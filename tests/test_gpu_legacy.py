"""The single-neighbourhood classes (spinterps_gb300.legacy, csrc/spi_legacy.cu)
against the reference's own compiled classes (tests/golden/legacy.npz, made
by running cyth/interpmthds.pyx:251-765) and against the oracle's
restatement on larger cases.

Bars:
- distances: within 1 ulp, at least 90% bit for bit (the reference's get_dist
  takes libm pow(s, 0.5), which is 1 ulp off the correctly rounded square
  root the GPU takes in ~0.1% of arguments);
- matrices and right-hand sides: 1e-13 relative (device exp / sin / pow
  against the host's libm);
- the inverse: 1e-9 of its largest entry;
- estimates, weights, multipliers and variances: 1e-9 of the field's
  largest magnitude, the FP64 bar of the step engine.
"""
import numpy as np
import pytest

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import port  # noqa: E402

ULP1 = ("in_dists",)
MATRIX = ("in_vars", "in_covars", "rhss", "out_covars")
INVERSE = ("in_vars_inv", "in_covars_inv")
INPUTS = ("xi", "yi", "zi", "xk", "yk", "si", "sk", "lim", "model", "cls")


def _make(cls_name, xi, yi, zi, xk, yk, model, si, sk, lim):
    import spinterps_gb300 as spi
    cls = getattr(spi, cls_name)
    if cls_name == "ExternalDriftKriging":
        obj = cls(xi, yi, zi, si[0].copy(), xk, yk, sk[0].copy(), model=model)
        obj.krige()
    elif cls_name == "ExternalDriftKriging_MD":
        obj = cls(xi, yi, zi, si, xk, yk, sk, model=model)
        obj.krige()
    elif cls_name.endswith("IndicatorKriging"):
        obj = cls(xi, yi, zi, xk, yk, lim=lim, model=model)
        obj.ikrige()
    else:
        obj = cls(xi, yi, zi, xk, yk, model=model)
        obj.krige()
    return obj


def _check(key, got, ref, tag):
    got = np.asarray(got, dtype=np.float64)
    assert got.shape == ref.shape, (tag, key)
    if key in ULP1:
        ulp = np.abs(got - ref) / np.spacing(np.maximum(ref, 1e-300))
        assert (ulp <= 1).all(), (tag, key)
        assert (got == ref).mean() >= 0.9, (tag, key)
        return
    scale = max(np.abs(ref).max(), 1e-300) if ref.size else 1.0
    if key in MATRIX:
        assert np.all(np.abs(got - ref) <= 1e-13 * np.maximum(np.abs(ref), 1e-300) + 1e-15 * scale), \
            (tag, key)
        return
    err = np.abs(got - ref).max() / scale if ref.size else 0.0
    assert err <= 1e-9, (tag, key, err)


def test_legacy_classes_match_reference(golden):
    g = golden
    routes = {}
    for ci in g["l_cases"]:
        p = f"l{ci}_"
        cls = str(g[p + "cls"])
        obj = _make(cls, g[p + "xi"], g[p + "yi"], g[p + "zi"], g[p + "xk"], g[p + "yk"],
                    str(g[p + "model"]), g[p + "si"], g[p + "sk"], float(g[p + "lim"]))
        routes[int(ci)] = obj.pinv_route
        keys = [k[len(p):] for k in g if k.startswith(p) and k[len(p):] not in INPUTS]
        for k in keys:
            _check(k, getattr(obj, k), g[p + k], f"{ci} {cls}")
        assert obj.vgs and len(obj.sills) == len(obj.ranges) == len(obj.vgs)
    # the duplicated-station OK case is exactly singular: the SVD route
    assert routes[10] == "pinv"
    assert all(r == "gj" for c, r in routes.items() if c != 10), routes


@pytest.mark.parametrize("cls", ["OrdinaryKriging", "SimpleKriging", "ExternalDriftKriging_MD",
                                 "OrdinaryIndicatorKriging"])
def test_legacy_larger_vs_oracle(cls):
    rng = np.random.default_rng(90)
    n, n_out = 220, 2500
    xi, yi = rng.uniform(0, 1e5, n), rng.uniform(0, 1e5, n)
    zi = rng.gamma(1.2, 3.0, n)
    xk, yk = rng.uniform(0, 1e5, n_out), rng.uniform(0, 1e5, n_out)
    xk[7], yk[7] = xi[11], yi[11]
    si, sk = rng.uniform(0, 2000, (2, n)), rng.uniform(0, 2000, (2, n_out))
    model = "0.1 Nug(0.0) + 0.9 Exp(30000)"
    lim = float(np.quantile(zi, 0.3))
    ref = port.legacy_krige(cls, xi, yi, zi, xk, yk, model, si=si, sk=sk, lim=lim)
    obj = _make(cls, xi, yi, zi, xk, yk, model, si, sk, lim)
    assert obj.pinv_route == "gj"
    for k, v in ref.items():
        if k == "covar":
            if cls == "SimpleKriging":
                assert obj.covar == v
            continue
        _check(k, getattr(obj, k), np.asarray(v), cls)


def test_legacy_device_entry_and_errors():
    import torch
    from spinterps_gb300 import legacy
    rng = np.random.default_rng(91)
    xi, yi, zi = rng.uniform(0, 5e4, 30), rng.uniform(0, 5e4, 30), rng.normal(size=30)
    xk, yk = rng.uniform(0, 5e4, 100), rng.uniform(0, 5e4, 100)
    model = "0.2 Nug(0.0) + 0.8 Gau(20000)"
    obj = legacy.OrdinaryKriging(xi, yi, zi, xk, yk, model=model)
    obj.krige()
    d = lambda a: torch.as_tensor(a, dtype=torch.float64, device="cuda")  # noqa: E731
    r = legacy.krige_points("OK", d(xi), d(yi), d(zi), d(xk), d(yk), model)
    torch.cuda.synchronize()
    assert np.array_equal(r["zk"].cpu().numpy(), obj.zk)
    assert np.array_equal(r["est"].cpu().numpy(), obj.est_vars)
    assert obj.vgs == [b"Nug", b"Gau"] and obj.sills == [0.2, 0.8]
    with pytest.raises(RuntimeError):
        obj.krige()
    with pytest.raises(KeyError):
        legacy.OrdinaryKriging(xi, yi, zi, xk, yk, model="1.0 Foo(3)").krige()
    with pytest.raises(ValueError):
        legacy.OrdinaryKriging(xi, yi, zi, xk, yk, model="1.0 Exp (3)").krige()
    with pytest.raises(AssertionError):
        legacy.ExternalDriftKriging_MD(xi, yi, zi, np.zeros((2, 29)), xk, yk, np.zeros((2, 100)))
    # no output points
    e = legacy.OrdinaryKriging(xi, yi, zi, xk[:0], yk[:0], model=model)
    e.krige()
    assert e.zk.shape == (0,) and e.lambdas.shape == (0, 30)


@pytest.mark.parametrize("m, rank", [(40, 40), (64, 61), (201, 197), (256, 250)])
def test_sym_pinv_matches_numpy(m, rank):
    """spi_sym_pinv (the legacy classes' pseudo-inverse) against numpy's
    pinv with the same cut-off (m eps of the largest singular value) on
    symmetric indefinite matrices of the given rank, saddle-like scales."""
    import ctypes
    import torch
    from spinterps_gb300 import _native as nat
    rng = np.random.default_rng(m + rank)
    q, _ = np.linalg.qr(rng.standard_normal((m, m)))
    lam = rng.uniform(0.1, 10.0, m) * rng.choice([-1.0, 1.0], m)
    lam[rank:] = 0.0
    a = (q * lam) @ q.T
    a = 0.5 * (a + a.T)
    ref = np.linalg.pinv(a, rcond=m * np.finfo(np.float64).eps)
    dev = torch.device("cuda")
    t = torch.as_tensor(a, device=dev)
    out = torch.empty_like(t)
    scratch = torch.empty(2 * m * m, dtype=torch.float64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    ptr = lambda x: ctypes.c_void_p(x.data_ptr())
    nat.call("spi_sym_pinv", ptr(t), m, m * float(np.finfo(np.float64).eps), ptr(out),
             ptr(scratch), ptr(status), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert int(status.item()) == m - rank
    err = np.abs(out.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err <= 1e-10, err
