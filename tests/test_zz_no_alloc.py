"""The allocation-free kriging entry point, spi_krige_ok_noalloc.

It is meant for callers that cannot allocate device memory (their own pool
allocator owns the GPU, or an allocation per call is too costly): it keeps
its workspace in a static device array instead of a caller-provided one.
Here it is called through the C ABI twice in a row, with different station
sets, variograms and step counts (the second call must not see the first
call's leftovers in the shared array), and each result is compared with the
regular entry points (spi_krige_factor / _duals / _cells through
interp_steps) at the FP64 parity tolerance of the other GPU tests. A third
call, on a station set with a duplicated station (an exactly singular
system), must give the regular path's fields and route: route 1 with
numpy.linalg.pinv's truncated inverse (spi_krige_factor's pinv check), or
route 2 exactly where the regular path lists the step as a problem step. Once the calls
above have run, a further call must leave the device's free memory
unchanged: it allocates nothing. Sizes beyond its limits must be rejected
before any work is launched.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FP64_TOL = 1e-9


def _err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    assert np.array_equal(np.isnan(a), np.isnan(b))
    m = ~np.isnan(b)
    d = float(np.abs(a[m] - b[m]).max())
    scale = float(np.abs(b[m]).max())
    return d / scale if scale > 0 else d


def _case(rng, n_all, subset, n_steps):
    z = np.full((n_steps, n_all), np.nan)
    z[:, subset] = 3.0 + rng.normal(size=(n_steps, subset.size))
    return z


def test_noalloc_matches_regular_entry_points_twice():
    import spinterps_gb300 as spi
    from spinterps_gb300 import _native as nat
    from spinterps_gb300.steps import _ptr, _stream, parse_vg

    dev = torch.device("cuda:0")
    rng = np.random.default_rng(5)
    n_all = 160
    sx, sy = rng.uniform(0, 8e4, n_all), rng.uniform(0, 8e4, n_all)
    gx, gy = np.meshgrid(np.arange(40) * 2000.0 + 1000.0, 8e4 - 1000.0 - np.arange(30) * 2000.0)
    cx, cy = gx.ravel(), gy.ravel()
    C = cx.size
    t_sx, t_sy, t_cx, t_cy = (torch.as_tensor(a, device=dev) for a in (sx, sy, cx, cy))
    dom = nat.DomainT(n_all, _ptr(t_sx), _ptr(t_sy), C, _ptr(t_cx), _ptr(t_cy), 0, None, None,
                      1e-4, None, None)
    calls = [
        (np.arange(0, 120), "0.05 Nug(0.0) + 0.95 Exp(20000)", 3),
        (np.sort(rng.choice(n_all, 150, replace=False)), "0.1 Nug(0.0) + 1.4 Sph(35000)", 5),
    ]
    args = [("OK", None, "OK"), ("EST_VARS_OK", None, "EST_VARS_OK")]
    for subset, vg, n_steps in calls:
        z = _case(rng, n_all, subset, n_steps)
        ref, _ = spi.interp_steps(sx, sy, z, cx, cy, [vg] * n_steps, args, est_vars=True,
                                  min_var_thr=-np.inf, min_vg_val=1e-4,
                                  intrp_dtype=np.float64)
        idx = torch.as_tensor(subset.astype(np.int32), device=dev)
        vals = torch.as_tensor(np.ascontiguousarray(z[:, subset]), device=dev)
        est = torch.full((n_steps, C), float("nan"), dtype=torch.float64, device=dev)
        var = torch.full((n_steps, C), float("nan"), dtype=torch.float64, device=dev)
        out = nat.OutT(1, _ptr(est), _ptr(var), 0, 0, 0.0, 0.0)
        v = parse_vg(vg)
        route = torch.full((1,), -1, dtype=torch.int32, device=dev)
        rc = nat.lib().spi_krige_ok_noalloc(ctypes.byref(dom), _ptr(idx), subset.size,
                                            ctypes.byref(v), _ptr(vals), n_steps, 1,
                                            ctypes.byref(out), _stream(), _ptr(route))
        assert rc == 0
        torch.cuda.synchronize()
        assert int(route.item()) == 0
        assert _err(est.cpu().numpy(), ref["OK"]) <= FP64_TOL
        assert _err(var.cpu().numpy(), ref["EST_VARS_OK"]) <= FP64_TOL


def test_noalloc_reports_a_singular_system_and_allocates_nothing():
    import spinterps_gb300 as spi
    from spinterps_gb300 import _native as nat
    from spinterps_gb300.steps import _ptr, _stream, parse_vg

    dev = torch.device("cuda:0")
    rng = np.random.default_rng(8)
    n_all = 60
    sx, sy = rng.uniform(0, 5e4, n_all), rng.uniform(0, 5e4, n_all)
    sx[7], sy[7] = sx[6], sy[6]          # a duplicated station: singular system
    gx, gy = np.meshgrid(np.arange(20) * 2500.0 + 1250.0, 5e4 - 1250.0 - np.arange(20) * 2500.0)
    cx, cy = gx.ravel(), gy.ravel()
    C = cx.size
    t_sx, t_sy, t_cx, t_cy = (torch.as_tensor(a, device=dev) for a in (sx, sy, cx, cy))
    dom = nat.DomainT(n_all, _ptr(t_sx), _ptr(t_sy), C, _ptr(t_cx), _ptr(t_cy), 0, None, None,
                      1e-4, None, None)
    vg = "0.1 Nug(0.0) + 0.9 Exp(15000)"
    n_steps = 2
    z = 2.0 + rng.normal(size=(n_steps, n_all))
    args = [("OK", None, "OK"), ("EST_VARS_OK", None, "EST_VARS_OK")]
    ref, prblm = spi.interp_steps(sx, sy, z, cx, cy, [vg] * n_steps, args, est_vars=True,
                                  min_var_thr=-np.inf, min_vg_val=1e-4,
                                  intrp_dtype=np.float64)
    idx = torch.arange(n_all, dtype=torch.int32, device=dev)
    vals = torch.as_tensor(z, device=dev)
    est = torch.full((n_steps, C), float("nan"), dtype=torch.float64, device=dev)
    var = torch.full((n_steps, C), float("nan"), dtype=torch.float64, device=dev)
    out = nat.OutT(1, _ptr(est), _ptr(var), 0, 0, 0.0, 0.0)
    route = torch.full((1,), -1, dtype=torch.int32, device=dev)
    v = parse_vg(vg)
    lib = nat.lib()

    def call():
        return lib.spi_krige_ok_noalloc(ctypes.byref(dom), _ptr(idx), n_all, ctypes.byref(v),
                                        _ptr(vals), n_steps, 1, ctypes.byref(out), _stream(),
                                        _ptr(route))

    assert call() == 0
    torch.cuda.synchronize()
    r = int(route.item())
    assert r in (1, 2)
    # route 2 is exactly the regular path's problem step
    assert (r == 2) == (prblm == [0, 1]), (r, prblm)
    assert _err(est.cpu().numpy(), ref["OK"]) <= FP64_TOL
    assert _err(var.cpu().numpy(), ref["EST_VARS_OK"]) <= FP64_TOL
    # the same call again, with nothing else running: no device memory
    # changes hands
    free0 = torch.cuda.mem_get_info(dev)[0]
    assert call() == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] == free0


def test_noalloc_rejects_sizes_beyond_its_limits():
    from spinterps_gb300 import _native as nat
    from spinterps_gb300.steps import _ptr, _stream, parse_vg

    dev = torch.device("cuda:0")
    x = torch.zeros(1000, dtype=torch.float64, device=dev)
    idx = torch.zeros(1000, dtype=torch.int32, device=dev)
    dom = nat.DomainT(1000, _ptr(x), _ptr(x), 10, _ptr(x), _ptr(x), 0, None, None, 0.0, None,
                      None)
    out = nat.OutT(1, _ptr(x), None, 0, 0, 0.0, 0.0)
    v = parse_vg("1.0 Exp(1000)")
    lib = nat.lib()
    too_many_stations = nat.SPI_NOALLOC_MAX_STNS + 1
    assert lib.spi_krige_ok_noalloc(ctypes.byref(dom), _ptr(idx), too_many_stations,
                                    ctypes.byref(v), _ptr(x), 1, 0, ctypes.byref(out),
                                    _stream(), None) == 5
    assert lib.spi_krige_ok_noalloc(ctypes.byref(dom), _ptr(idx), 10, ctypes.byref(v), _ptr(x),
                                    nat.SPI_NOALLOC_MAX_STEPS + 1, 0, ctypes.byref(out),
                                    _stream(), None) == 5
    # fewer than two stations: an argument error (the caller copies a
    # single station's value itself)
    assert lib.spi_krige_ok_noalloc(ctypes.byref(dom), _ptr(idx), 1, ctypes.byref(v), _ptr(x),
                                    1, 0, ctypes.byref(out), _stream(), None) == 1
