"""Steps in waves (spinterps_gb300.waves): a small budget forces several
waves; the fields handed to the sink, and the netCDF file nc_sink writes,
equal a one-shot interp_steps run (every step's system is its own, so only
the grouping of the launches differs)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import port  # noqa: E402


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_waves_equal_one_shot(tmp_path, precision):
    import spinterps_gb300 as spi
    from spinterps_gb300 import ncout, waves
    rng = np.random.default_rng(12)
    n, T, nx, ny = 150, 14, 40, 30
    sx, sy = rng.uniform(0, 8e4, n), rng.uniform(0, 8e4, n)
    gx, gy = np.meshgrid(np.arange(nx) * 2000.0 + 1000.0, 6e4 - 1000.0 - np.arange(ny) * 2000.0)
    cx, cy = gx.ravel(), gy.ravel()
    z = rng.gamma(0.8, 2.0, size=(T, n))
    z[rng.uniform(size=(T, n)) < 0.2] = np.nan
    z[5, :] = np.nan  # a step without stations: a problem step
    vgs = [f"0.1 Nug(0.0) + 0.9 {('Sph', 'Exp', 'Gau')[j % 3]}({15000 + 1000 * j})"
           for j in range(T)]
    args = port.interp_args_for(["OK", "SK", ("IDW", 2.0)], est_vars=True)
    kw = dict(est_vars=True, min_vg_val=1e-4, precision=precision)
    ref, rp = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    per = waves.step_bytes(n, cx.size, len(args), 4, ["OK", "SK"], True, precision == "mixed")
    got = {lab: np.full_like(v, np.nan) for lab, v in ref.items()}
    firsts = []

    def sink(first, flds):
        firsts.append(first)
        for lab, v in flds.items():
            got[lab][first:first + v.shape[0]] = v

    prblm, info = waves.interp_steps_waves(sx, sy, z, cx, cy, vgs, args, sink=sink,
                                           budget=3 * per, **kw)
    assert len(firsts) >= 4 and firsts == sorted(firsts)
    assert sorted(prblm) == sorted(rp) == [5]
    for lab in ref:
        m = np.isfinite(ref[lab])
        assert np.array_equal(m, np.isfinite(got[lab])), lab
        assert np.abs(got[lab][m] - ref[lab][m]).max() <= 1e-12 * np.abs(ref[lab][m]).max()
    # the same waves into the reference's netCDF layout
    path = tmp_path / "waves.nc"
    sink2 = waves.nc_sink(path, np.arange(nx) * 2000.0 + 1000.0,
                          6e4 - 1000.0 - np.arange(ny) * 2000.0, np.arange(T), args)
    waves.interp_steps_waves(sx, sy, z, cx, cy, vgs, args, sink=sink2, budget=3 * per, **kw)
    _, var, _ = ncout.read_nc(path)
    for lab in ref:
        a = var[lab][1].reshape(T, -1)
        assert np.array_equal(np.isfinite(a), np.isfinite(got[lab])), lab
        assert np.array_equal(a[np.isfinite(a)], got[lab][np.isfinite(a)]), lab


@pytest.mark.parametrize("mth,nn,npie", [("nrst", 10, 1), ("pie", 12, 4)])
def test_neighbour_waves_equal_one_shot(mth, nn, npie):
    """The neighbour methods in waves: every step's neighbour lists and
    group systems depend on its own stations and variogram only, so the
    waves' fields equal a one-shot run bit for bit."""
    import spinterps_gb300 as spi
    from spinterps_gb300 import waves
    rng = np.random.default_rng(13)
    n, T, nx, ny = 60, 11, 30, 20
    sx, sy = rng.uniform(0, 6e4, n), rng.uniform(0, 6e4, n)
    gx, gy = np.meshgrid(np.arange(nx) * 2000.0 + 1000.0, 4e4 - 1000.0 - np.arange(ny) * 2000.0)
    cx, cy = gx.ravel(), gy.ravel()
    z = rng.gamma(0.8, 2.0, size=(T, n))
    z[rng.uniform(size=(T, n)) < 0.2] = np.nan
    z[4, :] = np.nan  # a step without stations: a problem step
    vgs = [f"0.1 Nug(0.0) + 0.9 {('Sph', 'Exp')[j % 2]}({15000 + 1000 * j})" for j in range(T)]
    args = port.interp_args_for(["OK", "SK", ("IDW", 2.0)], est_vars=True)
    kw = dict(est_vars=True, min_vg_val=1e-4, neb_sel_mthd=mth, n_nebs=nn, n_pies=npie)
    ref, rp = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    got = {lab: np.full_like(v, np.nan) for lab, v in ref.items()}
    firsts = []

    def sink(first, flds):
        firsts.append(first)
        for lab, v in flds.items():
            got[lab][first:first + v.shape[0]] = v

    budget = waves.nebs_fixed_bytes(cx.size, nn) + 3 * cx.size * len(args) * 4
    prblm, info = waves.interp_steps_waves(sx, sy, z, cx, cy, vgs, args, sink=sink,
                                           budget=budget, **kw)
    assert firsts == [0, 3, 6, 9]
    assert sorted(prblm) == sorted(rp) == [4]
    for lab in ref:
        assert np.array_equal(got[lab], ref[lab], equal_nan=True), lab
