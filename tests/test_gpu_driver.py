"""GPU kernels of the driver flow (csrc/spi_driver.cu through
spinterps_gb300.driver): the polygon cell mask against the oracle's
restatement of ogr's strict containment, numpy.round bit for bit, the
per-step statistics against numpy's nan-statistics, and the whole flow
(grid, mask, drifts, interpolation, rounding, statistics) against the
oracle's step engine on the same cells."""
import numpy as np
import pytest

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import port  # noqa: E402


def _star(cx, cy, r0, r1, n, rng):
    a = np.sort(rng.uniform(0, 2 * np.pi, n))
    r = np.where(np.arange(n) % 2 == 0, r0, r1) * rng.uniform(0.8, 1.2, n)
    return cx + r * np.cos(a), cy + r * np.sin(a)


def test_polygon_mask_vs_oracle():
    from spinterps_gb300 import driver
    rng = np.random.default_rng(5)
    gx = np.arange(0.0, 100.0, 2.5) + 1.25
    cx, cy = np.meshgrid(gx, gx[::-1])
    cx, cy = cx.ravel(), cy.ravel()
    polys = [_star(30.0, 40.0, 25.0, 9.0, 14, rng), _star(70.0, 65.0, 20.0, 12.0, 10, rng),
             # an axis-aligned rectangle whose edges pass through cell centres
             ([51.25, 91.25, 91.25, 51.25], [3.75, 3.75, 28.75, 28.75])]
    got = driver.cells_in_polygons(cx, cy, polys)
    ref = port.points_in_polygons(cx, cy, polys)
    assert np.array_equal(got, ref)
    # cells on the rectangle's edges are outside, the ones just in are inside
    on = (np.isclose(cx, 51.25) & (cy >= 3.75) & (cy <= 28.75))
    assert on.any() and not got[on].any()
    assert got[np.isclose(cx, 53.75) & np.isclose(cy, 16.25)].all()


def test_round_fields_bit_exact():
    import torch
    from spinterps_gb300 import driver
    rng = np.random.default_rng(6)
    a = rng.normal(scale=50.0, size=200_003).astype(np.float32)
    a[:1000] = np.round(a[:1000], 1) + np.float32(0.05)   # near ties
    a[5] = np.nan
    for dt in (np.float32, np.float64):
        for d in (0, 1, 3, 5, -1, -2):
            t = torch.as_tensor(a.astype(dt), device="cuda")
            driver.round_fields_(t, d)
            assert np.array_equal(t.cpu().numpy(), np.round(a.astype(dt), d), equal_nan=True), \
                (dt, d)


def test_field_stats_vs_numpy():
    import torch
    from spinterps_gb300 import driver
    rng = np.random.default_rng(7)
    f = rng.gamma(1.5, 10.0, size=(9, 70_001)).astype(np.float32)
    f[rng.uniform(size=f.shape) < 0.3] = np.nan
    f[2] = np.nan                       # no finite entry
    f[3, :] = np.nan
    f[3, 17] = 4.5                      # one entry
    f[4] += 1e4                         # large mean against the spread
    t = torch.as_tensor(f, device="cuda")
    for ddof in (0, 1):
        got = driver.field_stats(t, ddof=ddof)
        ref = port.field_stats(f, ddof)
        assert np.array_equal(np.isnan(got), np.isnan(ref)), ddof
        # min, mean, max, count to FP64 rounding; std from FP64 sums of
        # squares loses ~ (mean^2 / var) eps (row 4: ~1e-10), far below the
        # float32 the reference keeps
        for j, rtol in ((0, 1e-12), (1, 1e-12), (2, 1e-12), (3, 1e-9), (4, 0)):
            m = ~np.isnan(ref[:, j])
            assert np.allclose(got[m, j], ref[m, j], rtol=rtol, atol=0), (ddof, j)
    # numpy's float32 nan-statistics, as the reference computes them per field
    got = driver.field_stats(t, ddof=0)
    with np.errstate(all="ignore"), __import__("warnings").catch_warnings():
        __import__("warnings").simplefilter("ignore")
        for r in (0, 1, 4, 8):
            ref = [np.nanmin(f[r]), np.nanmean(f[r]), np.nanmax(f[r]), np.nanstd(f[r]),
                   np.isfinite(f[r]).sum()]
            assert np.allclose(got[r].astype(np.float32), np.float32(ref), rtol=2e-6), r


def test_interpolate_grid_vs_oracle():
    from spinterps_gb300 import driver
    rng = np.random.default_rng(8)
    n, T, cs = 35, 5, 2000.0
    sx, sy = rng.uniform(2e3, 58e3, n), rng.uniform(2e3, 58e3, n)
    z = rng.gamma(1.4, 2.0, size=(T, n))
    z[rng.uniform(size=z.shape) < 0.15] = np.nan
    vgs = ["0.1 Nug(0.0) + 0.9 Exp(20000)", "1.0 Sph(30000)", "0.2 Nug(0.0) + 0.8 Exp(15000)",
           "0.5 Exp(25000)", "1.0 Nug(0.0)"]
    drift = dict(rasters=rng.uniform(0, 2000, (1, 34, 33)), x_min=0.0, y_max=66e3,
                 ndv=-9999.0)
    polys = [_star(30e3, 30e3, 28e3, 18e3, 16, rng)]
    args = port.interp_args_for(["OK", "EDK", ("IDW", 2.0)], est_vars=True)
    kw = dict(est_vars=True, min_vg_val=1e-4, intrp_dtype=np.float64)
    out, prblm, stats, grid = driver.interpolate_grid(
        sx, sy, z, vgs, args, cell_size=cs, bounds=(1e3, 61e3, 1e3, 61e3), polygons=polys,
        drift=drift, nmrl_prcn=None, **kw)
    mask = grid["mask"]
    assert mask.any() and not mask.all()
    db = driver.drift_bounds(0.0, 66e3, 34, 33, cs)
    cdr, sdr = port.sample_drifts(list(drift["rasters"]), db[0], db[3], cs, -9999.0,
                                  grid["rc"], sx, sy, cntn_idxs=mask)
    ref, rp = port.interp_steps(sx, sy, z, grid["cell_x"][mask], grid["cell_y"][mask], vgs,
                                args, stn_drifts=sdr, cell_drifts=cdr, **kw)
    assert sorted(prblm) == sorted(rp)
    ny, nx = grid["shape"]
    for lab, v in ref.items():
        got = out[lab].reshape(T, ny * nx)
        assert np.isnan(got[:, ~mask]).all()
        a, b = got[:, mask], v
        assert np.array_equal(np.isnan(a), np.isnan(b)), lab
        m = ~np.isnan(b)
        assert np.abs(a[m] - b[m]).max() <= 1e-9 * np.abs(b[m]).max(), lab
        if lab != "EST_VARS_OK":
            st = port.field_stats(b, 0)
            for j, s in enumerate(driver.STATS):
                assert np.allclose(stats[f"{lab}_{s}"], st[:, j].astype(np.float32),
                                   rtol=1e-6, equal_nan=True), (lab, s)
    dst = port.field_stats(z, 1)
    assert np.allclose(stats["data_std"], dst[:, 3].astype(np.float32), rtol=1e-6)
    # the output files: netCDF fields and stats.csv, read back
    import tempfile
    from spinterps_gb300 import ncout
    with tempfile.TemporaryDirectory() as td:
        nc_p, csv_p = driver.write_outputs(td, "interp.nc", out, grid, stats, args,
                                           np.arange(T), vlab="z", settings={"cell_size": cs})
        dims, var, gatt = ncout.read_nc(nc_p)
        assert dims == {"dimx": nx, "dimy": ny, "dimt": T}
        for lab in out:
            assert np.array_equal(var[lab][1], out[lab], equal_nan=True), lab
        assert len(open(csv_p).read().splitlines()) == T + 1
    # rounding as written: the rounded run equals numpy.round of the plain one
    out3, _, _, _ = driver.interpolate_grid(
        sx, sy, z, vgs, args, cell_size=cs, bounds=(1e3, 61e3, 1e3, 61e3), polygons=polys,
        drift=drift, nmrl_prcn=3, **kw)
    for lab in out:
        assert np.array_equal(out3[lab], np.round(out[lab], 3), equal_nan=True), lab
