"""Host logic of the driver flow (spinterps_gb300.driver) against the
reference's own grid and drift sampling (tests/golden/driver.npz, made by
running SpInterpPrepare._prepare_crds and KrigingDrift._prepare_stns_drift).
No GPU."""
import numpy as np

from spinterps_gb300 import driver


def test_grid_and_drifts_match_reference(golden):
    g = golden
    for ci in g["d_cases"]:
        p = f"d{ci}_"
        x0, x1, y0, y1, cs = g[p + "bounds"]
        db = None
        if p + "drift" in g:
            dx0, dy1 = g[p + "drift_origin"]
            nr, nc = g[p + "drift"].shape[1:]
            db = driver.drift_bounds(dx0, dy1, nr, nc, cs)
        r = driver.prepare_crds(x0, x1, y0, y1, cs, drift_bounds=db)
        assert tuple(r["rc"]) == tuple(g[p + "rc"])
        assert tuple(r["shape"]) == tuple(g[p + "shape"])
        for k in ("x_crds", "y_crds", "cell_x", "cell_y"):
            assert np.array_equal(r[k], g[p + k]), (ci, k)
        if db is not None:
            mask = g[p + "mask"] if p + "mask" in g else None
            cell, stn = driver.sample_drifts(list(g[p + "drift"]), db[0], db[3], cs,
                                             float(g[p + "ndv"]), r["rc"], g[p + "stn_x"],
                                             g[p + "stn_y"], cntn_idxs=mask)
            assert np.array_equal(cell, g[p + "cell_drift"], equal_nan=True), ci
            assert np.array_equal(stn, g[p + "stn_drift"]), ci


def test_corner_coordinates_and_stats_csv(tmp_path):
    b = driver.corner_coordinates([1.0, 5.0, 3.0], [2.0, -1.0, 4.0], cell_bdist=0.5)
    assert b == (0.5, 5.5, -1.5, 4.5)
    b = driver.corner_coordinates([1.0], [2.0], 1.0, poly_extent=(0.0, 10.0, 0.0, 20.0))
    assert b == (-1.0, 11.0, -1.0, 21.0)
    cols = {"data_min": np.array([1.0, np.nan], np.float32),
            "OK_mean": np.array([2.5, 3.25], np.float32)}
    f = tmp_path / "stats.csv"
    driver.write_stats_csv(f, ["t0", "t1"], cols)
    assert f.read_text().splitlines() == [";data_min;OK_mean", "t0;1.000000;2.500000",
                                          "t1;;3.250000"]


def test_grid_sweep_matches_reference(golden):
    """400 seeded extents and cell sizes, half inside drift rasters: the
    same row / column range, shape and coordinate vectors (by SHA-256 of
    their bytes) as the reference's _prepare_crds, and an AssertionError
    wherever the reference asserted (a grid outside its rasters)."""
    import hashlib

    import pytest
    g = golden
    for i, p in enumerate(g["sw_params"]):
        x0, x1, y0, y1, cs, edk = (float(v) for v in p[:6])
        db = tuple(float(v) for v in p[6:]) if edk else None
        if g["sw_raised"][i]:
            with pytest.raises(AssertionError):
                driver.prepare_crds(x0, x1, y0, y1, cs, drift_bounds=db)
            continue
        r = driver.prepare_crds(x0, x1, y0, y1, cs, drift_bounds=db)
        assert tuple(r["rc"]) == tuple(g["sw_rc"][i]), i
        assert tuple(r["shape"]) == tuple(g["sw_shape"][i]), i
        for k, key in enumerate(("x_crds", "y_crds")):
            d = hashlib.sha256(np.ascontiguousarray(r[key], dtype="<f8").tobytes()).digest()
            assert d == bytes(g["sw_digest"][i, k]), (i, key)


def test_drift_sweep_matches_reference(golden):
    """150 seeded drift windows (rasters from tests/golden/sweeps.py with
    no-data cells and values at the edge of np.isclose's reach; stations on
    cell edges and inside cells; with and without a cell mask): the same
    cell and station drifts as the reference's _prepare_stns_drift (by
    SHA-256), and the same exception where it raised."""
    import sys
    from pathlib import Path

    import pytest
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    from sweeps import NDV, cell_mask, digest, drift_rasters
    g = golden
    for i, p in enumerate(g["dw_params"]):
        cs, dx0, dy1, nr, nc, k, phase, x0, x1, y0, y1, masked = (float(v) for v in p)
        nr, nc, k = int(nr), int(nc), int(k)
        r = driver.prepare_crds(x0, x1, y0, y1, cs,
                                drift_bounds=(dx0, dx0 + nc * cs, dy1 - nr * cs, dy1))
        mask = cell_mask(r["cell_x"].size) if masked else None
        sx, sy = g["dw_stn"][i]
        run = lambda: driver.sample_drifts(  # noqa: E731
            drift_rasters(nr, nc, k, phase), dx0, dy1, cs, NDV, r["rc"], sx, sy,
            cntn_idxs=mask)
        if g["dw_raised"][i]:
            exc = AssertionError if g["dw_raised"][i] == 1 else IndexError
            with pytest.raises(exc):
                run()
            continue
        cell, stn = run()
        assert digest(cell) == bytes(g["dw_digest"][i, 0]), i
        assert digest(stn) == bytes(g["dw_digest"][i, 1]), i
