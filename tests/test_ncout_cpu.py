"""The netCDF classic writer (spinterps_gb300.ncout): the reference's file
layout (interp/prepare.py:290-432) read back by scipy's independent
netCDF-3 reader (CDF-2) and by the module's own reader (CDF-5, which keeps
the reference's int64 time). No GPU."""
import numpy as np
import pytest

from spinterps_gb300 import ncout

ARGS = [("OK", "", "OK"), ("IDW", "", "IDW_000", 2.0), ("OK", "", "EST_VARS_OK")]


def _case():
    rng = np.random.default_rng(3)
    T, ny, nx = 4, 5, 7
    xs = 250.0 + 500.0 * np.arange(nx)
    ys = 9750.0 - 500.0 * np.arange(ny)
    flds = {a[2]: np.round(rng.normal(size=(T, ny, nx)), 3).astype(np.float32) for a in ARGS}
    flds["OK"][1, 2, 3] = np.nan
    return xs, ys, np.arange(T), flds


def test_cdf2_read_by_scipy(tmp_path):
    sio = pytest.importorskip("scipy.io")
    xs, ys, t, flds = _case()
    p = tmp_path / "out.nc"
    ncout.write_interp_nc(p, xs, ys, t, flds, ARGS, xlab="X", ylab="Y", tlab="time",
                          vunits="mm", vlab="precipitation", settings={"cell_size": 500.0},
                          fmt=2)
    with sio.netcdf_file(str(p), "r", mmap=False) as f:
        assert f.dimensions == {"dimx": 7, "dimy": 5, "dimt": 4}
        assert np.array_equal(f.variables["X"][:], xs)
        assert np.array_equal(f.variables["Y"][:], ys)
        assert np.array_equal(f.variables["time"][:], t)
        for a in ARGS:
            v = f.variables[a[2]]
            assert v.dimensions == ("dimt", "dimy", "dimx")
            assert np.array_equal(v[:], flds[a[2]], equal_nan=True)
            assert v.units == b"mm"
        assert f.variables["IDW_000"].standard_name == b"precipitation (IDW_exp_2.0)"
        assert f.variables["OK"].standard_name == b"precipitation (OK)"
        assert f.sett_cell_size == b"500.0"
        assert f.Source == str(p).encode()


def test_cdf5_round_trip_int64_time(tmp_path):
    xs, ys, t, flds = _case()
    p = tmp_path / "out5.nc"
    ncout.write_interp_nc(p, xs, ys, t * 3600, flds, ARGS, tunits="seconds since 2000-01-01",
                          tcldr="gregorian", settings={"idw_exps": [2.0]})
    dims, var, gatt = ncout.read_nc(p)
    assert dims == {"dimx": 7, "dimy": 5, "dimt": 4}
    assert var["time"][1].dtype == np.int64 and np.array_equal(var["time"][1], t * 3600)
    assert var["time"][2] == {"units": "seconds since 2000-01-01", "calendar": "gregorian"}
    for a in ARGS:
        assert np.array_equal(var[a[2]][1], flds[a[2]], equal_nan=True)
    assert gatt["sett_idw_exps"] == "[2.0]"
    with open(p, "rb") as f:
        assert f.read(4) == b"CDF\x05"


def test_classic_fuzz_read_by_scipy(tmp_path):
    """Seeded random files (1 to 4 dimensions, scalar to 3-d variables of
    every classic type, odd byte counts that need padding, numeric and text
    attributes) written as CDF-1 and CDF-2 in turn and read back by scipy's
    independent netCDF-3 reader, value for value."""
    sio = pytest.importorskip("scipy.io")
    rng = np.random.default_rng(17)
    types = [np.int8, np.int16, np.int32, np.float32, np.float64]
    for case in range(40):
        dims = {f"d{k}": int(rng.integers(1, 7)) for k in range(int(rng.integers(1, 5)))}
        names = list(dims)
        variables = []
        for v in range(int(rng.integers(1, 5))):
            nd = int(rng.integers(0, min(3, len(names)) + 1))
            dn = tuple(rng.choice(names, nd, replace=False)) if nd else ()
            dt = types[rng.integers(len(types))]
            shape = tuple(dims[d] for d in dn)
            if np.issubdtype(dt, np.integer):
                arr = rng.integers(np.iinfo(dt).min, np.iinfo(dt).max, shape, endpoint=True)
            else:
                arr = rng.normal(size=shape) * 1e3
            attrs = {"units": "mm" * int(rng.integers(0, 3)) or "x",
                     "scale": np.array(rng.normal(size=int(rng.integers(1, 4))), dt)}
            variables.append((f"v{v}", dn, np.asarray(arr, dt), attrs))
        gatt = {"title": f"case {case}", "ver": np.int32(case)}
        p = tmp_path / f"f{case}.nc"
        ncout.write_nc(p, dims, variables, gatt, fmt=1 if case % 2 else 2)
        with sio.netcdf_file(p, "r", mmap=False) as f:
            assert {k: f.dimensions[k] for k in dims} == dims, case
            assert f.title == b"case %d" % case and f.ver == case
            for name, dn, arr, attrs in variables:
                got = f.variables[name]
                assert tuple(got.dimensions) == dn, (case, name)
                assert np.array_equal(got[...] if arr.ndim else got.getValue(), arr), (case, name)
                assert got.units.decode() == attrs["units"]
                assert np.array_equal(np.atleast_1d(got.scale), attrs["scale"]), (case, name)
