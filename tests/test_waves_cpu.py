"""The wave planner and the netCDF slab sink, on the CPU: waves cover
every step once, in order, each within the budget unless a single step
exceeds it; a file written wave by wave through nc_sink reads back as the
same file written at once (write_interp_nc with the whole fields)."""
import numpy as np

from spinterps_gb300 import ncout, waves


def test_plan_waves_cover_the_steps_within_the_budget():
    rng = np.random.default_rng(0)
    T, N, C = 40, 300, 5000
    data = rng.normal(size=(T, N))
    data[rng.uniform(size=(T, N)) < 0.3] = np.nan
    args = [("OK", None, "OK"), ("IDW", None, "IDW_000", 2.0),
            ("EST_VARS_OK", None, "EST_VARS_OK")]
    n_av = np.isfinite(data).sum(1)
    per = [waves.step_bytes(int(n), C, 3, 4, ["OK"], True, True) for n in n_av]
    for budget in (max(per) - 1, 3 * max(per), 10 * max(per), 10 ** 15):
        ws = waves.plan_waves(data, C, args, budget=budget, est_vars=True, precision="mixed")
        assert ws[0][0] == 0 and ws[-1][1] == T
        assert all(a < b for a, b in ws)
        assert all(ws[i][1] == ws[i + 1][0] for i in range(len(ws) - 1))
        for a, b in ws:
            assert b - a == 1 or sum(per[a:b]) <= budget
    assert len(waves.plan_waves(data, C, args, budget=10 ** 15)) == 1


def test_nc_sink_matches_the_whole_file(tmp_path):
    rng = np.random.default_rng(1)
    T, ny, nx = 7, 5, 6
    xc, yc = np.arange(nx) * 2.0, np.arange(ny)[::-1] * 2.0
    args = [("OK", None, "OK"), ("IDW", None, "IDW_000", 2.0)]
    mask = rng.uniform(size=ny * nx) < 0.7
    C = int(mask.sum())
    full = {a[2]: rng.normal(size=(T, C)).astype(np.float32) for a in args}
    whole = {}
    for lab, v in full.items():
        g = np.full((T, ny * nx), np.nan, dtype=np.float32)
        g[:, mask] = v
        whole[lab] = g.reshape(T, ny, nx)
    p1 = tmp_path / "whole.nc"
    p2 = tmp_path / "waves.nc"
    ncout.write_interp_nc(p1, xc, yc, np.arange(T), whole, args, vunits="mm")
    sink = waves.nc_sink(p2, xc, yc, np.arange(T), args, mask=mask, vunits="mm")
    for a, b in ((0, 3), (3, 4), (4, 7)):
        sink(a, {lab: v[a:b] for lab, v in full.items()})
    d1, v1, g1 = ncout.read_nc(p1)
    d2, v2, g2 = ncout.read_nc(p2)
    assert d1 == d2
    for k in v1:
        assert np.array_equal(v1[k][1], v2[k][1], equal_nan=True), k
        assert v1[k][2] == v2[k][2]
