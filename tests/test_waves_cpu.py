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


def test_neighbour_waves_slice_the_steps(monkeypatch):
    """With the neighbour methods every wave is one call of the neighbour
    step engine on its steps (replaced here by a stand-in that returns each
    cell's time step): waves fit the budget less the fixed neighbour
    bytes, each call gets its slice of the data, variograms and time steps
    with the method's keywords, the sink receives the waves in order, and
    the problem steps of all waves are merged."""
    from spinterps_gb300 import nebs
    calls = []

    def fake(stn_x, stn_y, data, cell_x, cell_y, vgs, interp_args, neb, n_nebs, n_pies, *,
             time_steps, **kw):
        calls.append(dict(neb=neb, n_nebs=n_nebs, n_pies=n_pies, steps=list(time_steps),
                          vgs=list(vgs), rows=data.shape[0], kw=kw))
        ts = np.asarray(time_steps, dtype=np.float64)
        flds = {a[2]: np.repeat(ts[:, None], cell_x.size, axis=1) for a in interp_args}
        return flds, [t for t in time_steps if t % 5 == 0]

    monkeypatch.setattr(nebs, "interp_steps_nebs", fake)
    monkeypatch.setattr(waves, "_require_cuda", lambda device: device)
    T, N, C = 23, 12, 50
    rng = np.random.default_rng(3)
    data = rng.normal(size=(T, N))
    sx, sy = rng.uniform(0, 1e4, N), rng.uniform(0, 1e4, N)
    cx, cy = rng.uniform(0, 1e4, C), rng.uniform(0, 1e4, C)
    vgs = [f"1.0 Exp({1000 + j})" for j in range(T)]
    args = [("OK", None, "OK"), ("IDW", None, "IDW_000", 2.0),
            ("EST_VARS_OK", None, "EST_VARS_OK")]
    per = C * len(args) * 4
    budget = waves.nebs_fixed_bytes(C, 8) + 4 * per
    got = {a[2]: np.full((T, C), np.nan) for a in args}
    firsts = []

    def sink(first, flds):
        firsts.append(first)
        for lab, v in flds.items():
            got[lab][first:first + v.shape[0]] = v

    steps = np.arange(100, 100 + T)
    prblm, info = waves.interp_steps_waves(
        sx, sy, data, cx, cy, vgs, args, sink=sink, budget=budget, est_vars=True,
        time_steps=steps, min_vg_val=1e-4, neb_sel_mthd="nrst", n_nebs=8, n_pies=1)
    assert firsts == [0, 4, 8, 12, 16, 20]
    assert [c["rows"] for c in calls] == [4, 4, 4, 4, 4, 3]
    assert [i["steps"] for i in info] == [[a, min(a + 4, T)] for a in firsts]
    for c, a in zip(calls, firsts):
        assert (c["neb"], c["n_nebs"], c["n_pies"]) == ("nrst", 8, 1)
        assert c["steps"] == list(steps[a:a + c["rows"]])
        assert c["vgs"] == vgs[a:a + c["rows"]]
        assert c["kw"]["est_vars"] and c["kw"]["min_vg_val"] == 1e-4
    for lab in got:
        assert np.array_equal(got[lab], np.repeat(steps[:, None], C, axis=1).astype(float))
    assert prblm == [100, 105, 110, 115, 120]
