"""Pin the oracle (oracle/port.py + oracle/vgfill.c) to the reference.

The golden vectors were produced by running the reference's own code
(tests/golden/make_golden.py). Distances, variogram fills, IDW primitives and
gathers must match bit for bit; kriging results go through LAPACK's pinv,
whose last bits depend on the BLAS build, so they are compared at 1e-11
relative to the field's scale.
"""
import numpy as np
import pytest

from oracle import port

KRIG_RTOL = 1e-11


def _close(a, b, rtol=KRIG_RTOL):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape
    assert np.array_equal(np.isnan(a), np.isnan(b))
    m = np.isfinite(b)
    scale = max(np.abs(b[m]).max(), 1e-300) if m.any() else 1.0
    err = np.abs(a[m] - b[m]).max() / scale if m.any() else 0.0
    assert err <= rtol, err


def test_dists_bit_exact(golden):
    g = golden
    d = port.get_dists_arr(g["k_cx"], g["k_cy"], g["k_sx"], g["k_sy"])
    assert np.array_equal(d, g["k_d_cs"])
    d = port.get_dists_arr(g["k_sx"], g["k_sy"], g["k_sx"], g["k_sy"])
    assert np.array_equal(d, g["k_d_ss"])


def test_vg_fill_bit_exact(golden):
    g = golden
    for vi, vg in enumerate(g["k_vgs"]):
        for covar in (0, 1):
            for mvv in (0.0, 1e-4, 0.05):
                a = port.fill_vg_var_arr(g["k_d_ss"], covar, 1, str(vg), mvv)
                assert np.array_equal(a, g[f"k_vg_ss_{vi}_{covar}_{mvv:g}"]), (vg, covar, mvv)
                b = port.fill_vg_var_arr(g["k_d_cs"], covar, 0, str(vg), mvv)
                assert np.array_equal(b, g[f"k_vg_cs_{vi}_{covar}_{mvv:g}"]), (vg, covar, mvv)


def test_idw_primitives_and_gather(golden):
    import ctypes
    from oracle import build
    lib = build.lib()
    g = golden
    for e in (1.0, 2.0, 3.5):
        d = g["k_d_cs"][5].copy() / g["k_d_cs"][5].max()
        w = np.empty_like(d)
        s = lib.orc_fill_wts_and_sum(ctypes.c_void_p(d.ctypes.data), d.size,
                                     ctypes.c_void_p(w.ctypes.data), e)
        assert np.array_equal(w, g[f"k_idw_w_{e:g}"])
        assert s == g[f"k_idw_s_{e:g}"]
        z = g[f"k_idw_z_{e:g}"]
        m = lib.orc_get_mults_sum(ctypes.c_void_p(w.ctypes.data),
                                  ctypes.c_void_p(z.ctypes.data), z.size)
        assert m == g[f"k_idw_m_{e:g}"]
    sub = port.get_2d_arr_subset(g["k_d_cs"], g["k_copy_ri"], g["k_copy_ci"], 2, 1)
    assert np.array_equal(np.isnan(sub), np.isnan(g["k_copy_sub"]))
    assert np.array_equal(np.nan_to_num(sub), np.nan_to_num(g["k_copy_sub"]))


def test_nuggetness(golden):
    g = golden
    for s, r4, r0 in zip(g["k_nug_strs"], g["k_nug_1e-4"], g["k_nug_0"]):
        assert port.check_full_nuggetness(str(s), 1e-4) == bool(r4), s
        assert port.check_full_nuggetness(str(s), 0.0) == bool(r0), s


def _interp(g, itype, vgs, *, cx="i_cx", cy="i_cy", z=None, n=None, flags=None,
            idw_exp=5.0, sd=None, cd=None):
    sx, sy = g["i_sx"], g["i_sy"]
    z = g["i_z"] if z is None else z
    if n is not None:
        sx, sy, z = sx[:n], sy[:n], z[:, :n]
    cxv, cyv = g[cx], g[cy]
    t = z.shape[0]
    vgs = [str(v) for v in vgs]
    krig = itype in ("OK", "SK", "EDK")
    d_cs = port.get_dists_arr(cxv, cyv, sx, sy)
    d_ss = port.get_dists_arr(sx, sy, sx, sy)
    uv = list(dict.fromkeys(vgs))
    rr = port.get_svars_arr(d_ss, uv, [itype], 1, 1e-4) if krig else None
    dr = port.get_svars_arr(d_cs, uv, [itype], 0, 1e-4) if krig else None
    if flags is None:
        flags = np.ones(t, dtype=bool)
    nug = np.array([port.check_full_nuggetness(v, 1e-4) for v in vgs])
    return port.get_interp(z.copy("c"), itype, sd, cd, idw_exp, np.array(vgs, dtype=object),
                           flags, nug, np.arange(t), [], d_cs.copy(), rr, dr,
                           np.arange(sx.size), np.arange(cxv.size), est_vars_flag=True)


def test_get_interp_ok_sk(golden):
    g = golden
    for itype in ("OK", "SK"):
        est, var = _interp(g, itype, g["i_vgs_mixed"], flags=g["i_flags"])
        _close(est, g[f"i_{itype}_est"])
        if itype == "OK":
            _close(var, g["i_OK_var"], 1e-6)   # float32 storage
    est, var = _interp(g, "OK", g["i_vgs_other"])
    _close(est, g["i_OKo_est"])
    _close(var, g["i_OKo_var"], 1e-6)


def test_get_interp_edk(golden):
    g = golden
    elev = g["i_EDK1_sd"][:, 0]
    for k in (1, 2):
        est, _ = _interp(g, "EDK", g["i_vgs_mixed"], z=g["i_z"] + 1e-3 * elev,
                         flags=g["i_flags"], sd=g[f"i_EDK{k}_sd"], cd=g[f"i_EDK{k}_cd"])
        _close(est, g[f"i_EDK{k}_est"])


def test_get_interp_idw_nnb_one(golden):
    g = golden
    t = g["i_z"].shape[0]
    vg0 = "0.05 Nug(0.0) + 0.95 Exp(20000)"
    for e in (1.0, 2.0, 3.5):
        est, _ = _interp(g, "IDW", [vg0] * t, cx="i_cx2", cy="i_cy2", flags=g["i_flags"],
                         idw_exp=e)
        assert np.isnan(est[g["i_flags"], 0]).all()
        _close(est, g[f"i_IDW_{e:g}_est"], 1e-15)
    est, _ = _interp(g, "NNB", [vg0] * t, cx="i_cx2", cy="i_cy2")
    assert np.array_equal(est, g["i_NNB_est"])
    est, var = _interp(g, "OK", [vg0] * t, n=1)
    assert np.array_equal(est, g["i_one_est"])
    assert np.isnan(var).all() and np.isnan(g["i_one_var"]).all()


@pytest.mark.parametrize("tag", ["okidw", "edk"])
def test_interp_steps(golden, tag):
    _check_steps(golden, tag)


def test_interp_steps_sweep(golden):
    """16 multi-step runs with seeded random settings
    (tests/golden/steps_sweep.npz): methods, missingness, thresholds and
    cut-offs."""
    for tag in golden["ss_tags"]:
        _check_steps(golden, str(tag))


def _check_steps(golden, tag):
    g = golden
    p = f"s_{tag}_"
    methods = []
    for m in g[p + "methods"]:
        m = str(m)
        methods.append(("IDW", float(m.split(":")[1])) if m.startswith("IDW:") else m)
    thr, mn, mx, mvv = g[p + "params"]
    args = port.interp_args_for(methods, est_vars="OK" in methods)
    flds, prblm = port.interp_steps(
        g[p + "sx"], g[p + "sy"], g[p + "z"], g[p + "cx"], g[p + "cy"],
        [str(v) for v in g[p + "vgs"]], args, est_vars="OK" in methods,
        stn_drifts=g.get(p + "sd"), cell_drifts=g.get(p + "cd"),
        min_var_thr=thr, min_var_cut=None if np.isnan(mn) else mn,
        max_var_cut=None if np.isnan(mx) else mx, min_vg_val=mvv)
    assert sorted(set(prblm)) == g[p + "prblm"].tolist()
    for lab, f in flds.items():
        ref = g[p + "out_" + lab]
        _close(f, ref, 1e-6)


def test_config1_subset(golden):
    g = golden
    sx, sy, z = g["c1_sx"], g["c1_sy"], g["c1_z"]
    cx, cy = g["c1_cx"], g["c1_cy"]
    vg = "0.05 Nug(0.0) + 0.95 Exp(20000)"
    args = port.interp_args_for(["OK", ("IDW", 2.0)], est_vars=True)
    flds, _ = port.interp_steps(sx, sy, z, cx, cy, [vg] * z.shape[0], args, est_vars=True,
                                min_vg_val=1e-4, intrp_dtype=np.float64)
    _close(flds["OK"], g["c1_ok_est"])
    _close(flds["EST_VARS_OK"], g["c1_ok_var"], 1e-6)
    _close(flds["IDW_000"], g["c1_idw_est"], 1e-14)


def test_oracle_neighbours_match_reference(golden):
    """nrst / pie neighbour lists and cell groups (interp/grps.py) as the
    reference computes them (tests/golden/nebs.npz), bit for bit."""
    g = golden
    sx, sy, cx, cy = g["n_sx"], g["n_sy"], g["n_cx"], g["n_cy"]
    for mth, nn, npie in (("nrst", 8, 1), ("pie", 8, 4), ("pie", 12, 6)):
        tag = f"{mth}_{nn}_{npie}"
        idx = port.neb_idxs(mth, cx, cy, sx, sy, nn, npie)
        lab, _ = port.neb_groups(idx)
        assert np.array_equal(idx, g[f"n_{tag}_idxs"]), tag
        assert np.array_equal(lab, g[f"n_{tag}_grp"]), tag


def test_oracle_neighbour_sweep_matches_reference(golden):
    """nrst / pie neighbour lists and cell groups on 60 seeded random station
    and cell sets (tests/golden/nebs_sweep.npz), bit for bit."""
    g = golden
    for i in g["ns_cases"]:
        p = f"ns{i}_"
        kind, nn, npie = (int(v) for v in g[p + "cfg"])
        mth = "nrst" if kind == 0 else "pie"
        idx = port.neb_idxs(mth, g[p + "cx"], g[p + "cy"], g[p + "sx"], g[p + "sy"], nn, npie)
        lab, _ = port.neb_groups(idx)
        assert np.array_equal(idx, g[p + "idxs"].astype(np.int64)), (i, mth, nn, npie)
        assert np.array_equal(lab, g[p + "grp"].astype(np.int64)), (i, mth, nn, npie)


LEGACY_INPUTS = ("xi", "yi", "zi", "xk", "yk", "si", "sk", "lim", "model", "cls")


def test_oracle_legacy_classes_match_reference(golden):
    """The restatement of OrdinaryKriging, SimpleKriging,
    ExternalDriftKriging(_MD) and the indicator classes
    (cyth/interpmthds.pyx:251-765) reproduces every array the reference's
    compiled classes expose (tests/golden/legacy.npz), bit for bit."""
    g = golden
    for ci in g["l_cases"]:
        p = f"l{ci}_"
        cls = str(g[p + "cls"])
        got = port.legacy_krige(cls, g[p + "xi"], g[p + "yi"], g[p + "zi"], g[p + "xk"],
                                g[p + "yk"], str(g[p + "model"]), si=g[p + "si"],
                                sk=g[p + "sk"], lim=float(g[p + "lim"]))
        keys = [k[len(p):] for k in g if k.startswith(p) and k[len(p):] not in LEGACY_INPUTS]
        assert keys, cls
        for k in keys:
            assert np.array_equal(np.asarray(got[k]), g[p + k]), (ci, cls, k)


def test_oracle_legacy_sweep_matches_reference(golden):
    """The same restatement on 48 seeded random cases of the six classes
    (tests/golden/legacy_sweep.npz: model nests, drifts, indicator limits):
    estimates, variances, multipliers, weights and indicators bit for bit."""
    g = golden
    for ci in g["ls_cases"]:
        p = f"ls{ci}_"
        cls = str(g[p + "cls"])
        got = port.legacy_krige(cls, g[p + "xi"], g[p + "yi"], g[p + "zi"], g[p + "xk"],
                                g[p + "yk"], str(g[p + "model"]), si=g[p + "si"],
                                sk=g[p + "sk"], lim=float(g[p + "lim"]))
        keys = [k[len(p):] for k in g if k.startswith(p) and k[len(p):] not in LEGACY_INPUTS]
        assert "zk" in keys or "ik" in keys, (ci, cls)
        for k in keys:
            assert np.array_equal(np.asarray(got[k]), g[p + k]), (ci, cls, k)


def test_oracle_driver_grid_and_drifts_match_reference(golden):
    """The grid (SpInterpPrepare._prepare_crds) and the drift sampling
    (KrigingDrift._prepare_stns_drift) as the reference computes them
    (tests/golden/driver.npz), bit for bit."""
    g = golden
    for ci in g["d_cases"]:
        p = f"d{ci}_"
        x0, x1, y0, y1, cs = g[p + "bounds"]
        db = None
        if p + "drift" in g:
            dx0, dy1 = g[p + "drift_origin"]
            nr, nc = g[p + "drift"].shape[1:]
            db = (dx0, dx0 + nc * cs, dy1 - nr * cs, dy1)
        r = port.prepare_crds(x0, x1, y0, y1, cs, drift_bounds=db)
        assert tuple(r["rc"]) == tuple(g[p + "rc"])
        assert tuple(r["shape"]) == tuple(g[p + "shape"])
        for k in ("x_crds", "y_crds", "cell_x", "cell_y"):
            assert np.array_equal(r[k], g[p + k]), (ci, k)
        if db is not None:
            mask = g[p + "mask"] if p + "mask" in g else None
            cell, stn = port.sample_drifts(list(g[p + "drift"]), dx0, dy1, cs,
                                           float(g[p + "ndv"]), r["rc"], g[p + "stn_x"],
                                           g[p + "stn_y"], cntn_idxs=mask)
            assert np.array_equal(cell, g[p + "cell_drift"], equal_nan=True), ci
            assert np.array_equal(stn, g[p + "stn_drift"]), ci


def test_oracle_polygon_mask_known_answers():
    """Strict containment after rounding to 1e-6: inside, outside, on an
    edge, on a vertex, in and on the edge of a concave notch, and just
    inside an edge."""
    sq = ([0.0, 10.0, 10.0, 0.0], [0.0, 0.0, 10.0, 10.0])
    notch = ([20.0, 30.0, 30.0, 25.0, 20.0], [0.0, 0.0, 10.0, 5.0, 10.0])
    px = np.array([5.0, 11.0, 10.0, 0.0, 5.0, 25.0, 25.0, 9.9999996, 9.9999994, 21.0, 22.0])
    py = np.array([5.0, 5.0, 5.0, 0.0, 10.0, 7.0, 4.0, 5.0, 5.0, 8.0, 8.0])
    want = np.array([1, 0, 0, 0, 0, 0, 1, 0, 1, 1, 0], dtype=bool)
    got = port.points_in_polygons(px, py, [sq, notch])
    assert np.array_equal(got, want), got


def test_get_interp_sweep(golden):
    """The oracle's get_interp against the reference's _get_interp on 80
    seeded random one-group cases (tests/golden/interp_sweep.npz): every
    variogram model in nests of up to three, flags off and nugget-only
    steps, OK / SK / EDK with 1 to 3 drifts / IDW / NNB."""
    g = golden
    for i in g["w_cases"]:
        p = f"w{i}_"
        itype = str(g[p + "type"])
        sx, sy, cx, cy, z = (g[p + k] for k in ("sx", "sy", "cx", "cy", "z"))
        vgs = [str(v) for v in g[p + "vgs"]]
        t = z.shape[0]
        krig = itype in ("OK", "SK", "EDK")
        d_cs = port.get_dists_arr(cx, cy, sx, sy)
        d_ss = port.get_dists_arr(sx, sy, sx, sy)
        uv = list(dict.fromkeys(vgs))
        rr = port.get_svars_arr(d_ss, uv, [itype], 1, 1e-4) if krig else None
        dr = port.get_svars_arr(d_cs, uv, [itype], 0, 1e-4) if krig else None
        nug = np.array([port.check_full_nuggetness(v, 1e-4) for v in vgs])
        prblm = []
        est, var = port.get_interp(
            z.copy("c"), itype, g.get(p + "sd"), g.get(p + "cd"), float(g[p + "idw_exp"]),
            np.array(vgs, dtype=object), g[p + "flags"], nug, np.arange(t), prblm, d_cs.copy(),
            rr, dr, np.arange(sx.size), np.arange(cx.size), est_vars_flag=True)
        assert sorted(prblm) == g[p + "prblm"].tolist(), i
        if itype == "NNB":
            assert np.array_equal(est, g[p + "est"], equal_nan=True), i
        else:
            _close(est, g[p + "est"], 1e-15 if itype == "IDW" else KRIG_RTOL)
        if p + "var" in g:
            _close(var, g[p + "var"], 1e-6)   # float32 storage


def test_vg_fill_edges_bit_exact(golden):
    """The C restatement of fill_vg_var_arr at every model's branch points
    (tests/golden/vg_edges.npz): h = 0, the smallest subnormal, each range
    and its neighbouring doubles, 1e300 and inf, ranges under the 1e-5 clamp."""
    g = golden
    for vi, vg in enumerate(g["ve_vgs"]):
        h = g[f"ve_h_{vi}"]
        row = h[None, :].copy()
        with np.errstate(invalid="ignore"):  # inf - inf
            sq = np.abs(h[:, None] - h[None, :])
        sq[~np.isfinite(sq)] = np.inf
        for covar in (0, 1):
            for mvv in (0.0, 0.05):
                a = port.fill_vg_var_arr(row, covar, 0, str(vg), mvv)
                assert np.array_equal(a, g[f"ve_row_{vi}_{covar}_{mvv:g}"], equal_nan=True), \
                    (vg, covar, mvv)
                b = port.fill_vg_var_arr(sq, covar, 1, str(vg), mvv)
                assert np.array_equal(b, g[f"ve_sq_{vi}_{covar}_{mvv:g}"], equal_nan=True), \
                    (vg, covar, mvv)
