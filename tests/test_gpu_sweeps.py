"""The CUDA path against the golden sweeps made by running the reference
(tests/golden/*_sweep.npz, vg_edges.npz).

Bars:
- neighbour lists and cell groups: exact;
- the variogram fill at the branch points: 1e-13 relative (device exp / sin
  / pow against the host's libm), the same non-finite entries;
- the legacy classes' outputs: 1e-9 of the field's largest magnitude, on
  the cases whose matrix condition is under 1e6. Above that, the
  reference's pinv and the Gauss-Jordan inverse both carry errors near
  cond * eps;
- the multi-step runs: 2e-6 (float32 fields) on the FP64 path, 1e-5 on the
  mixed path;
- the one-group runs of _get_interp (interp_sweep.npz): 1e-9 on regular
  systems (or 10x the reference's own spread under 1e-15 perturbations of
  its matrix, where that is larger), exact for NNB; systems that pinv
  treats as singular are set apart and held to the reference's outcomes
  under those perturbations (tests/envelope.py).
"""
import numpy as np
import pytest

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import port  # noqa: E402

import envelope  # noqa: E402


def test_neb_select_sweep(golden):
    from spinterps_gb300 import nebs
    g = golden
    for i in g["ns_cases"]:
        p = f"ns{i}_"
        kind, nn, npie = (int(v) for v in g[p + "cfg"])
        mth = "nrst" if kind == 0 else "pie"
        grp = nebs.SpInterpNeighborGrouping(mth, nn, npie, g[p + "cx"], g[p + "cy"])
        idxs, grps = grp.get_neb_idxs_and_grps(g[p + "sx"], g[p + "sy"])
        lab = np.full(g[p + "cx"].size, -1, dtype=np.int64)
        for gi, gr in enumerate(grps):
            lab[gr] = gi
        assert np.array_equal(np.asarray(idxs, np.int64), g[p + "idxs"].astype(np.int64)), i
        assert np.array_equal(lab, g[p + "grp"].astype(np.int64)), i


def test_vg_fill_edges(golden):
    import spinterps_gb300 as spi
    g = golden
    for vi, vg in enumerate(g["ve_vgs"]):
        h = g[f"ve_h_{vi}"]
        row = h[None, :].copy()
        with np.errstate(invalid="ignore"):  # inf - inf
            sq = np.abs(h[:, None] - h[None, :])
        sq[~np.isfinite(sq)] = np.inf
        for covar, types in ((0, ["OK"]), (1, ["SK"])):
            for mvv in (0.0, 0.05):
                st = spi.SpInterpSteps(min_vg_val=mvv)
                for arr, diag, key in ((row, 0, "row"), (sq, 1, "sq")):
                    got = st._get_svars_arr(arr, [str(vg)], types, diag)[(str(vg), covar)]
                    ref = g[f"ve_{key}_{vi}_{covar}_{mvv:g}"]
                    fin = np.isfinite(ref)
                    assert np.array_equal(np.isfinite(got), fin), (vg, covar, mvv, key)
                    assert np.array_equal(got[~fin], ref[~fin], equal_nan=True), (vg, key)
                    assert np.all(np.abs(got[fin] - ref[fin])
                                  <= 1e-13 * np.abs(ref[fin]) + 1e-300), (vg, covar, mvv, key)


def test_legacy_sweep(golden):
    import spinterps_gb300 as spi
    g = golden
    checked = 0
    for ci in g["ls_cases"]:
        p = f"ls{ci}_"
        cls = str(g[p + "cls"])
        args = (g[p + "xi"], g[p + "yi"], g[p + "zi"], g[p + "xk"], g[p + "yk"])
        model, si, sk, lim = str(g[p + "model"]), g[p + "si"], g[p + "sk"], float(g[p + "lim"])
        mats = port.legacy_krige(cls, *args, model, si=si, sk=sk, lim=lim)
        a = mats.get("in_vars", mats.get("in_covars"))
        if a is None or np.linalg.cond(a) > 1e6:
            continue
        c = getattr(spi, cls)
        if cls == "ExternalDriftKriging":
            obj = c(*args[:3], si[0].copy(), *args[3:], sk[0].copy(), model=model)
            obj.krige()
        elif cls == "ExternalDriftKriging_MD":
            obj = c(*args[:3], si, *args[3:], sk, model=model)
            obj.krige()
        elif cls.endswith("IndicatorKriging"):
            obj = c(*args, lim=lim, model=model)
            obj.ikrige()
        else:
            obj = c(*args, model=model)
            obj.krige()
        for k in ("zk", "est_vars", "est_covars", "mus", "mus_1", "mus_2", "mus_arr",
                  "lambdas", "ik"):
            if p + k not in g:
                continue
            ref = g[p + k]
            got = np.asarray(getattr(obj, k), dtype=np.float64)
            scale = max(np.abs(ref).max(), 1e-300) if ref.size else 1.0
            assert np.abs(got - ref).max() <= 1e-9 * scale if ref.size else True, (ci, cls, k)
        checked += 1
    assert checked >= 20, checked


def _err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape
    assert np.array_equal(np.isnan(a), np.isnan(b))
    m = ~np.isnan(b)
    if not m.any():
        return 0.0
    return float(np.abs(a[m] - b[m]).max() / max(np.abs(b[m]).max(), 1e-300))


def test_multi_step_sweep(golden):
    """The step engine on the 16 random multi-step runs
    (tests/golden/steps_sweep.npz), FP64 path at the float32 fields' bar and
    mixed path at 1e-5, as the hand-built multi-step cases."""
    import spinterps_gb300 as spi
    g = golden
    for tag in g["ss_tags"]:
        p = f"s_{tag}_"
        methods = []
        for m in g[p + "methods"]:
            m = str(m)
            methods.append(("IDW", float(m.split(":")[1])) if m.startswith("IDW:") else m)
        thr, mn, mx, mvv = g[p + "params"]
        args = port.interp_args_for(methods, est_vars="OK" in methods)
        for precision, tol in (("fp64", 2e-6), ("mixed", 1e-5)):
            flds, prblm = spi.interp_steps(
                g[p + "sx"], g[p + "sy"], g[p + "z"], g[p + "cx"], g[p + "cy"],
                [str(v) for v in g[p + "vgs"]], args, est_vars="OK" in methods,
                stn_drifts=g.get(p + "sd"), cell_drifts=g.get(p + "cd"), min_var_thr=thr,
                min_var_cut=None if np.isnan(mn) else mn,
                max_var_cut=None if np.isnan(mx) else mx, min_vg_val=mvv, precision=precision)
            assert sorted(set(prblm)) == g[p + "prblm"].tolist(), (tag, precision)
            for lab, f in flds.items():
                e = _err(f, g[p + "out_" + lab])
                assert e <= tol, (tag, precision, lab, e)


def test_interp_sweep(golden):
    """The step engine on the 80 one-group _get_interp runs
    (tests/golden/interp_sweep.npz): OK (with variance) / SK / EDK with 1
    to 3 drifts / IDW / NNB, nests of up to three of the eight models,
    cells on stations, flag-off and nugget-only steps. The reference got
    its per-step flags as an argument; here the flagged steps come from a
    run with min_value_to_interp_thresh -inf and the others from a run with
    +inf (every step then takes the step mean)."""
    import spinterps_gb300 as spi
    g = golden
    mvv = 1e-4
    n_regular = n_singular = 0
    sing_cells = sing_ok = 0
    for i in g["w_cases"]:
        p = f"w{i}_"
        itype = str(g[p + "type"])
        sx, sy, cx, cy, z = (g[p + k] for k in ("sx", "sy", "cx", "cy", "z"))
        vgs = [str(v) for v in g[p + "vgs"]]
        flags = g[p + "flags"].astype(bool)
        sd, cd = g.get(p + "sd"), g.get(p + "cd")
        ref_est = g[p + "est"]
        ref_var = g.get(p + "var")
        m = ("IDW", float(g[p + "idw_exp"])) if itype == "IDW" else itype
        args = port.interp_args_for([m], est_vars=itype == "OK")
        lab = args[0][2]
        kw = dict(est_vars=itype == "OK", stn_drifts=sd, cell_drifts=cd, min_vg_val=mvv,
                  intrp_dtype=np.float64)
        on, prblm = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, min_var_thr=-np.inf, **kw)
        off, _ = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, min_var_thr=np.inf, **kw)
        want_prblm = g[p + "prblm"].tolist()
        assert sorted(j for j in prblm if flags[j]) == want_prblm, i
        for j in range(z.shape[0]):
            got = (on if flags[j] else off)[lab][j]
            want = ref_est[j]
            if itype == "NNB":
                assert np.array_equal(got, want, equal_nan=True), (i, j)
                continue
            scale = max(float(np.nanmax(np.abs(want))), 1e-300) if np.isfinite(want).any() \
                else 1.0
            assert np.array_equal(np.isnan(got), np.isnan(want)), (i, j)
            if itype == "IDW" or not flags[j] or port.check_full_nuggetness(vgs[j], mvv):
                assert np.nanmax(np.abs(got - want), initial=0.0) <= 1e-9 * scale, (i, j)
                if ref_var is not None and not flags[j]:
                    assert np.all((on if flags[j] else off)["EST_VARS_OK"][j] == 0.0)
                continue
            idx = np.arange(sx.size)
            lhs, rhs, d_cs = envelope.system(itype, sx, sy, idx, cx, cy, vgs[j], mvv, sd, cd)
            sing, _ = envelope.singular_to_pinv(lhs)
            rs = envelope.runs(lhs, rhs, sx.size, z[j][None], d_cs, itype == "OK", k=4,
                               seed=int(i) * 10 + j)
            if not sing:
                n_regular += 1
                de, dv = envelope.spread(rs, scale)
                assert np.nanmax(np.abs(got - want), initial=0.0) \
                    <= max(1e-9, 10 * de) * scale, (i, j, itype, vgs[j])
                if ref_var is not None:
                    gv = on["EST_VARS_OK"][j]
                    vs = max(float(np.abs(ref_var[j]).max()), 1e-300)
                    # the reference stores its variance in float32
                    assert np.abs(gv - ref_var[j]).max() <= max(1e-6, 10 * dv) * vs, (i, j)
            else:
                n_singular += 1
                ok = envelope.consistent(got[None], rs, z[j][None], d_cs, 1e-9 * scale)[0]
                sing_cells += ok.size
                sing_ok += int(ok.sum())
    print(f"\ninterp sweep: {n_regular} regular kriging steps, {n_singular} singular "
          f"({sing_ok} of {sing_cells} cells inside the reference's perturbed outcomes)")
    assert n_regular >= 40
    if sing_cells:
        assert sing_ok >= 0.9 * sing_cells
