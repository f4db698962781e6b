"""Generate golden vectors by running the REFERENCE's own code.

TEST INFRASTRUCTURE. Run only where the reference tree exists::

    python tests/golden/make_golden.py REFERENCE_ROOT

(or with the root in $SPINTERPS_REFERENCE_ROOT)

It loads the unmodified reference (interp/steps.py, interp/grps.py, misc.py
and cyth/interpmthds.pyx compiled by oracle/build_ref.py, see refharness.py)
and writes small seeded cases to tests/golden/*.npz:

- kernels.npz   fill_dists_2d_mat, fill_vg_var_arr (every model, covar and
                diagonal flags, min_vg_val zeroing), fill_wts_and_sum,
                get_mults_sum, copy_2d_arr_at_idxs, check_full_nuggetness
- interp.npz    SpInterpSteps._get_interp for OK (+variance), SK, EDK (1 and 2
                drifts), IDW (several exponents, a cell on a station), NNB,
                one station, flags off, nugget-only variograms, mixed models
- steps.npz     whole multi-step runs with missing stations: the reference's
                _get_interp called per station group by the same loop as
                interp/steps.py:673-835 (that loop needs pandas, which is not
                installed, so its few lines of bookkeeping are restated here)
- nebs.npz      SpInterpNeighborGrouping.get_neb_idxs_and_grps for 'nrst' and
                'pie' (interp/grps.py:103-288, cyth sel_equidist_refs)
- fitter.npz    variograms/vgs.py Variogram: empirical variogram (pairs,
                clipping, equal-count bins, robust estimator), the objective,
                and whole fits with numpy's global RNG seeded
- driver.npz    the driver flow's grid (SpInterpPrepare._prepare_crds,
                interp/prepare.py:148-241) and drift sampling
                (KrigingDrift._prepare_stns_drift, interp/drift.py:165-227),
                plus sweeps of 400 seeded grids (ranges, shapes, digests of
                the coordinate vectors, and where the reference asserts) and
                of 150 drift windows (inputs from sweeps.py, digests of the
                cell and station drifts, the reference's exceptions)
- legacy.npz    the single-neighbourhood classes of cyth/interpmthds.pyx:
                OrdinaryKriging, SimpleKriging, ExternalDriftKriging(_MD),
                OrdinaryIndicatorKriging, SimpleIndicatorKriging
- interp_sweep.npz  SpInterpSteps._get_interp on 80 seeded random one-group
                cases (every model, nests of up to three, all five methods)
- nebs_sweep.npz    SpInterpNeighborGrouping on 60 seeded random station and
                cell sets, 'nrst' and 'pie'
- legacy_sweep.npz  the six single-neighbourhood classes on 48 seeded random
                cases (model nests, drifts, indicator limits)
- vg_edges.npz      fill_vg_var_arr at every model's branch points (h = 0,
                subnormal, the range and its neighbouring doubles, inf)
- empirical_sweep.npz  the Variogram's empirical variogram on 40 seeded random
                station sets (lattices with tied distances, nk, mdr)
- steps_sweep.npz   16 multi-step runs as steps.npz with seeded random settings
                (methods, missingness, thresholds, cut-offs)

``python tests/golden/make_golden.py REFERENCE_ROOT legacy`` writes only
legacy.npz (``driver``, ``interp_sweep``, ``nebs_sweep``, ``legacy_sweep``,
``vg_edges``, ``empirical_sweep``, ``steps_sweep``: only that file).
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
from refharness import (LocFrame, load_prepare, load_reference, load_variogram,  # noqa: E402
                        make_steps)

VG_STRS = [
    "0.05 Nug(0.0) + 0.95 Exp(20000)",
    "1.0 Sph(30000)",
    "0.2 Nug(0.0) + 0.8 Gau(15000)",
    "0.7 Lin(40000)",
    "0.5 Pow(1.2)",
    "1.5 Hol(25000)",
    "0.3 Nug(0.0) + 0.4 Sph(10000) + 0.3 Exp(50000)",
    "2.0 Rng(1.0)",
    "1.0 Exp(0.0)",
]


def grid_cells(x0, y1, cs, nx, ny):
    """Cell centres as interp/prepare.py:193-234 builds them (row-major,
    y descending)."""
    xs = np.linspace(x0 + 0.5 * cs, x0 + 0.5 * cs + (nx - 1) * cs, nx)
    ys = np.linspace(y1 - 0.5 * cs, y1 - 0.5 * cs - (ny - 1) * cs, ny)
    mx, my = np.meshgrid(xs, ys)
    return mx.ravel(), my.ravel()


def grf_values(rng, xs, ys, vg_str, n_steps, mean, ref):
    """Values = mean + GRF with the covariance of ``vg_str`` (Cholesky)."""
    d = np.hypot(xs[:, None] - xs[None], ys[:, None] - ys[None])
    g = ref.misc.get_theo_vg_vals(vg_str, d.ravel()).reshape(d.shape)
    sill = sum(float(p.strip().split(" ")[0]) for p in vg_str.split("+"))
    c = sill - g
    c[np.diag_indices_from(c)] = sill
    ll = np.linalg.cholesky(c + 1e-10 * np.eye(c.shape[0]))
    return mean + (ll @ rng.standard_normal((xs.size, n_steps))).T


def kernels_case(ref, out):
    cy = ref.cy
    rng = np.random.default_rng(11)
    n, c = 23, 41
    sx, sy = rng.uniform(0, 1e5, n), rng.uniform(0, 1e5, n)
    cx, cy_ = rng.uniform(0, 1e5, c), rng.uniform(0, 1e5, c)
    cx[:3], cy_[:3] = sx[:3], sy[:3]  # cells on stations: zero distances
    d_cs = np.full((c, n), np.nan)
    cy.fill_dists_2d_mat(cx, cy_, sx, sy, d_cs)
    d_ss = np.full((n, n), np.nan)
    cy.fill_dists_2d_mat(sx, sy, sx, sy, d_ss)
    out.update(k_sx=sx, k_sy=sy, k_cx=cx, k_cy=cy_, k_d_cs=d_cs, k_d_ss=d_ss)
    out["k_vgs"] = np.array(VG_STRS)
    for vi, vg in enumerate(VG_STRS):
        for covar in (0, 1):
            for mvv in (0.0, 1e-4, 0.05):
                a = np.full_like(d_ss, np.nan)
                cy.fill_vg_var_arr(d_ss, a, covar, 1, vg, mvv)
                b = np.full_like(d_cs, np.nan)
                cy.fill_vg_var_arr(d_cs, b, covar, 0, vg, mvv)
                out[f"k_vg_ss_{vi}_{covar}_{mvv:g}"] = a
                out[f"k_vg_cs_{vi}_{covar}_{mvv:g}"] = b
    # IDW primitives on one row of distances
    for e in (1.0, 2.0, 3.5):
        dist = d_cs[5].copy() / d_cs[5].max()
        w = np.full(n, np.nan)
        s = cy.fill_wts_and_sum(dist, w, e)
        z = rng.normal(size=n)
        out[f"k_idw_w_{e:g}"] = w
        out[f"k_idw_s_{e:g}"] = np.array(s)
        out[f"k_idw_z_{e:g}"] = z
        out[f"k_idw_m_{e:g}"] = np.array(cy.get_mults_sum(w, z))
    ri = np.array([4, 0, 17, 3], dtype=np.int64)
    ci = np.array([22, 1, 5], dtype=np.int64)
    sub = np.full((ri.size + 2, ci.size + 1), np.nan)
    cy.copy_2d_arr_at_idxs(d_cs, ri, ci, sub)
    out.update(k_copy_ri=ri, k_copy_ci=ci, k_copy_sub=sub)
    nug_cases = VG_STRS + ["1.0 Nug(0.0)", "0.00001 Exp(1000)", "1.0 Exp(0.00001)",
                           "0.5 Nug(0.0) + 0.5 Nug(0.0)"]
    out["k_nug_strs"] = np.array(nug_cases)
    out["k_nug_1e-4"] = np.array(
        [ref.misc.check_full_nuggetness(s, 1e-4) for s in nug_cases])
    out["k_nug_0"] = np.array([ref.misc.check_full_nuggetness(s, 0.0) for s in nug_cases])


VG_EDGE_STRS = [
    "1.0 Nug(0.0)", "0.7 Sph(1000.0)", "1.3 Exp(2500.5)", "0.4 Lin(777.0)", "2.0 Gau(3000.0)",
    "0.5 Pow(0.5)", "0.5 Pow(1.0)", "0.5 Pow(1.9)", "1.5 Hol(1200.0)", "2.0 Rng(1.0)",
    "1.0 Sph(1e-07)", "1.0 Exp(0.0)", "0.2 Nug(0.0) + 0.5 Sph(1000.0) + 0.3 Lin(777.0)",
]


def vg_edges(ref, out):
    """fill_vg_var_arr at the models' branch points: for each string, the
    distances 0, the smallest subnormal, each component's range and its two
    neighbouring doubles, half and twice the range, 1e300 and inf; covariance
    and semivariance, min_vg_val 0 and 0.05, as a row (diag flag 0) and as a
    symmetric square of the same values (diag flag 1)."""
    cy = ref.cy
    for vi, vg in enumerate(VG_EDGE_STRS):
        rs = []
        for part in vg.split("+"):
            r = max(1e-5, float(part.strip().split("(")[1].split(")")[0]))
            rs += [r, np.nextafter(r, 0.0), np.nextafter(r, np.inf), 0.5 * r, 2.0 * r]
        h = np.array([0.0, 5e-324, *rs, 1e300, np.inf])
        row = h[None, :].copy()
        with np.errstate(invalid="ignore"):  # inf - inf
            sq = np.abs(h[:, None] - h[None, :])
        sq[~np.isfinite(sq)] = np.inf
        out[f"ve_h_{vi}"] = h
        for covar in (0, 1):
            for mvv in (0.0, 0.05):
                a = np.full_like(row, np.nan)
                cy.fill_vg_var_arr(row, a, covar, 0, vg, mvv)
                b = np.full_like(sq, np.nan)
                cy.fill_vg_var_arr(sq, b, covar, 1, vg, mvv)
                out[f"ve_row_{vi}_{covar}_{mvv:g}"] = a
                out[f"ve_sq_{vi}_{covar}_{mvv:g}"] = b
    out["ve_vgs"] = np.array(VG_EDGE_STRS)


def interp_one(ref, st, sx, sy, cx, cy, z, itype, vgs, *, idw_exp=5.0,
               flags=None, nug=None, drifts=None, cell_drifts=None, mvv=1e-4):
    """One _get_interp call over all stations/cells (one group)."""
    n, c, t = sx.size, cx.size, z.shape[0]
    d_cs = st._get_dists_arr(cx, cy, sx, sy)
    d_ss = st._get_dists_arr(sx, sy, sx, sy)
    uv = list(dict.fromkeys(vgs))
    rr = st._get_svars_arr(d_ss, uv, [itype], 1) if itype in ("OK", "SK", "EDK") else None
    dr = st._get_svars_arr(d_cs, uv, [itype], 0) if itype in ("OK", "SK", "EDK") else None
    if flags is None:
        flags = np.ones(t, dtype=bool)
    if nug is None:
        nug = np.array([ref.misc.check_full_nuggetness(v, mvv) for v in vgs])
    prblm = []
    est, var = st._get_interp(
        z.copy("c"), itype, drifts, cell_drifts, idw_exp, np.array(vgs, dtype=object),
        flags, nug, np.arange(t), prblm, d_cs.copy(), rr, dr, np.arange(n),
        np.arange(c))
    return est, var, prblm


def interp_case(ref, out):
    rng = np.random.default_rng(22)
    n, t = 31, 5
    sx, sy = rng.uniform(0, 1e5, n), rng.uniform(0, 1e5, n)
    cx, cy = grid_cells(0.0, 1e5, 5000.0, 20, 20)
    cx = cx.copy()
    cy = cy.copy()
    vg0 = "0.05 Nug(0.0) + 0.95 Exp(20000)"
    z = grf_values(rng, sx, sy, vg0, t, 5.0, ref)
    out.update(i_sx=sx, i_sy=sy, i_cx=cx, i_cy=cy, i_z=z)
    vgs_mixed = [vg0, "1.0 Sph(30000)", vg0, "0.2 Nug(0.0) + 0.8 Gau(15000)", "1.0 Nug(0.0)"]
    out["i_vgs_mixed"] = np.array(vgs_mixed)
    flags = np.array([True, True, False, True, True])
    out["i_flags"] = flags
    st = make_steps(ref, min_vg_val=1e-4, est_vars=True)
    for itype in ("OK", "SK"):
        est, var, prblm = interp_one(ref, st, sx, sy, cx, cy, z, itype, vgs_mixed, flags=flags)
        out[f"i_{itype}_est"] = est
        if var is not None:
            out[f"i_{itype}_var"] = var
    # models exercising Lin / Pow / Hol / three components on OK
    vgs_other = ["0.7 Lin(40000)", "0.5 Pow(1.2)", "1.5 Hol(25000)",
                 "0.3 Nug(0.0) + 0.4 Sph(10000) + 0.3 Exp(50000)", vg0]
    out["i_vgs_other"] = np.array(vgs_other)
    est, var, _ = interp_one(ref, st, sx, sy, cx, cy, z, "OK", vgs_other)
    out["i_OKo_est"] = est
    out["i_OKo_var"] = var
    # EDK with one and two drifts
    elev = 1000 + 5e-3 * sx + 3e-3 * sy + rng.normal(0, 20, n)
    cel = 1000 + 5e-3 * cx + 3e-3 * cy
    for k in (1, 2):
        sd = np.stack([elev, sx / 1e3], 1)[:, :k].copy()
        cd = np.stack([cel, cx / 1e3], 0)[:k].copy()
        est, _, _ = interp_one(ref, st, sx, sy, cx, cy, z + 1e-3 * elev, "EDK",
                               vgs_mixed, flags=flags, drifts=sd, cell_drifts=cd)
        out[f"i_EDK{k}_est"] = est
        out[f"i_EDK{k}_sd"] = sd
        out[f"i_EDK{k}_cd"] = cd
    # IDW with several exponents; cell 0 moved onto station 0 -> NaN
    cx2, cy2 = cx.copy(), cy.copy()
    cx2[0], cy2[0] = sx[0], sy[0]
    out.update(i_cx2=cx2, i_cy2=cy2)
    for e in (1.0, 2.0, 3.5):
        est, _, _ = interp_one(ref, st, sx, sy, cx2, cy2, z, "IDW", [vg0] * t,
                               idw_exp=e, flags=flags)
        out[f"i_IDW_{e:g}_est"] = est
    est, _, _ = interp_one(ref, st, sx, sy, cx2, cy2, z, "NNB", [vg0] * t)
    out["i_NNB_est"] = est
    # a single station
    est, var, _ = interp_one(ref, st, sx[:1], sy[:1], cx, cy, z[:, :1], "OK", [vg0] * t)
    out["i_one_est"] = est
    out["i_one_var"] = var


def steps_case(ref, out, tag, *, n, t, nx, ny, cs, box, p_miss, vgs, methods,
               seed, min_var_thr=0.0, min_var_cut=None, max_var_cut=None,
               mvv=1e-4, edk=False):
    """A multi-step run: per station group, the reference's _get_interp for
    every method, clipped by _mod_min_max and cast to float32 as in
    interp/steps.py:673-835."""
    rng = np.random.default_rng(seed)
    sx, sy = rng.uniform(0, box, n), rng.uniform(0, box, n)
    cx, cy = grid_cells(0.0, box, cs, nx, ny)
    z = grf_values(rng, sx, sy, "0.1 Nug(0.0) + 0.9 Sph(40000)", t, 3.0, ref)
    if p_miss > 0:
        miss = rng.uniform(size=(t, n)) < p_miss
        z[miss] = np.nan
        z[2, :] = np.nan            # one step without any station
        z[3, :] = np.nan
        z[3, 4] = 1.25              # one step with a single station
        z[5, :] = z[4, :]           # two steps sharing a station set
    z[1, np.isfinite(z[1])] = -1.0  # a step under min_var_thr (flags off)
    sd = cd = None
    if edk:
        sd = (100 + 2e-3 * sx + rng.normal(0, 5, n))[:, None].copy()
        cd = (100 + 2e-3 * cx)[None].copy()
    st = make_steps(ref, min_vg_val=mvv, est_vars=True, min_var_thr=min_var_thr,
                    min_var_cut=min_var_cut, max_var_cut=max_var_cut)
    d_cs = st._get_dists_arr(cx, cy, sx, sy)
    d_ss = st._get_dists_arr(sx, sy, sx, sy)
    types = [m if isinstance(m, str) else m[0] for m in methods]
    uv = list(dict.fromkeys(vgs))
    rr = st._get_svars_arr(d_ss, uv, types, 1)
    dr = st._get_svars_arr(d_cs, uv, types, 0)
    labels = []
    for m in methods:
        if isinstance(m, tuple):
            labels.append(f"IDW_{sum(1 for l in labels if l.startswith('IDW')):03d}")
        else:
            labels.append(m)
    flds = {lab: np.full((t, cx.size), np.nan, dtype=np.float32) for lab in labels}
    flds["EST_VARS_OK"] = np.full((t, cx.size), np.nan, dtype=np.float32)
    avail = np.isfinite(z)
    keys = [avail[i].tobytes() for i in range(t)]
    done = set()
    prblm = []
    vgs_arr = np.array(vgs, dtype=object)
    for i0 in range(t):
        if keys[i0] in done:
            continue
        done.add(keys[i0])
        mask = np.array([k == keys[i0] for k in keys])
        stn = np.where(avail[i0])[0]
        if not stn.size:
            prblm.extend(np.where(mask)[0].tolist())
            continue
        vals = z[mask][:, stn].copy("c")
        flags = np.array([np.any(v >= min_var_thr) for v in vals])
        nug = np.array([ref.misc.check_full_nuggetness(v, mvv) for v in vgs_arr[mask]])
        dsub = st._get_2d_arr_subset(d_cs, np.arange(cx.size), stn, 0, 0)
        tid = np.where(mask)[0]
        for m, lab in zip(methods, labels):
            itype = m if isinstance(m, str) else m[0]
            e = m[1] if isinstance(m, tuple) else 5
            est, var = st._get_interp(
                vals, itype, sd[stn] if edk else None, cd if edk else None, e,
                vgs_arr[mask], flags, nug, tid, prblm, dsub, rr, dr, stn,
                np.arange(cx.size))
            st._mod_min_max(est)
            for j, ti in enumerate(tid):
                flds[lab][ti] = est[j].astype(np.float32)
                if itype == "OK":
                    flds["EST_VARS_OK"][ti] = var[j]
    out[f"s_{tag}_sx"] = sx
    out[f"s_{tag}_sy"] = sy
    out[f"s_{tag}_cx"] = cx
    out[f"s_{tag}_cy"] = cy
    out[f"s_{tag}_z"] = z
    out[f"s_{tag}_vgs"] = np.array(vgs)
    out[f"s_{tag}_methods"] = np.array([m if isinstance(m, str) else f"IDW:{m[1]}"
                                        for m in methods])
    out[f"s_{tag}_params"] = np.array(
        [min_var_thr, np.nan if min_var_cut is None else min_var_cut,
         np.nan if max_var_cut is None else max_var_cut, mvv])
    if edk:
        out[f"s_{tag}_sd"] = sd
        out[f"s_{tag}_cd"] = cd
    out[f"s_{tag}_prblm"] = np.array(sorted(set(prblm)), dtype=np.int64)
    for lab, f in flds.items():
        out[f"s_{tag}_out_{lab}"] = f


STEPS_SWEEP_VGS = ["0.05 Nug(0.0) + 0.95 Exp(20000)", "1.0 Sph(30000)",
                   "0.2 Nug(0.0) + 0.8 Gau(15000)", "1.0 Nug(0.0)", "0.7 Lin(40000)",
                   "0.1 Nug(0.0) + 0.5 Exp(8000) + 0.4 Sph(50000)"]


def steps_sweep(ref, out, n_cases=16, seed=1010):
    """steps_case with seeded random settings: 8 to 40 stations, 6 to 10
    steps, grids of 4 to 10 cells a side, missingness 0 to 0.35, per-step
    variograms from STEPS_SWEEP_VGS (nugget-only steps among them), a random
    subset of OK / SK / EDK / IDW (one or two exponents) / NNB, min_var_thr
    and both cut-offs on or off."""
    rng = np.random.default_rng(seed)
    tags = []
    for i in range(n_cases):
        n, t = int(rng.integers(8, 41)), int(rng.integers(6, 11))
        nx, ny = int(rng.integers(4, 11)), int(rng.integers(4, 11))
        box = float(rng.uniform(3e4, 1.5e5))
        methods = [m for m in ("OK", "SK", "EDK") if rng.uniform() < 0.5]
        for e in rng.choice([0.5, 1.0, 2.0, 3.0], int(rng.integers(0, 3)), replace=False):
            methods.append(("IDW", float(e)))
        if rng.uniform() < 0.4 or not methods:
            methods.append("NNB")
        vgs = [STEPS_SWEEP_VGS[k] for k in rng.integers(len(STEPS_SWEEP_VGS), size=t)]
        thr = float(rng.choice([0.0, 0.5, 3.0]))
        mn = float(rng.choice([0.0, 1.0])) if rng.uniform() < 0.5 else None
        mx = float(rng.choice([4.0, 6.0])) if rng.uniform() < 0.5 else None
        tag = f"sw{i}"
        steps_case(ref, out, tag, n=n, t=t, nx=nx, ny=ny, cs=box / max(nx, ny), box=box,
                   p_miss=float(rng.choice([0.0, 0.15, 0.35])), vgs=vgs, methods=methods,
                   seed=int(rng.integers(1 << 30)), min_var_thr=thr, min_var_cut=mn,
                   max_var_cut=mx, edk="EDK" in methods)
        tags.append(tag)
    out["ss_tags"] = np.array(tags)


class _NumpyLLP64:
    """numpy with ``uint32`` mapped to ``uint64``.

    interp/grps.py:176-178 allocates ``np.uint32`` buffers for arguments that
    cyth/interpmthds.pyx:811-823 types as ``unsigned long``. That matches on
    the reference author's Windows (LLP64, 32-bit long) but raises a buffer
    dtype error on Linux (LP64). Running the reference's own module with this
    shim as its ``np`` reproduces what it computes where it works."""

    def __getattr__(self, item):
        if item == "uint32":
            return np.uint64
        return getattr(np, item)


def nebs_case(ref, out):
    ref.grps.np = _NumpyLLP64()
    rng = np.random.default_rng(33)
    n = 40
    sx, sy = rng.uniform(0, 5e4, n), rng.uniform(0, 5e4, n)
    cx, cy = grid_cells(0.0, 5e4, 2500.0, 20, 20)
    out.update(n_sx=sx, n_sy=sy, n_cx=cx, n_cy=cy)
    for mth, nn, npie in (("nrst", 8, 1), ("pie", 8, 4), ("pie", 12, 6)):
        g = ref.grps.SpInterpNeighborGrouping(mth, nn, npie, cx.copy(), cy.copy(),
                                              verbose=False)
        idxs, grps = g.get_neb_idxs_and_grps(sx.copy(), sy.copy())
        tag = f"{mth}_{nn}_{npie}"
        out[f"n_{tag}_idxs"] = idxs.astype(np.int64)
        lab = np.full(cx.size, -1, dtype=np.int64)
        for gi, gr in enumerate(grps):
            lab[gr] = gi
        out[f"n_{tag}_grp"] = lab


def nebs_sweep(ref, out, n_cases=60, seed=707):
    """SpInterpNeighborGrouping.get_neb_idxs_and_grps over seeded random
    station and cell sets (3 to 50 stations, 5 to 60 cells, some cells on
    stations), 'nrst' with 1 to 16 neighbours and 'pie' with 1 to 8 sectors.
    Stored: the inputs, the neighbour lists and the cell groups (int16)."""
    ref.grps.np = _NumpyLLP64()
    rng = np.random.default_rng(seed)
    for i in range(n_cases):
        n, c = int(rng.integers(3, 51)), int(rng.integers(5, 61))
        box = float(rng.uniform(1e3, 1e5))
        sx, sy = rng.uniform(0, box, n), rng.uniform(0, box, n)
        cx, cy = rng.uniform(0, box, c), rng.uniform(0, box, c)
        on = int(rng.integers(0, 3))
        cx[:on], cy[:on] = sx[:on], sy[:on]
        if i % 2 == 0:
            mth, npie = "nrst", 1
            nn = int(rng.integers(1, min(16, n) + 1))
        else:
            mth = "pie"
            npie = int(rng.integers(1, min(8, n) + 1))
            nn = int(rng.integers(npie, min(16, n) + 1))
        g = ref.grps.SpInterpNeighborGrouping(mth, nn, npie, cx.copy(), cy.copy(),
                                              verbose=False)
        idxs, grps = g.get_neb_idxs_and_grps(sx.copy(), sy.copy())
        lab = np.full(c, -1, dtype=np.int16)
        for gi, gr in enumerate(grps):
            lab[gr] = gi
        p = f"ns{i}_"
        out.update({p + "sx": sx, p + "sy": sy, p + "cx": cx, p + "cy": cy,
                    p + "cfg": np.array([0 if mth == "nrst" else 1, nn, npie]),
                    p + "idxs": idxs.astype(np.int16), p + "grp": lab})
    out["ns_cases"] = np.arange(n_cases)


def empirical_sweep(ref_root, out, n_cases=40, seed=909):
    """The reference Variogram's empirical variogram (_max_dist_est and
    _vg_var_raw, variograms/vgs.py:320-520, 597-659) on seeded random
    station sets: 5 to 80 stations, a third of them on a lattice (many tied
    distances), nk 10 / 25 / 50, mdr 0.3 to 1.0. Stored: the inputs, the bin
    distances, the robust semivariances, the pair counts, the max distance."""
    vgs_mod = load_variogram(ref_root)
    rng = np.random.default_rng(seed)
    for i in range(n_cases):
        n = int(rng.integers(5, 81))
        box = float(rng.uniform(1e3, 1e5))
        if i % 3 == 0:
            m = int(np.ceil(np.sqrt(n))) + 1
            pts = rng.choice(m * m, n, replace=False)
            x, y = (pts % m) * box / m, (pts // m) * box / m
        else:
            x, y = rng.uniform(0, box, n), rng.uniform(0, box, n)
        z = rng.gamma(1.2, 2.0, n)
        nk = int(rng.choice([10, 25, 50]))
        mdr = float(rng.choice([0.3, 0.5, 0.7, 1.0]))
        v = vgs_mod.Variogram(x=x, y=y, z=z, mdr=mdr, nk=nk, typ="var", perm_r_list=[1, 2],
                              fil_nug_vg="Nug", ld=None, uh=None, h_itrs=100,
                              opt_meth="L-BFGS-B", opt_iters=10000, fit_vgs=["Sph", "Exp"],
                              n_best=1, evg_name="robust", use_wts=False, ngp=5,
                              fit_thresh=0.01)
        v._max_dist_est()
        v._vg_var_raw()
        p = f"fe{i}_"
        out.update({p + "x": x, p + "y": y, p + "z": z, p + "nk": np.array(nk),
                    p + "mdr": np.array(mdr), p + "h": v.vg_h_arr.copy(),
                    p + "g": v.vg_vg_arr.copy(), p + "np": v.pairs_no.copy(),
                    p + "maxd": np.array(v.max_dist)})
    out["fe_cases"] = np.arange(n_cases)


def fitter_case(ref_root, out):
    """variograms/vgs.py: empirical variogram, objective and fit, with the
    settings FitVariogramsSteps passes (variograms/fitvgs.py:187-206) and the
    reference test driver's choices (test/test_fitvgs.py:125-131: mdr 0.7,
    perm_r_list [1, 2], fit_vgs Sph/Exp, nugget 'Nug', n_best 1) and nk 50
    (variograms/vgsinput.py:207). DE draws from numpy's global RNG (the
    reference passes no seed), so seeding it makes the fit reproducible."""
    vgs_mod = load_variogram(ref_root)
    rng = np.random.default_rng(66)
    cases = []
    for ci, (n, vg, box) in enumerate(((40, "0.1 Nug(0.0) + 0.9 Exp(15000)", 6e4),
                                       (90, "0.2 Nug(0.0) + 1.3 Sph(40000)", 1.2e5),
                                       (150, "1.0 Gau(20000)", 1e5))):
        x, y = rng.uniform(0, box, n), rng.uniform(0, box, n)
        d = np.hypot(x[:, None] - x[None], y[:, None] - y[None])
        # covariance of the generating model (semivariogram -> covariance)
        comps = [(float(p.split()[0]), p.split()[1].split("(")[0], float(p.split("(")[1][:-1]))
                 for p in (q.strip() for q in vg.split("+"))]
        cov = np.zeros_like(d)
        for s, name, r in comps:
            if name == "Nug":
                cov += s * (d == 0)
            elif name == "Exp":
                cov += s * np.exp(-3 * d / r)
            elif name == "Gau":
                cov += s * np.exp(-3 * (d / r) ** 2)
            elif name == "Sph":
                t = np.minimum(d / r, 1.0)
                cov += s * (1 - 1.5 * t + 0.5 * t ** 3)
        z = np.linalg.cholesky(cov + 1e-8 * np.eye(n)) @ rng.standard_normal(n)
        v = vgs_mod.Variogram(x=x, y=y, z=z, mdr=0.7, nk=50, typ="var", perm_r_list=[1, 2],
                              fil_nug_vg="Nug", ld=None, uh=None, h_itrs=100,
                              opt_meth="L-BFGS-B", opt_iters=10000, fit_vgs=["Sph", "Exp"],
                              n_best=1, evg_name="robust", use_wts=False, ngp=5,
                              fit_thresh=0.01)
        v._max_dist_est()
        v._vg_var_raw()
        out[f"f{ci}_x"], out[f"f{ci}_y"], out[f"f{ci}_z"] = x, y, z
        out[f"f{ci}_h"] = v.vg_h_arr.copy()
        out[f"f{ci}_g"] = v.vg_vg_arr.copy()
        out[f"f{ci}_np"] = v.pairs_no.copy()
        out[f"f{ci}_maxd"] = np.array(v.max_dist)
        # objective at a few parameter sets
        prm = np.array([[v.vg_h_arr[0], v.vg_vg_arr[0], 2e4, 0.7],
                        [v.vg_h_arr[0], v.vg_vg_arr[0], 5e4, 1.2]])
        objs = []
        for p4 in prm:
            objs.append(v._vg_calib(p4[2:], ("Sph", v.sph_vg)))
            objs.append(v._vg_calib(p4[2:], ("Exp", v.exp_vg)))
            objs.append(v._vg_calib(p4, ("Nug", v.nug_vg), ("Exp", v.exp_vg)))
        out[f"f{ci}_prm"] = prm
        out[f"f{ci}_obj"] = np.array(objs)
        # a full fit with numpy's global RNG seeded
        v2 = vgs_mod.Variogram(x=x, y=y, z=z, mdr=0.7, nk=50, typ="var", perm_r_list=[1, 2],
                               fil_nug_vg="Nug", ld=None, uh=None, h_itrs=100,
                               opt_meth="L-BFGS-B", opt_iters=10000, fit_vgs=["Sph", "Exp"],
                               n_best=1, evg_name="robust", use_wts=False, ngp=5,
                               fit_thresh=0.01)
        np.random.seed(1000 + ci)
        v2.fit()
        out[f"f{ci}_vgstr"] = np.array(v2.vg_str_list)
        out[f"f{ci}_bestobj"] = np.array(v2.n_best_objs)
        out[f"f{ci}_bestprm"] = np.array(v2.best_vg_params[-1])
        cases.append(ci)
    out["f_cases"] = np.array(cases)


LEGACY_CASES = [
    # (class, model, n stations, n points, n drifts, seed)
    ("OrdinaryKriging", "0.1 Nug(0.0) + 0.9 Exp(20000)", 12, 15, 0, 71),
    ("OrdinaryKriging", "0.5 Pow(1.2)", 10, 9, 0, 72),
    ("OrdinaryKriging", "1.5 Hol(25000) + 0.2 Lin(40000)", 14, 11, 0, 73),
    ("SimpleKriging", "0.2 Nug(0.0) + 1.0 Sph(30000)", 12, 15, 0, 74),
    ("SimpleKriging", "1.0 Exp(15000)", 9, 8, 0, 75),
    ("ExternalDriftKriging", "1.0 Gau(25000)", 11, 10, 1, 76),
    ("ExternalDriftKriging_MD", "0.1 Nug(0.0) + 0.5 Exp(10000) + 0.4 Sph(40000)", 16, 13, 2,
     77),
    ("ExternalDriftKriging_MD", "1.0 Sph(35000)", 13, 12, 3, 78),
    ("OrdinaryIndicatorKriging", "0.1 Nug(0.0) + 0.9 Exp(20000)", 12, 15, 0, 79),
    ("SimpleIndicatorKriging", "1.0 Exp(15000)", 12, 10, 0, 80),
    # a duplicated station: exactly singular matrices (pinv's cut-off acts)
    ("OrdinaryKriging", "1.0 Exp(20000)", 12, 9, 0, 81),
    ("SimpleKriging", "0.3 Nug(0.0) + 0.7 Sph(30000)", 12, 9, 0, 82),
]
LEGACY_DUPLICATED = (10, 11)


def legacy_case(ref, out):
    """The classes of cyth/interpmthds.pyx:251-765, each on small seeded
    inputs with one output point on a station. Every readonly array the
    class exposes after krige()/ikrige() is stored."""
    cy = ref.cy
    for ci, (cls, model, n, n_out, n_drift, seed) in enumerate(LEGACY_CASES):
        rng = np.random.default_rng(seed)
        xi, yi = rng.uniform(0, 6e4, n), rng.uniform(0, 6e4, n)
        if ci in LEGACY_DUPLICATED:
            xi[5], yi[5] = xi[1], yi[1]
        zi = rng.gamma(1.5, 2.0, n)
        xk, yk = rng.uniform(0, 6e4, n_out), rng.uniform(0, 6e4, n_out)
        xk[0], yk[0] = xi[3], yi[3]
        si = rng.uniform(0, 1500, (n_drift, n))
        sk = rng.uniform(0, 1500, (n_drift, n_out))
        lim = float(np.median(zi))
        if cls in ("OrdinaryKriging", "SimpleKriging"):
            obj = getattr(cy, cls)(xi, yi, zi, xk, yk, model=model)
            obj.krige()
        elif cls == "ExternalDriftKriging":
            obj = cy.ExternalDriftKriging(xi, yi, zi, si[0].copy(), xk, yk, sk[0].copy(),
                                          model=model)
            obj.krige()
        elif cls == "ExternalDriftKriging_MD":
            obj = cy.ExternalDriftKriging_MD(xi, yi, zi, si, xk, yk, sk, model=model)
            obj.krige()
        else:
            obj = getattr(cy, cls)(xi, yi, zi, xk, yk, lim=lim, model=model)
            obj.ikrige()
        p = f"l{ci}_"
        out.update({p + "xi": xi, p + "yi": yi, p + "zi": zi, p + "xk": xk, p + "yk": yk,
                    p + "si": si, p + "sk": sk, p + "lim": np.array(lim),
                    p + "model": np.array(model), p + "cls": np.array(cls)})
        for attr in ("zk", "est_vars", "est_covars", "mus", "mus_1", "mus_2", "mus_arr",
                     "lambdas", "rhss", "in_dists", "in_vars", "in_vars_inv", "in_covars",
                     "in_covars_inv", "out_covars", "ik", "ixi"):
            if hasattr(obj, attr) and getattr(obj, attr) is not None:
                out[p + attr] = np.asarray(getattr(obj, attr)).copy()
    out["l_cases"] = np.arange(len(LEGACY_CASES))


LEGACY_CLASSES = ["OrdinaryKriging", "SimpleKriging", "ExternalDriftKriging",
                  "ExternalDriftKriging_MD", "OrdinaryIndicatorKriging",
                  "SimpleIndicatorKriging"]
LEGACY_SWEEP_OUT = ("zk", "est_vars", "est_covars", "mus", "mus_1", "mus_2", "mus_arr",
                    "lambdas", "ik")


def legacy_sweep(ref, out, n_cases=48, seed=808):
    """The six classes in turn on seeded random cases: 3 to 16 stations, 1 to
    16 output points (one on a station), nests of 1 to 3 of the eight
    models, 1 to 3 drifts for ExternalDriftKriging_MD, the median as the
    indicator limit. Stored: the inputs and the outputs callers read
    (estimates, variances, multipliers, weights, indicators)."""
    cy = ref.cy
    rng = np.random.default_rng(seed)
    for i in range(n_cases):
        cls = LEGACY_CLASSES[i % len(LEGACY_CLASSES)]
        n, n_out = int(rng.integers(3, 17)), int(rng.integers(1, 17))
        box = float(rng.uniform(1e3, 1e5))
        xi, yi = rng.uniform(0, box, n), rng.uniform(0, box, n)
        zi = rng.gamma(1.5, 2.0, n)
        xk, yk = rng.uniform(0, box, n_out), rng.uniform(0, box, n_out)
        xk[0], yk[0] = xi[1], yi[1]
        comps = []
        for _ in range(int(rng.integers(1, 4))):
            nm = SWEEP_MODELS[rng.integers(len(SWEEP_MODELS))]
            sill = round(float(rng.uniform(0.05, 2.0)), 4)
            r = (0.0 if nm == "Nug" else round(float(rng.uniform(0.1, 1.9)), 3) if nm == "Pow"
                 else round(float(rng.uniform(0.05, 1.0)) * box, 1))
            comps.append(f"{sill} {nm}({r})")
        model = " + ".join(comps)
        n_drift = int(rng.integers(1, 4)) if cls == "ExternalDriftKriging_MD" else (
            1 if cls == "ExternalDriftKriging" else 0)
        si = rng.uniform(0, 1500, (n_drift, n))
        sk = rng.uniform(0, 1500, (n_drift, n_out))
        lim = float(np.median(zi))
        if cls in ("OrdinaryKriging", "SimpleKriging"):
            obj = getattr(cy, cls)(xi, yi, zi, xk, yk, model=model)
            obj.krige()
        elif cls == "ExternalDriftKriging":
            obj = cy.ExternalDriftKriging(xi, yi, zi, si[0].copy(), xk, yk, sk[0].copy(),
                                          model=model)
            obj.krige()
        elif cls == "ExternalDriftKriging_MD":
            obj = cy.ExternalDriftKriging_MD(xi, yi, zi, si, xk, yk, sk, model=model)
            obj.krige()
        else:
            obj = getattr(cy, cls)(xi, yi, zi, xk, yk, lim=lim, model=model)
            obj.ikrige()
        p = f"ls{i}_"
        out.update({p + "xi": xi, p + "yi": yi, p + "zi": zi, p + "xk": xk, p + "yk": yk,
                    p + "si": si, p + "sk": sk, p + "lim": np.array(lim),
                    p + "model": np.array(model), p + "cls": np.array(cls)})
        for attr in LEGACY_SWEEP_OUT:
            if hasattr(obj, attr) and getattr(obj, attr) is not None:
                out[p + attr] = np.asarray(getattr(obj, attr)).copy()
    out["ls_cases"] = np.arange(n_cases)


DRIVER_CASES = [
    # (edk, x_min, x_max, y_min, y_max, cell size, polygon mask)
    (False, 1000.3, 26110.0, -5000.0, 14321.7, 500.0, False),
    (True, 3120.0, 41200.5, 2000.0, 30750.0, 1000.0, False),
    (True, 3120.0, 41200.5, 2000.0, 30750.0, 1000.0, True),
]


def driver_case(ref, out):
    """SpInterpPrepare._prepare_crds and KrigingDrift._prepare_stns_drift on a
    bare object with the attributes they read: a grid without drift, and
    with two drift rasters (no-data cells included), with and without a cell
    mask."""
    prep = load_prepare()
    rng = np.random.default_rng(88)
    for ci, (edk, x0, x1, y0, y1, cs, masked) in enumerate(DRIVER_CASES):
        obj = prep.SpInterpPrepare.__new__(prep.SpInterpPrepare)
        obj._edk_flag = edk
        obj._x_min, obj._x_max, obj._y_min, obj._y_max = x0, x1, y0, y1
        obj._cell_size = cs
        obj._plot_figs_flag = False
        p = f"d{ci}_"
        if edk:
            dx0, dy1, nr, nc_ = 0.0, 40000.0, 45, 50
            obj._drft_x_min, obj._drft_y_max = dx0, dy1
            obj._drft_x_max = dx0 + nc_ * cs
            obj._drft_y_min = dy1 - nr * cs
            ndv = -9999.0
            rasters = rng.uniform(0, 3000, (2, nr, nc_))
            rasters[0, 30:, :4] = ndv
            rasters[1, :3, 40:] = ndv
            obj._drft_oarrs = [r.copy() for r in rasters]
            obj._drft_ndv = ndv
            out.update({p + "drift": rasters, p + "ndv": np.array(ndv),
                        p + "drift_origin": np.array([dx0, dy1])})
        obj._prepare_crds()
        out.update({p + "bounds": np.array([x0, x1, y0, y1, cs]),
                    p + "rc": np.array([obj._min_col, obj._max_col, obj._min_row,
                                        obj._max_row]),
                    p + "x_crds": obj._nc_x_crds, p + "y_crds": obj._nc_y_crds,
                    p + "cell_x": obj._interp_x_crds_msh, p + "cell_y": obj._interp_y_crds_msh,
                    p + "shape": np.array(obj._interp_crds_orig_shape)})
        if edk:
            n = 30
            sx = rng.uniform(x0 + 1, x1 - 1, n)
            sy = rng.uniform(y0 + 1, y1 - 1, n)
            obj._crds_df = LocFrame({"X": sx, "Y": sy}, index=np.array(
                [f"s{i}" for i in range(n)]))
            obj._cell_sel_prms_set = masked
            mask = None
            if masked:
                mask = rng.uniform(size=obj._interp_x_crds_msh.size) < 0.6
            obj._cntn_idxs = mask
            obj._prepare_stns_drift()
            out.update({p + "stn_x": sx, p + "stn_y": sy,
                        p + "cell_drift": obj._drft_arrs,
                        p + "stn_drift": obj._stns_drft_df.values.copy()})
            if masked:
                out[p + "mask"] = mask
    out["d_cases"] = np.arange(len(DRIVER_CASES))
    driver_sweep(prep, out)


def driver_sweep(prep, out, n_cases=400, seed=404):
    """SpInterpPrepare._prepare_crds over seeded random extents and cell
    sizes, half of them inside drift rasters (EDK), some with the grid
    reaching outside the rasters (the reference asserts). Stored compactly:
    the inputs, whether the reference raised, the row / column range, the
    shape and SHA-256 digests of the x and y coordinate vectors."""
    import hashlib
    rng = np.random.default_rng(seed)
    sizes = [0.5, 1.0, 25.0, 100.0, 250.0, 333.3, 500.0, 1000.0, 1234.567]
    params = np.zeros((n_cases, 10))
    raised = np.zeros(n_cases, dtype=bool)
    rcs = np.full((n_cases, 4), -1, dtype=np.int64)
    shapes = np.zeros((n_cases, 2), dtype=np.int64)
    digests = np.zeros((n_cases, 2, 32), dtype=np.uint8)
    for i in range(n_cases):
        cs = float(sizes[rng.integers(len(sizes))])
        x0 = round(float(rng.uniform(-2e5, 2e5)), int(rng.integers(0, 4)))
        y0 = round(float(rng.uniform(-2e5, 2e5)), int(rng.integers(0, 4)))
        if rng.uniform() < 0.3:  # extents on the cell lattice: ceil at its edge
            w, h = cs * int(rng.integers(1, 150)), cs * int(rng.integers(1, 150))
        else:
            w, h = cs * float(rng.uniform(0.3, 150)), cs * float(rng.uniform(0.3, 150))
        x1, y1 = x0 + w, y0 + h
        edk = bool(rng.uniform() < 0.5)
        db = (np.nan,) * 4
        obj = prep.SpInterpPrepare.__new__(prep.SpInterpPrepare)
        obj._edk_flag = edk
        obj._x_min, obj._x_max, obj._y_min, obj._y_max = x0, x1, y0, y1
        obj._cell_size = cs
        obj._plot_figs_flag = False
        if edk:
            off = lambda: cs * int(rng.integers(0, 4)) + (  # noqa: E731
                float(rng.uniform(0, cs)) if rng.uniform() < 0.5 else 0.0)
            dx0, dy1 = x0 - off(), y1 + off()
            nc = int(np.ceil((x1 - dx0) / cs)) + int(rng.integers(0, 4))
            nr = int(np.ceil((dy1 - y0) / cs)) + int(rng.integers(0, 4))
            if rng.uniform() < 0.1:  # the grid reaches outside the rasters
                nc = max(1, nc - int(rng.integers(2, 6)))
            db = (dx0, dx0 + nc * cs, dy1 - nr * cs, dy1)
            obj._drft_x_min, obj._drft_x_max, obj._drft_y_min, obj._drft_y_max = db
        params[i] = [x0, x1, y0, y1, cs, float(edk), *db]
        try:
            obj._prepare_crds()
        except AssertionError:
            raised[i] = True
            continue
        rcs[i] = [obj._min_col, obj._max_col, obj._min_row, obj._max_row]
        shapes[i] = obj._interp_crds_orig_shape
        for k, v in enumerate((obj._nc_x_crds, obj._nc_y_crds)):
            digests[i, k] = np.frombuffer(
                hashlib.sha256(np.ascontiguousarray(v, dtype="<f8").tobytes()).digest(),
                dtype=np.uint8)
    out.update(sw_params=params, sw_raised=raised, sw_rc=rcs, sw_shape=shapes,
               sw_digest=digests)
    drift_sweep(prep, out)


def drift_sweep(prep, out, n_cases=150, n_stn=15, seed=505):
    """KrigingDrift._prepare_stns_drift over seeded grids inside drift
    rasters made by sweeps.drift_rasters (no-data cells, values at the edge
    of np.isclose's reach), stations on cell edges and inside cells, with
    and without the cell mask of sweeps.cell_mask. Stored: the inputs but
    the rasters, whether the reference raised (AssertionError: a station on
    no-data; IndexError: rounding put the window's last column or row past
    the rasters), and digests of the cell and station drift arrays."""
    from sweeps import NDV, cell_mask, digest, drift_rasters
    rng = np.random.default_rng(seed)
    sizes = [1.0, 25.0, 100.0, 250.0, 333.3, 1000.0]
    params = np.zeros((n_cases, 12))  # cs, dx0, dy1, nr, nc, k, phase, x0, x1, y0, y1, masked
    stn = np.zeros((n_cases, 2, n_stn))
    raised = np.zeros(n_cases, dtype=np.int8)  # 1 AssertionError, 2 IndexError
    digests = np.zeros((n_cases, 2, 32), dtype=np.uint8)
    for i in range(n_cases):
        cs = float(sizes[rng.integers(len(sizes))])
        dx0 = round(float(rng.uniform(-1e5, 1e5)), int(rng.integers(0, 3)))
        dy1 = round(float(rng.uniform(-1e5, 1e5)), int(rng.integers(0, 3)))
        nr, nc = int(rng.integers(6, 40)), int(rng.integers(6, 40))
        k = int(rng.integers(1, 3))
        phase = float(rng.uniform(0, 6))
        # the grid: a window of the rasters, its edges on or off the lattice
        c0, r0 = int(rng.integers(0, 3)), int(rng.integers(0, 3))
        fx = float(rng.uniform(0, 0.9)) if rng.uniform() < 0.5 else 0.0
        fy = float(rng.uniform(0, 0.9)) if rng.uniform() < 0.5 else 0.0
        x0 = dx0 + (c0 + fx) * cs
        y1 = dy1 - (r0 + fy) * cs
        x1 = dx0 + (nc - int(rng.integers(0, 3))) * cs
        y0 = dy1 - (nr - int(rng.integers(0, 3))) * cs
        masked = bool(rng.uniform() < 0.3)
        params[i] = [cs, dx0, dy1, nr, nc, k, phase, x0, x1, y0, y1, float(masked)]
        # stations: in cells that hold a value in every raster (a station on
        # an edge may still read its neighbour, as the reference's int()
        # rounds), half on cell edges (exact lattice points), half inside
        rasters = drift_rasters(nr, nc, k, phase)
        ok = np.all([~np.isclose(NDV, r) for r in rasters], axis=0)
        ok[:r0 + 1, :] = False
        ok[:, :c0 + 1] = False
        ok[nr - 2:, :] = False
        ok[:, nc - 2:] = False
        cand = np.argwhere(ok)
        pick = cand[rng.integers(len(cand), size=n_stn)]
        rows, cols = pick[:, 0], pick[:, 1]
        on_edge = rng.uniform(size=n_stn) < 0.5
        sx = dx0 + (cols + np.where(on_edge, 0.0, rng.uniform(0.05, 0.95, n_stn))) * cs
        sy = dy1 - (rows + np.where(on_edge, 0.0, rng.uniform(0.05, 0.95, n_stn))) * cs
        stn[i] = [sx, sy]
        obj = prep.SpInterpPrepare.__new__(prep.SpInterpPrepare)
        obj._edk_flag = True
        obj._x_min, obj._x_max, obj._y_min, obj._y_max = x0, x1, y0, y1
        obj._cell_size = cs
        obj._plot_figs_flag = False
        obj._drft_x_min, obj._drft_y_max = dx0, dy1
        obj._drft_x_max, obj._drft_y_min = dx0 + nc * cs, dy1 - nr * cs
        obj._drft_oarrs = rasters
        obj._drft_ndv = NDV
        obj._prepare_crds()
        obj._crds_df = LocFrame({"X": sx, "Y": sy},
                                index=np.array([f"s{j}" for j in range(n_stn)]))
        obj._cell_sel_prms_set = masked
        obj._cntn_idxs = cell_mask(obj._interp_x_crds_msh.size) if masked else None
        try:
            obj._prepare_stns_drift()
        except AssertionError:
            raised[i] = 1
            continue
        except IndexError:  # the window's last column or row past the rasters
            raised[i] = 2
            continue
        digests[i, 0] = np.frombuffer(digest(obj._drft_arrs), dtype=np.uint8)
        digests[i, 1] = np.frombuffer(digest(obj._stns_drft_df.values), dtype=np.uint8)
    out.update(dw_params=params, dw_stn=stn, dw_raised=raised, dw_digest=digests)


SWEEP_MODELS = ["Nug", "Sph", "Exp", "Lin", "Gau", "Pow", "Hol", "Rng"]
SWEEP_TYPES = ["OK", "SK", "EDK", "IDW", "NNB"]


def interp_sweep(ref, out, n_cases=80, seed=606):
    """SpInterpSteps._get_interp on one group over seeded random cases: 2 to
    35 stations, 5 to 40 cells (some on stations), 1 to 4 steps, each step
    a random nest of 1 to 3 of the eight models, flags off on some steps
    (nugget-only steps follow from the strings), OK / SK / EDK (1 to 3
    drifts) / IDW (exponents 0.5 to 3.7) / NNB in turn. Stored: the inputs,
    the estimates, the OK variances and the problem steps."""
    rng = np.random.default_rng(seed)
    st = make_steps(ref, min_vg_val=1e-4, est_vars=True)
    for i in range(n_cases):
        itype = SWEEP_TYPES[i % len(SWEEP_TYPES)]
        n, c, t = int(rng.integers(2, 36)), int(rng.integers(5, 41)), int(rng.integers(1, 5))
        box = float(rng.uniform(1e3, 2e5))
        sx, sy = rng.uniform(0, box, n), rng.uniform(0, box, n)
        cx, cy = rng.uniform(0, box, c), rng.uniform(0, box, c)
        on = int(rng.integers(0, 3))
        cx[:on], cy[:on] = sx[:on], sy[:on]
        z = rng.normal(3.0, 2.0, (t, n))
        vgs = []
        for _ in range(t):
            comps = []
            for _ in range(int(rng.integers(1, 4))):
                nm = SWEEP_MODELS[rng.integers(len(SWEEP_MODELS))]
                sill = round(float(rng.uniform(0.01, 2.0)), 4)
                if nm == "Nug":
                    r = 0.0
                elif nm == "Pow":
                    r = round(float(rng.uniform(0.1, 1.9)), 3)
                else:
                    r = round(float(rng.uniform(0.02, 1.0)) * box, 1)
                comps.append(f"{sill} {nm}({r})")
            vgs.append(" + ".join(comps))
        flags = rng.uniform(size=t) < 0.85
        sd = cd = None
        if itype == "EDK":
            kd = int(rng.integers(1, 4))
            sd = rng.uniform(0, 1000, (n, kd))
            cd = rng.uniform(0, 1000, (kd, c))
        idw_exp = float(rng.choice([0.5, 1.0, 2.0, 3.7]))
        est, var, prblm = interp_one(ref, st, sx, sy, cx, cy, z, itype, vgs, idw_exp=idw_exp,
                                     flags=flags, drifts=sd, cell_drifts=cd)
        p = f"w{i}_"
        out.update({p + "sx": sx, p + "sy": sy, p + "cx": cx, p + "cy": cy, p + "z": z,
                    p + "vgs": np.array(vgs), p + "flags": flags,
                    p + "type": np.array(itype), p + "idw_exp": np.array(idw_exp),
                    p + "est": est, p + "prblm": np.array(sorted(prblm), dtype=np.int64)})
        if var is not None:
            out[p + "var"] = var
        if sd is not None:
            out.update({p + "sd": sd, p + "cd": cd})
    out["w_cases"] = np.arange(n_cases)


def main(ref_root=None, only=None):
    ref = load_reference(ref_root)
    if only == "driver":
        out = {}
        driver_case(ref, out)
        np.savez_compressed(HERE / "driver.npz", **out)
        return
    if only == "legacy":
        out = {}
        legacy_case(ref, out)
        np.savez_compressed(HERE / "legacy.npz", **out)
        return
    if only == "interp_sweep":
        out = {}
        interp_sweep(ref, out)
        np.savez_compressed(HERE / "interp_sweep.npz", **out)
        return
    if only == "nebs_sweep":
        out = {}
        nebs_sweep(ref, out)
        np.savez_compressed(HERE / "nebs_sweep.npz", **out)
        return
    if only == "legacy_sweep":
        out = {}
        legacy_sweep(ref, out)
        np.savez_compressed(HERE / "legacy_sweep.npz", **out)
        return
    if only == "vg_edges":
        out = {}
        vg_edges(ref, out)
        np.savez_compressed(HERE / "vg_edges.npz", **out)
        return
    if only == "empirical_sweep":
        out = {}
        empirical_sweep(ref_root, out)
        np.savez_compressed(HERE / "empirical_sweep.npz", **out)
        return
    if only == "steps_sweep":
        out = {}
        steps_sweep(ref, out)
        np.savez_compressed(HERE / "steps_sweep.npz", **out)
        return
    out = {}
    kernels_case(ref, out)
    np.savez_compressed(HERE / "kernels.npz", **out)
    out = {}
    interp_case(ref, out)
    np.savez_compressed(HERE / "interp.npz", **out)
    out = {}
    vg_mix = ["0.05 Nug(0.0) + 0.95 Exp(20000)", "1.0 Sph(30000)",
              "0.2 Nug(0.0) + 0.8 Gau(15000)", "1.0 Nug(0.0)"]
    t = 12
    vgs = [vg_mix[i % len(vg_mix)] for i in range(t)]
    steps_case(ref, out, "okidw", n=40, t=t, nx=24, ny=18, cs=2500.0, box=6e4,
               p_miss=0.25, vgs=vgs, seed=44,
               methods=["OK", "SK", ("IDW", 2.0), ("IDW", 1.0), "NNB"],
               min_var_thr=0.0, min_var_cut=0.0, max_var_cut=None)
    steps_case(ref, out, "edk", n=35, t=t, nx=20, ny=20, cs=3000.0, box=6e4,
               p_miss=0.2, vgs=vgs, seed=55, methods=["EDK", "OK"], edk=True,
               min_var_thr=0.5, min_var_cut=None, max_var_cut=4.5)
    # config-1 shapes (150 stations, 100 km box, Exp vg, all stations present)
    # on a sub-sampled grid: every 8th row and column of the 200 x 200 grid.
    rng = np.random.default_rng(1)
    n1 = 150
    sx, sy = rng.uniform(0, 1e5, n1), rng.uniform(0, 1e5, n1)
    vg1 = "0.05 Nug(0.0) + 0.95 Exp(20000)"
    z1 = grf_values(rng, sx, sy, vg1, 4, 5.0, ref)
    cx, cy = grid_cells(0.0, 1e5, 500.0, 200, 200)
    sel = (np.arange(200)[:, None] % 8 == 0) & (np.arange(200)[None] % 8 == 0)
    cx, cy = cx[sel.ravel()].copy(), cy[sel.ravel()].copy()
    st = make_steps(ref, min_vg_val=1e-4, est_vars=True)
    est, var, _ = interp_one(ref, st, sx, sy, cx, cy, z1, "OK", [vg1] * 4)
    est_idw, _, _ = interp_one(ref, st, sx, sy, cx, cy, z1, "IDW", [vg1] * 4, idw_exp=2.0)
    out.update(c1_sx=sx, c1_sy=sy, c1_z=z1, c1_cx=cx, c1_cy=cy, c1_ok_est=est,
               c1_ok_var=var, c1_idw_est=est_idw)
    np.savez_compressed(HERE / "steps.npz", **out)
    out = {}
    nebs_case(ref, out)
    np.savez_compressed(HERE / "nebs.npz", **out)
    out = {}
    fitter_case(ref_root, out)
    np.savez_compressed(HERE / "fitter.npz", **out)
    out = {}
    legacy_case(ref, out)
    np.savez_compressed(HERE / "legacy.npz", **out)
    out = {}
    driver_case(ref, out)
    np.savez_compressed(HERE / "driver.npz", **out)
    out = {}
    interp_sweep(ref, out)
    np.savez_compressed(HERE / "interp_sweep.npz", **out)
    out = {}
    nebs_sweep(ref, out)
    np.savez_compressed(HERE / "nebs_sweep.npz", **out)
    out = {}
    legacy_sweep(ref, out)
    np.savez_compressed(HERE / "legacy_sweep.npz", **out)
    out = {}
    vg_edges(ref, out)
    np.savez_compressed(HERE / "vg_edges.npz", **out)
    out = {}
    empirical_sweep(ref_root, out)
    np.savez_compressed(HERE / "empirical_sweep.npz", **out)
    out = {}
    steps_sweep(ref, out)
    np.savez_compressed(HERE / "steps_sweep.npz", **out)
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main(*sys.argv[1:])
