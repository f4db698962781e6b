"""CPU restatement (numpy + the C kernels of ``oracle/vgfill.c``) of the
reference's gridded-interpolation step engine.

TEST INFRASTRUCTURE ONLY. This module is the oracle that the CUDA path is
checked against and the CPU baseline that ``bench.py`` times beside it; the
product package never imports it.

It follows the reference's algorithm step for step, including its loop
structure (a Python loop over cells calling ``np.matmul(pinv, rhs)``), so its
timing is a fair stand-in for the reference's own CPU path:

- ``parse_vg_str``          cyth/interpmthds.pyx:174-184 (split rules, max(1e-5, r))
- ``check_full_nuggetness`` misc.py:1074-1105
- ``get_dists_arr``         interp/steps.py:73-86 over cyth/interpmthds.pyx:123-143
- ``get_svars_arr``         interp/steps.py:88-138 over cyth/interpmthds.pyx:146-226
- ``get_2d_arr_subset``     interp/steps.py:140-168 over cyth/interpmthds.pyx:229-248
- ``get_vars_arr_subset``   interp/steps.py:170-243
- ``get_interp``            interp/steps.py:245-401
- ``fill_krig_idw_dst_data`` interp/steps.py:403-435
- ``mod_min_max``           interp/steps.py:466-476
- ``interp_steps``          interp/steps.py:478-835 (neighbour method 'all')
- ``get_grps_in_time``      interp/grps.py:57-101 (without pandas)
- ``ret_mp_idxs``           misc.py:601-613
- ``legacy_krige``          cyth/interpmthds.pyx:251-765 (the single-neighbourhood
                            kriging classes)
- ``prepare_crds``          interp/prepare.py:148-241 (the grid)
- ``sample_drifts``         interp/drift.py:165-227 (drift values at cells and stations)
- ``points_in_polygons``    interp/prepare.py:244-288, misc.py:407-500, 617-627
- ``field_stats``           interp/main.py:474-525 (per-step statistics)

Parity status: pinned against fixtures generated by running the reference's
own code (tests/golden/make_golden.py); see tests/test_oracle_golden.py.
"""
import ctypes
import math

import numpy as np

from . import build as _build

MODEL_CODES = {
    "Rng": 0, "Nug": 1, "Sph": 2, "Exp": 3, "Lin": 4, "Gau": 5, "Pow": 6, "Hol": 7,
}


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def parse_vg_str(vg_str):
    """Components ``[(code, sill, range)]`` of a variogram string.

    Same split rules as ``fill_vg_var_arr`` (cyth/interpmthds.pyx:174-184):
    split on '+', strip, split on ' ' into sill and 'Name(range', then on '('
    and ')'. The range is clamped to ``max(1e-5, range)``. An unknown model
    name raises (the reference's C++ map would return a null function).
    """
    comps = []
    for part in str(vg_str).encode().split(b"+"):
        part = part.strip()
        sill_s, vg_s = part.split(b" ")
        vg_s, range_s = vg_s.split(b"(")
        range_s = range_s.split(b")")[0]
        name = vg_s.decode()
        if name not in MODEL_CODES:
            raise KeyError(f"unknown variogram model {name!r}")
        comps.append((MODEL_CODES[name], float(sill_s), max(1e-5, float(range_s))))
    return comps


def check_full_nuggetness(in_model, min_vg_val):
    """misc.py:1074-1105. True when the total sill or the largest range is
    <= min_vg_val. (The reference's second test compares the whole
    sub-model string with 'Nug', which never matches.)"""
    in_model = str(in_model)
    nuggetness = False
    if in_model == "nan":
        return nuggetness
    models = in_model.split("+")
    sill = 0.0
    rng = 0.0
    for submodel in models:
        submodel = submodel.strip()
        sill += float(submodel.split("(")[0].strip()[:-3].strip())
        rng = max(rng, float(submodel.split("(")[1].split(")")[0]))
    if np.any(np.array([sill, rng]) <= min_vg_val):
        nuggetness = True
    if (len(models) == 1) and models[0] == "Nug":
        nuggetness = True
    return nuggetness


def get_dists_arr(x1s, y1s, x2s, y2s):
    x1s, y1s, x2s, y2s = (np.ascontiguousarray(a, dtype=np.float64)
                          for a in (x1s, y1s, x2s, y2s))
    out = np.full((x1s.size, x2s.size), np.nan)
    _build.lib().orc_fill_dists_2d_mat(
        _ptr(x1s), _ptr(y1s), x1s.size, _ptr(x2s), _ptr(y2s), x2s.size, _ptr(out))
    return out


def fill_vg_var_arr(dists, covar_flag, diag_mat_flag, vg_str, min_vg_val):
    dists = np.ascontiguousarray(dists, dtype=np.float64)
    comps = parse_vg_str(vg_str)
    codes = np.array([c[0] for c in comps], dtype=np.int32)
    sills = np.array([c[1] for c in comps], dtype=np.float64)
    ranges = np.array([c[2] for c in comps], dtype=np.float64)
    out = np.full_like(dists, np.nan)
    _build.lib().orc_fill_vg_var_arr(
        _ptr(dists), dists.shape[0], dists.shape[1], _ptr(out), int(covar_flag),
        int(diag_mat_flag), len(comps), _ptr(codes), _ptr(sills), _ptr(ranges),
        float(min_vg_val))
    return out


def get_svars_arr(dists_arr, vgs, interp_types, diag_mat_flag, min_vg_val):
    var_flag = any(t in interp_types for t in ("OK", "EDK"))
    covar_flag = "SK" in interp_types
    out = {}
    for vg in vgs:
        assert vg != "nan"
        if var_flag:
            out[(vg, 0)] = fill_vg_var_arr(dists_arr, 0, diag_mat_flag, vg, min_vg_val)
        if covar_flag:
            out[(vg, 1)] = fill_vg_var_arr(dists_arr, 1, diag_mat_flag, vg, min_vg_val)
    return out


def get_2d_arr_subset(arr, row_idxs, col_idxs, rows_add_rc=0, cols_add_rc=0):
    row_idxs = np.ascontiguousarray(row_idxs, dtype=np.int64)
    col_idxs = np.ascontiguousarray(col_idxs, dtype=np.int64)
    arr = np.ascontiguousarray(arr, dtype=np.float64)
    sub = np.full((row_idxs.size + rows_add_rc, col_idxs.size + cols_add_rc), np.nan)
    _build.lib().orc_copy_2d_arr_at_idxs(
        _ptr(arr), arr.shape[1], _ptr(row_idxs), row_idxs.size, _ptr(col_idxs),
        col_idxs.size, _ptr(sub), sub.shape[1])
    return sub


def get_vars_arr_subset(model, interp_type, ref_drfts, rr_all, dr_all,
                        ref_ref_sub_idxs, time_neb_idxs_grp, dst_drfts):
    if interp_type == "OK":
        add_rc, covar_flag = 1, 0
    elif interp_type == "SK":
        add_rc, covar_flag = 0, 1
    elif interp_type == "EDK":
        add_rc, covar_flag = 1 + ref_drfts.shape[1], 0
    else:
        raise NotImplementedError(interp_type)
    rr = get_2d_arr_subset(rr_all[(model, covar_flag)], ref_ref_sub_idxs,
                           ref_ref_sub_idxs, add_rc, add_rc)
    dr = get_2d_arr_subset(dr_all[(model, covar_flag)], time_neb_idxs_grp,
                           ref_ref_sub_idxs, 0, add_rc)
    n = ref_ref_sub_idxs.size
    if interp_type == "OK":
        rr[n, :n] = 1.0
        rr[:, n] = 1.0
        rr[n, n] = 0.0
        dr[:, n] = 1.0
    elif interp_type == "EDK":
        rr[n, :n] = 1.0
        rr[:n, n] = 1.0
        dr[:, n] = 1.0
        rr[n:, n:] = 0.0
        for k in range(ref_drfts.shape[1]):
            rr[n + 1 + k, :n] = ref_drfts[:, k]
            rr[:n, n + 1 + k] = ref_drfts[:, k]
            dr[:, n + 1 + k] = dst_drfts[k, :]
    return rr, dr


def fill_krig_idw_dst_data(n_refs, n_dsts, inv, dr_sub, dists_sub, ref_data, j,
                           dst_data, est_vars):
    for i in range(n_dsts):
        lmds = np.matmul(inv, dr_sub[i])
        if not np.isclose(lmds[:n_refs].sum(), 1.0):
            dst_data[j, i] = ref_data[j, np.argmin(dists_sub[i])]
            if est_vars is not None:
                est_vars[j, i] = 0.0
        else:
            dst_data[j, i] = (lmds[:n_refs] * ref_data[j]).sum()
            if est_vars is not None:
                est_vars[j, i] = (lmds * dr_sub[i]).sum() + lmds[n_refs]


def get_interp(ref_data, interp_type, ref_drfts, dst_drfts, idw_exp, models,
               interp_steps_flags, nuggetness_flags, sub_time_steps,
               prblm_time_steps, dists_sub, rr_all, dr_all, ref_ref_sub_idxs,
               time_neb_idxs_grp, *, est_vars_flag, intrp_dtype=np.float32):
    """interp/steps.py:245-401. ``dists_sub`` is modified in place by IDW,
    as in the reference."""
    n_dsts = dists_sub.shape[0]
    n_refs = ref_data.shape[1]
    n_time = ref_data.shape[0]
    dst_data = np.full((n_time, n_dsts), np.nan)
    est_vars = (np.full((n_time, n_dsts), np.nan, dtype=intrp_dtype)
                if (est_vars_flag and interp_type == "OK") else None)
    ref_means = ref_data.mean(axis=1)
    if n_refs == 1:
        for j in range(n_time):
            dst_data[j, :] = ref_data[j, :]
    elif interp_type == "NNB":
        for i in range(n_dsts):
            k = np.argmin(dists_sub[i])
            for j in range(n_time):
                dst_data[j, i] = ref_data[j, k]
    elif interp_type == "IDW":
        wts = np.full(n_refs, np.nan)
        flags = np.ascontiguousarray(interp_steps_flags, dtype=np.uint8)
        rd = np.ascontiguousarray(ref_data, dtype=np.float64)
        rm = np.ascontiguousarray(ref_means, dtype=np.float64)
        assert dists_sub.flags.c_contiguous
        bad = _build.lib().orc_idw_group(
            _ptr(dists_sub), n_dsts, n_refs, _ptr(rd), n_time, _ptr(flags),
            _ptr(rm), float(idw_exp), _ptr(wts), _ptr(dst_data))
        assert bad < 0, "IDW weight sum below 1e-14"
    elif interp_type in ("OK", "SK", "EDK"):
        old_model = ""
        last_failed = False
        inv = None
        dr_sub = None
        for j in np.argsort(models):
            model = models[j]
            if (not interp_steps_flags[j]) or nuggetness_flags[j]:
                dst_data[j, :] = ref_means[j]
                if est_vars is not None:
                    est_vars[j, :] = 0.0
                continue
            if model == "nan":
                raise ValueError("NaN VG!")
            if model != old_model:
                rr_sub, dr_sub = get_vars_arr_subset(
                    model, interp_type, ref_drfts, rr_all, dr_all,
                    ref_ref_sub_idxs, time_neb_idxs_grp, dst_drfts)
                old_model = model
                try:
                    inv = np.linalg.pinv(rr_sub)
                    last_failed = False
                except Exception:
                    last_failed = True
                    if sub_time_steps[j] not in prblm_time_steps:
                        prblm_time_steps.append(sub_time_steps[j])
                    inv = np.nan
            if last_failed:
                for i in range(n_dsts):
                    dst_data[j, i] = ref_data[j, np.argmin(dists_sub[i])]
                if est_vars is not None:
                    est_vars[j, :] = 0.0
            else:
                fill_krig_idw_dst_data(n_refs, n_dsts, inv, dr_sub, dists_sub,
                                       ref_data, j, dst_data, est_vars)
    else:
        raise NotImplementedError(interp_type)
    return dst_data, est_vars


def mod_min_max(fld, min_var_cut, max_var_cut):
    """interp/steps.py:466-476 (in place; NaN stays NaN)."""
    with np.errstate(invalid="ignore"):
        if min_var_cut is not None:
            fld[fld < min_var_cut] = min_var_cut
        if max_var_cut is not None:
            fld[fld > max_var_cut] = max_var_cut


def get_grps_in_time(data):
    """interp/grps.py:57-101 without pandas: steps with the same set of
    non-NaN stations, in order of first appearance.
    Returns [(station_idxs, step_mask)]."""
    avail = np.isfinite(data)
    keys = [avail[i].tobytes() for i in range(data.shape[0])]
    grps = []
    seen = {}
    for i, k in enumerate(keys):
        if k in seen:
            continue
        mask = np.array([kk == k for kk in keys])
        seen[k] = True
        grps.append((np.where(avail[i])[0], mask))
    return grps


def interp_args_for(methods, est_vars):
    """The (type, fig_dir, label[, idw_exp]) list of interp/prepare.py:638-695
    for a list of methods like ['OK', 'SK', 'EDK', ('IDW', 2.0), 'NNB']."""
    args = []
    for t in ("OK", "SK", "EDK"):
        if t in methods:
            args.append((t, None, t))
    idw = [m[1] for m in methods if isinstance(m, tuple) and m[0] == "IDW"]
    for i, e in enumerate(idw):
        args.append(("IDW", None, f"IDW_{i:03d}", float(e)))
    if "NNB" in methods:
        args.append(("NNB", None, "NNB"))
    if est_vars:
        args.append(("EST_VARS_OK", None, "EST_VARS_OK"))
    return args


def interp_steps(stn_x, stn_y, data, cell_x, cell_y, vgs, interp_args, *,
                 est_vars=False, stn_drifts=None, cell_drifts=None,
                 min_var_thr=0.0, min_var_cut=None, max_var_cut=None,
                 min_vg_val=0.0, intrp_dtype=np.float32, time_steps=None,
                 neb_sel_mthd="all", n_nebs=None, n_pies=None):
    """interp/steps.py:478-835 for one grid chunk.

    data [T, N] (NaN = station missing), vgs [T] strings (or None when no
    kriging is asked for), stn_drifts [N, k], cell_drifts [k, C].
    Returns ({label: [T, C] fields}, problem time steps).
    """
    if neb_sel_mthd != "all":
        return _interp_steps_nebs(stn_x, stn_y, data, cell_x, cell_y, vgs, interp_args,
                                  neb_sel_mthd, n_nebs, n_pies, est_vars=est_vars,
                                  stn_drifts=stn_drifts, cell_drifts=cell_drifts,
                                  min_var_thr=min_var_thr, min_var_cut=min_var_cut,
                                  max_var_cut=max_var_cut, min_vg_val=min_vg_val,
                                  intrp_dtype=intrp_dtype, time_steps=time_steps)
    data = np.asarray(data, dtype=np.float64)
    n_steps = data.shape[0]
    n_cells = cell_x.size
    if time_steps is None:
        time_steps = np.arange(n_steps)
    interp_types = [a[0] for a in interp_args]
    interp_labels = [a[2] for a in interp_args]
    krg = any(t in interp_types for t in ("OK", "SK", "EDK"))
    if krg:
        vgs = np.asarray(vgs, dtype=object)
        assert np.all(vgs != "nan")
        uniq_vgs = list(dict.fromkeys(vgs.tolist()))
        dr = get_dists_arr(stn_x, stn_y, stn_x, stn_y)
        rr_all = get_svars_arr(dr, uniq_vgs, interp_types, 1, min_vg_val)
    dd = get_dists_arr(cell_x, cell_y, stn_x, stn_y)
    if krg:
        dr_all = get_svars_arr(dd, uniq_vgs, interp_types, 0, min_vg_val)
    else:
        rr_all = dr_all = None
    flds = {lab: np.full((n_steps, n_cells), np.nan, dtype=intrp_dtype)
            for lab in interp_labels}
    prblm = []
    all_cells = np.arange(n_cells)
    for stn_idxs, step_mask in get_grps_in_time(data):
        sub_time_steps = time_steps[step_mask]
        if not stn_idxs.size:
            for s in sub_time_steps:
                if s not in prblm:
                    prblm.append(s)
            continue
        vals = data[step_mask][:, stn_idxs]
        drifts = stn_drifts[stn_idxs, :] if "EDK" in interp_types else None
        if krg:
            models = vgs[step_mask]
            nug = np.array([check_full_nuggetness(m, min_vg_val) for m in models])
        else:
            models = nug = None
        time_idxs = np.where(step_mask)[0]
        # neighbour method 'all': one cell group holding every cell, every
        # station of the group is a neighbour.
        sub_ref_data = vals.copy("c")
        dists_sub = get_2d_arr_subset(dd, all_cells, stn_idxs, 0, 0)
        flags = np.array([np.any(sub_ref_data[j] >= min_var_thr)
                          for j in range(sub_ref_data.shape[0])])
        sub_dst_drifts = cell_drifts[:, all_cells] if "EDK" in interp_types else None
        for i, t in enumerate(interp_types):
            if interp_labels[i] == "EST_VARS_OK":
                continue
            idw_exp = interp_args[i][3] if t == "IDW" else 5
            vals_i, ev = get_interp(
                sub_ref_data, t, drifts, sub_dst_drifts, idw_exp, models, flags,
                nug, sub_time_steps, prblm, dists_sub, rr_all, dr_all, stn_idxs,
                all_cells, est_vars_flag=est_vars, intrp_dtype=intrp_dtype)
            mod_min_max(vals_i, min_var_cut, max_var_cut)
            for j, ti in enumerate(time_idxs):
                flds[interp_labels[i]][ti, :] = vals_i[j].astype(intrp_dtype)
                if est_vars and t == "OK":
                    flds["EST_VARS_OK"][ti, :] = ev[j]
    return flds, prblm


def ret_mp_idxs(n_vals, n_cpus):
    """misc.py:601-613."""
    idxs = np.linspace(0, n_vals, n_cpus + 1, endpoint=True, dtype=np.int64)
    idxs = np.unique(idxs)
    if idxs.shape[0] == 1:
        idxs = np.concatenate((np.array([0]), idxs))
    return idxs


# ---- neighbour selection 'nrst' / 'pie' (interp/grps.py:103-288) ----------

def nebs_nrst(dst_xs, dst_ys, ref_xs, ref_ys, n_nebs):
    """interp/grps.py:147-163: per destination the n_nebs nearest references
    (numpy's argsort of the distances), as sorted indices."""
    n = ref_xs.size
    out = np.empty((dst_xs.size, min(n_nebs, n)), dtype=np.int64)
    for i in range(dst_xs.size):
        d = ((dst_xs[i] - ref_xs) ** 2 + (dst_ys[i] - ref_ys) ** 2) ** 0.5
        out[i] = np.sort(np.argsort(d)[:n_nebs])
    return out


def _pie_ranks(dst_x, dst_y, ref_xs, ref_ys, n_pies):
    """cyth/interpmthds.pyx:768-781 and 811-890 (sel_equidist_refs with
    min_dist_thresh -1): C pow distances, the angle of every reference
    (atan(dy/dx) with the reference's quadrant rules: dx == 0 gives 0, and
    dx < 0 with dy == 0 stays at 0), its pie int(angle * n_pies / 2 pi), and
    each reference's rank by distance within its pie (numpy argsort)."""
    n = ref_xs.size
    dists = np.array([math.pow(math.pow(dst_x - ref_xs[i], 2.0) +
                               math.pow(dst_y - ref_ys[i], 2.0), 0.5) for i in range(n)])
    pies = np.empty(n, dtype=np.int64)
    two_pi = 2 * math.pi
    for j in range(n):
        xd, yd = ref_xs[j] - dst_x, ref_ys[j] - dst_y
        if not xd:
            ang = 0.0
        else:
            ang = math.atan(yd / xd)
            if xd < 0 and yd > 0:
                ang = math.pi + ang
            elif xd < 0 and yd < 0:
                ang = math.pi + ang
            elif xd > 0 and yd < 0:
                ang = two_pi + ang
        pies[j] = int(ang * n_pies / two_pi)
    ranks = np.full(n, -1, dtype=np.int64)
    for j in range(n_pies):
        if not np.any(pies == j):
            continue
        tem = np.where(pies == j, dists, np.inf)
        order = np.argsort(tem)
        for i in range(n):
            if tem[order[i]] == np.inf:
                break
            ranks[order[i]] = i
    return dists, ranks


def nebs_pie(dst_xs, dst_ys, ref_xs, ref_ys, n_nebs, n_pies):
    """interp/grps.py:165-247: references ordered by their rank within their
    pie, then by distance within a rank (the nearest of every pie first);
    the first n_nebs, as sorted indices."""
    out = np.empty((dst_xs.size, n_nebs), dtype=np.int64)
    for i in range(dst_xs.size):
        dists, ranks = _pie_ranks(dst_xs[i], dst_ys[i], ref_xs, ref_ys, n_pies)
        seq = []
        for r in np.unique(ranks[ranks != -1]):
            same = np.where(ranks == r)[0]
            seq.extend(same[np.argsort(dists[same])].tolist())
        out[i, :] = np.sort(np.array(seq)[:n_nebs])
    return out


def neb_groups(all_neb_idxs):
    """interp/grps.py:103-138: destinations with identical neighbour lists,
    groups in order of first occurrence; returns the group label of every
    destination and the list of groups (destination indices)."""
    _, first, inv = np.unique(all_neb_idxs, axis=0, return_index=True, return_inverse=True)
    inv = np.asarray(inv).ravel()
    rank = np.empty(first.size, dtype=np.int64)
    rank[np.argsort(first)] = np.arange(first.size)
    lab = rank[inv]
    return lab, [np.where(lab == g)[0] for g in range(first.size)]


def neb_idxs(method, dst_xs, dst_ys, ref_xs, ref_ys, n_nebs, n_pies):
    """SpInterpNeighborGrouping.get_neb_idxs_and_grps (interp/grps.py:249-288)
    for the given references: the neighbour lists of every destination."""
    if method == "all":
        return np.tile(np.arange(ref_xs.size), (dst_xs.size, 1))
    if method == "nrst":
        return nebs_nrst(dst_xs, dst_ys, ref_xs, ref_ys, n_nebs)
    if method == "pie":
        return nebs_pie(dst_xs, dst_ys, ref_xs, ref_ys, n_nebs, n_pies)
    raise NotImplementedError(method)


def _interp_steps_nebs(stn_x, stn_y, data, cell_x, cell_y, vgs, interp_args, method,
                       n_nebs, n_pies, *, stn_drifts=None, cell_drifts=None, intrp_dtype=np.float32,
                       time_steps=None, **kw):
    """interp/steps.py:584-606 (stations that are nobody's neighbour with all
    stations present are dropped) and 673-833 (per group of steps with the
    same stations, every group of cells with the same neighbours is a
    group of _get_interp with those stations)."""
    data = np.asarray(data, dtype=np.float64)
    T, C = data.shape[0], cell_x.size
    if time_steps is None:
        time_steps = np.arange(T)
    keep = np.unique(neb_idxs(method, cell_x, cell_y, stn_x, stn_y, n_nebs, n_pies))
    sx, sy, data = stn_x[keep], stn_y[keep], data[:, keep]
    sd = None if stn_drifts is None else np.asarray(stn_drifts)[keep]
    vgs = None if vgs is None else np.asarray(vgs, dtype=object)
    labels = [a[2] for a in interp_args]
    flds = {lab: np.full((T, C), np.nan, dtype=intrp_dtype) for lab in labels}
    prblm = []
    for stn_idxs, step_mask in get_grps_in_time(data):
        sub_t = time_steps[step_mask]
        if not stn_idxs.size:
            for t in sub_t:
                if t not in prblm:
                    prblm.append(t)
            continue
        rows = np.where(step_mask)[0]
        nidx = neb_idxs(method, cell_x, cell_y, sx[stn_idxs], sy[stn_idxs], n_nebs, n_pies)
        _, groups = neb_groups(nidx)
        for grp in groups:
            sub = stn_idxs[nidx[grp[0]]]
            out, pr = interp_steps(
                sx[sub], sy[sub], data[rows][:, sub], cell_x[grp], cell_y[grp],
                None if vgs is None else vgs[rows], interp_args,
                stn_drifts=None if sd is None else sd[sub],
                cell_drifts=None if cell_drifts is None else np.asarray(cell_drifts)[:, grp],
                intrp_dtype=intrp_dtype, time_steps=sub_t, **kw)
            for lab in labels:
                flds[lab][np.ix_(rows, grp)] = out[lab]
            for t in pr:
                if t not in prblm:
                    prblm.append(t)
    return flds, prblm


# ---- the single-neighbourhood classes of cyth/interpmthds.pyx:251-765 ------

LEGACY_CLASSES = ("OrdinaryKriging", "SimpleKriging", "ExternalDriftKriging",
                  "ExternalDriftKriging_MD", "OrdinaryIndicatorKriging",
                  "SimpleIndicatorKriging")


def _vg_comp_arr(dists, comp):
    """gamma of one variogram component at every entry (the reference's
    vg_ftn(h, range, sill) of cyth/interpmthds.pyx:38-84)."""
    code, sill, rng = comp
    dists = np.ascontiguousarray(dists, dtype=np.float64)
    out = np.empty_like(dists)
    codes = np.array([code], dtype=np.int32)
    sills = np.array([sill], dtype=np.float64)
    ranges = np.array([rng], dtype=np.float64)
    _build.lib().orc_fill_vg_var_arr(
        _ptr(dists), dists.shape[0], dists.shape[1], _ptr(out), 0, 0, 1, _ptr(codes),
        _ptr(sills), _ptr(ranges), float("-inf"))
    return out


def legacy_krige(cls, xi, yi, zi, xk, yk, model, si=None, sk=None, lim=None):
    """What ``cls(...).krige()`` (``ikrige()`` for the indicator classes)
    leaves in the object's arrays, as a dict keyed by attribute name.

    Follows cyth/interpmthds.pyx:251-765:
    - components parsed with the split rules of parse_vg_str (lines 294-303),
      ranges clamped to max(1e-5, r);
    - station distances for j > i, mirrored; the semivariogram matrix sums
      the components in order for i != j and keeps 0 on the diagonal, so a
      nugget is a discontinuity at h = 0 (not the sill, as in
      fill_vg_var_arr);
    - OK: [[G, 1], [1', 0]]; EDK: [[G, 1, S'], [1', 0, 0], [S, 0, 0]] with
      S = si [k, n] (ExternalDriftKriging: k = 1); SK: the matrix starts at
      the fill value 0.0 that __init__ gave it before krige() summed the
      sills, so it is -G with a zero diagonal (lines 397-399, 413, 432-442);
    - P = numpy.linalg.pinv of that matrix; per point, the right-hand side
      sums gamma over components where the distance is not 0 (SK: total
      sill minus them, the total sill where the distance is 0) plus 1 and
      the point's drifts; lambda = P r by np.matmul per point;
    - zk = sum(lambda[:n] z); OK: est_vars = max(0, lambda'r + mu);
      SK: est_covars = max(0, total sill - lambda'c);
    - indicator classes: ixi = (z <= lim), ik = max(0, sum(lambda ixi)),
      est = max(0, ik (1 - ik)).
    """
    assert cls in LEGACY_CLASSES, cls
    xi, yi, zi, xk, yk = (np.ascontiguousarray(a, dtype=np.float64)
                          for a in (xi, yi, zi, xk, yk))
    comps = parse_vg_str(model)
    n, n_out = xi.size, xk.size
    sk_kind = cls in ("SimpleKriging", "SimpleIndicatorKriging")
    edk = cls.startswith("ExternalDrift")
    if edk:
        si = np.atleast_2d(np.asarray(si, dtype=np.float64))
        sk = np.atleast_2d(np.asarray(sk, dtype=np.float64))
    n_drift = si.shape[0] if edk else 0
    a = 0 if sk_kind else 1 + n_drift
    m = n + a
    covar = 0.0
    for c in comps:
        covar += c[1]
    in_dists = get_dists_arr(xi, yi, xi, yi)
    off = ~np.eye(n, dtype=bool)
    g = np.zeros((n, n))
    for c in comps:
        gc = _vg_comp_arr(in_dists, c)
        if sk_kind:
            g[off] -= gc[off]
        else:
            g[off] += gc[off]
    lhs = np.zeros((m, m))
    lhs[:n, :n] = g
    if not sk_kind:
        lhs[n, :n] = 1.0
        lhs[:n, n] = 1.0
        for k in range(n_drift):
            lhs[n + 1 + k, :n] = si[k]
            lhs[:n, n + 1 + k] = si[k]
    inv = np.linalg.pinv(lhs)
    d_out = get_dists_arr(xi, yi, xk, yk)            # [n, n_out]
    gam = [_vg_comp_arr(d_out, c) for c in comps]
    rhss = np.zeros((n_out, m))
    lambdas = np.zeros((n_out, n))
    mus = np.zeros((a, n_out))
    zk = np.zeros(n_out)
    est = np.zeros(n_out)
    for k in range(n_out):
        r = np.zeros(m)
        for lo in range(n):
            if d_out[lo, k] == 0.0:
                r[lo] = covar if sk_kind else 0.0
                continue
            t = covar if sk_kind else 0.0
            for gc in gam:
                t = t - gc[lo, k] if sk_kind else t + gc[lo, k]
            r[lo] = t
        if not sk_kind:
            r[n] = 1.0
            for q in range(n_drift):
                r[n + 1 + q] = sk[q, k]
        lam = np.matmul(inv, r)
        mus[:, k] = lam[n:]
        lk = lam[:n]
        zk[k] = np.sum(lk * zi)
        if sk_kind:
            est[k] = max(0.0, covar - np.sum(lk * r[:n]))
        elif not edk:
            est[k] = max(0.0, np.sum(lk * r[:n]) + lam[n])
        lambdas[k] = lk
        rhss[k] = r
    out = dict(zk=zk, lambdas=lambdas, rhss=rhss, in_dists=in_dists, covar=covar)
    if sk_kind:
        out.update(est_covars=est, in_covars=lhs, in_covars_inv=inv, out_covars=rhss.copy())
    else:
        out.update(in_vars=lhs, in_vars_inv=inv)
    if cls == "ExternalDriftKriging":
        out.update(mus_1=mus[0].copy(), mus_2=mus[1].copy())
    elif cls == "ExternalDriftKriging_MD":
        out.update(mus_arr=mus)
    elif not sk_kind:
        out.update(est_vars=est, mus=mus[0].copy())
    if cls.endswith("IndicatorKriging"):
        ixi = np.where(zi <= lim, 1.0, 0.0)
        ik = np.zeros(n_out)
        for o in range(n_out):
            ik[o] = max(0.0, np.sum(lambdas[o, :] * ixi))
            est[o] = max(0.0, ik[o] * (1.0 - ik[o]))
        out.update(ixi=ixi, ik=ik)
    return out


# ---- the driver flow around the step engine ---------------------------------

def prepare_crds(x_min, x_max, y_min, y_max, cell_size, drift_bounds=None):
    """SpInterpPrepare._prepare_crds (interp/prepare.py:148-241): the column
    and row range of the grid (inside the drift rasters when drift_bounds =
    (x_min, x_max, y_min, y_max) of the rasters is given, EDK), cell-centre
    coordinates by np.linspace from (x_min + cs / 2, y_max - cs / 2), and
    the row-major cell mesh."""
    if drift_bounds is not None:
        dx0, dx1, dy0, dy1 = drift_bounds
        assert x_min >= dx0 and x_max <= dx1 and y_min >= dy0 and y_max <= dy1
        min_col = int(math.floor((x_min - dx0) / cell_size))
        max_col = int(math.ceil((x_max - dx0) / cell_size)) - 1
        min_row = int(math.floor((dy1 - y_max) / cell_size))
        max_row = int(math.ceil((dy1 - y_min) / cell_size)) - 1
    else:
        min_col, min_row = 0, 0
        max_col = int(math.ceil((x_max - x_min) / cell_size)) - 1
        max_row = int(math.ceil((y_max - y_min) / cell_size)) - 1
    assert 0 <= min_col <= max_col and 0 <= min_row <= max_row
    sx = x_min + 0.5 * cell_size
    ex = sx + (max_col - min_col) * cell_size
    sy = y_max - 0.5 * cell_size
    ey = sy - (max_row - min_row) * cell_size
    xs = np.linspace(sx, ex, max_col - min_col + 1)
    ys = np.linspace(sy, ey, max_row - min_row + 1)
    mx, my = np.meshgrid(xs, ys)
    return dict(rc=(min_col, max_col, min_row, max_row), x_crds=xs, y_crds=ys,
                cell_x=mx.ravel(), cell_y=my.ravel(), shape=mx.shape)


def sample_drifts(rasters, drift_x_min, drift_y_max, cell_size, ndv, rc, stn_x, stn_y,
                  cntn_idxs=None):
    """KrigingDrift._prepare_stns_drift (interp/drift.py:165-227): every
    raster read at the grid's rows and columns (no-data, by np.isclose, to
    NaN), then at each station's cell int((x - x_min) / cs),
    int((y_max - y) / cs); station drifts must be finite."""
    min_col, max_col, min_row, max_row = rc
    cm, rm = np.meshgrid(np.arange(min_col, max_col + 1), np.arange(min_row, max_row + 1))
    cm, rm = cm.ravel(), rm.ravel()
    if cntn_idxs is not None:
        cm, rm = cm[cntn_idxs], rm[cntn_idxs]
    cell = []
    for r in rasters:
        v = r[rm, cm]
        v[np.isclose(ndv, v)] = np.nan
        cell.append(v)
    cell = np.array(cell, dtype=float)
    stn = np.full((len(stn_x), len(rasters)), np.nan)
    for i, (x, y) in enumerate(zip(stn_x, stn_y)):
        col = int((x - drift_x_min) / cell_size)
        row = int((drift_y_max - y) / cell_size)
        for k, r in enumerate(rasters):
            d = r[row, col]
            stn[i, k] = np.nan if np.isclose(ndv, d) else d
    assert np.all(np.isfinite(stn)), "Invalid value(s) of drift(s) for stations in drift rasters!"
    return cell, stn


def _orient(a, b, c, d):
    """exact sign of a*b - c*d for the float64 values a, b, c, d."""
    from fractions import Fraction
    r = Fraction(float(a)) * Fraction(float(b)) - Fraction(float(c)) * Fraction(float(d))
    return (r > 0) - (r < 0)


def points_in_polygons(px, py, polygons):
    """The cell selection of _select_nearby_cells (interp/prepare.py:244-288
    over chk_pt_cntmnt_in_polys_mp / chk_pt_cntmnt_in_poly / cnvt_to_pt /
    chk_cntmt, misc.py:407-500, 617-627): a point, rounded to 1e-6 as
    "POINT (%f %f)" prints it, is kept when it lies strictly inside one of
    the single-ring polygons (ogr Contains: boundary points are outside).
    polygons: list of (xs, ys) vertex arrays, closed from the last vertex
    to the first. Pure-Python loops (small cases only).

    Parity unpinned against the reference itself: ogr is not importable
    here. The crossing-number rule and the boundary test restate the
    definition of Contains."""
    out = np.zeros(len(px), dtype=bool)
    for i, (x0, y0) in enumerate(zip(px, py)):
        x = float(np.rint(x0 * 1e6) / 1e6)
        y = float(np.rint(y0 * 1e6) / 1e6)
        for vx, vy in polygons:
            vx, vy = np.asarray(vx, float), np.asarray(vy, float)
            if not (vx.min() <= x <= vx.max() and vy.min() <= y <= vy.max()):
                continue
            odd, onb = False, False
            nv = len(vx)
            for e in range(nv):
                x1, y1 = vx[e], vy[e]
                x2, y2 = vx[(e + 1) % nv], vy[(e + 1) % nv]
                up1, up2 = y1 > y, y2 > y
                inbox = min(x1, x2) <= x <= max(x1, x2) and min(y1, y2) <= y <= max(y1, y2)
                if up1 == up2 and not inbox:
                    continue
                s = _orient(x2 - x1, y - y1, y2 - y1, x - x1)
                if s == 0 and inbox:
                    onb = True
                    break
                if up1 != up2 and ((s > 0) if y2 > y1 else (s < 0)):
                    odd = not odd
            if odd and not onb:
                out[i] = True
                break
    return out


def field_stats(fld, ddof):
    """Per-row (min, mean, max, std, count) over the finite entries of fld
    [rows, n] (interp/main.py:474-525): numpy's nanmin / nanmean / nanmax /
    nanstd (ddof 0) and isfinite().sum() for the interpolated fields,
    pandas' skip-NaN min / mean / max / std (ddof 1) / count for the station
    data; computed in float64 here."""
    f = np.asarray(fld, dtype=np.float64)
    out = np.full((f.shape[0], 5), np.nan)
    for r in range(f.shape[0]):
        v = f[r][np.isfinite(f[r])]
        out[r, 4] = v.size
        if v.size:
            out[r, 0], out[r, 1], out[r, 2] = v.min(), v.mean(), v.max()
            if v.size > ddof:
                out[r, 3] = v.std(ddof=ddof)
    return out
