"""The reference's answer for one kriging system, and its spread under tiny
perturbations of the system matrix.

TEST INFRASTRUCTURE ONLY (built on the oracle, oracle/port.py).

The reference inverts every kriging system with numpy.linalg.pinv
(interp/steps.py:351-352) and applies it per cell (interp/steps.py:403-435:
lambda = P r, the isclose(sum(lambda[:n]), 1) check with nearest-station
fallback, est = lambda[:n] . z, var = lambda . r + lambda[n]). Where the
matrix is badly conditioned that answer is set by rounding. This module
measures how far: it re-runs the same per-cell formulas with pinv of the
matrix under K symmetric relative perturbations of 1e-15 (a few ulp of
every entry) and returns every run, so a test can ask whether the GPU's
answer lies inside the reference's own spread.

The per-cell formulas are applied to all cells at once (one matrix
product) instead of the reference's cell loop; that changes only the
order of the additions (~1e-16 relative), far below the spreads measured.
"""
import warnings

import numpy as np

from oracle import port

def system(kind, sx, sy, idx, cx, cy, vg, min_vg_val, stn_drifts=None, cell_drifts=None):
    """The reference's system for station subset ``idx``: (LHS [m, m], cell
    right-hand sides [C, m], cell-station distances [C, n]), built with the
    oracle's restatement of interp/steps.py:170-243."""
    idx = np.asarray(idx)
    d_ss = port.get_dists_arr(sx[idx], sy[idx], sx[idx], sy[idx])
    d_cs = port.get_dists_arr(cx, cy, sx[idx], sy[idx])
    flag = 1 if kind == "SK" else 0
    rr_all = {(vg, flag): port.fill_vg_var_arr(d_ss, flag, 1, vg, min_vg_val)}
    dr_all = {(vg, flag): port.fill_vg_var_arr(d_cs, flag, 0, vg, min_vg_val)}
    sd = None if stn_drifts is None else np.asarray(stn_drifts)[idx]
    lhs, rhs = port.get_vars_arr_subset(vg, kind, sd, rr_all, dr_all, np.arange(idx.size),
                                        np.arange(cx.size), cell_drifts)
    return lhs, rhs, d_cs


def singular_to_pinv(lhs):
    """Whether numpy.linalg.pinv's default cut-off (rcond 1e-15: singular
    values <= 1e-15 s_max are dropped) drops a singular value of ``lhs``,
    and its condition number. The singular values come from the same SVD
    call pinv makes (with singular vectors): for an exactly singular
    matrix the null singular value is rounding noise of a few eps s_max,
    near the cut-off, and the SVD without vectors computes a different
    one."""
    s = np.linalg.svd(lhs, full_matrices=False)[1]
    return bool((s <= 1e-15 * s[0]).any()), float(s[0] / max(s[-1], 1e-300))


def outcome(P, rhs, n, vals, d_cs, want_var):
    """interp/steps.py:403-435 for every cell and step: (est [T, C],
    var [C] or None, passed [C]); ``vals`` [T, n]."""
    lam = rhs @ P.T
    passed = np.isclose(lam[:, :n].sum(1), 1.0)
    nearest = vals[:, np.argmin(d_cs, 1)]
    est = np.where(passed[None], vals @ lam[:, :n].T, nearest)
    var = None
    if want_var:
        var = np.where(passed, (lam * rhs).sum(1) + lam[:, n], 0.0)
    return est, var, passed


def runs(lhs, rhs, n, vals, d_cs, want_var, k=4, seed=0):
    """The reference's outcome on the matrix as given, then under ``k``
    symmetric relative perturbations of 1e-15 (a pinv failure gives the
    reference's nearest-station fill for every cell)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(k + 1):
        m = lhs
        if i:
            e = rng.standard_normal(lhs.shape)
            m = lhs * (1.0 + 1e-15 * (e + e.T) / 2)
        try:
            P = np.linalg.pinv(m)
        except np.linalg.LinAlgError:
            c = d_cs.shape[0]
            out.append((vals[:, np.argmin(d_cs, 1)], np.zeros(c) if want_var else None,
                        np.zeros(c, dtype=bool)))
            continue
        out.append(outcome(P, rhs, n, vals, d_cs, want_var))
    return out


def spread(rs, scale):
    """Largest change of the estimates (and variances) over the perturbed
    runs, relative to ``scale`` (estimates) and the variance's largest
    magnitude."""
    e0, v0, _ = rs[0]
    de = max(float(np.abs(r[0] - e0).max()) for r in rs[1:]) / scale
    dv = 0.0
    if v0 is not None:
        vs = max(float(np.abs(v0).max()), 1e-300)
        dv = max(float(np.abs(r[1] - v0).max()) for r in rs[1:]) / vs
    return de, dv


def consistent(got, rs, vals, d_cs, slack):
    """Per (step, cell): whether the GPU's estimate ``got`` [T, C] is one
    of the reference's outcomes across the runs: the nearest station's
    value (exactly) where some run fell back, or a value inside the passing
    runs' range widened by its own width plus ``slack``."""
    nearest = vals[:, np.argmin(d_cs, 1)]
    passed = np.array([r[2] for r in rs])              # [K+1, C]
    ests = np.array([r[0] for r in rs])                # [K+1, T, C]
    any_fail = (~passed).any(0)[None]
    big = np.where(passed[:, None, :], ests, np.nan)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)  # cells no run passed
        lo = np.nanmin(big, 0)
        hi = np.nanmax(big, 0)
    w = np.nan_to_num(hi - lo) + slack
    inside = np.isfinite(lo) & (got >= lo - w) & (got <= hi + w)
    return (any_fail & (got == nearest)) | inside
