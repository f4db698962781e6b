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
every entry), with numpy's cut-off and with one at 1e-13 (singular values
that close to zero are rounding noise, and where they fall against the
1e-15 cut-off depends on the platform's LAPACK), and returns every run, so
a test can ask whether the GPU's answer lies inside the reference's own
spread.

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


# numpy.linalg.pinv's default cut-off, and the widest cut-off within
# rounding reach of it: an exactly singular matrix's null singular values
# come out of the SVD as rounding noise of about eps to 16 eps times s_max
# (the LAPACK build and the platform decide where), on either side of
# numpy's 1e-15
RCOND = 1e-15
RCOND_NOISE = 1e-13


def singular_to_pinv(lhs):
    """Whether ``lhs`` has singular values within rounding reach of
    numpy.linalg.pinv's cut-off (<= 1e-13 s_max; pinv itself drops those
    <= 1e-15 s_max, decided there by rounding), and its condition number."""
    s = np.linalg.svd(lhs, full_matrices=False)[1]
    return bool((s <= RCOND_NOISE * s[0]).any()), float(s[0] / max(s[-1], 1e-300))


def pinv_cuts(lhs):
    """Whether numpy.linalg.pinv (rcond 1e-15) drops a singular value of
    ``lhs`` on this platform: the same SVD call pinv makes."""
    s = np.linalg.svd(lhs, full_matrices=False)[1]
    return bool((s <= RCOND * s[0]).any())


def _pinvs(m, rconds):
    """numpy.linalg.pinv's computation (the SVD with vectors, singular
    values <= rcond s_max dropped) for several cut-offs from one SVD."""
    u, s, vt = np.linalg.svd(m, full_matrices=False)
    out = []
    for rc in rconds:
        inv = np.where(s > rc * s[0], 1.0 / np.where(s > 0, s, 1.0), 0.0)
        out.append((vt.T * inv) @ u.T)
    return out


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
    symmetric relative perturbations of 1e-15, each with numpy's cut-off
    (1e-15) and, after those, each again with the cut-off at 1e-13 (an
    SVD failure gives the reference's nearest-station fill for every
    cell). Runs 0 .. k are numpy.linalg.pinv's own; the others add the
    outcomes in which the singular values within rounding reach of the
    cut-off are dropped."""
    rng = np.random.default_rng(seed)
    own, wide = [], []
    c = d_cs.shape[0]
    fail = (vals[:, np.argmin(d_cs, 1)], np.zeros(c) if want_var else None,
            np.zeros(c, dtype=bool))
    for i in range(k + 1):
        m = lhs
        if i:
            e = rng.standard_normal(lhs.shape)
            m = lhs * (1.0 + 1e-15 * (e + e.T) / 2)
        try:
            P, Pw = _pinvs(m, (RCOND, RCOND_NOISE))
        except np.linalg.LinAlgError:
            own.append(fail)
            wide.append(fail)
            continue
        own.append(outcome(P, rhs, n, vals, d_cs, want_var))
        wide.append(outcome(Pw, rhs, n, vals, d_cs, want_var))
    return own + wide


def spread(rs, scale):
    """Largest change of the estimates (and variances) over the runs,
    relative to ``scale`` (estimates) and the variance's largest
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
