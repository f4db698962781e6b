"""CPU restatement of the reference's variogram fitter (variograms/vgs.py).

TEST INFRASTRUCTURE ONLY: the oracle that the GPU fitter is checked against
and the CPU baseline of the fitting benchmark. It follows the reference
step for step for the settings FitVariogramsSteps uses
(variograms/fitvgs.py:187-206: typ 'var', robust estimator, no weights,
opt_iters 10000, fit_thresh 0.01):

- ``pairs``             vgs.py:311-391  all pairs i > j, sorted by distance
                         (numpy quicksort, as pandas sort_values does)
- ``clip_pairs``        vgs.py:597-659  mdr cut-off (numeric mdr branch)
- ``equal_count_bins``  vgs.py:495-520  bins of nk pairs, mean distance
- ``evg_robust``        vgs.py:414-422  Cressie-Hawkins estimator
- ``MODELS``            vgs.py:553-595  model functions, arg = (range, sill)
- ``objective``         vgs.py:661-678  sum of squared differences
- ``fit``               vgs.py:680-870  permutations, bounds, DE, AIC pick,
                         range ordering, n_best, output strings

scipy's differential_evolution is called with the reference's arguments;
the reference passes no seed, so DE draws from numpy's global RNG, which
``fit(seed=...)`` seeds first (pinned against fixtures made the same way by
running the reference, tests/golden/make_golden.py).
"""
from itertools import permutations
from math import pi

import numpy as np


def pairs(x, y, z):
    """[z_i, z_j, d_ij] for i > j (row order), sorted by d."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    z = np.asarray(z, dtype=np.float64)
    i, j = np.tril_indices(z.size, -1)
    d = np.sqrt((x[i] - x[j]) ** 2 + (y[i] - y[j]) ** 2)
    p = np.stack([z[i], z[j], d], axis=1)
    return p[np.argsort(p[:, 2], kind="quicksort")]


def clip_pairs(p, mdr):
    """vgs.py:597-659 for a numeric mdr (uh None). Returns (pairs, max_dist)."""
    act_max = p[:, 2].max()
    max_dist = act_max * mdr
    idx_clip = np.argmin(np.abs(p[:, 2] - max_dist))
    clip_ul = p[idx_clip, 2]
    if not (clip_ul - max_dist) > 0:
        clip_ul = max_dist
    if idx_clip != p.shape[0] - 1:
        d = np.clip(p[:, 2], 0, clip_ul)
        keep = d != clip_ul
        p = p[keep]
    return p, max_dist


def evg_robust(xs, ys):
    nh = xs.shape[0]
    if nh == 0:
        return 0
    evg = ((np.sum((np.abs(xs - ys)) ** 0.5, axis=0)) / nh) ** 4
    return np.divide(evg, (0.457 + (0.494 / nh))) / 2


def evg_classic(xs, ys):
    if xs.shape[0] == 0:
        return np.nan
    return np.median((np.subtract(xs, ys)) ** 2)


def equal_count_bins(p, nk, evg_name="robust"):
    """vgs.py:495-520: (h = mean distance, gamma, pairs per bin)."""
    est = evg_robust if evg_name == "robust" else evg_classic
    h, g, cnt = [], [], []
    for m in range(0, p.shape[0], nk):
        n = p[m:m + nk]
        h.append(np.mean(n[:, 2]))
        g.append(est(n[:, 0], n[:, 1]))
        cnt.append(n.shape[0])
    return np.array(h), np.array(g, dtype=np.float64), np.array(cnt, dtype=np.float64)


def nug_vg(h, arg):
    return np.full(h.shape, arg[1])


def sph_vg(h, arg):
    a = (1.5 * h) / arg[0]
    b = h ** 3 / (2 * arg[0] ** 3)
    out = arg[1] * (a - b)
    out[h > arg[0]] = arg[1]
    return out


def exp_vg(h, arg):
    return arg[1] * (1 - np.exp(-3 * (h / arg[0])))


def lin_vg(h, arg):
    out = arg[1] * (h / arg[0])
    out[h > arg[0]] = arg[1]
    return out


def gau_vg(h, arg):
    return arg[1] * (1 - np.exp(-3 * ((h ** 2 / arg[0] ** 2))))


def pow_vg(h, arg):
    return arg[1] * (h ** arg[0])


def hol_vg(h, arg):
    out = np.zeros(h.shape[0])
    idx = np.where(h > 0)
    a = (pi * h[idx]) / arg[0]
    out[idx] = arg[1] * (1 - (np.sin(a) / a))
    return out


MODELS = {"Nug": nug_vg, "Sph": sph_vg, "Exp": exp_vg, "Lin": lin_vg, "Gau": gau_vg,
          "Pow": pow_vg, "Hol": hol_vg}


def objective(arg, names, h, g, cnt=None, use_wts=False):
    """vgs.py:661-678."""
    mix = np.zeros(h.shape)
    for i, name in enumerate(names):
        mix += MODELS[name](h, arg[i * 2:i * 2 + 2])
    if use_wts:
        return np.sum(cnt / mix ** 2 * np.square(g - mix))
    return np.sum(np.square(g - mix))


def empirical(x, y, z, nk=50, mdr=0.7, evg_name="robust"):
    """Pairs, mdr clip and equal-count bins: (h, gamma, counts, max_dist,
    variance of z)."""
    p = pairs(x, y, z)
    p, max_dist = clip_pairs(p, mdr)
    h, g, cnt = equal_count_bins(p, nk, evg_name)
    return h, g, cnt, max_dist, np.var(np.asarray(z, dtype=np.float64))


def perm_problems(fit_vgs, perm_r_list, fil_nug_vg, h, g, variance):
    """The (names, bounds) of every DE problem _vg_get_vg solves, in order
    (vgs.py:700-760); the range-ordering skip list is applied by ``fit``."""
    mix_list = list(fit_vgs)
    if fil_nug_vg is not None:
        mix_list.append(fil_nug_vg)
    prl = [min(r, len(mix_list)) for r in perm_r_list]
    prl = np.array(np.unique(prl), dtype=int)
    out = []
    lb = 1e-5
    for n in prl:
        for o in permutations(mix_list, int(n)):
            c1 = n == 1
            c2 = (n > 1) and (o[0] == fil_nug_vg)
            if not (c1 or c2):
                continue
            bounds = []
            for pidx, name in enumerate(o):
                if name == "Pow":
                    bounds += [(lb, 2), (lb, 2 * variance)]
                elif c2 and pidx == 0:
                    bounds += [(h[0], h[0]), (g[0], g[0])]
                else:
                    bounds += [(h[0], 1e9), (lb, 2 * variance)]
            out.append((int(n), tuple(o), bounds))
    return out


def fit(x, y, z, *, nk=50, mdr=0.7, perm_r_list=(1, 2), fil_nug_vg="Nug",
        fit_vgs=("Sph", "Exp"), n_best=1, opt_iters=10000, fit_thresh=0.01, seed=None,
        evg_name="robust"):
    """Variogram.fit for FitVariogramsSteps' settings. Returns
    (vg strings best-last, AIC list, best params, names)."""
    from scipy.optimize import differential_evolution

    h, g, cnt, max_dist, variance = empirical(x, y, z, nk, mdr, evg_name)
    tot_pts = np.asarray(z).size
    if seed is not None:
        np.random.seed(seed)
    min_obj = np.inf
    best_names, best_params, best_objs = [], [], []
    skip = []
    for n, o, bounds in perm_problems(fit_vgs, list(perm_r_list), fil_nug_vg, h, g, variance):
        if o in skip:
            continue
        opt = differential_evolution(
            lambda a, names=o: objective(a, names, h, g), tuple(bounds),
            maxiter=opt_iters, popsize=len(bounds) * 50, polish=False)
        rngs = opt.x[0::2].copy()
        sills = opt.x[1::2].copy()
        aic = (tot_pts * np.log(opt.fun)) + (2 * opt.x.shape[0])
        c1 = aic < min_obj * (1.0 - fit_thresh)
        names = list(o)
        if not np.all(np.ediff1d(rngs) >= 0):
            order = np.argsort(rngs)
            rngs, sills = rngs[order], sills[order]
            skip.append(tuple(np.array(o)[order]))
            names = [names[k] for k in order]
        prms = np.zeros(2 * rngs.shape[0])
        prms[0::2] = rngs
        prms[1::2] = sills
        if c1:
            min_obj = aic
            best_names.append(names)
            best_params.append(prms)
            best_objs.append(min_obj)
        if len(best_names) > n_best:
            del best_names[0], best_params[0], best_objs[0]
    strs = []
    for names, prms in zip(best_names, best_params):
        s = ""
        for m, name in enumerate(names):
            s += " + %0.5f %s(%0.5f)" % (prms[2 * m + 1], name, prms[2 * m])
        strs.append(s[3:])
    return strs, best_objs, (best_params[-1] if best_params else None), best_names
