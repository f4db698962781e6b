"""GPU variogram fitting: the reference's FitVariograms for all steps at once.

Mirrors ``variograms/fitvgs.py`` (FitVariogramsSteps._fit_vgs_step,
143-278) and ``variograms/vgs.py`` (Variogram with fitvgs' settings):

- per step, the stations with a value (optionally without zeros, 164-178);
  steps with fewer than ``min_vld_stns`` stations or with numpy.isclose(std,
  0) get no variogram (160-184);
- empirical variograms of every step in one batch on the GPU
  (``spi_vg_empirical``: pairs, sort, mdr cut-off, bins of nk pairs, robust
  estimator);
- every model permutation of ``vgs.py:_vg_get_vg`` (680-764) for every
  step as one batched differential-evolution launch (``spi_vg_de``);
- the AIC selection, range ordering, skip list, n_best bookkeeping and the
  ``'%0.5f %s(%0.5f)'`` strings of vgs.py:766-848, on the host (a few
  numbers per step).

The DE is the reference's algorithm family (scipy's best1bin, population
50 D^2, dithered F, CR 0.7, same stopping rule) but not scipy's random
stream, so fits agree with the reference in objective value, not bit for bit.
"""
import ctypes
from itertools import permutations

import numpy as np
import torch

from . import _native as nat
from .steps import _ptr, _require_cuda, _stream

CODES = {"Rng": 0, "Nug": 1, "Sph": 2, "Exp": 3, "Lin": 4, "Gau": 5, "Pow": 6, "Hol": 7}


class DeProblem(ctypes.Structure):
    _fields_ = [("step", ctypes.c_int32), ("n_comp", ctypes.c_int32),
                ("code", ctypes.c_int32 * 2), ("fixed_first", ctypes.c_int32),
                ("warm", ctypes.c_int32), ("var2", ctypes.c_double), ("seed", ctypes.c_uint64),
                ("warm_lo", ctypes.c_double * 4), ("warm_hi", ctypes.c_double * 4)]


class VgEmpWs(ctypes.Structure):
    _fields_ = [("pd", ctypes.c_void_p), ("pp", ctypes.c_void_p), ("sd", ctypes.c_void_p),
                ("bcnt", ctypes.c_void_p), ("bstart", ctypes.c_void_p),
                ("bcur", ctypes.c_void_p)]


def perm_list(fit_vgs, perm_r_list, fil_nug_vg):
    """The permutations _vg_get_vg fits, in its order (vgs.py:700-730)."""
    mix = list(fit_vgs)
    if fil_nug_vg is not None:
        mix.append(fil_nug_vg)
    prl = np.array(np.unique([min(r, len(mix)) for r in perm_r_list]), dtype=int)
    out = []
    for n in prl:
        for o in permutations(mix, int(n)):
            if n == 1 or o[0] == fil_nug_vg:
                out.append(tuple(o))
    return out


def step_points(stn_x, stn_y, data, drop_zeros=False, min_vld_stns=1):
    """Per step, the (x, y, z) of the stations with a value, as
    FitVariogramsSteps selects them (variograms/fitvgs.py:149-184); steps
    that get no variogram map to None."""
    data = np.asarray(data, dtype=np.float64)
    stn_x = np.asarray(stn_x, dtype=np.float64)
    stn_y = np.asarray(stn_y, dtype=np.float64)
    pts = []
    for t in range(data.shape[0]):
        idx = np.where(np.isfinite(data[t]))[0]
        z = data[t, idx]
        if drop_zeros:
            keep = z != 0
            idx, z = idx[keep], z[keep]
        if idx.size < max(min_vld_stns, 2) or np.isclose(z.std(), 0.0):
            pts.append(None)
            continue
        pts.append((stn_x[idx], stn_y[idx], z))
    return pts


class Empirical:
    """Device-resident empirical variograms of a batch of steps."""

    def __init__(self, stn_x, stn_y, data, *, nk=50, mdr=0.7, drop_zeros=False,
                 min_vld_stns=1, device="cuda", points=None):
        dev = self.dev = _require_cuda(device)
        if points is None:
            points = step_points(stn_x, stn_y, data, drop_zeros, min_vld_stns)
        self.T = len(points)
        self.nk, self.mdr = int(nk), float(mdr)
        steps, xs, ys, zs, var2 = [], [], [], [], []
        for t, p in enumerate(points):
            if p is None:
                continue
            x, y, z = (np.asarray(a, dtype=np.float64) for a in p)
            steps.append(t)
            xs.append(x)
            ys.append(y)
            zs.append(z)
            var2.append(2 * np.var(z))
        self.steps = np.array(steps, dtype=np.int64)
        self.var2 = np.array(var2)
        self.n_pts = np.array([z.size for z in zs], dtype=np.int64)
        S = self.S = len(steps)
        if S == 0:
            return
        npair = self.n_pts * (self.n_pts - 1) // 2
        nbkt = np.maximum(1, npair // 4)
        nbin = (npair + nk - 1) // nk
        off = lambda a: np.concatenate([[0], np.cumsum(a)]).astype(np.int64)
        self.pt_off, self.pair_off, self.bkt_off, self.bin_off = (
            off(self.n_pts), off(npair), off(nbkt), off(nbin))
        dmax = np.array([np.hypot(np.ptp(x), np.ptp(y)) for x, y in zip(xs, ys)])
        dmax = np.maximum(dmax, 1e-300) * (1 + 1e-9)
        t = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt,
                                                        device=dev)
        self.d_pt_off, self.d_pair_off = t(self.pt_off, torch.int64), t(self.pair_off, torch.int64)
        self.d_bkt_off, self.d_bin_off = t(self.bkt_off, torch.int64), t(self.bin_off, torch.int64)
        self.d_x, self.d_y, self.d_z = t(np.concatenate(xs)), t(np.concatenate(ys)), t(
            np.concatenate(zs))
        self.d_dmax = t(dmax)
        P, B, NB = int(self.pair_off[-1]), int(self.bkt_off[-1]), int(self.bin_off[-1])
        self.pd = torch.empty(P, dtype=torch.float64, device=dev)
        self.pp = torch.empty(P, dtype=torch.int32, device=dev)
        self.sd = torch.empty(P, dtype=torch.float64, device=dev)
        self.bcnt = torch.zeros(B, dtype=torch.int32, device=dev)
        self.bstart = torch.empty(B, dtype=torch.int32, device=dev)
        self.bcur = torch.empty(B, dtype=torch.int32, device=dev)
        self.bin_h = torch.zeros(NB, dtype=torch.float64, device=dev)
        self.bin_g = torch.zeros(NB, dtype=torch.float64, device=dev)
        self.bin_n = torch.zeros(NB, dtype=torch.float64, device=dev)
        self.n_bins = torch.zeros(S, dtype=torch.int32, device=dev)
        self.max_dist = torch.zeros(S, dtype=torch.float64, device=dev)
        self.ws = VgEmpWs(*[_ptr(a) for a in (self.pd, self.pp, self.sd, self.bcnt,
                                               self.bstart, self.bcur)])
        self._max_p, self._max_b = int(npair.max()), int(nbkt.max())

    def run(self):
        if self.S == 0:
            return self
        self.bcnt.zero_()
        nat.call("spi_vg_empirical", self.S, _ptr(self.d_pt_off), _ptr(self.d_x), _ptr(self.d_y),
                 _ptr(self.d_z), _ptr(self.d_pair_off), _ptr(self.d_bkt_off), _ptr(self.d_dmax),
                 self._max_p, self._max_b, self.nk, self.mdr, ctypes.byref(self.ws),
                 _ptr(self.d_bin_off), _ptr(self.bin_h), _ptr(self.bin_g), _ptr(self.bin_n),
                 _ptr(self.n_bins), _ptr(self.max_dist), _stream())
        return self

    def bins(self, k):
        """(h, gamma, counts) of the k-th fitted step, as numpy."""
        nb = int(self.n_bins[k].item())
        o = int(self.bin_off[k])
        return (self.bin_h[o:o + nb].cpu().numpy(), self.bin_g[o:o + nb].cpu().numpy(),
                self.bin_n[o:o + nb].cpu().numpy())


def fit_steps(stn_x, stn_y, data, *, nk=50, mdr=0.7, perm_r_list=(1, 2), fil_nug_vg="Nug",
              fit_vgs=("Sph", "Exp"), n_best=1, opt_iters=10000, tol=0.01, fit_thresh=0.01,
              drop_zeros=False, min_vld_stns=1, seed=0, warm=None, step_perms=None,
              emp=None, device="cuda", return_details=False):
    """Fit every step's variogram. Returns a list (one per step) of the
    n_best variogram strings, best last (None where the reference fits
    nothing). ``warm``: optional {(step, perm tuple): (lo[4], hi[4])} initial
    population boxes in unit-cube coordinates; ``step_perms``: optional
    {step: [perm tuples]} to fit only those permutations of a step (both for
    the learned warm start); ``emp``: an already computed Empirical."""
    if emp is None:
        emp = Empirical(stn_x, stn_y, data, nk=nk, mdr=mdr, drop_zeros=drop_zeros,
                        min_vld_stns=min_vld_stns, device=device).run()
    T = emp.T
    out = [None] * T
    details = {}
    if emp.S == 0:
        return (out, details) if return_details else out
    perms = perm_list(fit_vgs, perm_r_list, fil_nug_vg)
    if any(len(o) > 2 for o in perms):
        raise ValueError("the GPU fitter fits at most two nested components (perm_r_list <= 2)")
    probs, plist = [], []
    for k in range(emp.S):
        sp = perms if step_perms is None else step_perms.get(int(emp.steps[k]), perms)
        plist.append(sp)
        for o in sp:
            pi = perms.index(o)
            p = DeProblem()
            p.step = k
            p.n_comp = len(o)
            for c, name in enumerate(o):
                p.code[c] = CODES[name]
            p.fixed_first = 1 if (len(o) > 1 and o[0] == fil_nug_vg) else 0
            p.var2 = float(emp.var2[k])
            p.seed = (int(seed) * 1000003 + int(emp.steps[k]) * 131 + pi) & 0xFFFFFFFFFFFFFFFF
            box = None if warm is None else warm.get((int(emp.steps[k]), o))
            if box is not None:
                p.warm = 1
                for j in range(4):
                    p.warm_lo[j], p.warm_hi[j] = float(box[0][j]), float(box[1][j])
            probs.append(p)
    raw = bytes((DeProblem * len(probs))(*probs))
    d_prob = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(emp.dev)
    best_x = torch.zeros((len(probs), 4), dtype=torch.float64, device=emp.dev)
    best_f = torch.zeros(len(probs), dtype=torch.float64, device=emp.dev)
    n_gen = torch.zeros(len(probs), dtype=torch.int32, device=emp.dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    nat.call("spi_vg_de", len(probs), _ptr(d_prob), _ptr(emp.d_bin_off), _ptr(emp.n_bins),
             _ptr(emp.bin_h), _ptr(emp.bin_g), int(opt_iters), float(tol), _ptr(best_x),
             _ptr(best_f), _ptr(n_gen), _stream())
    ev1.record()
    bx = best_x.cpu().numpy()
    bf = best_f.cpu().numpy()
    ng = n_gen.cpu().numpy()
    details["_de_ms"] = ev0.elapsed_time(ev1)
    details["_de_problems"] = len(probs)
    details["_de_member_evals"] = int(sum(50 * (2 * p.n_comp) ** 2 * int(g_)
                                          for p, g_ in zip(probs, ng)))
    q = 0
    for k in range(emp.S):
        tot_pts = int(emp.n_pts[k])
        min_obj = np.inf
        best_names, best_params, best_objs, skip = [], [], [], []
        sp = plist[k]
        for o in sp:
            x, f = bx[q], bf[q]
            q += 1
            if o in skip:
                continue
            nc = len(o)
            rngs = x[0:2 * nc:2].copy()
            sills = x[1:2 * nc:2].copy()
            aic = tot_pts * np.log(f) + 2 * (2 * nc)
            c1 = aic < min_obj * (1.0 - fit_thresh)
            names = list(o)
            if not np.all(np.ediff1d(rngs) >= 0):
                order = np.argsort(rngs)
                rngs, sills = rngs[order], sills[order]
                skip.append(tuple(np.array(o)[order]))
                names = [names[i] for i in order]
            prms = np.zeros(2 * nc)
            prms[0::2], prms[1::2] = rngs, sills
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
        t = int(emp.steps[k])
        out[t] = strs
        details[t] = {"aic": best_objs, "params": best_params[-1] if best_params else None,
                      "names": best_names[-1] if best_names else None,
                      "objective": {sp[i]: float(bf[q - len(sp) + i]) for i in range(len(sp))},
                      "generations": {sp[i]: int(ng[q - len(sp) + i]) for i in range(len(sp))}}
    return (out, details) if return_details else out
