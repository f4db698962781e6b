"""Learned warm start of the variogram fitter (no counterpart in the reference).

The reference fits every step from scratch: a differential evolution over
each model permutation's whole parameter box (variograms/vgs.py:731-764,
ranges up to 1e9). Here a small MLP (20 -> 128 -> 128 -> logits of the
permutations + 3 parameters, FP32, trained and evaluated by the kernels of
csrc/spi_mlp.cu) reads 20 lag-bin features of a step's values and proposes
the permutation the fitter would choose and its parameters. The fitter then
fits only the ``topk`` most likely permutations, each from a narrow initial
box around the proposal (the DE still searches the full bounds), and falls
back to the plain cold fit of every permutation when the proposal explains
the empirical variogram poorly (its objective above ``fallback`` times the
bins' total sum of squares).

Parameters are normalised as (log10(range) - 4, structured sill / variance,
nugget / variance).
"""
import ctypes
import time
from pathlib import Path

import numpy as np
import torch

from . import _native as nat
from .fitvgs import CODES, DeProblem, Empirical, fit_steps, perm_list
from .steps import _ptr, _require_cuda, _stream

DEFAULT_WEIGHTS = Path(__file__).resolve().parent / "data" / "warmstart_mlp.npz"
N_FEAT = 20
N_PAR = 3


def default_perms():
    return perm_list(("Sph", "Exp"), (1, 2), "Nug")


class WarmStartMLP:
    def __init__(self, perms=None, h1=128, h2=128, seed=0, device="cuda"):
        self.dev = _require_cuda(device)
        self.perms = list(perms or default_perms())
        self.n_class = len(self.perms)
        self.dims = (N_FEAT, h1, h2, self.n_class + N_PAR)
        self.n_par = int(nat.lib().spi_mlp_n_params(*self.dims))
        rng = np.random.default_rng(seed)
        p = np.zeros(self.n_par, dtype=np.float32)
        k = 0
        for nin, nout in ((N_FEAT, h1), (h1, h2), (h2, self.dims[3])):
            p[k:k + nin * nout] = rng.normal(0, 1.0 / np.sqrt(nin), nin * nout)
            k += nin * nout + nout
        self.params = torch.as_tensor(p, device=self.dev)
        self.mu = np.zeros(N_FEAT, dtype=np.float32)
        self.sd = np.ones(N_FEAT, dtype=np.float32)

    # ---- persistence
    def save(self, path):
        np.savez(path, params=self.params.cpu().numpy(), mu=self.mu, sd=self.sd,
                 dims=np.array(self.dims), perms=np.array(["+".join(o) for o in self.perms]))

    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS, device="cuda"):
        z = np.load(path)
        perms = [tuple(s.split("+")) for s in z["perms"]]
        m = cls(perms=perms, h1=int(z["dims"][1]), h2=int(z["dims"][2]), device=device)
        m.params = torch.as_tensor(z["params"], device=m.dev)
        m.mu, m.sd = z["mu"].astype(np.float32), z["sd"].astype(np.float32)
        return m

    # ---- kernels
    def _x(self, feat):
        x = (np.asarray(feat, dtype=np.float32) - self.mu) / self.sd
        return torch.as_tensor(np.ascontiguousarray(x), device=self.dev)

    def forward(self, feat):
        X = self._x(feat)
        B = X.shape[0]
        d = self.dims
        ws = torch.empty(B * (d[1] + d[2] + 2 * d[3] + d[2] + d[1]), dtype=torch.float32,
                         device=self.dev)
        O = torch.empty((B, d[3]), dtype=torch.float32, device=self.dev)
        nat.call("spi_mlp_forward", *d, self.n_class, _ptr(self.params), _ptr(X), B, _ptr(ws),
                 _ptr(O), _stream())
        return O.cpu().numpy()

    def loss_grad(self, X, cls, yp, mask, wp=1.0):
        B = X.shape[0]
        d = self.dims
        ws = torch.empty(B * (d[1] + d[2] + 2 * d[3] + d[2] + d[1]), dtype=torch.float32,
                         device=self.dev)
        grad = torch.empty(self.n_par, dtype=torch.float32, device=self.dev)
        loss = torch.empty(B, dtype=torch.float32, device=self.dev)
        nat.call("spi_mlp_grad", *d, self.n_class, _ptr(self.params), _ptr(X), _ptr(cls),
                 _ptr(yp), _ptr(mask), float(wp), B, _ptr(ws), _ptr(grad), _ptr(loss),
                 _stream())
        return loss, grad

    def train(self, feat, cls, yp, mask, *, epochs=200, batch=256, lr=2e-3, wp=1.0, seed=0):
        """Adam on minibatches; returns the per-epoch mean loss."""
        feat = np.asarray(feat, dtype=np.float32)
        self.mu = feat.mean(0)
        self.sd = feat.std(0) + 1e-6
        X = self._x(feat)
        C = torch.as_tensor(np.asarray(cls, dtype=np.int32), device=self.dev)
        Y = torch.as_tensor(np.asarray(yp, dtype=np.float32), device=self.dev)
        M = torch.as_tensor(np.asarray(mask, dtype=np.float32), device=self.dev)
        m = torch.zeros_like(self.params)
        v = torch.zeros_like(self.params)
        rng = np.random.default_rng(seed)
        n = X.shape[0]
        t = 0
        hist = []
        for _ in range(epochs):
            order = torch.as_tensor(rng.permutation(n), device=self.dev)
            tot = 0.0
            for s in range(0, n, batch):
                idx = order[s:s + batch]
                xb, cb = X[idx].contiguous(), C[idx].contiguous()
                yb, mb = Y[idx].contiguous(), M[idx].contiguous()
                loss, grad = self.loss_grad(xb, cb, yb, mb, wp)
                t += 1
                nat.call("spi_mlp_adam", _ptr(self.params), _ptr(grad), _ptr(m), _ptr(v),
                         self.n_par, lr, 0.9, 0.999, 1e-8, t, _stream())
                tot += float(loss.sum()) * xb.shape[0]
            hist.append(tot / n)
        return hist


def step_features(points, steps, device="cuda"):
    """Features [len(steps), 20] of the given steps' points (GPU)."""
    dev = _require_cuda(device)
    xs, ys, zs = [], [], []
    for t in steps:
        x, y, z = points[t]
        xs.append(np.asarray(x, dtype=np.float64))
        ys.append(np.asarray(y, dtype=np.float64))
        zs.append(np.asarray(z, dtype=np.float64))
    off = np.concatenate([[0], np.cumsum([z.size for z in zs])]).astype(np.int64)
    t_ = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    d_off, dx, dy, dz = t_(off, torch.int64), t_(np.concatenate(xs)), t_(np.concatenate(ys)), t_(
        np.concatenate(zs))
    feat = torch.empty((len(steps), N_FEAT), dtype=torch.float32, device=dev)
    nat.call("spi_vg_features", len(steps), _ptr(d_off), _ptr(dx), _ptr(dy), _ptr(dz), N_FEAT,
             _ptr(feat), _stream())
    return feat.cpu().numpy()


def labels(details, points, perms):
    """Training labels from the plain fitter's choices: class = chosen
    permutation, parameters (log10 range - 4, structured sill / var,
    nugget / var) with a mask of the ones the class has. points: per-step
    (x, y, z) as fitted."""
    cls, yp, mk, keep = [], [], [], []
    for t, det in details.items():
        if not isinstance(t, int) or det["names"] is None:
            continue
        names, prm = tuple(det["names"]), det["params"]
        if names not in perms:
            continue
        z = np.asarray(points[t][2])
        var = max(np.var(z), 1e-300)
        y = np.zeros(N_PAR)
        m = np.zeros(N_PAR)
        for k, name in enumerate(names):
            r, s = prm[2 * k], prm[2 * k + 1]
            if name == "Nug":
                y[2], m[2] = s / var, 1
            else:
                y[0], m[0] = np.log10(max(r, 1.0)) - 4.0, 1
                y[1], m[1] = s / var, 1
        cls.append(perms.index(names))
        yp.append(y)
        mk.append(m)
        keep.append(t)
    return (np.array(keep), np.array(cls, dtype=np.int32), np.array(yp, dtype=np.float32),
            np.array(mk, dtype=np.float32))


def _unit(v, lo, hi):
    return float(np.clip((v - lo) / (hi - lo), 0.0, 1.0)) if hi > lo else 0.0


def _model(name, h, r, s):
    """The fitter's models (variograms/vgs.py:553-595), arg (range, sill)."""
    if name == "Nug":
        return np.full(h.shape, s)
    if name == "Exp":
        return s * (1 - np.exp(-3 * (h / r)))
    if name == "Gau":
        return s * (1 - np.exp(-3 * (h / r) ** 2))
    if name == "Sph":
        out = s * (1.5 * h / r - h ** 3 / (2 * r ** 3))
        out[h > r] = s
        return out
    if name == "Lin":
        out = s * (h / r)
        out[h > r] = s
        return out
    raise ValueError(name)


def _proposal(o, h0, g0, var, rng, ssill, nug, fil_nug_vg="Nug"):
    """(range, sill) per component of permutation o for the proposal."""
    prm = []
    for k, name in enumerate(o):
        if len(o) > 1 and k == 0 and name == fil_nug_vg:
            prm.append((h0, g0))
        elif name == "Nug":
            prm.append((h0, ssill + nug))
        else:
            prm.append((rng, ssill))
    return prm


def warm_fit_steps(stn_x, stn_y, data, mlp, *, topk=1, fallback=0.5, range_fac=1.6,
                   sill_fac=0.3, seed=0, opt_iters=10000, tol=0.01, nk=50, mdr=0.7,
                   device="cuda", points=None):
    """Warm-started fit: the MLP's top-k permutations from narrow initial
    boxes, the plain cold fit of all permutations where the proposal's
    objective exceeds ``fallback`` times the bins' total sum of squares.
    Returns (strings per step, details) like fit_steps, with
    details["_fallback_steps"] and details["_ms"] (features, network, DE)."""
    from .fitvgs import step_points
    t0 = time.perf_counter()
    if points is None:
        points = step_points(stn_x, stn_y, data)
    emp = Empirical(None, None, None, nk=nk, mdr=mdr, device=device, points=points).run()
    steps = [int(s) for s in emp.steps]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    feat = step_features(points, steps, device=device)
    O = mlp.forward(feat)
    e1.record()
    logits, pr = O[:, :mlp.n_class], O[:, mlp.n_class:]
    warm, step_perms, fall = {}, {}, []
    for k, t in enumerate(steps):
        h, g, _ = emp.bins(k)
        var = emp.var2[k] / 2
        lo_r, hi_r, lo_s, hi_s = h[0], 1e9, 1e-5, 2 * var
        order = [int(i) for i in np.argsort(-logits[k])[:topk]]
        rng = 10 ** (float(pr[k, 0]) + 4.0)
        ssill = max(float(pr[k, 1]), 1e-6) * var
        nug = max(float(pr[k, 2]), 0.0) * var
        o = mlp.perms[order[0]]
        prm = _proposal(o, h[0], g[0], var, rng, ssill, nug)
        model = sum(_model(name, h, r, s) for name, (r, s) in zip(o, prm))
        obj = np.sum((g - model) ** 2)
        tss = np.sum((g - g.mean()) ** 2)
        if not (obj <= fallback * tss):
            fall.append(t)
            continue
        step_perms[t] = [mlp.perms[i] for i in order]
        for i in order:
            oi = mlp.perms[i]
            lo, hi = np.zeros(4), np.ones(4)
            for c, ((r, sl), name) in enumerate(zip(_proposal(oi, h[0], g[0], var, rng, ssill,
                                                              nug), oi)):
                if len(oi) > 1 and c == 0 and name == "Nug":
                    continue
                if name != "Nug":
                    lo[2 * c] = _unit(r / range_fac, lo_r, hi_r)
                    hi[2 * c] = _unit(r * range_fac, lo_r, hi_r)
                lo[2 * c + 1] = _unit(sl * (1 - sill_fac), lo_s, hi_s)
                hi[2 * c + 1] = _unit(sl * (1 + sill_fac), lo_s, hi_s)
            warm[(t, oi)] = (lo, hi)
    out, det = fit_steps(stn_x, stn_y, data, seed=seed, warm=warm, step_perms=step_perms,
                         emp=emp, opt_iters=opt_iters, tol=tol, device=device,
                         return_details=True)
    torch.cuda.synchronize()
    det["_fallback_steps"] = fall
    det["_ms"] = {"features_and_network": e0.elapsed_time(e1), "de": det["_de_ms"],
                  "wall": (time.perf_counter() - t0) * 1e3}
    return out, det
