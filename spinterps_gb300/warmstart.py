"""Learned warm start of the variogram fitter (no counterpart in the reference).

The reference fits every step from scratch: a differential evolution over
each model permutation's whole parameter box (variograms/vgs.py:731-764,
ranges up to 1e9). Here a small MLP (20 -> 128 -> 128 -> logits of the
permutations + 3 parameters, FP32, trained and evaluated by the kernels of
csrc/spi_mlp.cu) reads 20 lag-bin features of a step's values and proposes
the permutation the fitter would choose and its parameters. Each proposal
is refined on the GPU (spi_vg_refine: for the proposed permutation's one
free structure the least-squares sill is closed form at any range, so the
range is searched within a factor ``span`` of the network's). The fitter
then fits only the ``topk`` most likely permutations, each from a narrow
initial box around its refined proposal (the DE still searches the full
bounds), and falls back to the plain cold fit of every permutation when
the refined top proposal explains the empirical variogram poorly: its
objective (the fitter's sum of squared bin residuals) above ``fallback``
times the bins' noise, the sum of squares that scatter alone leaves,
estimated from successive bin differences as
nb/(nb-1) * sum((g[i+1] - g[i])^2) / 2 (bin_noise). A correct model scores
about 1 on that scale.

Parameters are normalised as (log10(range / hmax), structured sill /
variance, nugget / variance), hmax = half the diagonal of the stations'
bounding box (the features' lag scale), so the network does not depend on
the size of the station network's box.
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


def lag_scale(x, y):
    """hmax of the features: half the diagonal of the points' bounding box."""
    x, y = np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64)
    return max(0.5 * float(np.hypot(np.ptp(x), np.ptp(y))), 1e-300)


def labels(details, points, perms):
    """Training labels from the plain fitter's choices: class = chosen
    permutation, parameters (log10(range / hmax), structured sill / var,
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
        hmax = lag_scale(points[t][0], points[t][1])
        y = np.zeros(N_PAR)
        m = np.zeros(N_PAR)
        for k, name in enumerate(names):
            r, s = prm[2 * k], prm[2 * k + 1]
            if name == "Nug":
                y[2], m[2] = s / var, 1
            else:
                y[0], m[0] = np.log10(max(r, 1e-300) / hmax), 1
                y[1], m[1] = s / var, 1
        cls.append(perms.index(names))
        yp.append(y)
        mk.append(m)
        keep.append(t)
    return (np.array(keep), np.array(cls, dtype=np.int32), np.array(yp, dtype=np.float32),
            np.array(mk, dtype=np.float32))


def _unit(v, lo, hi):
    return float(np.clip((v - lo) / (hi - lo), 0.0, 1.0)) if hi > lo else 0.0


def bin_noise(g):
    """Sum of squares of the bins' scatter about a smooth curve, from
    successive differences (a smooth trend adds only second-order terms)."""
    g = np.asarray(g, dtype=np.float64)
    nb = g.size
    if nb < 3:
        return 0.0
    return 0.5 * float(np.sum(np.diff(g) ** 2)) * nb / (nb - 1)


def warm_fit_steps(stn_x, stn_y, data, mlp, *, topk=1, fallback=4.0, span=4.0, range_fac=1.25,
                   sill_fac=0.1, seed=0, opt_iters=10000, tol=0.01, nk=50, mdr=0.7,
                   device="cuda", points=None):
    """Warm-started fit. Per step: the MLP's top-k permutations, each with its
    proposal refined on the GPU (spi_vg_refine: least-squares sill, range
    searched within a factor ``span`` of the network's), then the fitter's
    differential evolution from a box of ``range_fac`` / ``sill_fac`` around
    it. Steps whose refined top proposal has an objective above ``fallback``
    times the bins' noise get the plain cold fit of every permutation.
    Returns (strings per step, details) like fit_steps, with
    details["_fallback_steps"] and details["_ms"] (features + network +
    refinement, DE, wall)."""
    from .fitvgs import step_points
    t0 = time.perf_counter()
    if points is None:
        points = step_points(stn_x, stn_y, data)
    emp = Empirical(None, None, None, nk=nk, mdr=mdr, device=device, points=points).run()
    steps = [int(s) for s in emp.steps]
    S = len(steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    feat = step_features(points, steps, device=device)
    O = mlp.forward(feat)
    logits, pr = O[:, :mlp.n_class], O[:, mlp.n_class:]
    order = np.argsort(-logits, axis=1)[:, :topk]
    probs, r0 = [], []
    for k, t in enumerate(steps):
        hmax = lag_scale(points[t][0], points[t][1])
        for i in order[k]:
            o = mlp.perms[int(i)]
            p = DeProblem()
            p.step = k
            p.n_comp = len(o)
            for c, name in enumerate(o):
                p.code[c] = CODES[name]
            p.fixed_first = 1 if (len(o) > 1 and o[0] == "Nug") else 0
            p.var2 = float(emp.var2[k])
            probs.append(p)
            r0.append(10 ** float(pr[k, 0]) * hmax)
    raw = bytes((DeProblem * len(probs))(*probs))
    d_prob = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(emp.dev)
    d_r0 = torch.as_tensor(np.array(r0, dtype=np.float64), device=emp.dev)
    P = len(probs)
    x = torch.empty((P, 4), dtype=torch.float64, device=emp.dev)
    f = torch.empty(P, dtype=torch.float64, device=emp.dev)
    nz = torch.empty(P, dtype=torch.float64, device=emp.dev)
    nat.call("spi_vg_refine", P, _ptr(d_prob), _ptr(emp.d_bin_off), _ptr(emp.n_bins),
             _ptr(emp.bin_h), _ptr(emp.bin_g), _ptr(d_r0), float(span), _ptr(x), _ptr(f),
             _ptr(nz), _stream())
    e1.record()
    x, f, nz = x.cpu().numpy(), f.cpu().numpy(), nz.cpu().numpy()
    h0 = emp.bin_h[emp.d_bin_off[:S]].cpu().numpy() if S else np.zeros(0)
    warm, step_perms, fall = {}, {}, []
    q = 0
    for k, t in enumerate(steps):
        q0 = q
        q += topk
        if not (f[q0] <= fallback * nz[q0]):
            fall.append(t)
            continue
        step_perms[t] = [mlp.perms[int(i)] for i in order[k]]
        var2 = float(emp.var2[k])
        for j, i in enumerate(order[k]):
            oi = mlp.perms[int(i)]
            xi = x[q0 + j]
            if not np.all(np.isfinite(xi)):
                continue
            lo, hi = np.zeros(4), np.ones(4)
            for c in range(len(oi)):
                if len(oi) > 1 and c == 0 and oi[0] == "Nug":
                    continue
                r, sl = xi[2 * c], xi[2 * c + 1]
                if oi[c] != "Nug":
                    lo[2 * c] = _unit(r / range_fac, h0[k], 1e9)
                    hi[2 * c] = _unit(r * range_fac, h0[k], 1e9)
                lo[2 * c + 1] = _unit(sl * (1 - sill_fac), 1e-5, var2)
                hi[2 * c + 1] = _unit(sl * (1 + sill_fac), 1e-5, var2)
            warm[(t, oi)] = (lo, hi)
    out, det = fit_steps(stn_x, stn_y, data, seed=seed, warm=warm, step_perms=step_perms,
                         emp=emp, opt_iters=opt_iters, tol=tol, device=device,
                         return_details=True)
    torch.cuda.synchronize()
    det["_fallback_steps"] = fall
    det["_ms"] = {"features_network_refine": e0.elapsed_time(e1), "de": det["_de_ms"],
                  "wall": (time.perf_counter() - t0) * 1e3}
    return out, det
