"""Train the fitter's warm-start network (spinterps_gb300.warmstart).

Training data: Gaussian random fields on 300-1500 stations uniform in a
box of 100-400 km (aspect 0.5-1), each with a random Sph / Exp / Gau model
(range 2-40% of the box, sill 0.5-2) and, for half of them, a nugget of up
to 30% of the sill; half of the fields are then made precipitation-like
(zero below a random 20-70% quantile, gamma amounts above it). Each field is fitted by the project's own GPU fitter
(spinterps_gb300.fitvgs, the reference's fitvgs settings); its choice
(permutation and parameters) is the label, its 20 lag-bin features the
input. The network is trained by the kernels of csrc/spi_mlp.cu (FP32 Adam).
Field synthesis (a Cholesky factor of each field's covariance) uses torch:
it only makes training data.

    python -m spinterps_gb300.train_warmstart [n_fields] [out.npz]
"""
import sys
import time

import numpy as np
import torch

from .fitvgs import Empirical, fit_steps
from .warmstart import DEFAULT_WEIGHTS, WarmStartMLP, default_perms, labels, step_features


def _cov(typ, d, rng, sill):
    if typ == "Exp":
        return sill * torch.exp(-3 * d / rng)
    if typ == "Gau":
        return sill * torch.exp(-3 * (d / rng) ** 2)
    t = torch.clamp(d / rng, max=1.0)
    return sill * (1 - 1.5 * t + 0.5 * t ** 3)


def synth_points(n_fields, seed=0, n_lo=300, n_hi=1500, device="cuda"):
    """[(x, y, z)] of n_fields synthetic fields and their generating models
    (type, range, sill, nugget fraction, dry fraction or 0)."""
    from scipy.stats import gamma, norm
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    pts, models = [], []
    for _ in range(n_fields):
        n = int(rng.integers(n_lo, n_hi + 1))
        box = rng.uniform(100e3, 400e3)
        x, y = rng.uniform(0, box, n), rng.uniform(0, box * rng.uniform(0.5, 1.0), n)
        typ = str(rng.choice(["Sph", "Exp", "Gau"]))
        r = rng.uniform(0.02, 0.4) * box
        sill = rng.uniform(0.5, 2.0)
        nugf = rng.uniform(0.0, 0.3) if rng.uniform() < 0.5 else 0.0
        X = torch.as_tensor(np.stack([x, y], 1), device=device)
        d = torch.cdist(X, X)
        c = _cov(typ, d, r, sill * (1 - nugf))
        jitter = max(sill * nugf, 1e-6 * sill)
        for _ in range(6):
            try:
                L = torch.linalg.cholesky(c + jitter * torch.eye(n, device=device,
                                                                   dtype=torch.float64))
                break
            except RuntimeError:
                jitter *= 10
        z = (L @ torch.randn(n, generator=gen, device=device, dtype=torch.float64)).cpu().numpy()
        dry = 0.0
        if rng.uniform() < 0.5:
            # precipitation-like: dry below a quantile, gamma amounts above it
            dry = rng.uniform(0.2, 0.7)
            u = norm.cdf(z / np.sqrt(sill))
            z = np.where(u > dry, gamma.ppf(np.clip((u - dry) / (1 - dry), 1e-12, 1 - 1e-12),
                                            rng.uniform(0.5, 2.0), scale=2.0), 0.0)
        pts.append((x, y, z))
        models.append((typ, r, sill, nugf, dry))
    return pts, models


def make_training_set(n_fields, seed=0, chunk=200, device="cuda"):
    """Features and fitter labels of n_fields synthetic fields."""
    perms = default_perms()
    feats, cls, yp, mk = [], [], [], []
    t0 = time.time()
    for c0 in range(0, n_fields, chunk):
        pts, _ = synth_points(min(chunk, n_fields - c0), seed=seed + c0, device=device)
        emp = Empirical(None, None, None, points=pts, device=device).run()
        _, det = fit_steps(None, None, None, emp=emp, seed=seed + c0, return_details=True,
                           device=device)
        keep, c, y, m = labels(det, pts, perms)
        feats.append(step_features(pts, [int(k) for k in keep], device=device))
        cls.append(c)
        yp.append(y)
        mk.append(m)
        print(f"  fields {c0 + len(pts)}/{n_fields} fitted, {time.time() - t0:.1f}s "
              f"(DE {det['_de_ms'] / 1e3:.1f}s)", flush=True)
    return (np.concatenate(feats), np.concatenate(cls), np.concatenate(yp),
            np.concatenate(mk))


def main(n_fields=50000, out=DEFAULT_WEIGHTS, epochs=300, seed=0):
    t0 = time.time()
    F, C, Y, M = make_training_set(n_fields, seed=seed)
    t1 = time.time()
    n_val = max(1, len(F) // 10)
    mlp = WarmStartMLP(seed=seed)
    hist = mlp.train(F[n_val:], C[n_val:], Y[n_val:], M[n_val:], epochs=epochs)
    O = mlp.forward(F[:n_val])
    acc = float(np.mean(np.argmax(O[:, :mlp.n_class], 1) == C[:n_val]))
    rng_err = float(np.sqrt(np.mean(((O[:, mlp.n_class] - Y[:n_val, 0]) ** 2)[M[:n_val, 0] > 0])))
    out = str(out)
    mlp.save(out)
    print(f"fields {n_fields} samples {len(F)} synth+fit {t1 - t0:.1f}s train "
          f"{time.time() - t1:.1f}s loss {hist[0]:.3f}->{hist[-1]:.3f} val class acc {acc:.3f} "
          f"val log10-range rmse {rng_err:.3f} -> {out}")
    return mlp


if __name__ == "__main__":
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 50000
    dst = sys.argv[2] if len(sys.argv) > 2 else DEFAULT_WEIGHTS
    main(n, dst)
