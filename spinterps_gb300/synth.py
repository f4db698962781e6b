"""Seeded synthetic inputs with the shapes and distributions of the
reference's benchmark configurations (no dataset ships with it).

stress_edk: the precision-stress case for external-drift kriging: stations
clustered by a Thomas process (parents uniform in the box, children
Gaussian around their parent), a Gaussian variogram with a 1e-6 nugget,
which makes the kriging matrices nearly singular (condition numbers
1e8-1e11), and one drift, an fBm elevation raster sampled at the stations
and given at every cell.

The nugget is written as a micro-range exponential, "1e-06 Exp(1.0)": 0 at
h = 0 and 1e-6 from a few metres on. The reference's own Nug model is its
sill at every distance, h = 0 included (cyth/interpmthds.pyx:38-84), so a
"Nug" term only shifts the semivariance matrix by a constant that the
Lagrange row absorbs and never reaches the diagonal: with it these systems
are singular to FP64 (condition ~1e20). The micro-range form is the
regularising nugget the configuration describes, in the reference's own
variogram language.
"""
import numpy as np


def thomas_points(rng, n, n_parents, sigma, box):
    """n points: parents uniform in [0, box)^2, each point a parent plus
    N(0, sigma^2) offsets."""
    px, py = rng.uniform(0, box, n_parents), rng.uniform(0, box, n_parents)
    k = rng.integers(0, n_parents, n)
    return px[k] + rng.normal(0, sigma, n), py[k] + rng.normal(0, sigma, n)


def fbm_raster(rng, ny, nx, hurst, lo, hi):
    """[ny, nx] fractional Brownian surface by spectral synthesis (amplitude
    ~ |k|^-(H+1)), scaled to [lo, hi]."""
    ky = np.fft.fftfreq(ny)[:, None]
    kx = np.fft.fftfreq(nx)[None, :]
    k = np.hypot(kx, ky)
    k[0, 0] = 1.0
    amp = k ** -(hurst + 1.0)
    amp[0, 0] = 0.0
    noise = rng.normal(size=(ny, nx)) + 1j * rng.normal(size=(ny, nx))
    f = np.real(np.fft.ifft2(noise * amp))
    f = (f - f.min()) / (f.max() - f.min())
    return lo + (hi - lo) * f


def bilinear(raster, x0, ytop, cell, x, y):
    """raster[row, col] holds the value at cell centre (x0 + (col + 0.5) cell,
    ytop - (row + 0.5) cell); bilinear sample at (x, y), edges clamped."""
    ny, nx = raster.shape
    c = np.clip((np.asarray(x) - x0) / cell - 0.5, 0, nx - 1)
    r = np.clip((ytop - np.asarray(y)) / cell - 0.5, 0, ny - 1)
    c0, r0 = np.minimum(c.astype(int), nx - 2), np.minimum(r.astype(int), ny - 2)
    fc, fr = c - c0, r - r0
    return ((1 - fr) * ((1 - fc) * raster[r0, c0] + fc * raster[r0, c0 + 1])
            + fr * ((1 - fc) * raster[r0 + 1, c0] + fc * raster[r0 + 1, c0 + 1]))


def stress_edk(seed=20261204, n_stns=400, n_parents=20, sigma=300.0, box=100e3, n_steps=200,
               nx=500, ny=500, rng_m=30e3, nugget=1e-6):
    """Stations, values, grid and drift of the precision-stress EDK case.
    Values per step: 5 + 1e-3 * elevation + a Gaussian random field with the
    step's variogram (all stations present)."""
    rng = np.random.default_rng(seed)
    sx, sy = thomas_points(rng, n_stns, n_parents, sigma, box)
    cell = box / nx
    elev = fbm_raster(rng, ny, nx, 0.8, 0.0, 3000.0)
    xs = cell / 2 + cell * np.arange(nx)
    ys = box - cell / 2 - cell * np.arange(ny)
    gx, gy = np.meshgrid(xs, ys)
    s_el = bilinear(elev, 0.0, box, cell, sx, sy)
    d = np.hypot(sx[:, None] - sx[None], sy[:, None] - sy[None])
    cov = (1.0 - nugget) * np.exp(-3.0 * (d / rng_m) ** 2) + nugget * np.eye(n_stns)
    w, V = np.linalg.eigh(cov)
    root = V * np.sqrt(np.clip(w, 0.0, None))
    grf = (root @ rng.standard_normal((n_stns, n_steps))).T
    z = 5.0 + 1e-3 * s_el[None] + grf
    vg = f"{nugget:.6g} Exp(1.0) + {1.0 - nugget:.6f} Gau({rng_m:.1f})"
    return dict(sx=sx, sy=sy, z=z, cx=gx.ravel().copy(), cy=gy.ravel().copy(),
                vgs=[vg] * n_steps, stn_drift=s_el[:, None].copy(),
                cell_drift=elev.ravel()[None].copy())


def large_edk(n_steps=152, seed=20261205, n_stns=4000, box=500e3, nx=2000, ny=2000,
              n_models=8, device="cuda"):
    """The large hourly external-drift case: n_stns stations uniform in a
    box x box square, each missing per step with a per-station probability
    ~ U(0.05, 0.5); two drifts, an fBm elevation raster (H = 0.8, 0-3000 m)
    and the easting, sampled at the stations and given at every cell of an
    nx x ny grid; values per step 5 + 1e-3 * elevation + 2e-6 * easting + a
    Gaussian random field drawn from one of n_models Sph / Exp models (range
    20-100 km, sill 0.5-2, nugget fraction 0-0.2). The steps' variograms
    are left to the fitter. The field factors are Cholesky factors computed
    with torch on ``device`` (test data only)."""
    import torch
    rng = np.random.default_rng(seed)
    sx, sy = rng.uniform(0, box, n_stns), rng.uniform(0, box, n_stns)
    p_miss = rng.uniform(0.05, 0.5, n_stns)
    cell = box / nx
    elev = fbm_raster(rng, ny, nx, 0.8, 0.0, 3000.0)
    xs = cell / 2 + cell * np.arange(nx)
    ys = box - cell / 2 - cell * np.arange(ny)
    gx, gy = np.meshgrid(xs, ys)
    cx, cy = gx.ravel().copy(), gy.ravel().copy()
    s_el = bilinear(elev, 0.0, box, cell, sx, sy)
    X = torch.as_tensor(np.stack([sx, sy], 1), device=device)
    d = torch.cdist(X, X)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    model = rng.integers(0, n_models, n_steps)
    grf = np.empty((n_steps, n_stns))
    for k in range(n_models):
        typ = ("Sph", "Exp")[int(rng.integers(2))]
        r, s, nf = rng.uniform(20e3, 100e3), rng.uniform(0.5, 2.0), rng.uniform(0.0, 0.2)
        if typ == "Exp":
            c = torch.exp(-3.0 * d / r)
        else:
            t = torch.clamp(d / r, max=1.0)
            c = 1.0 - 1.5 * t + 0.5 * t ** 3
        c = (1 - nf) * s * c + (nf * s + 1e-9 * s) * torch.eye(n_stns, device=device,
                                                               dtype=torch.float64)
        L = torch.linalg.cholesky(c)
        sel = np.where(model == k)[0]
        if sel.size:
            e = torch.randn((n_stns, sel.size), generator=gen, device=device, dtype=torch.float64)
            grf[sel] = (L @ e).T.cpu().numpy()
    z = 5.0 + 1e-3 * s_el[None] + 2e-6 * sx[None] + grf
    z[rng.uniform(size=z.shape) < p_miss[None]] = np.nan
    return dict(sx=sx, sy=sy, z=z, cx=cx, cy=cy, stn_drift=np.stack([s_el, sx], 1),
                cell_drift=np.stack([elev.ravel(), cx], 0))
