"""Systems too large for the shared-memory right-hand side of the cell kernel
(spi_cells_stream.cu): external-drift kriging with 3500 stations and two
drifts (elevation, easting in metres), the scale of the reference's large
hourly configuration. Both the FP64 and the mixed path take the streamed
kernel at this size.

At this size the reference's own pinv (oracle/port.py) is ~1e-8 away from the
exact kriging estimate (the saddle matrix mixes variogram entries ~1 with
easting drifts ~5e5), so the yardstick is the exact estimate: LU with
iterative refinement, residuals in long double. Bars relative to the field's
largest magnitude: FP64 path 1e-9, mixed path 1e-5, the oracle 1e-7.
"""
import numpy as np
import pytest

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import port  # noqa: E402


def test_large_edk_streamed():
    import spinterps_gb300 as spi
    rng = np.random.default_rng(41)
    n, box = 3500, 500e3
    sx, sy = rng.uniform(0, box, n), rng.uniform(0, box, n)
    cx, cy = rng.uniform(0, box, 400), rng.uniform(0, box, 400)

    def elev(x, y):
        return 1500 + 800 * np.sin(x / 7e4) * np.cos(y / 9e4) + 300 * np.sin((x + y) / 3e4)

    sd = np.stack([elev(sx, sy), sx], 1)
    cd = np.stack([elev(cx, cy), cx], 0)
    z = (5 + 1e-3 * sd[:, 0] + 2e-6 * sx + rng.normal(0, 1, n))[None].copy()
    z[0, rng.uniform(size=n) < 0.02] = np.nan
    vgs = ["0.1 Nug(0.0) + 0.9 Exp(60000.0)"]
    args = port.interp_args_for(["EDK"], est_vars=False)
    kw = dict(stn_drifts=sd, cell_drifts=cd, intrp_dtype=np.float64)
    ref, _ = port.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    exact = _exact(sx, sy, z[0], sd, cx, cy, cd)
    scale = np.abs(exact).max()
    f64, _ = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    mixed, _, info = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, precision="mixed",
                                      return_info=True, **kw)
    assert info["fp32_tier_steps"]["EDK"] == [0]  # the FP32 tier ran
    assert np.abs(f64["EDK"][0] - exact).max() / scale <= 1e-9
    assert np.abs(mixed["EDK"][0] - exact).max() / scale <= 1e-5
    assert np.abs(ref["EDK"][0] - exact).max() / scale <= 1e-7


def _exact(sx, sy, z, sd, cx, cy, cd):
    """EDK estimates of "0.1 Nug(0.0) + 0.9 Exp(60000.0)" from the present
    stations by LU with iterative refinement (long-double residuals)."""
    idx = np.isfinite(z)
    x, y, zz, S = sx[idx], sy[idx], z[idx], sd[idx]
    m = x.size

    def gam(d):
        return 0.1 + 0.9 * (1 - np.exp(-3 * d / 60000.0))

    d = np.hypot(x[:, None] - x[None], y[:, None] - y[None])
    A = np.zeros((m + 3, m + 3))
    A[:m, :m] = gam(d)
    A[:m, m], A[m, :m] = 1, 1
    A[:m, m + 1:], A[m + 1:, :m] = S, S.T
    dc = np.hypot(cx[:, None] - x[None], cy[:, None] - y[None])
    R = np.concatenate([gam(dc), np.ones((cx.size, 1)), cd.T], 1)
    B = np.concatenate([zz, np.zeros(3)])[:, None]
    AL = A.astype(np.longdouble)
    xs = np.linalg.solve(A, B).astype(np.longdouble)
    for _ in range(4):
        r = B.astype(np.longdouble) - AL @ xs
        xs = xs + np.linalg.solve(A, r.astype(np.float64)).astype(np.longdouble)
    return (R.astype(np.longdouble) @ xs).astype(np.float64)[:, 0]
