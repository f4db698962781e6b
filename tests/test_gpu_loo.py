"""Leave-one-out kriging residuals (steps.krige_loo) against brute force.

The closed form reads every station's residual off one factorisation of the
step's full ordinary-kriging system. The oracle re-solves the system without
the station (oracle/port.py interp_steps, the reference's OK at one cell
placed on the left-out station), once per station. Tolerance 1e-9 relative
to the data's scale, the FP64 bar of the kriging path.
"""
import numpy as np
import pytest

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import port  # noqa: E402


def test_loo_matches_brute_force():
    from spinterps_gb300 import steps
    rng = np.random.default_rng(11)
    n, T = 45, 3
    sx, sy = rng.uniform(0, 8e4, n), rng.uniform(0, 6e4, n)
    z = rng.gamma(1.5, 2.0, size=(T, n))
    z[rng.uniform(size=z.shape) < 0.2] = np.nan
    vgs = ["0.2 Nug(0.0) + 1.1 Sph(30000.0)", "1.0 Exp(15000.0)",
           "0.05 Nug(0.0) + 0.8 Gau(25000.0)"]
    res, rmse = steps.krige_loo(sx, sy, z, vgs)
    args = port.interp_args_for(["OK"], est_vars=False)
    for t in range(T):
        idx = np.where(np.isfinite(z[t]))[0]
        assert res[t] is not None and res[t].size == idx.size
        want = np.empty(idx.size)
        for k, i in enumerate(idx):
            zt = z[t:t + 1].copy()
            zt[0, i] = np.nan
            out, _ = port.interp_steps(sx, sy, zt, sx[i:i + 1], sy[i:i + 1], vgs[t:t + 1], args,
                                       intrp_dtype=np.float64)
            want[k] = z[t, i] - out["OK"][0, 0]
        scale = np.nanmax(np.abs(z[t]))
        assert np.abs(res[t] - want).max() <= 1e-9 * scale, (t, np.abs(res[t] - want).max())
        assert abs(rmse[t] - np.sqrt(np.mean(want ** 2))) <= 1e-9 * scale
