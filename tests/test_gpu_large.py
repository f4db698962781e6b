"""Systems too large for the shared-memory right-hand side of the cell kernel
(spi_cells_stream.cu): external-drift kriging with 3500 stations and two
drifts, the scale of the reference's large hourly configuration, against the
oracle (oracle/port.py, the reference's pinv per system). With n = 3500 both
the FP64 launch (n > ~1600) and the FP32 launch (n > ~3300) take the streamed
kernel. Tolerances as the other parity tests: FP64 1e-9, mixed 1e-5,
relative to the field's largest magnitude.
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
    scale = np.abs(ref["EDK"]).max()
    f64, _ = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    mixed, _, info = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, precision="mixed",
                                      return_info=True, **kw)
    assert info["fp32_tier_steps"]["EDK"] == [0]  # the FP32 tier ran
    assert np.abs(f64["EDK"] - ref["EDK"]).max() / scale <= 1e-9
    assert np.abs(mixed["EDK"] - ref["EDK"]).max() / scale <= 1e-5
