"""Neighbour selection 'nrst' / 'pie' (spinterps_gb300.nebs, csrc/spi_nebs.cu)
and the step engine through neighbour groups.

Neighbour lists and cell groups must equal the reference's bit for bit
(tests/golden/nebs.npz, made by running interp/grps.py) and the oracle's on a
larger random case. Interpolation through neighbour groups is compared with
the oracle's restatement of interp/steps.py:584-833 at the FP64 (1e-9) and
mixed (1e-5) bars, relative to the field's largest magnitude.
"""
import numpy as np
import pytest

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import port  # noqa: E402


def test_neb_select_matches_reference(golden):
    from spinterps_gb300.nebs import SpInterpNeighborGrouping
    g = golden
    sx, sy, cx, cy = g["n_sx"], g["n_sy"], g["n_cx"], g["n_cy"]
    for mth, nn, npie in (("nrst", 8, 1), ("pie", 8, 4), ("pie", 12, 6)):
        tag = f"{mth}_{nn}_{npie}"
        grp = SpInterpNeighborGrouping(mth, nn, npie, cx, cy)
        idx = grp.neb_idxs(sx, sy)
        lab, _ = grp.groups(idx)
        assert np.array_equal(idx, g[f"n_{tag}_idxs"]), tag
        assert np.array_equal(lab, g[f"n_{tag}_grp"]), tag


def test_neb_select_larger_vs_oracle():
    from spinterps_gb300.nebs import SpInterpNeighborGrouping
    rng = np.random.default_rng(8)
    sx, sy = rng.uniform(0, 2e5, 300), rng.uniform(0, 2e5, 300)
    cx, cy = rng.uniform(0, 2e5, 1500), rng.uniform(0, 2e5, 1500)
    for mth, nn, npie in (("nrst", 16, 1), ("pie", 16, 8), ("pie", 20, 5)):
        got = SpInterpNeighborGrouping(mth, nn, npie, cx, cy).neb_idxs(sx, sy)
        ref = port.neb_idxs(mth, cx, cy, sx, sy, nn, npie)
        assert np.array_equal(got, ref), mth


@pytest.mark.parametrize("mth,nn,npie", [("nrst", 8, 1), ("pie", 8, 4)])
def test_interp_through_neighbours_vs_oracle(mth, nn, npie):
    import spinterps_gb300 as spi
    rng = np.random.default_rng(9)
    sx, sy = rng.uniform(0, 6e4, 45), rng.uniform(0, 6e4, 45)
    cx, cy = rng.uniform(0, 6e4, 300), rng.uniform(0, 6e4, 300)
    z = rng.gamma(1.3, 2.0, size=(4, 45))
    z[rng.uniform(size=z.shape) < 0.2] = np.nan
    vgs = ["0.1 Nug(0.0) + 1.0 Exp(20000.0)", "0.8 Sph(30000.0)",
           "0.2 Nug(0.0) + 0.9 Exp(15000.0)", "1.0 Exp(25000.0)"]
    args = port.interp_args_for(["OK", "SK", ("IDW", 2.0), "NNB"], est_vars=True)
    kw = dict(est_vars=True, min_vg_val=1e-4, intrp_dtype=np.float64, neb_sel_mthd=mth,
              n_nebs=nn, n_pies=npie)
    ref, rp = port.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    for prec, tol in (("fp64", 1e-9), ("mixed", 1e-5)):
        got, gp = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, precision=prec, **kw)
        assert sorted(gp) == sorted(rp)
        for lab in ref:
            a, b = got[lab], ref[lab]
            assert np.array_equal(np.isnan(a), np.isnan(b)), (prec, lab)
            m = ~np.isnan(b)
            assert np.abs(a[m] - b[m]).max() <= tol * np.abs(b[m]).max(), (prec, lab)
