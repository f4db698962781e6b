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


def test_group_solve_vs_oracle_edk_and_wide_lists():
    """Kriging through neighbour groups (spi_local_groups: one inverse per
    group and step) against the oracle's per-group _get_interp: EDK with
    two drifts over 12 'pie' neighbours, and OK / SK over 40 nearest, at
    the FP64 bar."""
    import spinterps_gb300 as spi
    rng = np.random.default_rng(21)
    ns, nc, T = 90, 700, 5
    sx, sy = rng.uniform(0, 8e4, ns), rng.uniform(0, 8e4, ns)
    cx, cy = rng.uniform(0, 8e4, nc), rng.uniform(0, 8e4, nc)
    z = rng.gamma(1.1, 3.0, size=(T, ns))
    z[rng.uniform(size=z.shape) < 0.15] = np.nan
    z[3] = 0.0  # no value reaches the threshold: the mean
    vgs = ["0.1 Nug(0.0) + 1.0 Exp(25000.0)", "1.0 Sph(40000.0)",
           "0.2 Nug(0.0) + 0.9 Gau(20000.0)", "1.0 Exp(30000.0)", "1.0 Nug(0.0)"]
    sd = np.stack([sx / 1e4 + rng.normal(0, 0.5, ns), np.sqrt(sy / 1e3)], axis=1)
    cd = np.stack([cx / 1e4 + rng.normal(0, 0.5, nc), np.sqrt(cy / 1e3)], axis=0)
    cases = [("pie", 12, 4, ["EDK"], dict(stn_drifts=sd, cell_drifts=cd)),
             ("nrst", 40, 1, ["OK", "SK"], {})]
    for mth, nn, npie, methods, extra in cases:
        args = port.interp_args_for(methods, est_vars=True)
        kw = dict(est_vars=True, min_vg_val=1e-4, intrp_dtype=np.float64, neb_sel_mthd=mth,
                  n_nebs=nn, n_pies=npie, min_var_thr=0.01, **extra)
        ref, rp = port.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
        got, gp = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
        assert sorted(gp) == sorted(rp), (mth, methods)
        for lab in ref:
            a, b = got[lab], ref[lab]
            assert np.array_equal(np.isnan(a), np.isnan(b)), (mth, lab)
            m = ~np.isnan(b)
            if m.any():  # EDK leaves EST_VARS_OK at NaN
                assert np.abs(a[m] - b[m]).max() <= 1e-9 * np.abs(b[m]).max(), (mth, lab)


def test_group_solve_singular_groups_take_pinv():
    """Co-located stations make their groups' saddle matrices exactly
    singular: the reference's pinv still succeeds there (no problem step),
    and so does the group solve, with pinv's truncated inverse. Where a
    co-located pair ties for the last neighbour slot, the reference's
    unstable argsort and the index order of spi_neb_select may keep
    different twins; those cells are left out of the comparison."""
    import spinterps_gb300 as spi
    from spinterps_gb300.nebs import SpInterpNeighborGrouping
    rng = np.random.default_rng(22)
    ns, nc, T = 40, 500, 3
    sx, sy = rng.uniform(0, 5e4, ns), rng.uniform(0, 5e4, ns)
    sx[1::5], sy[1::5] = sx[0::5], sy[0::5]  # every fifth pair shares a site
    cx, cy = rng.uniform(0, 5e4, nc), rng.uniform(0, 5e4, nc)
    z = rng.gamma(1.5, 2.0, size=(T, ns))
    vgs = ["1.0 Exp(20000.0)", "0.1 Nug(0.0) + 0.9 Sph(30000.0)",
           "0.05 Nug(0.0) + 1.0 Gau(15000.0)"]
    args = port.interp_args_for(["OK", "SK"], est_vars=True)
    kw = dict(est_vars=True, min_vg_val=1e-4, intrp_dtype=np.float64, neb_sel_mthd="nrst",
              n_nebs=10, n_pies=1)
    ref, rp = port.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    got, gp = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    assert sorted(gp) == sorted(rp) == []
    same = np.all(SpInterpNeighborGrouping("nrst", 10, 1, cx, cy).neb_idxs(sx, sy) ==
                  port.neb_idxs("nrst", cx, cy, sx, sy, 10, 1), axis=1)
    for c in np.where(~same)[0]:
        d = np.sort(np.hypot(cx[c] - sx, cy[c] - sy))
        assert d[9] == d[10], c  # an exact tie for the last slot
    assert same.sum() >= nc // 2
    for lab in ref:
        a, b = got[lab][:, same], ref[lab][:, same]
        assert np.array_equal(np.isnan(a), np.isnan(b)), lab
        m = ~np.isnan(b)
        assert np.abs(a[m] - b[m]).max() <= 1e-6 * np.abs(b[m]).max(), lab


def _local_case(kind_name, nn, seed):
    """One step group's inputs for the C entries, all stations present."""
    import torch
    from spinterps_gb300 import nebs
    from spinterps_gb300.steps import _Domain, _vg_tensor, check_full_nuggetness, parse_vg
    rng = np.random.default_rng(seed)
    ns, nc, T = 70, 900, 6
    sx, sy = rng.uniform(0, 6e4, ns), rng.uniform(0, 6e4, ns)
    cx, cy = rng.uniform(0, 6e4, nc), rng.uniform(0, 6e4, nc)
    z = rng.gamma(1.2, 2.5, size=(T, ns))
    vgs = ["0.1 Nug(0.0) + 1.0 Exp(20000.0)", "1.0 Sph(35000.0)",
           "0.1 Nug(0.0) + 0.9 Gau(18000.0)",
           "1.0 Exp(12000.0)", "0.3 Nug(0.0) + 0.7 Sph(25000.0)", "1.0 Exp(40000.0)"]
    dev = torch.device("cuda")
    sd = cd = None
    if kind_name == "EDK":
        sd = np.stack([sx / 1e4, rng.normal(0, 1, ns)], axis=1)
        cd = np.stack([cx / 1e4, rng.normal(0, 1, nc)], axis=0)
    dom = _Domain(dev, sx, sy, cx, cy, sd, cd, 1e-4, 0)
    grp = nebs.SpInterpNeighborGrouping("nrst", nn, None, cx, cy)
    nb = grp.neb_idxs_device(sx, sy)
    vg = _vg_tensor([parse_vg(v) for v in vgs], dev).view(T, -1)
    nug = torch.as_tensor(np.array([check_full_nuggetness(v, 1e-4) for v in vgs],
                                   dtype=np.int32), device=dev)
    return dom, nb, torch.as_tensor(z, device=dev), vg, nug, T, nc


@pytest.mark.parametrize("kind_name", ["OK", "SK", "EDK"])
def test_local_groups_match_per_cell_solve(kind_name):
    """spi_local_groups (one inverse per group and step, applied per cell)
    against spi_local_cells (one Gauss-Jordan solve per cell and step) on
    the same neighbour lists: the same fields at rounding level, and the
    same again when the scratch holds one step at a time."""
    import ctypes
    import torch
    from spinterps_gb300 import _native as nat
    from spinterps_gb300.nebs import LOCAL_KIND, device_groups
    from spinterps_gb300.steps import _out_struct, _ptr, _stream
    dom, nb, z, vg, nug, T, C = _local_case(kind_name, 16, 30 + LOCAL_KIND[kind_name])
    kind, k = LOCAL_KIND[kind_name], nb.shape[1]
    steps = torch.arange(T, dtype=torch.int32, device="cuda")
    want = int(kind_name == "OK")
    nd = int(dom.st.n_drift)

    def fields():
        est = torch.full((T, C), float("nan"), dtype=torch.float64, device="cuda")
        var = torch.full((T, C), float("nan"), dtype=torch.float64, device="cuda")
        return est, var, torch.zeros(T, dtype=torch.int32, device="cuda")

    e0, v0, p0 = fields()
    nat.call("spi_local_cells", ctypes.byref(dom.st), kind, k, _ptr(nb), T, _ptr(steps),
             _ptr(steps), _ptr(z), z.shape[1], _ptr(vg), _ptr(nug), 0.0, 0.0, want,
             ctypes.byref(_out_struct(e0, v0 if want else None, None, None)), _ptr(p0),
             _stream())
    g_nebs, cell_grp, order = device_groups(nb)
    G = g_nebs.shape[0]
    assert G < C
    res = []
    for n_at_once in (T, 1):
        nbytes = nat.lib().spi_local_groups_scratch_bytes(kind, k, nd, G, n_at_once)
        scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        e1, v1, p1 = fields()
        nat.call("spi_local_groups", ctypes.byref(dom.st), kind, k, _ptr(g_nebs), G,
                 _ptr(cell_grp), _ptr(order), T, _ptr(steps), _ptr(steps), _ptr(z),
                 z.shape[1], _ptr(vg), _ptr(nug), 0.0, want,
                 ctypes.byref(_out_struct(e1, v1 if want else None, None, None)),
                 _ptr(scratch), nbytes, _ptr(p1), _stream())
        torch.cuda.synchronize()
        res.append((e1.cpu().numpy(), v1.cpu().numpy(), p1.cpu().numpy()))
    e0, v0, p0 = e0.cpu().numpy(), v0.cpu().numpy(), p0.cpu().numpy()
    for e1, v1, p1 in res:
        assert not p0.any() and not p1.any()
        assert not np.isnan(e1).any()
        assert np.abs(e1 - e0).max() <= 1e-10 * np.abs(e0).max(), kind_name
        if want:
            assert np.abs(v1 - v0).max() <= 1e-9 * np.abs(v0).max()
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1],
                                                                   equal_nan=True)
