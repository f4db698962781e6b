"""Parity of the CUDA path (through the C ABI) with the reference.

Golden vectors come from the reference's own code (tests/golden); larger
cases are checked against the oracle (oracle/port.py, pinned to the same
vectors). Tolerances, relative to the largest magnitude of the field:
  FP64 path  1e-9  (spec bar for the plain FP64 GPU path)
  mixed path 1e-5  (spec bar for split-precision FP32)
  float32 output fields: 2e-6 (one float32 rounding of either side)
Distances are the correctly rounded root; the reference's glibc pow(x, 0.5)
differs from it by one ulp on ~0.1% of inputs.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import port  # noqa: E402

FP64_TOL = 1e-9
MIXED_TOL = 1e-5
F32_TOL = 2e-6


def _spi():
    import spinterps_gb300 as spi
    return spi


def _err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    nan_a, nan_b = np.isnan(a), np.isnan(b)
    assert np.array_equal(nan_a, nan_b), (nan_a.sum(), nan_b.sum())
    m = ~nan_b
    if not m.any():
        return 0.0
    scale = max(np.abs(b[m]).max(), 1e-300)
    return float(np.abs(a[m] - b[m]).max() / scale)


def test_dists_drop_in(golden):
    spi = _spi()
    st = spi.SpInterpSteps(min_vg_val=1e-4)
    g = golden
    d = st._get_dists_arr(g["k_cx"], g["k_cy"], g["k_sx"], g["k_sy"])
    ref = g["k_d_cs"]
    ulp = np.abs(d - ref) / np.spacing(np.maximum(ref, 1e-300))
    assert (ulp <= 1).all()
    assert (d == ref).mean() > 0.98
    assert (d[:3, :3].diagonal() == 0).all()


def test_vg_fill_drop_in(golden):
    spi = _spi()
    st = spi.SpInterpSteps(min_vg_val=0.0)
    g = golden
    for vi, vg in enumerate(g["k_vgs"]):
        vg = str(vg)
        for covar in (0, 1):
            for mvv in (0.0, 1e-4, 0.05):
                st._min_vg_val = mvv
                types = ["SK"] if covar else ["OK"]
                a = st._get_svars_arr(g["k_d_ss"], [vg], types, 1)[(vg, covar)]
                b = st._get_svars_arr(g["k_d_cs"], [vg], types, 0)[(vg, covar)]
                for got, key in ((a, f"k_vg_ss_{vi}_{covar}_{mvv:g}"),
                                 (b, f"k_vg_cs_{vi}_{covar}_{mvv:g}")):
                    ref = g[key]
                    # values within the zeroing threshold may flip by one ulp
                    near = np.abs(ref - mvv) <= 1e-12 * max(1.0, abs(mvv))
                    diff = np.abs(got - ref)
                    scale = max(np.abs(ref).max(), 1e-300)
                    assert (diff[~near] <= 1e-13 * scale).all(), (vg, covar, mvv)


def test_copy_subset_drop_in(golden):
    spi = _spi()
    st = spi.SpInterpSteps()
    g = golden
    sub = st._get_2d_arr_subset(g["k_d_cs"], g["k_copy_ri"], g["k_copy_ci"], 2, 1)
    ref = g["k_copy_sub"]
    assert np.array_equal(np.isnan(sub), np.isnan(ref))
    assert np.array_equal(np.nan_to_num(sub), np.nan_to_num(ref))


def _one_group(g, methods, vgs, *, cx="i_cx", cy="i_cy", z=None, n=None, sd=None, cd=None,
               precision="fp64"):
    """Run interp_steps on the fixture's single station group with every
    step flagged for interpolation (the fixture passed its flags directly to
    _get_interp; callers compare the steps whose flag was on)."""
    spi = _spi()
    sx, sy = g["i_sx"], g["i_sy"]
    z = (g["i_z"] if z is None else z).copy()
    if n is not None:
        sx, sy, z = sx[:n], sy[:n], z[:, :n]
    args = port.interp_args_for(methods, est_vars="OK" in methods)
    return spi.interp_steps(sx, sy, z, g[cx], g[cy], [str(v) for v in vgs], args,
                            est_vars="OK" in methods, stn_drifts=sd, cell_drifts=cd,
                            min_var_thr=-np.inf, min_vg_val=1e-4, intrp_dtype=np.float64,
                            precision=precision)[0]


def test_ok_sk_single_group_vs_reference(golden):
    g = golden
    flags = g["i_flags"]
    for itype in ("OK", "SK"):
        got = _one_group(g, [itype], g["i_vgs_mixed"])
        ref = g[f"i_{itype}_est"]
        on = np.where(flags)[0]
        assert _err(got[itype][on], ref[on]) <= FP64_TOL, itype
        if itype == "OK":
            assert _err(got["EST_VARS_OK"][on], g["i_OK_var"][on]) <= F32_TOL
    got = _one_group(g, ["OK"], g["i_vgs_other"])
    assert _err(got["OK"], g["i_OKo_est"]) <= FP64_TOL
    assert _err(got["EST_VARS_OK"], g["i_OKo_var"]) <= F32_TOL


def test_edk_single_group_vs_reference(golden):
    g = golden
    flags = g["i_flags"]
    on = np.where(flags)[0]
    elev = g["i_EDK1_sd"][:, 0]
    for k in (1, 2):
        got = _one_group(g, ["EDK"], g["i_vgs_mixed"], z=g["i_z"] + 1e-3 * elev,
                         sd=g[f"i_EDK{k}_sd"], cd=g[f"i_EDK{k}_cd"])
        assert _err(got["EDK"][on], g[f"i_EDK{k}_est"][on]) <= FP64_TOL, k


def test_idw_nnb_single_group_vs_reference(golden):
    g = golden
    flags = g["i_flags"]
    on = np.where(flags)[0]
    t = g["i_z"].shape[0]
    vg0 = "0.05 Nug(0.0) + 0.95 Exp(20000)"
    for e in (1.0, 2.0, 3.5):
        got = _one_group(g, [("IDW", e)], [vg0] * t, cx="i_cx2", cy="i_cy2")
        assert _err(got["IDW_000"][on], g[f"i_IDW_{e:g}_est"][on]) <= FP64_TOL, e
    got = _one_group(g, ["NNB"], [vg0] * t, cx="i_cx2", cy="i_cy2")
    assert np.array_equal(got["NNB"], g["i_NNB_est"])
    got = _one_group(g, ["OK"], [vg0] * t, n=1)
    assert np.array_equal(got["OK"], g["i_one_est"])
    assert np.isnan(got["EST_VARS_OK"]).all()


@pytest.mark.parametrize("tag", ["okidw", "edk"])
def test_multi_step_runs_vs_reference(golden, tag):
    spi = _spi()
    g = golden
    p = f"s_{tag}_"
    methods = []
    for m in g[p + "methods"]:
        m = str(m)
        methods.append(("IDW", float(m.split(":")[1])) if m.startswith("IDW:") else m)
    thr, mn, mx, mvv = g[p + "params"]
    args = port.interp_args_for(methods, est_vars="OK" in methods)
    for precision, tol in (("fp64", F32_TOL), ("mixed", MIXED_TOL)):
        flds, prblm = spi.interp_steps(
            g[p + "sx"], g[p + "sy"], g[p + "z"], g[p + "cx"], g[p + "cy"],
            [str(v) for v in g[p + "vgs"]], args, est_vars="OK" in methods,
            stn_drifts=g.get(p + "sd"), cell_drifts=g.get(p + "cd"), min_var_thr=thr,
            min_var_cut=None if np.isnan(mn) else mn, max_var_cut=None if np.isnan(mx) else mx,
            min_vg_val=mvv, precision=precision)
        assert sorted(set(prblm)) == g[p + "prblm"].tolist()
        for lab, f in flds.items():
            assert f.dtype == np.float32
            e = _err(f, g[p + "out_" + lab])
            assert e <= tol, (precision, lab, e)


def test_config1_subset_vs_reference(golden):
    spi = _spi()
    g = golden
    vg = "0.05 Nug(0.0) + 0.95 Exp(20000)"
    args = port.interp_args_for(["OK", ("IDW", 2.0)], est_vars=True)
    for precision, tol, vtol in (("fp64", FP64_TOL, F32_TOL), ("mixed", MIXED_TOL, MIXED_TOL)):
        flds, _ = spi.interp_steps(g["c1_sx"], g["c1_sy"], g["c1_z"], g["c1_cx"], g["c1_cy"],
                                   [vg] * 4, args, est_vars=True, min_vg_val=1e-4,
                                   intrp_dtype=np.float64, precision=precision)
        assert _err(flds["OK"], g["c1_ok_est"]) <= tol, precision
        assert _err(flds["EST_VARS_OK"], g["c1_ok_var"]) <= vtol, precision
        assert _err(flds["IDW_000"], g["c1_idw_est"]) <= tol, precision


def _random_case(seed, n=120, t=6, nx=40, ny=30, p_miss=0.3, box=1.2e5):
    rng = np.random.default_rng(seed)
    sx, sy = rng.uniform(0, box, n), rng.uniform(0, box, n)
    gx, gy = np.meshgrid(np.arange(nx) * (box / nx) + box / nx / 2,
                         box - box / ny / 2 - np.arange(ny) * (box / ny))
    z = rng.gamma(0.8, 2.0, size=(t, n)) * (rng.uniform(size=(t, n)) < 0.6)
    z[rng.uniform(size=(t, n)) < p_miss] = np.nan
    types = ["Sph", "Exp", "Gau"]
    vgs = []
    for j in range(t):
        r = rng.uniform(10e3, 40e3)
        s = rng.uniform(0.5, 2.0)
        nf = rng.uniform(0, 0.2)
        vgs.append(f"{nf * s:.5f} Nug(0.0) + {s - nf * s:.5f} {types[j % 3]}({r:.1f})")
    elev = 500 + 4e-3 * sx + rng.normal(0, 30, n)
    celev = 500 + 4e-3 * gx.ravel()
    return sx, sy, z, gx.ravel(), gy.ravel(), vgs, elev[:, None], celev[None]


def test_random_steps_vs_oracle():
    spi = _spi()
    sx, sy, z, cx, cy, vgs, sd, cd = _random_case(7)
    methods = ["OK", "SK", "EDK", ("IDW", 2.0), ("IDW", 1.5), "NNB"]
    args = port.interp_args_for(methods, est_vars=True)
    kw = dict(est_vars=True, stn_drifts=sd, cell_drifts=cd, min_var_thr=0.1, min_vg_val=1e-4,
              intrp_dtype=np.float64)
    ref, rp = port.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    got, gp, info = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, return_info=True, **kw)
    assert gp == rp
    for lab in ref:
        assert _err(got[lab], ref[lab]) <= FP64_TOL, lab
    mixed, _ = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, precision="mixed", **kw)
    for lab in ref:
        assert _err(mixed[lab], ref[lab]) <= MIXED_TOL, lab


def test_float32_fields_and_clipping():
    spi = _spi()
    sx, sy, z, cx, cy, vgs, _, _ = _random_case(9, t=4)
    args = port.interp_args_for(["OK", ("IDW", 2.0)], est_vars=True)
    kw = dict(est_vars=True, min_var_cut=0.5, max_var_cut=3.0, min_vg_val=1e-4)
    ref, _ = port.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    got, _ = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    for lab in ref:
        assert got[lab].dtype == np.float32
        assert _err(got[lab], ref[lab]) <= F32_TOL, lab
    assert np.nanmin(got["OK"]) >= 0.5 and np.nanmax(got["OK"]) <= 3.0


def test_mixed_zeroes_the_same_entries_at_the_cut():
    """SK zeroes covariances <= min_vg_val (OK: semivariances). Cells are
    placed within 1e-9 relative of that cut from every station, so FP32
    arithmetic alone would zero a different set of entries than FP64 and
    miss by min_vg_val * |w_i|; the mixed path must agree with the oracle."""
    spi = _spi()
    rng = np.random.default_rng(21)
    n, mvv, r = 40, 1e-3, 10000.0
    sx, sy = rng.uniform(0, 2e4, n), rng.uniform(0, 2e4, n)
    z = rng.gamma(1.2, 2.0, size=(3, n))
    dcut = -np.log(mvv) * r / 3.0  # exp(-3 d / r) == mvv
    k = np.repeat(np.arange(n), 50)
    ang = rng.uniform(0, 2 * np.pi, k.size)
    d = dcut * (1 + rng.uniform(-1e-9, 1e-9, k.size))
    cx, cy = sx[k] + d * np.cos(ang), sy[k] + d * np.sin(ang)
    vgs = ["1.0 Exp(10000.0)"] * 3
    args = port.interp_args_for(["SK", "OK"], est_vars=True)
    kw = dict(est_vars=True, min_vg_val=mvv, intrp_dtype=np.float64)
    ref, _ = port.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    got, _, info = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, precision="mixed",
                                    return_info=True, **kw)
    assert info["fp32_tier_steps"]["SK"] == [0, 1, 2]  # the FP32 tier ran
    for lab in ref:
        assert _err(got[lab], ref[lab]) <= MIXED_TOL, lab


def test_mixed_vs_fp64_on_the_batched_workload():
    """The bench's batched workload (1000 stations, per-step missingness and
    variograms, zero-inflated values), 4 steps incl. a Gaussian one, a
    quarter of the grid: every mixed field within 1e-5 of the FP64 GPU path.
    SK cells whose sum of weights sits at the check's boundary are the
    delicate case (estimate vs nearest station)."""
    import bench
    spi = _spi()
    w = bench.make_workload()
    steps = [0, 4, 150, 300]
    cells = np.arange(0, w["cx"].size, 4)
    args = bench.interp_args()
    kw = dict(bench.KW)
    z = w["z"][steps]
    vgs = [w["vgs"][s] for s in steps]
    f64, _ = spi.interp_steps(w["sx"], w["sy"], z, w["cx"][cells], w["cy"][cells], vgs, args,
                              **kw)
    mixed, _ = spi.interp_steps(w["sx"], w["sy"], z, w["cx"][cells], w["cy"][cells], vgs, args,
                                precision="mixed", **kw)
    for lab in f64:
        assert _err(mixed[lab], f64[lab]) <= MIXED_TOL, lab


def test_mixed_without_tensor_cores():
    """The FP32 tier on CUDA cores only (tensor_cores=False: k_krige_cells
    <float> with its own variance pass) at the mixed bar."""
    spi = _spi()
    sx, sy, z, cx, cy, vgs, sd, cd = _random_case(7)
    args = port.interp_args_for(["OK", "SK", ("IDW", 2.0)], est_vars=True)
    kw = dict(est_vars=True, min_var_thr=0.1, min_vg_val=1e-4, intrp_dtype=np.float64)
    ref, _ = port.interp_steps(sx, sy, z, cx, cy, vgs, args, **kw)
    got, _ = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, precision="mixed",
                              tensor_cores=False, **kw)
    for lab in ref:
        assert _err(got[lab], ref[lab]) <= MIXED_TOL, lab


def test_pinv_route_on_rank_deficient_systems():
    """Exactly singular systems: a duplicated station (OK and SK with Exp,
    Sph and Gau variograms) and an EDK drift equal to a constant. The
    reference inverts them with numpy.linalg.pinv (interp/steps.py:351),
    which drops singular values <= 1e-15 s_max; the null direction's
    computed singular value is rounding noise of about eps to 16 eps s_max,
    so whether pinv drops it depends on the rounding of its SVD (on x86 and
    on Arm the same matrix falls on different sides). Where the oracle's
    pinv drops it here (checked with the same SVD call) its answer is the
    truncated pseudo-inverse's, which the exact-inverse route must give
    (spi_krige_factor's pinv check), not a problem step: 1e-9 against the
    oracle. Where it does not, the GPU's answer must be one of the
    reference's outcomes under 1e-15 perturbations with the cut-off within
    rounding reach (tests/envelope.py)."""
    import envelope
    spi = _spi()
    rng = np.random.default_rng(31)
    n = 60
    sx, sy = rng.uniform(0, 6e4, n), rng.uniform(0, 6e4, n)
    sx[7], sy[7] = sx[6], sy[6]
    gx, gy = np.meshgrid(np.arange(24) * 2500.0 + 1250.0, 6e4 - 1250.0 - np.arange(24) * 2500.0)
    cx, cy = gx.ravel(), gy.ravel()
    vgs = ["0.1 Nug(0.0) + 0.9 Exp(15000)", "1.2 Sph(25000)", "0.05 Nug(0.0) + 0.8 Gau(12000)"]
    t = len(vgs)
    z = 3.0 + rng.normal(size=(t, n))
    const = dict(stn_drifts=np.full((n, 1), 5.0), cell_drifts=np.full((1, cx.size), 5.0))
    zc = z.copy()
    zc[:, 7] = np.nan  # no duplicate: the constant drift alone is singular
    matched = 0
    for kind, zz, drifts in (("OK", z, {}), ("SK", z, {}), ("EDK", zc, const)):
        args = port.interp_args_for([kind], est_vars=kind == "OK")
        kw = dict(est_vars=kind == "OK", min_var_thr=-np.inf, min_vg_val=1e-4,
                  intrp_dtype=np.float64, **drifts)
        ref, rp = port.interp_steps(sx, sy, zz, cx, cy, vgs, args, **kw)
        got, gp, info = spi.interp_steps(sx, sy, zz, cx, cy, vgs, args, return_info=True, **kw)
        assert gp == rp == [], kind
        assert info["pinv_steps"][kind] == [0, 1, 2], (kind, info["pinv_steps"])
        idx = np.where(np.isfinite(zz[0]))[0]
        for j, vg in enumerate(vgs):
            lhs, rhs, d_cs = envelope.system(kind, sx, sy, idx, cx, cy, vg, 1e-4,
                                             drifts.get("stn_drifts"),
                                             drifts.get("cell_drifts"))
            if envelope.pinv_cuts(lhs):
                matched += 1
                for lab in ref:
                    scale = max(float(np.abs(ref[lab][j]).max()), 1e-300)
                    e = float(np.abs(got[lab][j] - ref[lab][j]).max()) / scale
                    assert e <= FP64_TOL, (kind, vg, lab, e)
            else:
                rs = envelope.runs(lhs, rhs, idx.size, zz[j, idx][None], d_cs, kind == "OK")
                ok = envelope.consistent(got[kind][j][None], rs, zz[j, idx][None], d_cs, 1e-9)
                assert ok.mean() >= 0.98, (kind, vg, ok.mean())
    print(f"\npinv route: {matched} of 9 systems cut by this platform's pinv, checked at "
          "1e-9; the others inside the reference's rounding envelope")


@pytest.mark.parametrize("case", ["singular_gau_750", "duplicate_60"])
def test_step_by_step_elimination_is_bit_identical(monkeypatch, case):
    """The exact-inverse path's Gauss-Jordan elimination spread over the GPU
    (spi_gj_multi.cu, systems of >= 256 rows) performs gj_invert's
    operations one for one: forcing either form on the same systems gives
    identical fields, problem steps and routes."""
    import bench
    from spinterps_gb300 import steps as st
    spi = _spi()
    if case == "singular_gau_750":
        w = bench.make_workload()
        sel = [4, 10]   # Gaussian variograms, numerically singular OK systems
        sx, sy, z = w["sx"], w["sy"], w["z"][sel]
        vgs = [w["vgs"][s] for s in sel]
        cells = np.arange(0, w["cx"].size, 997)
        cx, cy = w["cx"][cells], w["cy"][cells]
        kw = dict(bench.KW, intrp_dtype=np.float64)
        args = bench.interp_args()
    else:
        rng = np.random.default_rng(4)
        sx, sy = rng.uniform(0, 5e4, 60), rng.uniform(0, 5e4, 60)
        sx[9], sy[9] = sx[8], sy[8]
        gx, gy = np.meshgrid(np.arange(30) * 1700.0, np.arange(20) * 2500.0)
        cx, cy = gx.ravel(), gy.ravel()
        z = 2.0 + rng.normal(size=(2, 60))
        vgs = ["0.1 Nug(0.0) + 0.9 Exp(15000)", "1.0 Gau(9000)"]
        kw = dict(est_vars=True, min_vg_val=1e-4, intrp_dtype=np.float64)
        args = port.interp_args_for(["OK", "SK"], est_vars=True)
    out = []
    for min_m in (10 ** 9, 0):
        monkeypatch.setattr(st, "GJ_MULTI_MIN_M", min_m)
        f, p, info = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, return_info=True, **kw)
        out.append((f, p, info))
    (f0, p0, i0), (f1, p1, i1) = out
    assert p0 == p1
    assert i0["exact_inverse_steps"] == i1["exact_inverse_steps"]
    assert any(i0["exact_inverse_steps"].values())
    for lab in f0:
        assert np.array_equal(f0[lab], f1[lab], equal_nan=True), lab


def test_fp32_factor_with_fp64_refinement():
    """The mixed path's FP32 factorisation with FP64 iterative refinement of
    the duals (systems without the OK variance; EDK and SK here): every
    well-conditioned system keeps its FP32 factor, its duals converge to
    FP64 accuracy in a few iterations, and the fields equal those of the
    FP64 factorisation (refine=False) to the FP64 bar, 1e-9 of the field
    (both solves carry errors near cond * eps), within the mixed bar of
    the oracle."""
    spi = _spi()
    sx, sy, z, cx, cy, vgs, sd, cd = _random_case(17, n=300, t=6)
    args = port.interp_args_for(["SK", "EDK"], est_vars=False)
    kw = dict(stn_drifts=sd, cell_drifts=cd, min_var_thr=0.1, min_vg_val=1e-4,
              intrp_dtype=np.float64, precision="mixed")
    got, _, info = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, return_info=True, **kw)
    ref64, _ = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, refine=False, **kw)
    ora, _ = port.interp_steps(sx, sy, z, cx, cy, vgs, args, **{k: v for k, v in kw.items()
                                                                 if k != "precision"})
    kept = info["ir_steps"]["EDK"]
    assert len(kept) >= 3, (info["ir_steps"], info["ir_fallback_steps"])
    its = info["ir_iters"]["EDK"]
    assert all(0 <= its[j] <= 6 for j in kept), its
    for lab in ref64:
        assert _err(got[lab], ref64[lab]) <= FP64_TOL, lab
        assert _err(got[lab], ora[lab]) <= MIXED_TOL, lab


@pytest.mark.parametrize("p", [1.0, 2.0, 3.5])
def test_idw_on_tensor_cores(p):
    """IDW as the masked GEMM pair on the tensor cores (spi_idw_cells_tc,
    the mixed path) against the FP64 path: 150 steps (five groups of 32),
    missing stations, steps under min_var_thr (the step mean), a cell on a
    station (NaN where that station is present), float64 fields, within
    the mixed bar of the field's largest magnitude."""
    spi = _spi()
    rng = np.random.default_rng(int(p * 10))
    N, T, C = 500, 150, 6000
    sx, sy = rng.uniform(0, 2e5, N), rng.uniform(0, 2e5, N)
    z = rng.gamma(0.6, 4.0, (T, N))
    z[rng.uniform(size=(T, N)) < 0.3] = np.nan
    z[5] = np.where(np.isnan(z[5]), np.nan, 0.01)        # under the threshold
    cx, cy = rng.uniform(0, 2e5, C), rng.uniform(0, 2e5, C)
    cx[17], cy[17] = sx[3], sy[3]                         # a cell on station 3
    z[7, 3] = np.nan                                      # missing at step 7
    z[8, 3] = 2.5                                         # present at step 8
    args = port.interp_args_for([("IDW", p)], est_vars=False)
    kw = dict(min_var_thr=0.1, intrp_dtype=np.float64)
    f64, _ = spi.interp_steps(sx, sy, z, cx, cy, [None] * T, args, **kw)
    mixed, _ = spi.interp_steps(sx, sy, z, cx, cy, [None] * T, args, precision="mixed", **kw)
    lab = "IDW_000"
    assert np.isnan(mixed[lab][8, 17]) and np.isfinite(mixed[lab][7, 17])
    assert np.all(mixed[lab][5] == f64[lab][5])
    assert _err(mixed[lab], f64[lab]) <= MIXED_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nugget_only_variogram_any_size(precision):
    """A nugget-only variogram with a range (as fits can return): the
    reference's saddle matrix is then rank 2a and its pinv gives the
    minimum-norm weights: OK the mean of the values (variance: the sill),
    EDK the drifts' least-squares fit, SK zero weights (every cell falls
    back to its nearest station). 300 stations, above the pinv check's 256
    rows; no problem steps."""
    spi = _spi()
    rng = np.random.default_rng(77)
    N, T, C = 300, 3, 900
    sx, sy = rng.uniform(0, 1e5, N), rng.uniform(0, 1e5, N)
    z = rng.gamma(1.5, 2.0, (T, N))
    z[1, rng.choice(N, 40, replace=False)] = np.nan
    cx, cy = rng.uniform(0, 1e5, C), rng.uniform(0, 1e5, C)
    sd = rng.uniform(0, 500, (N, 1))
    cd = rng.uniform(0, 500, (1, C))
    vgs = ["0.9 Nug(2000.0)"] * T
    args = port.interp_args_for(["OK", "SK", "EDK"], est_vars=True)
    got, prblm = spi.interp_steps(sx, sy, z, cx, cy, vgs, args, stn_drifts=sd, cell_drifts=cd,
                                  est_vars=True, min_vg_val=1e-4, intrp_dtype=np.float64,
                                  precision=precision)
    assert prblm == []
    d = np.hypot(cx[:, None] - sx[None], cy[:, None] - sy[None])
    for t in range(T):
        idx = np.where(np.isfinite(z[t]))[0]
        zt = z[t, idx]
        ok = np.full(C, zt.mean())
        F = np.column_stack([np.ones(idx.size), sd[idx, 0]])
        beta = np.linalg.lstsq(F, zt, rcond=None)[0]
        edk = beta[0] + beta[1] * cd[0]
        sk = zt[np.argmin(d[:, idx], 1)]
        assert _err(got["OK"][t], ok) <= FP64_TOL
        assert _err(got["EST_VARS_OK"][t], np.full(C, 0.9)) <= FP64_TOL
        assert _err(got["EDK"][t], edk) <= FP64_TOL
        assert np.array_equal(got["SK"][t], sk)
