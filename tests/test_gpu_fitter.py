"""GPU variogram fitting (spinterps_gb300.fitvgs) against the reference.

Empirical variograms must match the reference's bins (tests/golden/fitter.npz,
made by running variograms/vgs.py): distances, counts and bin means bit for
bit, the Cressie-Hawkins estimate to RTOL. The kernel rounds x^4 correctly;
numpy's ``** 4`` (a vectorised pow on x86) is off by one ulp in about 0.07% of
values, which the two divides that follow can widen to two ulps, so RTOL is
1e-15 (2 ulp is at most 4.4e-16 relative).

Whole fits: the GPU differential evolution draws its own random stream, so it
is compared by outcome under the reference's own selection score, the AIC
n*log(objective) + 2*params of vgs.py: the GPU's pick must score no worse
than the reference's seeded scipy pick (plus n*log(1.02), i.e. an objective
at most 2% above it). Names are not compared: on near-nugget fields the
reference's own pick flips between models with its seed (golden case 0: Nug
for seeds 0 and 2, Exp for 1, 3, 4, 5).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import fitter  # noqa: E402

RTOL = 1e-15


def test_empirical_bins_match_reference(golden):
    from spinterps_gb300 import fitvgs
    g = golden
    cases = [int(c) for c in g["f_cases"]]
    # all golden point sets as the steps of one batch (stations = union)
    xs = np.concatenate([g[f"f{c}_x"] for c in cases])
    ys = np.concatenate([g[f"f{c}_y"] for c in cases])
    data = np.full((len(cases), xs.size), np.nan)
    o = 0
    for k, c in enumerate(cases):
        n = g[f"f{c}_z"].size
        data[k, o:o + n] = g[f"f{c}_z"]
        o += n
    emp = fitvgs.Empirical(xs, ys, data, nk=50, mdr=0.7).run()
    torch.cuda.synchronize()
    for k, c in enumerate(cases):
        h, gam, cnt = emp.bins(k)
        assert np.array_equal(h, g[f"f{c}_h"])
        assert np.array_equal(cnt, g[f"f{c}_np"])
        assert np.allclose(gam, g[f"f{c}_g"], rtol=RTOL, atol=0)
        assert float(emp.max_dist[k]) == float(g[f"f{c}_maxd"])


def test_empirical_bins_match_oracle_larger():
    from spinterps_gb300 import fitvgs
    rng = np.random.default_rng(3)
    n = 600
    x, y = rng.uniform(0, 2e5, n), rng.uniform(0, 2e5, n)
    data = rng.gamma(0.8, 2.0, size=(3, n))
    data[rng.uniform(size=data.shape) < 0.3] = np.nan
    emp = fitvgs.Empirical(x, y, data, nk=50, mdr=0.7).run()
    for k in range(3):
        idx = np.isfinite(data[k])
        h, gam, cnt, md, _ = fitter.empirical(x[idx], y[idx], data[k, idx], nk=50, mdr=0.7)
        gh, gg, gc = emp.bins(k)
        assert np.array_equal(gh, h)
        assert np.array_equal(gc, cnt)
        assert np.allclose(gg, gam, rtol=RTOL, atol=0)


def test_fits_match_reference_outcome(golden):
    from spinterps_gb300 import fitvgs
    g = golden
    for c in [int(c) for c in g["f_cases"]]:
        x, y, z = g[f"f{c}_x"], g[f"f{c}_y"], g[f"f{c}_z"]
        strs, det = fitvgs.fit_steps(x, y, z[None], seed=7, return_details=True)
        ref_names = [s.split(" ")[1].split("(")[0] for s in str(g[f"f{c}_vgstr"][-1]).split(" + ")]
        h, gam = g[f"f{c}_h"], g[f"f{c}_g"]
        f_gpu = fitter.objective(det[0]["params"], det[0]["names"], h, gam)
        f_ref = fitter.objective(g[f"f{c}_bestprm"], ref_names, h, gam)
        n = z.size
        aic_gpu = n * np.log(f_gpu) + 2 * len(det[0]["params"])
        aic_ref = n * np.log(f_ref) + 2 * len(g[f"f{c}_bestprm"])
        assert aic_gpu <= aic_ref + n * np.log(1.02), (c, strs, g[f"f{c}_vgstr"], aic_gpu,
                                                        aic_ref)
