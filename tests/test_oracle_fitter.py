"""Pin the fitter oracle (oracle/fitter.py) to the reference's Variogram
(variograms/vgs.py), run on the same seeded points by
tests/golden/make_golden.py: the empirical variogram and the objective must
match exactly; whole fits (scipy DE drawing from the same seeded global RNG)
must give the same variogram strings and AIC."""
import numpy as np
import pytest

from oracle import fitter


def _cases(golden):
    return [int(c) for c in golden["f_cases"]]


def test_empirical_variogram_exact(golden):
    g = golden
    for c in _cases(g):
        h, gam, cnt, max_dist, _ = fitter.empirical(g[f"f{c}_x"], g[f"f{c}_y"], g[f"f{c}_z"],
                                                    nk=50, mdr=0.7)
        assert np.array_equal(h, g[f"f{c}_h"])
        assert np.array_equal(gam, g[f"f{c}_g"])
        assert np.array_equal(cnt, g[f"f{c}_np"])
        assert max_dist == g[f"f{c}_maxd"]


def test_empirical_variogram_sweep_exact(golden):
    """The same on 40 seeded random station sets (tests/golden/
    empirical_sweep.npz): lattices with many tied distances, nk 10 / 25 /
    50, mdr 0.3 to 1.0."""
    g = golden
    for c in g["fe_cases"]:
        p = f"fe{c}_"
        h, gam, cnt, max_dist, _ = fitter.empirical(g[p + "x"], g[p + "y"], g[p + "z"],
                                                    nk=int(g[p + "nk"]), mdr=float(g[p + "mdr"]))
        assert np.array_equal(h, g[p + "h"]), c
        assert np.array_equal(gam, g[p + "g"]), c
        assert np.array_equal(cnt, g[p + "np"]), c
        assert max_dist == g[p + "maxd"], c


def test_objective_exact(golden):
    g = golden
    for c in _cases(g):
        h, gam = g[f"f{c}_h"], g[f"f{c}_g"]
        got = []
        for p4 in g[f"f{c}_prm"]:
            got.append(fitter.objective(p4[2:], ("Sph",), h, gam))
            got.append(fitter.objective(p4[2:], ("Exp",), h, gam))
            got.append(fitter.objective(p4, ("Nug", "Exp"), h, gam))
        assert np.array_equal(np.array(got), g[f"f{c}_obj"])


@pytest.mark.parametrize("c", [0, 1, 2])
def test_seeded_fit_matches_reference(golden, c):
    pytest.importorskip("scipy")
    g = golden
    strs, objs, prms, _ = fitter.fit(g[f"f{c}_x"], g[f"f{c}_y"], g[f"f{c}_z"], seed=1000 + c)
    assert strs == [str(s) for s in g[f"f{c}_vgstr"]]
    assert np.allclose(objs, g[f"f{c}_bestobj"], rtol=1e-12)
    assert np.allclose(prms, g[f"f{c}_bestprm"], rtol=1e-12)
