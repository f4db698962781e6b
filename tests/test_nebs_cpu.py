"""Host logic of the neighbour methods (spinterps_gb300.nebs) without a GPU:
the device grouping of cells by identical neighbour lists that
spi_local_groups consumes, against the oracle's grouping of
interp/grps.py:103-138 on the neighbour lists the oracle selects."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import port  # noqa: E402


@pytest.mark.parametrize("mth,nn,npie", [("nrst", 8, 1), ("pie", 12, 4), ("nrst", 3, 1)])
def test_device_groups_partition_like_the_reference(mth, nn, npie):
    from spinterps_gb300.nebs import device_groups
    rng = np.random.default_rng(40 + nn)
    sx, sy = rng.uniform(0, 5e4, 30), rng.uniform(0, 5e4, 30)
    cx, cy = rng.uniform(0, 5e4, 600), rng.uniform(0, 5e4, 600)
    idx = port.neb_idxs(mth, cx, cy, sx, sy, nn, npie)
    nb = torch.as_tensor(idx.astype(np.int32))
    grp_nebs, cell_grp, order = device_groups(nb)
    for t in (grp_nebs, cell_grp, order):
        assert t.dtype == torch.int32 and t.is_contiguous()
    g, c, o = grp_nebs.numpy(), cell_grp.numpy(), order.numpy()
    # every cell's list is its group's list, and the groups' lists are distinct
    assert np.array_equal(g[c], idx)
    assert np.unique(g, axis=0).shape[0] == g.shape[0]
    # the order lists each group's cells together, cells ascending within a group
    assert np.array_equal(np.sort(o), np.arange(cx.size))
    assert np.all(np.diff(c[o]) >= 0)
    same = np.diff(c[o]) == 0
    assert np.all(np.diff(o)[same] > 0)
    # the same partition of the cells as the reference's grouping
    _, ref_groups = port.neb_groups(idx)
    ours = sorted(tuple(np.where(c == k)[0]) for k in range(g.shape[0]))
    assert ours == sorted(tuple(x) for x in ref_groups)


def test_device_groups_with_empty_slots():
    """'pie' lists can end in empty slots (-1): they group like any value."""
    from spinterps_gb300.nebs import device_groups
    nb = torch.tensor([[0, 3, -1], [1, 2, 4], [0, 3, -1], [1, 2, 4], [5, -1, -1]],
                      dtype=torch.int32)
    g, c, o = (t.numpy() for t in device_groups(nb))
    assert g.shape == (3, 3)
    assert np.array_equal(g[c], nb.numpy())
    assert c[0] == c[2] and c[1] == c[3] and len({c[0], c[1], c[4]}) == 3
    assert list(o[np.argsort(c[o], kind="stable")]) == list(o)
