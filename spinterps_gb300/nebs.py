"""Neighbour selection and grouping of destination cells (the reference's
SpInterpNeighborGrouping, interp/grps.py:13-288).

'all' uses every present station; 'nrst' the n_nebs nearest; 'pie' stations
nearest in each of n_pies angular sectors first. The selection runs on the
GPU (spi_neb_select, csrc/spi_nebs.cu); cells with identical neighbour lists
form the groups the step engine solves together, in order of first
occurrence as the reference's hash grouping (interp/grps.py:103-138).
"""
import numpy as np
import torch

from . import _native as nat
from .steps import _ptr, _require_cuda, _stream

METHODS = {"nrst": 1, "pie": 2}


class SpInterpNeighborGrouping:
    def __init__(self, neb_sel_method, n_nebs, n_pies, dst_xs, dst_ys, verbose=False,
                 device="cuda"):
        if neb_sel_method not in ("all", "nrst", "pie"):
            raise ValueError(neb_sel_method)
        if neb_sel_method == "nrst" and not (isinstance(n_nebs, int) and n_nebs > 0):
            raise ValueError("n_nebs must be a positive int")
        if neb_sel_method == "pie" and not (isinstance(n_pies, int) and n_nebs >= n_pies):
            raise ValueError("pie needs an int n_pies <= n_nebs")
        self.dev = _require_cuda(device)
        self._neb_sel_mthd = neb_sel_method
        self._n_nebs, self._n_pies = n_nebs, n_pies
        self._dst_xs = np.ascontiguousarray(dst_xs, dtype=np.float64)
        self._dst_ys = np.ascontiguousarray(dst_ys, dtype=np.float64)
        self._d = (torch.as_tensor(self._dst_xs, device=self.dev),
                   torch.as_tensor(self._dst_ys, device=self.dev))

    def neb_idxs(self, ref_xs, ref_ys):
        """[n_dst, k] neighbour indices into ref_xs (ascending per row)."""
        ref_xs = np.ascontiguousarray(ref_xs, dtype=np.float64)
        ref_ys = np.ascontiguousarray(ref_ys, dtype=np.float64)
        n, C = ref_xs.size, self._dst_xs.size
        if self._neb_sel_mthd == "all":
            return np.tile(np.arange(n), (C, 1))
        k = min(self._n_nebs, n) if self._neb_sel_mthd == "nrst" else self._n_nebs
        rx = torch.as_tensor(ref_xs, device=self.dev)
        ry = torch.as_tensor(ref_ys, device=self.dev)
        out = torch.empty((C, k), dtype=torch.int32, device=self.dev)
        nat.call("spi_neb_select", METHODS[self._neb_sel_mthd], _ptr(self._d[0]),
                 _ptr(self._d[1]), C, _ptr(rx), _ptr(ry), n, int(self._n_nebs),
                 int(self._n_pies or 0), _ptr(out), _stream())
        return out.cpu().numpy().astype(np.int64)

    @staticmethod
    def groups(all_neb_idxs):
        """Group label of every destination and the groups (destination
        indices), groups in order of first occurrence."""
        _, first, inv = np.unique(all_neb_idxs, axis=0, return_index=True, return_inverse=True)
        inv = np.asarray(inv).ravel()
        rank = np.empty(first.size, dtype=np.int64)
        rank[np.argsort(first)] = np.arange(first.size)
        lab = rank[inv]
        order = np.argsort(lab, kind="stable")
        bounds = np.searchsorted(lab[order], np.arange(first.size + 1))
        return lab, [order[bounds[g]:bounds[g + 1]] for g in range(first.size)]

    def get_neb_idxs_and_grps(self, ref_xs, ref_ys):
        """(all_neb_idxs, neb_idxs_grps) as interp/grps.py:249-288."""
        idx = self.neb_idxs(ref_xs, ref_ys)
        return idx, self.groups(idx)[1]


def interp_steps_nebs(stn_x, stn_y, data, cell_x, cell_y, vgs, interp_args, neb_sel_mthd,
                      n_nebs, n_pies, *, stn_drifts=None, cell_drifts=None,
                      intrp_dtype=np.float32, time_steps=None, device="cuda", **kw):
    """The step engine with 'nrst' / 'pie' neighbours (interp/steps.py:584-606,
    673-833): stations that are nobody's neighbour with every station present
    are dropped; then, per group of steps with the same stations, every group
    of cells with the same neighbours is interpolated from those neighbours
    alone (the batched plan of spinterps_gb300.steps on that cell subset).
    Returns (fields, problem steps) like steps.interp_steps."""
    from .steps import InterpPlan
    stn_x = np.ascontiguousarray(stn_x, dtype=np.float64)
    stn_y = np.ascontiguousarray(stn_y, dtype=np.float64)
    cell_x = np.ascontiguousarray(cell_x, dtype=np.float64)
    cell_y = np.ascontiguousarray(cell_y, dtype=np.float64)
    data = np.ascontiguousarray(data, dtype=np.float64)
    T, C = data.shape[0], cell_x.size
    if time_steps is None:
        time_steps = np.arange(T)
    g = SpInterpNeighborGrouping(neb_sel_mthd, n_nebs, n_pies, cell_x, cell_y, device=device)
    keep = np.unique(g.neb_idxs(stn_x, stn_y))
    sx, sy, data = stn_x[keep], stn_y[keep], data[:, keep]
    sd = None if stn_drifts is None else np.asarray(stn_drifts).reshape(stn_x.size, -1)[keep]
    cd = None if cell_drifts is None else np.asarray(cell_drifts).reshape(-1, C)
    vgs = None if vgs is None else np.asarray(vgs, dtype=object)
    labels = [a[2] for a in interp_args]
    flds = {lab: np.full((T, C), np.nan, dtype=intrp_dtype) for lab in labels}
    prblm = []
    avail = np.isfinite(data)
    _, first, inv = np.unique(np.packbits(avail, axis=1), axis=0, return_index=True,
                              return_inverse=True)
    inv = np.asarray(inv).ravel()
    for gi in np.argsort(first):
        rows = np.where(inv == gi)[0]
        stn_idxs = np.where(avail[rows[0]])[0]
        if not stn_idxs.size:
            for t in time_steps[rows]:
                if t not in prblm:
                    prblm.append(t)
            continue
        nidx = g.neb_idxs(sx[stn_idxs], sy[stn_idxs])
        for grp in g.groups(nidx)[1]:
            sub = stn_idxs[nidx[grp[0]]]
            plan = InterpPlan(sx[sub], sy[sub], data[rows][:, sub], cell_x[grp], cell_y[grp],
                              None if vgs is None else vgs[rows], interp_args,
                              stn_drifts=None if sd is None else sd[sub],
                              cell_drifts=None if cd is None else cd[:, grp],
                              intrp_dtype=intrp_dtype, time_steps=time_steps[rows],
                              device=device, **kw)
            plan.execute()
            out = plan.fields()
            for lab in labels:
                flds[lab][np.ix_(rows, grp)] = out[lab]
            for t in plan.problem_steps():
                if t not in prblm:
                    prblm.append(t)
    return flds, prblm
