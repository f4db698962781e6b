"""Neighbour selection and grouping of destination cells (the reference's
SpInterpNeighborGrouping, interp/grps.py:13-288).

'all' uses every present station; 'nrst' the n_nebs nearest; 'pie' stations
nearest in each of n_pies angular sectors first. The selection runs on the
GPU (spi_neb_select, csrc/spi_nebs.cu); cells with identical neighbour lists
form the groups the step engine solves together, in order of first
occurrence as the reference's hash grouping (interp/grps.py:103-138).
"""
import ctypes

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

    def neb_idxs_device(self, ref_xs, ref_ys):
        """[n_dst, k] int32 device tensor of neighbour indices into ref_xs
        (ascending per row, -1 in unused slots at the end)."""
        ref_xs = np.ascontiguousarray(ref_xs, dtype=np.float64)
        ref_ys = np.ascontiguousarray(ref_ys, dtype=np.float64)
        n, C = ref_xs.size, self._dst_xs.size
        if self._neb_sel_mthd == "all":
            return torch.arange(n, dtype=torch.int32, device=self.dev).expand(C, n).contiguous()
        k = min(self._n_nebs, n) if self._neb_sel_mthd == "nrst" else self._n_nebs
        rx = torch.as_tensor(ref_xs, device=self.dev)
        ry = torch.as_tensor(ref_ys, device=self.dev)
        out = torch.empty((C, k), dtype=torch.int32, device=self.dev)
        nat.call("spi_neb_select", METHODS[self._neb_sel_mthd], _ptr(self._d[0]),
                 _ptr(self._d[1]), C, _ptr(rx), _ptr(ry), n, int(self._n_nebs),
                 int(self._n_pies or 0), _ptr(out), _stream())
        return out

    def neb_idxs(self, ref_xs, ref_ys):
        """[n_dst, k] neighbour indices into ref_xs (ascending per row)."""
        return self.neb_idxs_device(ref_xs, ref_ys).cpu().numpy().astype(np.int64)

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


LOCAL_KIND = {"OK": 0, "SK": 1, "EDK": 2, "IDW": 3, "NNB": 4}


# Scratch for the per-group inverses of one call of spi_local_groups; steps
# beyond it are processed in chunks.
GRP_SCRATCH_BYTES = 2 << 30


def device_groups(nb):
    """Cells with identical neighbour lists, on the device: (grp_nebs [G, k],
    cell_grp [C], cell_order [C]) as int32, cell_order listing each group's
    cells together in ascending cell order."""
    grp_nebs, cell_grp = torch.unique(nb, dim=0, return_inverse=True)
    cell_order = torch.argsort(cell_grp, stable=True)
    return (grp_nebs.to(torch.int32).contiguous(), cell_grp.to(torch.int32).contiguous(),
            cell_order.to(torch.int32).contiguous())


def interp_steps_nebs(stn_x, stn_y, data, cell_x, cell_y, vgs, interp_args, neb_sel_mthd,
                      n_nebs, n_pies, *, stn_drifts=None, cell_drifts=None,
                      intrp_dtype=np.float32, time_steps=None, device="cuda", est_vars=False,
                      min_var_thr=0.0, min_var_cut=None, max_var_cut=None, min_vg_val=0.0,
                      **kw):
    """The step engine with 'nrst' / 'pie' neighbours (interp/steps.py:584-606,
    673-833). Stations that are nobody's neighbour with every station
    present are dropped. Then, per group of steps with the same stations,
    the neighbour lists are selected and grouped on the device, and
    - kriging (OK / SK / EDK) runs as the reference's _get_interp per group
      of cells with identical neighbour lists: spi_local_groups inverts
      each group's system once per step and applies it to the group's
      cells;
    - IDW and NNB run per cell (spi_local_cells, one warp per (cell, step)).
    FP64 in either precision; the other keywords of steps.interp_steps do
    not apply. Returns (fields, problem steps) like steps.interp_steps."""
    import torch
    from . import _native as nat
    from .steps import (_Domain, _out_struct, _ptr, _require_cuda, _stream, _vg_tensor,
                        check_full_nuggetness, parse_vg)
    dev = _require_cuda(device)
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
    keep = keep[keep >= 0]
    sx, sy, data = stn_x[keep], stn_y[keep], np.ascontiguousarray(data[:, keep])
    sd = None if stn_drifts is None else np.asarray(stn_drifts).reshape(stn_x.size, -1)[keep]
    cd = None if cell_drifts is None else np.asarray(cell_drifts).reshape(-1, C)
    dom = _Domain(dev, sx, sy, cell_x, cell_y, sd, cd, min_vg_val, 0)
    tdt = torch.float64 if np.dtype(intrp_dtype) == np.float64 else torch.float32
    labels = [a[2] for a in interp_args]
    flds = {lab: torch.full((T, C), float("nan"), dtype=tdt, device=dev) for lab in labels}
    d_data = torch.as_tensor(data, device=dev)
    krig = any(a[0] in ("OK", "SK", "EDK") for a in interp_args)
    vgt = nug = None
    if krig:
        vgl = [str(v) for v in vgs]
        vgt = _vg_tensor([parse_vg(v) for v in vgl], dev).view(T, -1)
        nug = torch.as_tensor(np.array([check_full_nuggetness(v, min_vg_val) for v in vgl],
                                       dtype=np.int32), device=dev)
    n_drift = int(dom.st.n_drift)
    prblm = []
    flags = torch.zeros(T, dtype=torch.int32, device=dev)
    avail = np.isfinite(data)
    _, first, inv = np.unique(np.packbits(avail, axis=1), axis=0, return_index=True,
                              return_inverse=True)
    inv = np.asarray(inv).ravel()
    s = _stream()
    held = []  # device arrays in use by queued launches
    for gi in np.argsort(first):
        rows = np.where(inv == gi)[0]
        stn_idxs = np.where(avail[rows[0]])[0]
        if not stn_idxs.size:
            prblm.extend(t for t in time_steps[rows] if t not in prblm)
            continue
        nidx = g.neb_idxs_device(sx[stn_idxs], sy[stn_idxs])
        k = nidx.shape[1]
        d_stn = torch.as_tensor(stn_idxs.astype(np.int32), device=dev)
        d_nb = torch.where(nidx >= 0, d_stn[nidx.clamp(min=0).long()], nidx).contiguous()
        d_rows = torch.as_tensor(rows.astype(np.int32), device=dev)
        d_vg = vgt[d_rows.long()].contiguous() if krig else None
        d_nug = nug[d_rows.long()].contiguous() if krig else None
        d_pr = torch.zeros(rows.size, dtype=torch.int32, device=dev)
        grp = scratch = None
        held.append((d_stn, d_nb, d_rows, d_vg, d_nug, d_pr))
        for a in interp_args:
            if a[0] == "EST_VARS_OK":  # written by the OK launch
                continue
            kind = LOCAL_KIND[a[0]]
            want_var = bool(est_vars and a[0] == "OK" and "EST_VARS_OK" in flds)
            out = _out_struct(flds[a[2]], flds["EST_VARS_OK"] if want_var else None,
                              min_var_cut, max_var_cut)
            if kind <= 2:
                if grp is None:
                    grp = device_groups(d_nb)
                    G = grp[0].shape[0]
                    held.append(grp)
                need = nat.lib().spi_local_groups_scratch_bytes(kind, k, n_drift, G, rows.size)
                one = nat.lib().spi_local_groups_scratch_bytes(kind, k, n_drift, G, 1)
                nbytes = max(one, min(need, GRP_SCRATCH_BYTES))
                if scratch is None or scratch.numel() < nbytes:
                    scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
                    held.append(scratch)
                nat.call("spi_local_groups", ctypes.byref(dom.st), kind, k, _ptr(grp[0]), G,
                         _ptr(grp[1]), _ptr(grp[2]), rows.size, _ptr(d_rows), _ptr(d_rows),
                         _ptr(d_data), data.shape[1], _ptr(d_vg), _ptr(d_nug),
                         float(min_var_thr), int(want_var), ctypes.byref(out), _ptr(scratch),
                         scratch.numel(), _ptr(d_pr), s)
            else:
                nat.call("spi_local_cells", ctypes.byref(dom.st), kind, k, _ptr(d_nb),
                         rows.size, _ptr(d_rows), _ptr(d_rows), _ptr(d_data), data.shape[1],
                         _ptr(d_vg), _ptr(d_nug), float(min_var_thr),
                         float(a[3]) if a[0] == "IDW" else 0.0, int(want_var),
                         ctypes.byref(out), _ptr(d_pr), s)
        flags.index_add_(0, d_rows.long(), d_pr)
    bad = np.where(flags.cpu().numpy() != 0)[0]
    prblm.extend(t for t in time_steps[bad] if t not in prblm)
    return {lab: v.cpu().numpy() for lab, v in flds.items()}, prblm
