"""Host side of the GB300 step engine: the reference's SpInterpSteps, batched.

Mirrors ``interp/steps.py`` of spinterps:

- :class:`SpInterpSteps` keeps the reference's method names for the
  materialising kernels (``_get_dists_arr`` 73-86, ``_get_svars_arr``
  88-138, ``_get_2d_arr_subset`` 140-168), computed on the GPU through the
  C ABI.
- :func:`interp_steps` replaces ``_get_all_interp_outputs`` (478-835) with
  its per-group ``_get_interp`` calls (245-401) for neighbour method 'all':
  it takes the same inputs (station coordinates, the station x step value
  matrix with NaN for missing, cell coordinates, drifts, one variogram
  string per step, the interp_args list of interp/prepare.py:638-695) and
  returns the same fields ({label: [steps, cells]}, float32 by default) plus
  the problem steps. All steps go to the GPU at once: steps are grouped into
  kriging systems (station set x variogram), every system is built and
  factored in FP64 in one launch, and one launch writes every cell of every
  step of every system.

Reference behaviours kept (file:line):
- steps without stations: outputs stay NaN, step reported as a problem
  step (673-690);
- one station: its value everywhere, OK variance NaN (282-283);
- no value >= min_value_to_interp_thresh, or a nugget-only variogram
  (misc.py:1074-1105): the step mean, variance 0 (325-331; IDW 311-313);
- the isclose(sum(lambda), 1) check with nearest-station fallback (418-426);
- the OK variance lambda'gamma + 2 mu (429-434);
- estimates clipped to [min_var_cut, max_var_cut] (466-476), fields cast to
  float32 (interp/prepare.py:42).
"""
import ctypes
from collections import OrderedDict

import numpy as np
import torch

from . import _native as nat

PRECISION = {"fp64": 0, "mixed": 1}


def _require_cuda(device):
    if not torch.cuda.is_available():
        raise RuntimeError("spinterps_gb300 needs a CUDA GPU; there is no CPU fallback")
    dev = torch.device(device)
    if dev.type != "cuda":
        raise ValueError("device must be a CUDA device")
    nat.lib()
    return dev


# Default condition cap of the double-float variance tier: its right-hand
# sides carry ~1e-9 relative error, which the probe checks system by
# system.
COND_DF = 1e13


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


_VG_CACHE = {}
_NUG_CACHE = {}
# the autotuner's cell tiles (InterpPlan.autotune)
_TILE_CACHE = {}
# systems of at least this many rows (stations + Lagrange / drift rows) take
# the step-by-step Gauss-Jordan elimination over the whole GPU on the
# exact-inverse path (2 launches per row); smaller ones one CTA each
GJ_MULTI_MIN_M = 256


def parse_vg(vg_str):
    """Parse a variogram string with the reference's rules (C ABI)."""
    v = _VG_CACHE.get(vg_str)
    if v is None:
        v = nat.VgT()
        nat.call("spi_parse_vg", str(vg_str).encode(), ctypes.byref(v))
        _VG_CACHE[vg_str] = v
    return v


def check_full_nuggetness(vg_str, min_vg_val):
    key = (vg_str, float(min_vg_val))
    r = _NUG_CACHE.get(key)
    if r is None:
        out = nat.c_i32(0)
        nat.call("spi_check_full_nuggetness", str(vg_str).encode(), float(min_vg_val),
                 ctypes.byref(out))
        r = bool(out.value)
        _NUG_CACHE[key] = r
    return r


def _vg_tensor(vgs, dev):
    arr = (nat.VgT * len(vgs))(*vgs)
    raw = bytes(arr)
    return torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(dev)


def _as_dev(x, dev, dtype=torch.float64):
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(x)).to(device=dev, dtype=dtype)


class SpInterpSteps:
    """GPU versions of the reference step engine's materialising kernels.

    Inputs may be numpy arrays (results come back as numpy) or CUDA tensors
    (results stay on the device).
    """

    def __init__(self, min_vg_val=0.0, device="cuda"):
        self._min_vg_val = float(min_vg_val)
        self._dev = _require_cuda(device)

    def _io(self, *arrs):
        host = not isinstance(arrs[0], torch.Tensor)
        return host, [_as_dev(a, self._dev) for a in arrs]

    @staticmethod
    def _back(t, host):
        if host:
            return t.cpu().numpy()
        return t

    def _get_dists_arr(self, x1s, y1s, x2s, y2s):
        host, (x1, y1, x2, y2) = self._io(x1s, y1s, x2s, y2s)
        assert x1.ndim == y1.ndim == x2.ndim == y2.ndim == 1
        assert x1.numel() == y1.numel() and x2.numel() == y2.numel()
        out = torch.full((x1.numel(), x2.numel()), float("nan"), dtype=torch.float64,
                         device=self._dev)
        nat.call("spi_fill_dists_2d_mat", _ptr(x1), _ptr(y1), x1.numel(), _ptr(x2), _ptr(y2),
                 x2.numel(), _ptr(out), _stream())
        return self._back(out, host)

    def _get_svars_arr(self, dists_arr, vgs, interp_types, diag_mat_flag):
        assert isinstance(interp_types, (list, tuple))
        host, (d,) = self._io(dists_arr)
        var_flag = any(t in interp_types for t in ("OK", "EDK"))
        covar_flag = "SK" in interp_types
        out = {}
        for vg in vgs:
            assert vg != "nan"
            for flag, on in ((0, var_flag), (1, covar_flag)):
                if not on:
                    continue
                a = torch.full_like(d, float("nan"))
                v = parse_vg(vg)
                nat.call("spi_fill_vg_var_arr", _ptr(d), d.shape[0], d.shape[1], _ptr(a), flag,
                         int(diag_mat_flag), ctypes.byref(v), self._min_vg_val, _stream())
                out[(vg, flag)] = self._back(a, host)
        return out

    def _get_2d_arr_subset(self, arr, row_idxs, col_idxs, rows_add_rc=0, cols_add_rc=0):
        host, (a,) = self._io(arr)
        ri = _as_dev(row_idxs, self._dev, torch.int64)
        ci = _as_dev(col_idxs, self._dev, torch.int64)
        assert a.ndim == 2 and ri.ndim == 1 and ci.ndim == 1
        assert a.numel() and ri.numel() and ci.numel()
        assert int(ri.min()) >= 0 and int(ri.max()) < a.shape[0]
        assert int(ci.min()) >= 0 and int(ci.max()) < a.shape[1]
        sub = torch.full((ri.numel() + rows_add_rc, ci.numel() + cols_add_rc), float("nan"),
                         dtype=torch.float64, device=self._dev)
        nat.call("spi_copy_2d_arr_at_idxs", _ptr(a), a.shape[0], a.shape[1], _ptr(ri),
                 ri.numel(), _ptr(ci), ci.numel(), _ptr(sub), sub.shape[1], _stream())
        return self._back(sub, host)


class _Domain:
    """Device copies of the coordinates/drifts and the spi_domain_t."""

    def __init__(self, dev, stn_x, stn_y, cell_x, cell_y, stn_drifts, cell_drifts,
                 min_vg_val, precision):
        self.sx = _as_dev(stn_x, dev)
        self.sy = _as_dev(stn_y, dev)
        self.cx = _as_dev(cell_x, dev)
        self.cy = _as_dev(cell_y, dev)
        self.N = self.sx.numel()
        self.C = self.cx.numel()
        self.sd = self.cd = None
        k = 0
        if stn_drifts is not None:
            self.sd = _as_dev(np.asarray(stn_drifts).reshape(self.N, -1), dev)
            self.cd = _as_dev(np.asarray(cell_drifts).reshape(-1, self.C), dev)
            k = self.sd.shape[1]
            if k > nat.SPI_MAX_DRIFT:
                raise ValueError(f"at most {nat.SPI_MAX_DRIFT} drifts")
        self.ssplit = self.csplit = None
        res = 0.0
        if precision == 1:
            ox = float(min(self.sx.min().item(), self.cx.min().item()))
            oy = float(min(self.sy.min().item(), self.cy.min().item()))
            ext = max(float(max(self.sx.max().item(), self.cx.max().item())) - ox,
                      float(max(self.sy.max().item(), self.cy.max().item())) - oy, 1e-300)
            # heads on a power-of-two grid with <= 22 significant bits
            res = 2.0 ** (np.ceil(np.log2(ext)) - 22)
            self.ssplit = torch.empty((self.N, 4), dtype=torch.float32, device=dev)
            self.csplit = torch.empty((self.C, 4), dtype=torch.float32, device=dev)
            nat.call("spi_split_coords", _ptr(self.sx), _ptr(self.sy), self.N, ox, oy, res,
                     _ptr(self.ssplit), _stream())
            nat.call("spi_split_coords", _ptr(self.cx), _ptr(self.cy), self.C, ox, oy, res,
                     _ptr(self.csplit), _stream())
        self.st = nat.DomainT(self.N, _ptr(self.sx), _ptr(self.sy), self.C, _ptr(self.cx),
                              _ptr(self.cy), k, _ptr(self.sd), _ptr(self.cd), float(min_vg_val),
                              _ptr(self.ssplit), _ptr(self.csplit), float(res))


class _DomainView:
    """A subset of a domain's cells (the mixed path's probe cells): the same
    stations and the same split coordinates (so FP32 entries are identical)."""

    def __init__(self, dom, idx):
        t = torch.as_tensor(np.asarray(idx, dtype=np.int64), device=dom.cx.device)
        self.C = int(t.numel())
        self.cx, self.cy = dom.cx[t].contiguous(), dom.cy[t].contiguous()
        self.cd = dom.cd[:, t].contiguous() if dom.cd is not None else None
        self.csplit = dom.csplit[t].contiguous() if dom.csplit is not None else None
        d = dom.st
        self.st = nat.DomainT(d.n_stns, d.stn_x, d.stn_y, self.C, _ptr(self.cx), _ptr(self.cy),
                              d.n_drift, d.stn_drift, _ptr(self.cd), d.min_vg_val, d.stn_split,
                              _ptr(self.csplit), d.split_res)


def _out_struct(est, var, min_var_cut, max_var_cut):
    return nat.OutT(1 if est.dtype == torch.float64 else 0, _ptr(est), _ptr(var),
                    0 if min_var_cut is None else 1, 0 if max_var_cut is None else 1,
                    0.0 if min_var_cut is None else float(min_var_cut),
                    0.0 if max_var_cut is None else float(max_var_cut))


def _align(x, a=32):
    return (x + a - 1) // a * a


class _KrigeBatch:
    """One chunk of kriging systems: device descriptors and workspaces."""

    def __init__(self, dev, dom, kind, systems, ch, data, T, val_off, beta, precision,
                 want_var=False, tensor_cores=True, n_probe=0, need_linv=None, pinv=None,
                 ir=True, cond_ir=1e10):
        self.ch = ch
        self.kind = kind
        self.precision = precision
        ns = np.array([len(systems[i][0]) for i in ch], dtype=np.int64)
        stn_off = np.concatenate([[0], np.cumsum(ns)]).astype(np.int64)
        stn_idx = np.concatenate([systems[i][0] for i in ch]).astype(np.int32)
        sizes = np.array([_align((n + nat.GA) * (n + nat.GA)) for n in ns], dtype=np.int64)
        mat_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
        self.arena = int(sizes.sum())
        steps_l = [systems[i][2] for i in ch]
        step_off = np.concatenate([[0], np.cumsum([len(x) for x in steps_l])]).astype(np.int64)
        steps = np.concatenate([np.asarray(x, dtype=np.int32) for x in steps_l])
        vals_l, off = [], 0
        for i, sl in zip(ch, steps_l):
            idx = systems[i][0]
            for j in sl:
                val_off[j] = off
                vals_l.append(data[j, idx])
                off += len(idx)
        self.steps_l = steps_l
        self.vals = torch.as_tensor(np.concatenate(vals_l), device=dev)
        self.vgt = _vg_tensor([parse_vg(systems[i][1]) for i in ch], dev)
        self.t = [torch.as_tensor(a, device=dev) for a in
                  (stn_off, stn_idx, mat_off, step_off, steps, val_off.copy())]
        self.out_row = torch.as_tensor(np.arange(T, dtype=np.int32), device=dev)
        t = self.t
        self.sy = nat.SystemsT(len(ch), nat.KIND[kind], _ptr(t[0]), _ptr(t[1]), _ptr(self.vgt),
                               _ptr(t[2]), _ptr(t[3]), _ptr(t[4]), _ptr(t[5]),
                               _ptr(self.out_row), int(ns.max()))
        n_sys = len(ch)
        self.L = torch.empty(self.arena, dtype=torch.float64, device=dev)
        # Linv only where the OK variance (or leave-one-out) reads it; other
        # systems get their duals and condition estimate from L by
        # triangular solves (spi_krige_factor / spi_krige_duals)
        if need_linv is None:
            need_linv = bool(want_var and kind == "OK")
        self.X = torch.empty(self.arena, dtype=torch.float64, device=dev) if need_linv else None
        self.status = torch.empty(n_sys, dtype=torch.int32, device=dev)
        self.route = torch.empty(n_sys, dtype=torch.int32, device=dev)
        self.cond = torch.empty(n_sys, dtype=torch.float64, device=dev)
        self.shift = torch.empty(n_sys, dtype=torch.float64, device=dev)
        self.g_cols = torch.zeros(int(stn_off[-1]) * nat.GA, dtype=torch.float64, device=dev)
        self.s_inv = torch.zeros(n_sys * nat.GA * nat.GA, dtype=torch.float64, device=dev)
        self.g_colsum = torch.zeros(n_sys * nat.GA, dtype=torch.float64, device=dev)
        self.w_hat = torch.zeros_like(self.vals)
        self.beta = beta
        self.pinv = pinv
        # cell tile per pass, from InterpPlan.autotune (0: the largest that
        # fits)
        self.tiles = {}
        self.split = None
        if precision == 1:
            # FP32 (hi, lo) pairs of Linv, G and w_hat for the split-precision kernel
            na = self.arena if self.X is not None else 0
            self.split = [torch.empty(k, dtype=torch.float32, device=dev)
                          for k in (na, na, self.g_cols.numel(), self.g_cols.numel(),
                                    self.w_hat.numel(), self.w_hat.numel())]
            if self.X is None:
                self.split[0] = self.split[1] = None
        # |Linv c|^2 per (system, cell) from the tensor cores (FP32 tier of
        # the OK variance)
        self.yy = None
        self.tc_err = None
        self.linv_tc = self.linv_tc_off = None
        if precision == 1 and want_var and kind == "OK" and tensor_cores:
            self.yy = torch.empty(len(ch) * dom.C, dtype=torch.float64, device=dev)
            self.tc_err = torch.zeros(1, dtype=torch.int32, device=dev)
            # Linv's TF32 terms in the tensor cores' tile order: per system,
            # per 256-row block, 8-column chunks up to the block's last row,
            # each with its stations' coordinates (spi_krige_var_tc_pack)
            kc = nat.SPI_VAR_TC_KC
            chunks = np.array([sum((min(int(n), rb + 256) + kc - 1) // kc
                                   for rb in range(0, int(n), 256)) for n in ns], dtype=np.int64)
            off = np.concatenate([[0], np.cumsum(chunks)]).astype(np.int64)
            self.linv_tc = torch.empty(int(off[-1]) * nat.SPI_VAR_TC_CHUNK_FLOATS,
                                       dtype=torch.float32, device=dev)
            self.linv_tc_off = torch.as_tensor(off, device=dev)
        # the probe (precision 1): both tiers on a few cells decide each
        # system's tier (spi_krige_tier)
        self.tier = self.probe = self.probe_df = None
        if precision == 1 and n_probe > 0:
            n_sys = len(ch)
            self.tier = torch.zeros(n_sys, dtype=torch.int32, device=dev)
            self.disc = torch.zeros((n_sys, 3), dtype=torch.float64, device=dev)
            f = lambda: torch.full((T, n_probe), float("nan"), dtype=torch.float64, device=dev)
            pe64, pe32 = f(), f()
            pv64, pv32 = (f(), f()) if want_var else (None, None)
            pyy = (torch.empty(n_sys * n_probe, dtype=torch.float64, device=dev)
                   if self.yy is not None else None)
            self.probe = (pe64, pe32, pv64, pv32, pyy, _out_struct(pe64, pv64, None, None),
                          _out_struct(pe32, pv32, None, None))
            if self.yy is not None:
                # the double-float variance on the probe cells (tier 2)
                pyy_d = torch.empty(n_sys * n_probe, dtype=torch.float64, device=dev)
                pe32d, pv32d = f(), f()
                self.probe_df = (pyy_d, pe32d, pv32d, _out_struct(pe32d, pv32d, None, None))
        ptrs = [_ptr(self.L), _ptr(self.X), _ptr(self.status), _ptr(self.route),
                _ptr(self.cond), _ptr(self.shift), _ptr(self.w_hat), _ptr(self.beta),
                _ptr(self.g_cols), _ptr(self.s_inv), _ptr(self.g_colsum),
                *[_ptr(t) for t in (self.split or [None] * 6)]]
        # cells of the exact-inverse variance passes that ran (main pass only)
        self.var_cells = torch.zeros(len(ch), dtype=torch.int32, device=dev)
        # numpy.linalg.pinv's cut-off on the exact-inverse systems
        # (spi_krige_factor with a pinv scratch): shared by the plan's
        # batches, which run in stream order
        self.pinv_used = torch.zeros(len(ch), dtype=torch.int32, device=dev)
        # exact-inverse systems of hundreds of rows: their Gauss-Jordan
        # elimination spread over the GPU, step by step (spi_gj_multi.cu);
        # smaller systems keep one CTA each
        self.a_rows = 0 if kind == "SK" else (1 + dom.st.n_drift if kind == "EDK" else 1)
        self.max_m = int(ns.max()) + self.a_rows
        self.gj = None
        if self.max_m >= GJ_MULTI_MIN_M:
            self.gj = torch.empty(1 + 2 * int(stn_off[-1]) + (2 * nat.GA + 1) * len(ch),
                                  dtype=torch.float64, device=dev)
        # the mixed path without the OK variance's inverse factor: every
        # system factored in FP32 first, its duals refined in FP64 where
        # the FP32 factor holds (cond <= cond_ir), FP64 otherwise
        self.l32 = self.ir = self.ir_iters = None
        if precision == 1 and self.X is None and ir:
            self.l32 = torch.empty(self.arena, dtype=torch.float32, device=dev)
            self.ir = torch.zeros(n_sys, dtype=torch.int32, device=dev)
            self.ir_iters = torch.zeros(n_sys, dtype=torch.int32, device=dev)
        extra = dict(pinv_scratch=_ptr(pinv), pinv_used=_ptr(self.pinv_used),
                     gj_scratch=_ptr(self.gj), l32=_ptr(self.l32), ir=_ptr(self.ir),
                     ir_iters=_ptr(self.ir_iters), cond_ir=float(cond_ir),
                linv_tc=_ptr(self.linv_tc), linv_tc_off=_ptr(self.linv_tc_off))
        self.ws = nat.KrigeWsT(*ptrs, _ptr(self.yy), _ptr(self.tier), _ptr(self.var_cells),
                               **extra)
        self.ws_probe = nat.KrigeWsT(*ptrs, _ptr(self.probe[4]) if self.probe else None, None,
                                     None, **extra)
        self.ws_probe_df = (nat.KrigeWsT(*ptrs, _ptr(self.probe_df[0]), None, None, **extra)
                            if self.probe_df else None)
        # algorithmic FLOP of the cell kernel: per (system, cell) the
        # triangular variance n(n+1), the dual columns 2na; per cell-step 2n
        self.n = ns
        self.n_steps = np.array([len(x) for x in steps_l], dtype=np.int64)

    def cell_flops(self, C, want_var, a):
        per = 2 * self.n * a + 2 * self.n * self.n_steps
        if want_var:
            per = per + self.n * (self.n + 1)
        return float(per.sum()) * C

    def kernel_flops(self, C, want_var, a, cond_split):
        """Algorithmic FLOP of each cell kernel of the last run: the OK
        variance n(n+1) per (system, cell), the dual columns 2na and 2n per
        cell-step; split by where each system ran (tensor-core variance,
        FP32 tier, FP64 tier)."""
        route = self.route.cpu().numpy()
        cond = self.cond.cpu().numpy()
        var = self.n * (self.n + 1) if want_var else np.zeros_like(self.n)
        rest = 2 * self.n * a + 2 * self.n * self.n_steps
        ok = route != 2
        # the exact-inverse path's variance (P r: 2 m^2 per cell) runs only
        # on tiles where a cell passes the sum check: counted from the
        # cells of the passes that ran (var_cells, last execution)
        vc = self.var_cells.cpu().numpy().astype(np.float64)
        m = self.n + (a if want_var else 0)
        prim_var = np.where(route == 1, 2.0 * m * m * vc, 0.0) if want_var else 0.0 * vc
        var = np.where(route == 1, 0, var)
        if self.precision == 1:
            tr = (self.tier.cpu().numpy() if self.tier is not None
                  else ((route == 0) & (cond <= cond_split)).astype(np.int32))
            fast = tr != 0
            tc = self.yy is not None and want_var
            return {"var_tc": float((var * (tr == 1)).sum()) * C if tc else 0.0,
                    "var_df": float((var * (tr == 2)).sum()) * C if tc else 0.0,
                    "cells_fp32": float(((rest + (0 if tc else var)) * fast).sum()) * C,
                    "cells_fp64": float(((rest + var) * (ok & ~fast)).sum()) * C
                    + float((prim_var * (ok & ~fast)).sum())}
        return {"cells_fp64": float(((rest + var) * ok).sum()) * C + float((prim_var * ok).sum())}

    def run(self, dom, out, want_var, cond_max, cond_split, ev=None, probe=None,
            cond_df=COND_DF):
        """Factor, duals, splits, (mixed) the probe that picks each system's
        tier, cell kernels. ``ev``: a list that receives (kernel name, start
        event, end event) per cell-kernel call; ``probe``: (probe domain,
        estimate tolerance, variance tolerance)."""
        s = _stream()
        ws = ctypes.byref(self.ws)

        def timed(name, fn):
            if ev is None:
                fn()
                return
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            ev.append((name, a, b))

        nat.call("spi_krige_factor", ctypes.byref(dom.st), ctypes.byref(self.sy), ws,
                 float(cond_max), s)
        nat.call("spi_krige_duals", ctypes.byref(dom.st), ctypes.byref(self.sy), _ptr(self.vals),
                 ws, s)
        if self.split is not None:
            xh, xl, gh, gl, wh, wl = self.split
            if self.X is not None:
                nat.call("spi_split_f64", _ptr(self.X), _ptr(xh), _ptr(xl), self.arena, s)
                if self.linv_tc is not None:
                    nat.call("spi_krige_var_tc_pack", ctypes.byref(dom.st), ctypes.byref(self.sy),
                             ws, s)
            nat.call("spi_split_f64", _ptr(self.g_cols), _ptr(gh), _ptr(gl), self.g_cols.numel(), s)
            nat.call("spi_split_f64", _ptr(self.w_hat), _ptr(wh), _ptr(wl), self.w_hat.numel(), s)
        if self.probe is not None and probe is not None:
            pdom, tol_e, tol_v = probe
            pe64, pe32, pv64, pv32, pyy, o64, o32 = self.probe
            wp = ctypes.byref(self.ws_probe)
            if pyy is not None and want_var:
                nat.call("spi_krige_var_tc", ctypes.byref(pdom.st), ctypes.byref(self.sy), wp,
                         float(cond_split), _ptr(self.tc_err), s)
            # the FP32-tier estimates of every double-float candidate (cond
            # up to cond_df); the tensor-core variance, and systems without
            # a variance, only under cond_split (the streamed estimate kernel
            # regenerates the right-hand sides for every four dual vectors:
            # slower than FP64 on systems shared by hundreds of steps)
            cap = max(float(cond_split), cond_df) if self.probe_df else float(cond_split)
            for prec, filt, o in ((1, 1, o32), (0, 0, o64)):
                nat.call("spi_krige_cells", ctypes.byref(pdom.st), ctypes.byref(self.sy),
                         _ptr(self.vals), wp, 1 if want_var else 0, prec, filt,
                         cap if prec == 1 else float(cond_split), ctypes.byref(o), s)
            pv32d = None
            if self.probe_df is not None and want_var:
                pyy_d, _, pv32d, o32d = self.probe_df
                wpd = ctypes.byref(self.ws_probe_df)
                nat.call("spi_krige_var_df", ctypes.byref(pdom.st), ctypes.byref(self.sy), wpd,
                         cap, s)
                nat.call("spi_krige_cells", ctypes.byref(pdom.st), ctypes.byref(self.sy),
                         _ptr(self.vals), wpd, 1, 1, 1, cap, ctypes.byref(o32d), s)
            nat.call("spi_krige_tier", ctypes.byref(self.sy), ws, pdom.C, _ptr(pe64), _ptr(pe32),
                     _ptr(pv64 if want_var else None), _ptr(pv32 if want_var else None),
                     _ptr(pv32d), float(tol_e), float(tol_v), float(cond_split), cap,
                     _ptr(self.tc_err), _ptr(self.tier), _ptr(self.disc), s)
        if self.yy is not None and want_var:
            timed("var_tc", lambda: nat.call(
                "spi_krige_var_tc", ctypes.byref(dom.st), ctypes.byref(self.sy), ws,
                float(cond_split), _ptr(self.tc_err), s))
            if self.tier is not None:
                timed("var_df", lambda: nat.call(
                    "spi_krige_var_df", ctypes.byref(dom.st), ctypes.byref(self.sy), ws,
                    float(cond_split), s))
        self.var_cells.zero_()
        for prec, filt in self.passes():
            tile = self.tiles.get((prec, filt), 0)
            timed("cells_fp32" if prec == 1 else "cells_fp64", lambda prec=prec, filt=filt,
                  tile=tile: nat.call(
                "spi_krige_cells_tiled", ctypes.byref(dom.st), ctypes.byref(self.sy),
                _ptr(self.vals), ws, 1 if want_var else 0, prec, filt, float(cond_split),
                ctypes.byref(out), tile, s))

    def gj_launches(self):
        """Kernels of the exact-inverse elimination in spi_krige_factor: one
        (one CTA per system), or, step by step over the GPU, set-up and
        finish plus two per row of the largest system that took the
        exact-inverse path (read from the routes of the last run)."""
        if self.gj is None:
            return 1
        route = self.route.cpu().numpy()
        pend = self.n[route != 0]
        return 2 + (2 * int(pend.max() + self.a_rows) if pend.size else 0)

    def passes(self):
        """The cell-kernel passes of run(): (precision, route filter)."""
        return [(1, 1), (0, 2)] if self.precision == 1 else [(0, 0)]

    def tiled(self, prec, want_var):
        """Whether the pass takes the shared-memory tile kernel (the FP32
        tier with a tensor-core variance, without a variance or SK, and
        systems too large for shared memory take the streamed kernel)."""
        if prec == 1 and (self.yy is not None or not want_var or self.kind == "SK"):
            return False
        return True


def _chunk_systems(systems, precision, arena_budget):
    order = sorted(range(len(systems)), key=lambda i: -len(systems[i][0]))
    chunks, cur, cur_bytes = [], [], 0
    for i in order:
        n = len(systems[i][0])
        b = _align((n + nat.GA) ** 2) * 8 * 2
        if cur and (cur_bytes + b > arena_budget or len(cur) >= 65535):
            chunks.append(cur)
            cur, cur_bytes = [], 0
        cur.append(i)
        cur_bytes += b
    if cur:
        chunks.append(cur)
    return chunks


class InterpPlan:
    """All host-side work of one interpolation job, done once: step
    grouping, flags, nugget checks, kriging systems, value gathering and
    the uploads. :meth:`execute` then runs only GPU work (factorisations,
    duals, cell kernels, IDW / NNB, row fills) on the current stream, from
    device-resident inputs into device-resident fields."""

    def __init__(self, stn_x, stn_y, data, cell_x, cell_y, vgs, interp_args, *,
                 est_vars=False, stn_drifts=None, cell_drifts=None, min_var_thr=0.0,
                 min_var_cut=None, max_var_cut=None, min_vg_val=0.0, intrp_dtype=np.float32,
                 time_steps=None, precision="fp64", device="cuda", arena_budget=8 << 30,
                 cond_max=1e13, cond_split=None, tensor_cores=True, probe_cells=1024,
                 probe_tol=2e-6, cond_df=COND_DF, refine=True, cond_ir=1e10):
        dev = self.dev = _require_cuda(device)
        if cond_split is None:
            # a cap under the probe; without it, the a-priori split
            cond_split = 1e10 if probe_cells > 0 else 1e7
        self.cond_max, self.cond_split = cond_max, cond_split
        self.cond_df = cond_df
        prec = self.prec = PRECISION[precision]
        data = np.ascontiguousarray(data, dtype=np.float64)
        T, N = data.shape
        self.T = T
        C = self.C = int(np.asarray(cell_x).size)
        if time_steps is None:
            time_steps = np.arange(T)
        types = self.types = [a[0] for a in interp_args]
        labels = self.labels = [a[2] for a in interp_args]
        self.interp_args = interp_args
        self.min_var_cut, self.max_var_cut = min_var_cut, max_var_cut
        tdt = torch.float64 if np.dtype(intrp_dtype) == np.float64 else torch.float32
        self.flds = OrderedDict((lab, torch.full((T, C), float("nan"), dtype=tdt, device=dev))
                                for lab in labels)
        avail = np.isfinite(data)
        n_av = avail.sum(1)
        means = np.full(T, np.nan)
        for j in np.where(n_av > 0)[0]:
            means[j] = data[j, avail[j]].mean()   # numpy's pairwise mean, as the reference
        flags = ((data >= min_var_thr) & avail).any(1)
        self.time_steps = time_steps
        self.prblm = [time_steps[j] for j in np.where(n_av == 0)[0]]
        self.single = np.where(n_av == 1)[0]
        self.single_val = np.array([data[j, avail[j]][0] for j in self.single], dtype=np.float64)
        multi = self.multi = np.where(n_av >= 2)[0]
        self.dom = _Domain(dev, stn_x, stn_y, cell_x, cell_y,
                           stn_drifts if "EDK" in types else None,
                           cell_drifts if "EDK" in types else None, min_vg_val, prec)
        self.krig = []
        krig = [t for t in ("OK", "SK", "EDK") if t in types]
        # the mixed path's probe: every system runs in both tiers on these
        # cells first; it takes the FP32 tier only where the two agree to
        # probe_tol of the fields' scale (the data's largest magnitude for
        # estimates, the largest total sill for variances)
        self.pdom = None
        n_probe = 0
        if krig and prec == 1 and probe_cells > 0:
            pidx = np.unique(np.linspace(0, C - 1, min(C, int(probe_cells))).round()
                             .astype(np.int64))
            self.pdom = _DomainView(self.dom, pidx)
            n_probe = self.pdom.C
            finite = data[avail]
            est_scale = float(np.abs(finite).max()) if finite.size else 1.0
            sills = [sum(parse_vg(v).sill[k] for k in range(parse_vg(v).n_comp))
                     for v in dict.fromkeys(np.asarray(vgs, dtype=object)[multi].tolist())
                     if v is not None]
            var_scale = max(sills) if sills else 1.0
            # variances get 2.5x the estimates' tolerance (still 2x under the
            # 1e-5 bar): the tensor-core TF32-split term carries ~2e-6 of the sill
            self.probe_args = (self.pdom, probe_tol * est_scale, 2.5 * probe_tol * var_scale)
        # scratch of the pinv check of exact-inverse systems (spi_krige_factor)
        self.pinv = (torch.empty(nat.SPI_PINV_SCRATCH_DOUBLES, dtype=torch.float64, device=dev)
                     if krig else None)
        # rows written after the kriging kernels: the OK variance of
        # nugget-only variograms (below)
        self.post_fills = []
        if krig:
            vgs = np.asarray(vgs, dtype=object)
            assert np.all(vgs != "nan"), "NaN VGs not allowed!"
            nug = np.array([check_full_nuggetness(v, min_vg_val) for v in vgs])
            packed = np.packbits(avail, axis=1)
            _, grp = np.unique(packed, axis=0, return_inverse=True)
            grp = grp.ravel()
            for kind in krig:
                est = self.flds[kind]
                var = self.flds["EST_VARS_OK"] if (kind == "OK" and est_vars) else None
                out = _out_struct(est, var, min_var_cut, max_var_cut)
                mean_steps = [j for j in multi if (not flags[j]) or nug[j]]
                systems = OrderedDict()
                for j in multi:
                    if (not flags[j]) or nug[j]:
                        continue
                    key = (int(grp[j]), vgs[j])
                    if key not in systems:
                        systems[key] = (np.where(avail[j])[0], vgs[j], [])
                    systems[key][2].append(int(j))
                systems = list(systems.values())
                if var is not None:
                    # nugget-only variograms (the cell kernels take the
                    # minimum-norm weights there, spi_krige_factor): the
                    # reference's variance lambda'gamma + mu is the total
                    # sill on every cell (lambda sums to 1, gamma is the
                    # sill everywhere, mu = 0)
                    rows, vv = [], []
                    for _, v, sl in systems:
                        pv = parse_vg(v)
                        if all(pv.code[c] == nat.VG_CODE["Nug"] for c in range(pv.n_comp)):
                            rows.extend(sl)
                            vv.extend([float(sum(pv.sill[c] for c in range(pv.n_comp)))] * len(sl))
                    if rows:
                        self.post_fills.append((_out_struct(var, None, None, None),
                                                _fill_args(dev, rows, vv, None)))
                val_off = np.zeros(T, dtype=np.int64)
                beta = torch.zeros((T, nat.GA), dtype=torch.float64, device=dev)
                batches = [_KrigeBatch(dev, self.dom, kind, systems, ch, data, T, val_off, beta,
                                       prec, want_var=var is not None,
                                       tensor_cores=tensor_cores, n_probe=n_probe,
                                       pinv=self.pinv, ir=refine, cond_ir=cond_ir)
                           for ch in _chunk_systems(systems, prec, arena_budget)]
                fills = (
                    _fill_args(dev, self.single, self.single_val,
                               None if var is None else np.full(self.single.size, np.nan)),
                    _fill_args(dev, mean_steps, means[mean_steps], np.zeros(len(mean_steps))))
                a = 1 + self.dom.st.n_drift if kind == "EDK" else 1
                self.krig.append((kind, out, var is not None, batches, fills, a))
        self.idw = []
        self.idw_pack = self.idw_err = None
        if any(t in ("IDW", "NNB") for t in types):
            self.data_d = torch.as_tensor(data, device=dev)
            self.data_hi = self.data_lo = None
            if prec == 1 and tensor_cores and "IDW" in types:
                # IDW as the masked GEMM pair on the tensor cores
                # (spi_idw_cells_tc): its packed B per 32 steps
                self.idw_pack_floats = nat.idw_tc_pack_floats(self.dom.N, len(multi))
                self.idw_pack = torch.empty(max(self.idw_pack_floats, 4), dtype=torch.float32,
                                            device=dev)
                self.idw_err = torch.zeros(1, dtype=torch.int32, device=dev)
            elif prec == 1:
                self.data_hi = torch.empty(data.size, dtype=torch.float32, device=dev)
                self.data_lo = torch.empty(data.size, dtype=torch.float32, device=dev)
            self.steps_t = torch.as_tensor(multi.astype(np.int32), device=dev)
            self.flag_t = torch.as_tensor(flags.astype(np.uint8), device=dev)
            self.mean_t = torch.as_tensor(np.nan_to_num(means), device=dev)
            n_present = n_av[multi].astype(np.float64)
            for i, t in enumerate(types):
                if t not in ("IDW", "NNB"):
                    continue
                out = _out_struct(self.flds[labels[i]], None, min_var_cut, max_var_cut)
                fill = _fill_args(dev, self.single, self.single_val, None)
                p = float(interp_args[i][3]) if t == "IDW" else 0.0
                self.idw.append((t, out, fill, p))
            # algorithmic work: 4 FLOP per present station and cell-step
            # (weighted values and weight sums); masked-out stations are not
            # counted
            self.idw_flops = 4.0 * float(n_present.sum()) * C
        self.info = {"failed_steps": {}, "cond": {}}

    def execute(self, timing=False):
        """Run the whole job on the GPU (current stream). With ``timing``,
        returns the CUDA events of every cell-kernel call (per batch:
        (batch, want_var, a, [(kernel, start, end)])) and of the IDW calls,
        read after a synchronisation (:meth:`kernel_times`)."""
        C = self.C
        evs = {"krige": [], "idw": []}
        s = _stream()
        for kind, out, want_var, batches, fills, a in self.krig:
            for f in fills:
                _fill_run(f, C, out, s)
            for b in batches:
                ev = [] if timing else None
                b.run(self.dom, out, want_var, self.cond_max, self.cond_split, ev,
                      self.probe_args if self.pdom is not None else None, self.cond_df)
                if timing:
                    evs["krige"].append((b, want_var, a, ev))
        for out, fill in self.post_fills:
            _fill_run(fill, C, out, s)
        for t, out, fill, p in self.idw:
            _fill_run(fill, C, out, s)
            if not len(self.multi):
                continue
            ev = None
            if timing:
                ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                ev[0].record()
            if t == "IDW" and self.idw_pack is not None:
                nat.call("spi_idw_cells_tc", ctypes.byref(self.dom.st), len(self.multi),
                         _ptr(self.steps_t), _ptr(self.steps_t), _ptr(self.data_d),
                         _ptr(self.flag_t), _ptr(self.mean_t), p, _ptr(self.idw_pack),
                         self.idw_pack_floats, ctypes.byref(out), _ptr(self.idw_err), s)
            elif t == "IDW":
                if self.data_hi is not None:
                    nat.call("spi_split_f64", _ptr(self.data_d), _ptr(self.data_hi),
                             _ptr(self.data_lo), self.data_d.numel(), s)
                nat.call("spi_idw_cells", ctypes.byref(self.dom.st), len(self.multi),
                         _ptr(self.steps_t), _ptr(self.steps_t), _ptr(self.data_d),
                         _ptr(self.data_hi), _ptr(self.data_lo), _ptr(self.flag_t),
                         _ptr(self.mean_t), p, self.prec, ctypes.byref(out), s)
            else:
                nat.call("spi_nnb_cells", ctypes.byref(self.dom.st), len(self.multi),
                         _ptr(self.steps_t), _ptr(self.steps_t), _ptr(self.data_d),
                         ctypes.byref(out), s)
            if timing:
                ev[1].record()
                evs["idw"].append(("idw", ev, self.idw_flops) if t == "IDW" else ("nnb", ev, 0.0))
        return evs

    def autotune(self, tiles=(16, 32, 64), cached_only=False):
        """Pick the cell tile of the shared-memory cell kernel per batch and
        pass: each candidate of ``tiles`` runs that pass (after one
        execute(): factors, duals and tiers in place; the pass rewrites the
        same fields), timed with CUDA events on the current stream after a
        warm-up launch of its own; the fastest is kept. Choices are cached
        process-wide per (precision, pass, kind, variance, station-count
        bucket of the next power of two), so later plans of the same shape
        reuse them untimed (``cached_only``: take cached choices only, for a
        plan not yet executed). Returns {(kind, batch, pass): tile}."""
        s = _stream()
        chosen = {}
        for kind, out, want_var, batches, fills, a in self.krig:
            for bi, b in enumerate(batches):
                bucket = 1 << int(np.ceil(np.log2(max(int(b.n.max()), 2))))
                for prec, filt in b.passes():
                    if not b.tiled(prec, want_var):
                        continue
                    key = (b.precision, prec, filt, kind, bool(want_var), bucket)
                    if key not in _TILE_CACHE and cached_only:
                        continue
                    if key not in _TILE_CACHE:
                        best, best_ms = 0, None
                        for tc in tiles:
                            ms = []
                            for _ in range(2):
                                e0 = torch.cuda.Event(enable_timing=True)
                                e1 = torch.cuda.Event(enable_timing=True)
                                e0.record()
                                rc = nat.lib().spi_krige_cells_tiled(
                                    ctypes.byref(self.dom.st), ctypes.byref(b.sy),
                                    _ptr(b.vals), ctypes.byref(b.ws), 1 if want_var else 0,
                                    prec, filt, float(self.cond_split), ctypes.byref(out), tc, s)
                                e1.record()
                                if rc:
                                    break
                                torch.cuda.synchronize()
                                ms.append(e0.elapsed_time(e1))
                            if rc == nat.SPI_ERR_TOO_LARGE:
                                continue
                            if rc:
                                raise nat.SpiError("spi_krige_cells_tiled", rc)
                            if best_ms is None or ms[-1] < best_ms:
                                best, best_ms = tc, ms[-1]
                        _TILE_CACHE[key] = best
                    b.tiles[(prec, filt)] = _TILE_CACHE[key]
                    chosen[(kind, bi, (prec, filt))] = _TILE_CACHE[key]
        return chosen

    def capture(self):
        """Record execute() in a CUDA graph (after one plain execution on the
        current stream, which sets the kernels' shared-memory attributes);
        replay() then runs the whole job with one launch from the host.
        The graph keeps the plan's device buffers and inputs: replay
        recomputes the same fields."""
        self.execute()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="thread_local"):
            self.execute()
        torch.cuda.synchronize()
        self._graph = g
        return g

    def replay(self):
        """Run the captured job (capture() first) on the current stream."""
        self._graph.replay()

    def collect_info(self):
        if self.idw_err is not None and int(self.idw_err.item()):
            raise RuntimeError("spi_idw_cells_tc: a tensor-core wait timed out (its cells hold "
                               "NaN)")
        for kind, out, want_var, batches, fills, a in self.krig:
            failed, routed, cond, pinv = [], [], {}, []
            for b in batches:
                if b.tc_err is not None and int(b.tc_err.item()):
                    raise RuntimeError("spi_krige_var_tc: a tensor-core wait timed out")
                rt = b.route.cpu().numpy()
                cn = b.cond.cpu().numpy()
                pu = b.pinv_used.cpu().numpy()
                for k, sl in enumerate(b.steps_l):
                    for j in sl:
                        cond[int(j)] = float(cn[k])
                        if rt[k] == 2:
                            failed.append(int(j))
                        elif rt[k] == 1:
                            routed.append(int(j))
                            if pu[k]:
                                pinv.append(int(j))
            fast, dfv, disc = [], [], []
            for b in batches:
                if b.tier is not None:
                    disc.append(b.disc.cpu().numpy())
                    tr = b.tier.cpu().numpy()
                    for k, sl in enumerate(b.steps_l):
                        if tr[k]:
                            fast.extend(int(j) for j in sl)
                        if tr[k] == 2:
                            dfv.extend(int(j) for j in sl)
            self.info.setdefault("fp32_tier_steps", {})[kind] = sorted(fast)
            self.info.setdefault("df_variance_steps", {})[kind] = sorted(dfv)
            if disc:
                # per system: largest probe discrepancy of estimates, variances
                self.info.setdefault("probe_disc", {})[kind] = np.concatenate(disc)
            self.info["failed_steps"][kind] = sorted(failed)
            self.info.setdefault("exact_inverse_steps", {})[kind] = sorted(routed)
            # exact-inverse steps whose inverse is pinv's truncated one
            self.info.setdefault("pinv_steps", {})[kind] = sorted(pinv)
            # the FP32 factor with FP64 refinement: steps and iterations
            # (ir 1: refined over the FP32 factor; 2: refinement did not
            # converge, factored and solved again in FP64)
            irs, iters, back = [], {}, []
            for b in batches:
                if b.ir is None:
                    continue
                kept = b.ir.cpu().numpy()
                its = b.ir_iters.cpu().numpy()
                for k, sl in enumerate(b.steps_l):
                    if kept[k] == 1:
                        for j in sl:
                            irs.append(int(j))
                            iters[int(j)] = int(its[k] & 0xFFFF)
                    elif kept[k] == 2:
                        back.extend(int(j) for j in sl)
            self.info.setdefault("ir_steps", {})[kind] = sorted(irs)
            self.info.setdefault("ir_iters", {})[kind] = iters
            self.info.setdefault("ir_fallback_steps", {})[kind] = sorted(back)
            self.info["cond"][kind] = cond
        return self.info

    def launches_per_execute(self):
        """Kernels of this library that one execute() launches, call by call
        as _KrigeBatch.run makes them: row fills; per batch the build,
        Cholesky, inverse (or condition estimate), Gauss-Jordan and the pinv
        check of the exact-inverse systems, the duals
        (plus two triangular-solve kernels without the inverse), the FP32
        splits, the probe (tensor-core and double-float variances, both
        tiers' cell kernels, the tier pick), the main variance kernels and
        one cell kernel per tier; per IDW / NNB field its fill, split (mixed
        IDW) and kernel."""
        n = 0
        for kind, out, want_var, batches, fills, a in self.krig:
            n += sum(f is not None for f in fills)
            for b in batches:
                # build, Cholesky, inverse or condition estimate, the
                # exact-inverse elimination (one kernel, or set-up + 2 per
                # row + finish), the pinv check
                n += 3 + b.gj_launches() + (b.pinv is not None)
                n += 1 if kind == "EDK" else 0  # the drift-dependence check
                # the FP32 factor of the refinement path: copy, Cholesky,
                # condition estimate, gate
                n += 4 if b.l32 is not None else 0
                # the refinement's fallback pass: gate, FP64 Cholesky,
                # condition estimate, the two dual kernels again
                n += 5 if b.l32 is not None else 0
                n += 1 if b.X is not None else 3
                if b.split is not None:
                    n += 2 + (b.X is not None) + (b.linv_tc is not None)
                if b.probe is not None and self.pdom is not None:
                    n += (b.probe[4] is not None and want_var) + 2 + 1
                    n += 2 if (b.probe_df is not None and want_var) else 0
                n += 1 if (b.yy is not None and want_var) else 0
                n += 1 if (b.yy is not None and want_var and b.tier is not None) else 0
                n += 2 if b.precision == 1 else 1
        n += len(self.post_fills)
        for t, out, fill, p in self.idw:
            n += (fill is not None) + (len(self.multi) > 0) * (
                1 + (t == "IDW" and (self.data_hi is not None or self.idw_pack is not None)))
        return int(n)

    def kernel_times(self, evs):
        """{kernel: [ms, launches, algorithmic FLOP]} of an execute(timing=True)."""
        out = {}
        for b, want_var, a, ev in evs["krige"]:
            fl = b.kernel_flops(self.C, want_var, a, self.cond_split)
            for name, e0, e1 in ev:
                t = out.setdefault(name, [0.0, 0, 0.0])
                t[0] += e0.elapsed_time(e1)
                t[1] += 1
                t[2] += fl.get(name, 0.0)
        for name, (e0, e1), fl in evs["idw"]:
            t = out.setdefault(name, [0.0, 0, 0.0])
            t[0] += e0.elapsed_time(e1)
            t[1] += 1
            t[2] += fl
        return out

    def problem_steps(self):
        """The reference's prblm_time_steps after an execution: steps without
        a present station, then steps whose kriging system is singular
        (filled by nearest station, as the reference's pinv-failure branch,
        interp/steps.py:362-372)."""
        out = list(self.prblm)
        info = self.collect_info()
        failed = sorted({j for v in info["failed_steps"].values() for j in v})
        for j in failed:
            t = self.time_steps[j]
            if t not in out:
                out.append(t)
        return out

    def fields(self, numpy=True):
        torch.cuda.current_stream().synchronize()
        if numpy:
            return OrderedDict((k, v.cpu().numpy()) for k, v in self.flds.items())
        return self.flds


def _fill_args(dev, rows, vals, vvals):
    if not len(rows):
        return None
    r = torch.as_tensor(np.asarray(rows, dtype=np.int32), device=dev)
    v = torch.as_tensor(np.asarray(vals, dtype=np.float64), device=dev)
    vv = None if vvals is None else torch.as_tensor(np.asarray(vvals, dtype=np.float64),
                                                    device=dev)
    return (len(rows), r, v, vv)


def _fill_run(f, C, out, s):
    if f is None:
        return
    n, r, v, vv = f
    nat.call("spi_fill_rows", n, _ptr(r), _ptr(v), _ptr(vv), C, ctypes.byref(out), s)


def interp_args_for(methods, est_vars=False, fig_dir=None):
    """The reference's interpolation tuples (interp/prepare.py:638-695) for
    a list of methods like ['OK', 'SK', 'EDK', ('IDW', 2.0), 'NNB']:
    (type, figure directory, label[, idw_exp]) in the reference's order,
    IDW labels 'IDW_000', 'IDW_001', ... in the order the exponents are
    given (not sorted), and ('EST_VARS_OK', ...) last when est_vars."""
    args = []
    for t in ("OK", "SK", "EDK"):
        if t in methods:
            args.append((t, fig_dir, t))
    idw = [m[1] for m in methods if isinstance(m, tuple) and m[0] == "IDW"]
    for i, e in enumerate(idw):
        args.append(("IDW", fig_dir, f"IDW_{i:03d}", float(e)))
    if "NNB" in methods:
        args.append(("NNB", fig_dir, "NNB"))
    if est_vars:
        args.append(("EST_VARS_OK", fig_dir, "EST_VARS_OK"))
    return args


def interp_steps(stn_x, stn_y, data, cell_x, cell_y, vgs, interp_args, *, est_vars=False,
                 stn_drifts=None, cell_drifts=None, min_var_thr=0.0, min_var_cut=None,
                 max_var_cut=None, min_vg_val=0.0, intrp_dtype=np.float32, time_steps=None,
                 precision="fp64", device="cuda", return_numpy=True, return_info=False,
                 arena_budget=8 << 30, cond_max=1e13, cond_split=None, tensor_cores=True,
                 probe_cells=1024, probe_tol=2e-6, neb_sel_mthd="all", n_nebs=None,
                 n_pies=None, refine=True, cond_ir=1e10):
    """Interpolate every step onto every cell on the GPU.

    ``neb_sel_mthd`` 'nrst' / 'pie' (with ``n_nebs``, ``n_pies``) selects
    each cell's neighbours as the reference does (spinterps_gb300.nebs).

    Same inputs and outputs as the reference step engine for one grid chunk
    (see the module docstring). ``precision`` is "fp64" (plain FP64) or
    "mixed" (FP32 right-hand sides and contractions over the FP64
    factorisation; with ``tensor_cores`` the OK variance of the FP32 tier
    runs on tcgen05 as split TF32 products). In the mixed path each system first runs in
    both tiers on ``probe_cells`` cells and takes the FP32 tier only where
    they agree to ``probe_tol`` of the fields' scale, and only on the
    Cholesky path with cond <= ``cond_split``. With ``refine`` the mixed
    path factors systems without the OK variance in FP32 and refines their
    duals in FP64 (tried where the FP32 factor's condition estimate is at
    most ``cond_ir``; systems whose refinement does not converge are
    factored and solved again in FP64). Returns ``(fields, problem_steps)``, plus an info
    dict (failed systems, condition estimates, tiers, refinement
    iterations) when ``return_info``.
    """
    if neb_sel_mthd != "all":
        from .nebs import interp_steps_nebs
        if return_info or not return_numpy:
            raise ValueError("neighbour methods return numpy fields only")
        return interp_steps_nebs(
            stn_x, stn_y, data, cell_x, cell_y, vgs, interp_args, neb_sel_mthd, n_nebs, n_pies,
            stn_drifts=stn_drifts, cell_drifts=cell_drifts, intrp_dtype=intrp_dtype,
            time_steps=time_steps, device=device, est_vars=est_vars, min_var_thr=min_var_thr,
            min_var_cut=min_var_cut, max_var_cut=max_var_cut, min_vg_val=min_vg_val,
            precision=precision, arena_budget=arena_budget, cond_max=cond_max,
            cond_split=cond_split, tensor_cores=tensor_cores, probe_cells=probe_cells,
            probe_tol=probe_tol)
    plan = InterpPlan(stn_x, stn_y, data, cell_x, cell_y, vgs, interp_args, est_vars=est_vars,
                      stn_drifts=stn_drifts, cell_drifts=cell_drifts, min_var_thr=min_var_thr,
                      min_var_cut=min_var_cut, max_var_cut=max_var_cut, min_vg_val=min_vg_val,
                      intrp_dtype=intrp_dtype, time_steps=time_steps, precision=precision,
                      device=device, arena_budget=arena_budget, cond_max=cond_max,
                      cond_split=cond_split, tensor_cores=tensor_cores,
                      probe_cells=probe_cells, probe_tol=probe_tol, refine=refine,
                      cond_ir=cond_ir)
    plan.execute()
    flds = plan.fields(numpy=return_numpy)
    prblm = plan.problem_steps()
    if return_info:
        return flds, prblm, plan.collect_info()
    return flds, prblm


def krige_loo(stn_x, stn_y, data, vgs, *, min_vg_val=0.0, device="cuda", cond_max=1e13):
    """Leave-one-out cross-validation of ordinary kriging per step.

    Returns (residuals, rmse): residuals[t] is z minus the kriging estimate
    at each present station of step t from the other stations (closed form
    from the step's FP64 factorisation, spi_krige_loo), rmse[t] their root
    mean square (NaN for steps with fewer than three stations, a nugget-only
    variogram, or a system off the Cholesky path)."""
    dev = _require_cuda(device)
    data = np.ascontiguousarray(data, dtype=np.float64)
    T = data.shape[0]
    avail = np.isfinite(data)
    sx = np.asarray(stn_x, dtype=np.float64)
    dom = _Domain(dev, stn_x, stn_y, sx[:1], np.asarray(stn_y, dtype=np.float64)[:1], None,
                  None, min_vg_val, 0)
    systems = []
    for t in range(T):
        idx = np.where(avail[t])[0]
        if idx.size < 3 or check_full_nuggetness(vgs[t], min_vg_val):
            continue
        systems.append((idx, vgs[t], [t]))
    res = [None] * T
    rmse = np.full(T, np.nan)
    val_off = np.zeros(T, dtype=np.int64)
    beta = torch.zeros((T, nat.GA), dtype=torch.float64, device=dev)
    for ch in _chunk_systems(systems, 0, 8 << 30):
        b = _KrigeBatch(dev, dom, "OK", systems, ch, data, T, val_off, beta, 0, need_linv=True)
        s = _stream()
        ws = ctypes.byref(b.ws)
        nat.call("spi_krige_factor", ctypes.byref(dom.st), ctypes.byref(b.sy), ws,
                 float(cond_max), s)
        nat.call("spi_krige_duals", ctypes.byref(dom.st), ctypes.byref(b.sy), _ptr(b.vals),
                 ws, s)
        r = torch.empty_like(b.vals)
        nat.call("spi_krige_loo", ctypes.byref(dom.st), ctypes.byref(b.sy), ws, _ptr(r), s)
        r = r.cpu().numpy()
        for i in ch:
            idx, _, (t,) = systems[i]
            e = r[val_off[t]:val_off[t] + idx.size]
            res[t] = e
            rmse[t] = float(np.sqrt(np.mean(e * e)))
    return res, rmse
