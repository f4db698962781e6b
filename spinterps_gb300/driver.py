"""The driver flow around the step engine, as ``SpInterpMain`` runs it
(interp/main.py, interp/prepare.py, interp/drift.py), with arrays in place of
the reference's files:
- the grid: ``corner_coordinates`` and ``prepare_crds``
  (interp/prepare.py:92-241);
- drift rasters at the cells and the stations: ``drift_bounds`` and
  ``sample_drifts`` (interp/drift.py:25-227);
- the polygon cell mask: ``cells_in_polygons``
  (interp/prepare.py:244-288, GPU);
- the interpolation of every step over the selected cells (``InterpPlan``);
- the rounding to ``nc_nmrl_prcn`` decimals before the fields are written
  (interp/steps.py:899-922, GPU);
- the per-step statistics of ``stats.csv`` (interp/main.py:474-525, GPU).

``interpolate_grid`` strings these together. It returns full [T, rows, cols]
float fields, NaN outside the mask. ``write_outputs`` writes them as the
reference's netCDF file (``ncout``, classic binary format) and stats.csv.

Reading GeoTIFF rasters and shapefiles (GDAL / ogr) is not here: those
libraries are absent. Callers pass arrays: raster values
with their origin, cell size and no-data value, and polygon vertex lists.
Buffering polygons (``ogr.Geometry.Buffer``) is the caller's job too.
"""
import ctypes
import math

import numpy as np
import torch

from . import _native as nat
from .steps import InterpPlan, _require_cuda


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def corner_coordinates(stn_x, stn_y, cell_bdist=0.0, poly_extent=None):
    """SpInterpPrepare._cmpt_corner_coordinates (interp/prepare.py:92-146):
    the bounds (x_min, x_max, y_min, y_max) from the polygons' extent when
    given (x_min, x_max, y_min, y_max), else from the stations, widened by
    cell_bdist on every side."""
    if poly_extent is not None:
        x0, x1, y0, y1 = poly_extent
    else:
        x0, x1 = float(np.min(stn_x)), float(np.max(stn_x))
        y0, y1 = float(np.min(stn_y)), float(np.max(stn_y))
    return x0 - cell_bdist, x1 + cell_bdist, y0 - cell_bdist, y1 + cell_bdist


def drift_bounds(x_min, y_max, n_rows, n_cols, cell_size):
    """The drift rasters' extent as KrigingDrift._assemble_drift_data
    computes it (interp/drift.py:136-152): from the origin, the shape and
    the cell size, rounded to 6 decimals. Returns (x_min, x_max, y_min,
    y_max)."""
    x_max = x_min + (n_cols * cell_size)
    y_min = y_max - (n_rows * cell_size)
    return tuple(float(v) for v in np.round((x_min, x_max, y_min, y_max), 6))


def prepare_crds(x_min, x_max, y_min, y_max, cell_size, drift_bounds=None):
    """SpInterpPrepare._prepare_crds (interp/prepare.py:148-241).

    Computes the column and row range of the grid. When ``drift_bounds``
    (the drift rasters' x_min, x_max, y_min, y_max) is given, the range is
    taken inside the rasters (EDK). Cell centres run from
    (x_min + cs/2, y_max - cs/2) by np.linspace, and the cell mesh is
    row-major with y descending.

    Returns a dict: rc (min_col, max_col, min_row, max_row), x_crds,
    y_crds, cell_x, cell_y, shape."""
    if drift_bounds is not None:
        dx0, dx1, dy0, dy1 = drift_bounds
        assert x_min >= dx0, "Grid x_min outside of the drift rasters!"
        assert x_max <= dx1, "Grid x_max outside of drift rasters!"
        assert y_min >= dy0, "Grid y_min outside of the drift rasters!"
        assert y_max <= dy1, "Grid y_max outside of drift rasters!"
        min_col = int(math.floor((x_min - dx0) / cell_size))
        max_col = int(math.ceil((x_max - dx0) / cell_size)) - 1
        min_row = int(math.floor((dy1 - y_max) / cell_size))
        max_row = int(math.ceil((dy1 - y_min) / cell_size)) - 1
    else:
        min_col, min_row = 0, 0
        max_col = int(math.ceil((x_max - x_min) / cell_size)) - 1
        max_row = int(math.ceil((y_max - y_min) / cell_size)) - 1
    assert 0 <= min_col <= max_col, (min_col, max_col)
    assert 0 <= min_row <= max_row, (min_row, max_row)
    sx = x_min + (0.5 * cell_size)
    ex = sx + ((max_col - min_col) * cell_size)
    sy = y_max - (0.5 * cell_size)
    ey = sy - ((max_row - min_row) * cell_size)
    xs = np.linspace(sx, ex, (max_col - min_col + 1))
    ys = np.linspace(sy, ey, (max_row - min_row + 1))
    mx, my = np.meshgrid(xs, ys)
    return dict(rc=(min_col, max_col, min_row, max_row), x_crds=xs, y_crds=ys,
                cell_x=mx.ravel(), cell_y=my.ravel(), shape=mx.shape)


def sample_drifts(rasters, drift_x_min, drift_y_max, cell_size, ndv, rc, stn_x, stn_y,
                  cntn_idxs=None):
    """KrigingDrift._prepare_stns_drift (interp/drift.py:165-227).

    Every raster is read at the grid's rows and columns (the selected cells
    only, with a mask); no-data values, matched by np.isclose, become NaN.
    Each station reads its cell int((x - x_min) / cs), int((y_max - y) / cs).
    Returns (cell_drifts [k, C], stn_drifts [N, k]). Raises AssertionError
    when a station's drift is not finite, as the reference does."""
    min_col, max_col, min_row, max_row = rc
    cols, rows = np.meshgrid(np.arange(min_col, max_col + 1, dtype=int),
                             np.arange(min_row, max_row + 1, dtype=int))
    cols, rows = cols.ravel(), rows.ravel()
    if cntn_idxs is not None:
        cols, rows = cols[cntn_idxs], rows[cntn_idxs]
    cell = []
    for r in rasters:
        v = np.asarray(r, dtype=float)[rows, cols]
        v[np.isclose(ndv, v)] = np.nan
        cell.append(v)
    cell = np.array(cell, dtype=float)
    stn_col = ((np.asarray(stn_x, float) - drift_x_min) / cell_size).astype(int)
    stn_row = ((drift_y_max - np.asarray(stn_y, float)) / cell_size).astype(int)
    stn = np.empty((len(stn_col), len(rasters)))
    for k, r in enumerate(rasters):
        d = np.asarray(r, dtype=float)[stn_row, stn_col]
        stn[:, k] = np.where(np.isclose(ndv, d), np.nan, d)
    assert np.all(np.isfinite(stn)), "Invalid value(s) of drift(s) for stations in drift rasters!"
    return cell, stn


def cells_in_polygons(cell_x, cell_y, polygons, device="cuda"):
    """The polygon cell mask of _select_nearby_cells (interp/prepare.py:244-288):
    True where a cell, its coordinates rounded to 1e-6, lies strictly inside
    one of the polygons (spi_points_in_polygons).

    polygons: a list of (xs, ys) vertex arrays, each one ring, closed from
    its last vertex to its first. Each polygon needs at least 3 vertices
    and a nonzero area, as the reference asserts. Raises AssertionError
    when no cell is selected, as the reference does."""
    device = _require_cuda(device)
    vx, vy, off, bbox = [], [], [0], []
    for xs, ys in polygons:
        xs, ys = np.asarray(xs, float).ravel(), np.asarray(ys, float).ravel()
        assert xs.size == ys.size and xs.size >= 3, \
            f"Polygon not having enough points ({xs.size})!"
        area = 0.5 * abs(np.dot(xs, np.roll(ys, -1)) - np.dot(ys, np.roll(xs, -1)))
        assert area > 0, "Polygon has no area!"
        vx.append(xs)
        vy.append(ys)
        off.append(off[-1] + xs.size)
        bbox.append((xs.min(), xs.max(), ys.min(), ys.max()))
    n = int(np.asarray(cell_x).size)
    d = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt,  # noqa
                                                     device=device)
    px, py = d(cell_x), d(cell_y)
    inside = torch.zeros(n, dtype=torch.uint8, device=device)
    if polygons:
        # every device array is held by a name until the kernel has run: a
        # temporary freed after its pointer was taken could hand its memory
        # to the next argument's allocation
        t_off = d(np.array(off, dtype=np.int64), torch.int64)
        t_vx, t_vy = d(np.concatenate(vx)), d(np.concatenate(vy))
        t_bb = d(np.array(bbox, dtype=np.float64))
        nat.call("spi_points_in_polygons", _ptr(px), _ptr(py), n, len(polygons), _ptr(t_off),
                 _ptr(t_vx), _ptr(t_vy), _ptr(t_bb), _ptr(inside), _stream())
    mask = inside.cpu().numpy().astype(bool)
    assert mask.any(), "No cells selected for interpolation!"
    return mask


def round_fields_(fld, decimals):
    """numpy.round(fld, decimals) in place on a CUDA float or double tensor
    (spi_round_fields), as the reference rounds its fields to nc_nmrl_prcn
    decimals before writing them."""
    assert fld.is_cuda and fld.is_contiguous() and fld.dtype in (torch.float32, torch.float64)
    nat.call("spi_round_fields", _ptr(fld), int(fld.dtype == torch.float64), fld.numel(),
             int(decimals), _stream())
    return fld


def field_stats(fld, ddof=0):
    """(min, mean, max, std, count) per row of a CUDA [rows, n] float or
    double tensor over its finite entries, as a numpy [rows, 5] array
    (spi_field_stats). ddof 0 is numpy's nanstd of the interpolated fields,
    ddof 1 pandas' std of the station data (interp/main.py:474-525)."""
    assert fld.is_cuda and fld.dim() == 2 and fld.dtype in (torch.float32, torch.float64)
    if fld.stride(1) != 1:
        fld = fld.contiguous()
    rows, n = fld.shape
    scratch = torch.empty(5 * (608 + rows), dtype=torch.float64, device=fld.device)
    out = torch.empty((rows, 5), dtype=torch.float64, device=fld.device)
    nat.call("spi_field_stats", _ptr(fld), int(fld.dtype == torch.float64), rows, n,
             fld.stride(0), int(ddof), _ptr(scratch), scratch.numel(), _ptr(out), _stream())
    return out.cpu().numpy()


STATS = ("min", "mean", "max", "std", "count")


def stats_table(data, flds, interp_args, device="cuda"):
    """The columns of the reference's stats.csv (interp/main.py:474-525), one
    float32 value per step. data_* are pandas' skip-NaN statistics of the
    station values (ddof 1). {label}_* are numpy's nan-statistics of every
    field except EST_VARS_OK (ddof 0). flds: label -> CUDA [T, C] tensor of
    the selected cells, already rounded as written."""
    device = _require_cuda(device)
    cols = {}
    dt = torch.as_tensor(np.ascontiguousarray(data, dtype=np.float64), device=device)
    st = field_stats(dt, ddof=1)
    for j, s in enumerate(STATS):
        cols[f"data_{s}"] = st[:, j].astype(np.float32)
    for a in interp_args:
        lab = a[2]
        if lab == "EST_VARS_OK":
            continue
        st = field_stats(flds[lab], ddof=0)
        for j, s in enumerate(STATS):
            cols[f"{lab}_{s}"] = st[:, j].astype(np.float32)
    return cols


def write_stats_csv(path, time_steps, cols):
    """stats.csv as the reference writes it: ';' separated, '%0.6f' floats,
    the time steps as the first column."""
    names = list(cols)
    with open(path, "w") as f:
        f.write(";" + ";".join(names) + "\n")
        for i, t in enumerate(time_steps):
            f.write(str(t) + ";" + ";".join(
                "" if not np.isfinite(cols[c][i]) else f"{float(cols[c][i]):0.6f}"
                for c in names) + "\n")


def interpolate_grid(stn_x, stn_y, data, vgs, interp_args, *, cell_size, bounds=None,
                     cell_bdist=0.0, polygons=None, drift=None, nmrl_prcn=3,
                     intrp_dtype=np.float32, est_vars=False, min_var_thr=0.0,
                     min_var_cut=None, max_var_cut=None, min_vg_val=0.0, precision="fp64",
                     time_steps=None, device="cuda", **plan_kw):
    """The whole driver flow over arrays.

    Steps:
    1. The bounds default to the stations' extent widened by cell_bdist, or
       to the polygons' extent when polygons are given.
    2. The grid is built inside the drift rasters when drift is given.
    3. The polygon mask selects the cells.
    4. The drifts are sampled at the cells and the stations.
    5. Every step is interpolated on the GPU over the selected cells.
    6. The fields are rounded to nmrl_prcn decimals (None: no rounding).
    7. The statistics are computed.

    ``drift``: a dict with rasters [k, rows, cols], x_min, y_max and ndv.
    Its cell size must be ``cell_size``.

    Returns ``(fields, problem_steps, stats, grid)``:
    - fields: label -> numpy [T, rows, cols], NaN outside the mask;
    - stats: the stats.csv columns;
    - grid: the prepare_crds dict plus 'mask'.
    """
    stn_x, stn_y = np.asarray(stn_x, float), np.asarray(stn_y, float)
    data = np.ascontiguousarray(data, dtype=np.float64)
    if bounds is None:
        ext = None
        if polygons:
            allx = np.concatenate([np.asarray(p[0], float) for p in polygons])
            ally = np.concatenate([np.asarray(p[1], float) for p in polygons])
            ext = (allx.min(), allx.max(), ally.min(), ally.max())
        bounds = corner_coordinates(stn_x, stn_y, cell_bdist, ext)
    db = None
    if drift is not None:
        r = np.asarray(drift["rasters"], float)
        db = drift_bounds(drift["x_min"], drift["y_max"], r.shape[1], r.shape[2], cell_size)
    grid = prepare_crds(*bounds, cell_size, drift_bounds=db)
    mask = None
    cx, cy = grid["cell_x"], grid["cell_y"]
    if polygons:
        mask = cells_in_polygons(cx, cy, polygons, device=device)
        cx, cy = cx[mask], cy[mask]
    grid["mask"] = mask
    stn_drifts = cell_drifts = None
    if drift is not None:
        cell_drifts, stn_drifts = sample_drifts(list(r), db[0], db[3], cell_size,
                                                drift["ndv"], grid["rc"], stn_x, stn_y,
                                                cntn_idxs=mask)
    plan = InterpPlan(stn_x, stn_y, data, cx, cy, vgs, interp_args, est_vars=est_vars,
                      stn_drifts=stn_drifts, cell_drifts=cell_drifts, min_var_thr=min_var_thr,
                      min_var_cut=min_var_cut, max_var_cut=max_var_cut, min_vg_val=min_vg_val,
                      intrp_dtype=intrp_dtype, time_steps=time_steps, precision=precision,
                      device=device, **plan_kw)
    plan.execute()
    flds = plan.fields(numpy=False)
    if nmrl_prcn is not None:
        for v in flds.values():
            if v.dtype in (torch.float32, torch.float64):
                round_fields_(v, nmrl_prcn)
    stats = stats_table(data, flds, interp_args, device=device)
    T = data.shape[0]
    ny, nx = grid["shape"]
    out = {}
    for lab, v in flds.items():
        h = v.cpu().numpy()
        if mask is None:
            out[lab] = h.reshape(T, ny, nx)
        else:
            full = np.full((T, ny * nx), np.nan, dtype=h.dtype)
            full[:, mask] = h
            out[lab] = full.reshape(T, ny, nx)
    return out, plan.problem_steps(), stats, grid


def write_outputs(out_dir, nc_name, fields, grid, stats, interp_args, time_vals, *,
                  time_steps=None, xlab="X", ylab="Y", tlab="time", tunits=None, tcldr=None,
                  vunits="", vlab="", settings=None, fmt=5):
    """The reference's two output files from interpolate_grid's results:
    the netCDF file of the fields (ncout.write_interp_nc; name as the
    reference forms it, interp/prepare.py:308-311) and stats.csv
    (interp/main.py:519-520). Returns the two paths."""
    from pathlib import Path
    from . import ncout
    out_dir = Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    nc_path = out_dir / (nc_name.split(".", 1)[0] + ".nc")
    ncout.write_interp_nc(nc_path, grid["x_crds"], grid["y_crds"], time_vals, fields,
                          interp_args, xlab=xlab, ylab=ylab, tlab=tlab, tunits=tunits,
                          tcldr=tcldr, vunits=vunits, vlab=vlab, settings=settings, fmt=fmt)
    csv_path = out_dir / "stats.csv"
    write_stats_csv(csv_path, time_steps if time_steps is not None else time_vals, stats)
    return nc_path, csv_path
