"""Jobs larger than one GPU's memory: the steps in waves sized to an HBM
budget, each wave's fields handed to a sink as soon as they are done.

The reference's driver sizes its work to the host's RAM: it cuts the steps
into chunks per process and the grid into row chunks until the cell x
station matrices and the output arrays of a pass fit
(``SpInterpMain._get_thread_steps_idxs``, interp/main.py:652-859), and each
pass writes its slab of the netCDF file (interp/steps.py:879-969). Here the
cell x station matrices never exist, so only the steps are cut: a wave
holds as many steps as its fields (cells x labels x the output type) and
its factor arenas ((n + 8)^2 doubles per system, twice with the OK
variance's inverse factor, plus the tensor-core variance's n_cells doubles
per OK system of the mixed path) leave within the budget. Every step's
system is its own (its station set and variogram), so cutting the steps
changes no result: a wave's fields equal the same rows of a one-shot run.

``interp_steps_waves`` builds the next wave's plan on the host while the
GPU runs the current one (``InterpPlan.execute`` only enqueues work), then
copies the finished wave's fields to the host and calls
``sink(first_step, fields)`` with numpy arrays [wave steps, cells].
``nc_sink`` returns a sink that writes those rows into a netCDF file laid
out as the reference's (``ncout.write_interp_nc`` with deferred fields).

With the neighbour methods (``neb_sel_mthd`` 'nrst' / 'pie') a wave is a
call of ``nebs.interp_steps_nebs`` on its steps: a step then costs only its
fields, and every wave also holds one step group's neighbour lists, their
grouping and the kriging scratch (``nebs_fixed_bytes``). The stations kept
and every cell's neighbours depend on the coordinates alone, so a wave's
fields again equal the same rows of a one-shot run.
"""
import numpy as np
import torch

from . import _native as nat
from .steps import InterpPlan, _require_cuda


def step_bytes(n_present, n_cells, n_labels, out_itemsize, krige_kinds, ok_var, mixed):
    """Device bytes one step adds to a wave: its fields, and per kriging
    kind its system's factor arena(s), per-cell variance buffer and the
    mixed path's FP32 factor."""
    b = n_cells * n_labels * out_itemsize
    arena = (n_present + nat.GA) ** 2 * 8
    for kind in krige_kinds:
        var = ok_var and kind == "OK"
        b += arena * (2 if var else 1)
        if mixed and var:
            # the tensor-core variance: per-cell |Linv c|^2, Linv's FP32
            # hi / lo copies and its packed TF32 terms
            kc = nat.SPI_VAR_TC_KC
            chunks = sum((min(n_present, rb + 256) + kc - 1) // kc
                         for rb in range(0, n_present, 256))
            b += n_cells * 8 + arena + chunks * nat.SPI_VAR_TC_CHUNK_FLOATS * 4
        if mixed and not var:
            b += arena // 2  # the FP32 factor of the refinement path
    return int(b)


def nebs_fixed_bytes(n_cells, k):
    """Device bytes a wave of the neighbour methods holds besides its
    fields: one step group's neighbour lists ([n_cells, k] int32, selected
    and mapped), their grouping (int64 inverse and order, int32 copies)
    and the kriging scratch of spi_local_groups (at most
    nebs.GRP_SCRATCH_BYTES)."""
    from .nebs import GRP_SCRATCH_BYTES
    return int(GRP_SCRATCH_BYTES + n_cells * (3 * 4 * max(int(k), 1) + 4 * 8))


def plan_waves(data, n_cells, interp_args, *, budget, out_itemsize=4, est_vars=False,
               precision="fp64", neighbours=False):
    """Cut the steps of ``data`` [T, N] (NaN = missing) into consecutive
    waves whose step_bytes add up to at most ``budget``; a step that alone
    exceeds it is a wave of its own. With ``neighbours`` (the neighbour
    methods) a step costs its fields only. Returns [(first, end), ...]."""
    types = [a[0] for a in interp_args]
    kinds = [t for t in ("OK", "SK", "EDK") if t in types]
    n_labels = len(interp_args)
    n_av = np.isfinite(np.asarray(data)).sum(1)
    waves, t0, acc = [], 0, 0
    for t in range(n_av.size):
        if neighbours:
            b = n_cells * n_labels * out_itemsize
        else:
            b = step_bytes(int(n_av[t]), n_cells, n_labels, out_itemsize, kinds, est_vars,
                           precision == "mixed")
        if t > t0 and acc + b > budget:
            waves.append((t0, t))
            t0, acc = t, 0
        acc += b
    if n_av.size:
        waves.append((t0, n_av.size))
    return waves


def interp_steps_waves(stn_x, stn_y, data, cell_x, cell_y, vgs, interp_args, *, sink,
                       budget=None, stn_drifts=None, cell_drifts=None, time_steps=None,
                       intrp_dtype=np.float32, est_vars=False, precision="fp64",
                       device="cuda", **plan_kw):
    """Interpolate every step in waves (see the module docstring), calling
    ``sink(first_step, fields)`` once per wave in step order with numpy
    fields {label: [wave steps, cells]}. ``budget``: device bytes per wave
    (default: a third of the free device memory; two waves' plans are alive
    at once while the next is built). The other arguments are
    ``interp_steps``'s, ``neb_sel_mthd`` / ``n_nebs`` / ``n_pies`` included.
    Returns (problem time steps, info per wave: steps, seconds of host
    planning, and the plan's collect_info(); with the neighbour methods the
    seconds of the wave's call)."""
    import time
    dev = _require_cuda(device)
    data = np.ascontiguousarray(data, dtype=np.float64)
    T = data.shape[0]
    C = int(np.asarray(cell_x).size)
    if time_steps is None:
        time_steps = np.arange(T)
    vgs = list(vgs) if vgs is not None else [None] * T
    if budget is None:
        budget = torch.cuda.mem_get_info(dev)[0] // 3
    itemsize = np.dtype(intrp_dtype).itemsize
    neb = plan_kw.pop("neb_sel_mthd", "all")
    n_nebs, n_pies = plan_kw.pop("n_nebs", None), plan_kw.pop("n_pies", None)
    prblm, info = [], []
    if neb != "all":
        from .nebs import interp_steps_nebs
        k = n_nebs if n_nebs else int(np.asarray(stn_x).size)
        waves = plan_waves(data, C, interp_args, out_itemsize=itemsize, neighbours=True,
                           budget=max(budget - nebs_fixed_bytes(C, k), 1))
        for a, b in waves:
            t0 = time.perf_counter()
            flds, pr = interp_steps_nebs(
                stn_x, stn_y, data[a:b], cell_x, cell_y, vgs[a:b], interp_args, neb, n_nebs,
                n_pies, stn_drifts=stn_drifts, cell_drifts=cell_drifts,
                intrp_dtype=intrp_dtype, time_steps=np.asarray(time_steps)[a:b],
                device=device, est_vars=est_vars, precision=precision, **plan_kw)
            sink(a, flds)
            for t in pr:
                if t not in prblm:
                    prblm.append(t)
            info.append({"steps": [int(a), int(b)], "call_s": time.perf_counter() - t0})
        return prblm, info
    waves = plan_waves(data, C, interp_args, budget=budget, out_itemsize=itemsize,
                       est_vars=est_vars, precision=precision)

    def build(w):
        a, b = w
        t0 = time.perf_counter()
        p = InterpPlan(stn_x, stn_y, data[a:b], cell_x, cell_y, vgs[a:b], interp_args,
                       stn_drifts=stn_drifts, cell_drifts=cell_drifts,
                       time_steps=np.asarray(time_steps)[a:b], intrp_dtype=intrp_dtype,
                       est_vars=est_vars, precision=precision, device=device, **plan_kw)
        return p, time.perf_counter() - t0

    def finish(p, w, host_s):
        flds = p.fields(numpy=True)
        sink(w[0], flds)
        for t in p.problem_steps():
            if t not in prblm:
                prblm.append(t)
        info.append({"steps": [int(w[0]), int(w[1])], "plan_s": host_s,
                     "info": p.collect_info()})

    cur = None
    for w in waves:
        p, host_s = build(w)          # overlaps the previous wave's GPU work
        if cur is not None:
            finish(*cur)
            cur = None
            torch.cuda.empty_cache()
        p.execute()
        cur = (p, w, host_s)
    if cur is not None:
        finish(*cur)
    return prblm, info


def nc_sink(path, x_crds, y_crds, time_vals, interp_args, mask=None, **nc_kw):
    """A sink for interp_steps_waves that writes each wave's rows into the
    reference's netCDF layout (ncout.write_interp_nc, float32 fields of
    [T, len(y_crds), len(x_crds)]); ``mask`` (optional, bool over the grid's
    cells) places the interpolated cells, NaN elsewhere."""
    from . import ncout
    T, ny, nx = len(time_vals), len(y_crds), len(x_crds)
    deferred = {a[2]: ncout.Deferred((T, ny, nx), np.float32) for a in interp_args}
    ncout.write_interp_nc(path, x_crds, y_crds, time_vals, deferred, interp_args, **nc_kw)
    begins = dict(ncout.write_nc.begins)

    def sink(first, flds):
        for lab, v in flds.items():
            v = np.asarray(v, dtype=np.float32)
            if mask is not None:
                full = np.full((v.shape[0], ny * nx), np.nan, dtype=np.float32)
                full[:, mask] = v
                v = full
            ncout.write_slab(path, begins[lab], v.reshape(-1, ny, nx), first)

    return sink
