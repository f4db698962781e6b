"""The bench's kernel accounting, on the CPU.

- InterpPlan.launches_per_execute must equal the kernels that
  _KrigeBatch.run actually launches. The batches are built on the CPU and
  run with the entry points recorded instead of called; each recorded entry
  point is then counted by the kernels its C source launches.
- InterpPlan.kernel_times files IDW and NNB under their own names, with
  IDW's algorithmic FLOP only.
- A whole plan runs its host logic end to end (construction, execute with
  and without timing, counters, problem steps) with the entry points
  recorded instead of called."""
import types

import numpy as np
import pytest
import torch

from spinterps_gb300 import _native as nat
from spinterps_gb300 import steps


def entry_kernels(name, batch):
    """Kernel launches per call of each entry point _KrigeBatch.run uses
    (csrc/spi_factor.cu, spi_cells.cu, spi_var_tc.cu, spi_var_df.cu)."""
    if name == "spi_krige_factor":
        # build, Cholesky, inverse or condition estimate, Gauss-Jordan (one
        # kernel, or set-up + 2 per row + finish over the GPU), and the pinv
        # check of exact-inverse systems when the batch has its scratch
        gj = batch.gj_launches()
        # + the FP32 factor of the refinement path (copy, Cholesky,
        # condition estimate, gate)
        return (3 + gj + (batch.pinv is not None) + (4 if batch.l32 is not None else 0)
                + (batch.kind == "EDK"))
    if name == "spi_krige_duals":
        # + the two triangular-solve kernels, + the refinement's fallback
        # pass (gate, Cholesky, condition estimate, both solve kernels)
        return 1 if batch.X is not None else (3 + (5 if batch.l32 is not None else 0))
    return {"spi_split_f64": 1, "spi_krige_var_tc": 1, "spi_krige_var_df": 1,
            "spi_krige_cells": 1, "spi_krige_cells_tiled": 1, "spi_krige_tier": 1,
            "spi_krige_var_tc_pack": 1}[name]


def make_batch(kind, precision, want_var, n_probe, tensor_cores=True):
    rng = np.random.default_rng(0)
    N, T, C = 12, 5, 40
    data = rng.normal(size=(T, N))
    systems = [(np.arange(N), "0.1 Nug(0.0) + 0.9 Exp(20000)", [0, 1, 2]),
               (np.arange(N - 3), "1.0 Gau(15000)", [3, 4])]
    dom = types.SimpleNamespace(C=C, st=nat.DomainT())
    val_off = np.zeros(T, dtype=np.int64)
    beta = torch.zeros(T * nat.GA, dtype=torch.float64)
    pinv = torch.empty(8, dtype=torch.float64)
    b = steps._KrigeBatch("cpu", dom, kind, systems, [0, 1], data, T, val_off, beta, precision,
                          want_var=want_var, tensor_cores=tensor_cores, n_probe=n_probe,
                          pinv=pinv)
    return dom, b


CASES = [(kind, prec, var, probe, tc)
         for kind in ("OK", "SK", "EDK") for prec in (0, 1) for var in (False, True)
         for probe in (0, 16) for tc in (True, False)
         if not (var and kind != "OK") and not (prec == 0 and (probe or not tc))]


@pytest.mark.parametrize("kind,prec,want_var,n_probe,tc", CASES)
def test_launch_count_follows_run(monkeypatch, kind, prec, want_var, n_probe, tc):
    dom, b = make_batch(kind, prec, want_var, n_probe, tc)
    calls = []
    monkeypatch.setattr(nat, "call", lambda name, *a: calls.append(name))
    monkeypatch.setattr(steps, "_stream", lambda: None)
    out = nat.OutT()
    probe = None
    pdom = None
    if n_probe:
        pdom = types.SimpleNamespace(C=n_probe, st=nat.DomainT())
        probe = (pdom, 1e-6, 1e-6)
    b.run(dom, out, want_var, 1e13, 1e10, None, probe)
    launched = sum(entry_kernels(c, b) for c in calls)
    plan = types.SimpleNamespace(krig=[(kind, out, want_var, [b], [None], 1)], idw=[],
                                 multi=[], pdom=pdom, data_hi=None, post_fills=[])
    assert steps.InterpPlan.launches_per_execute(plan) == launched, calls


class _Ev:
    def __init__(self, t):
        self.t = t

    def elapsed_time(self, other):
        return other.t - self.t


def test_kernel_times_keeps_nnb_apart_from_idw():
    """IDW carries its algorithmic FLOP (present stations only); NNB has its
    own entry and no FLOP."""
    evs = {"krige": [], "idw": [("idw", (_Ev(0.0), _Ev(2.0)), 40.0),
                                ("nnb", (_Ev(2.0), _Ev(3.0)), 0.0),
                                ("idw", (_Ev(3.0), _Ev(4.0)), 40.0)]}
    plan = types.SimpleNamespace(C=10, cond_split=1e10)
    out = steps.InterpPlan.kernel_times(plan, evs)
    assert out == {"idw": [3.0, 2, 80.0], "nnb": [1.0, 1, 0.0]}


class _FakeEvent:
    """Stands in for torch.cuda.Event on the CPU."""
    _t = 0.0

    def __init__(self, enable_timing=False):
        self.t = 0.0

    def record(self, stream=None):
        _FakeEvent._t += 1.0
        self.t = _FakeEvent._t

    def elapsed_time(self, other):
        return other.t - self.t


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_plan_dry_run(monkeypatch, precision):
    """A whole InterpPlan (OK + variance, SK, IDW, NNB; missing stations, a
    step without stations, a single-station step) built and executed with
    the entry points recorded instead of called: the host logic runs end to
    end, the launch count equals the kernels behind the recorded calls, and
    the timed execution files every kernel it times."""
    calls = []
    monkeypatch.setattr(steps, "_require_cuda", lambda device: torch.device("cpu"))
    monkeypatch.setattr(nat, "call", lambda name, *a: calls.append((name, a)))
    monkeypatch.setattr(steps, "_stream", lambda: None)
    monkeypatch.setattr(torch.cuda, "Event", _FakeEvent)
    rng = np.random.default_rng(3)
    N, T, C = 30, 6, 200
    sx, sy = rng.uniform(0, 1e5, N), rng.uniform(0, 1e5, N)
    z = rng.normal(size=(T, N))
    z[rng.uniform(size=(T, N)) < 0.2] = np.nan
    z[2] = np.nan
    z[3] = np.nan
    z[3, 4] = 1.0
    cx, cy = rng.uniform(0, 1e5, C), rng.uniform(0, 1e5, C)
    vgs = ["0.1 Nug(0.0) + 0.9 Exp(20000)", "1.0 Gau(30000)"] * (T // 2)
    args = steps.interp_args_for(["OK", "SK", ("IDW", 2.0), "NNB"], est_vars=True)
    plan = steps.InterpPlan(sx, sy, z, cx, cy, vgs, args, est_vars=True, precision=precision,
                            min_vg_val=1e-4)

    def kernels(name, a):
        if name == "spi_krige_factor":
            # + the pinv check when the workspace carries its scratch; the
            # step-by-step elimination with its scratch (systems >= 256 rows)
            ws, sy = a[2]._obj, a[1]._obj
            gj = 1
            assert not ws.gj_scratch  # small systems: one CTA each
            return (3 + gj + bool(ws.pinv_scratch) + (4 if ws.l32 and not ws.linv_arena else 0)
                    + (sy.kind == 2))
        if name == "spi_krige_duals":
            ws = a[3]._obj
            return 1 if ws.linv_arena else (3 + (5 if ws.l32 else 0))
        if name == "spi_idw_cells_tc":
            return 2  # the pack of B, the contraction
        return 1

    for timing in (False, True):
        calls.clear()
        evs = plan.execute(timing=timing)
        assert plan.launches_per_execute() == sum(kernels(n, a) for n, a in calls)
    names = {n for n, _ in calls}
    assert {"spi_krige_factor", "spi_krige_duals", "spi_krige_cells_tiled",
            "spi_nnb_cells", "spi_fill_rows"} <= names
    if precision == "mixed":
        assert {"spi_krige_tier", "spi_krige_var_tc", "spi_krige_var_df",
                "spi_idw_cells_tc"} <= names
        assert "spi_idw_cells" not in names
    else:
        assert "spi_idw_cells" in names
    times = plan.kernel_times(evs)
    assert {"idw", "nnb"} <= set(times)
    assert times["nnb"][2] == 0.0 and times["idw"][2] > 0.0
    assert plan.problem_steps()[0] == 2


def test_legacy_and_polygon_dry_run(monkeypatch):
    """The legacy classes and the polygon mask run their host logic with the
    entry points recorded instead of called (no GPU)."""
    from spinterps_gb300 import driver, legacy
    calls = []
    cpu = torch.device("cpu")

    class _Stream:
        cuda_stream = 0

        def synchronize(self):
            pass

    for mod in (steps, legacy, driver):
        monkeypatch.setattr(mod, "_require_cuda", lambda device: cpu)
    monkeypatch.setattr(driver, "_stream", lambda: None)
    monkeypatch.setattr(nat, "call", lambda name, *a: calls.append(name))
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a, **k: _Stream())
    monkeypatch.setattr(legacy, "_dev", lambda a: torch.as_tensor(
        np.ascontiguousarray(a, dtype=np.float64)))
    rng = np.random.default_rng(4)
    xi, yi, zi = rng.uniform(0, 5e4, 12), rng.uniform(0, 5e4, 12), rng.normal(size=12)
    xk, yk = rng.uniform(0, 5e4, 20), rng.uniform(0, 5e4, 20)
    for cls in ("OrdinaryKriging", "SimpleKriging", "OrdinaryIndicatorKriging"):
        obj = getattr(legacy, cls)(xi, yi, zi, xk, yk, model="0.1 Nug(0.0) + 0.9 Exp(20000)")
        if "Indicator" in cls:
            obj.ikrige()
        else:
            obj.krige()
        assert obj.pinv_route == "gj" and obj.zk.shape == (20,)
    assert calls.count("spi_legacy_system") == 3 and calls.count("spi_legacy_points") == 3
    calls.clear()
    ring = (np.array([0.0, 5e4, 5e4, 0.0]), np.array([0.0, 0.0, 5e4, 5e4]))
    with pytest.raises(AssertionError, match="No cells selected"):
        driver.cells_in_polygons(xk, yk, [ring])  # the recorded kernel selects nothing
    assert calls == ["spi_points_in_polygons"]
