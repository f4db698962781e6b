"""The bench's kernel accounting, on the CPU.

- InterpPlan.launches_per_execute must equal the kernels that
  _KrigeBatch.run actually launches. The batches are built on the CPU and
  run with the entry points recorded instead of called; each recorded entry
  point is then counted by the kernels its C source launches.
- InterpPlan.kernel_times files IDW and NNB under their own names, with
  IDW's algorithmic FLOP only."""
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
        return 4  # build, Cholesky, inverse or condition estimate, Gauss-Jordan
    if name == "spi_krige_duals":
        return 1 if batch.X is not None else 3  # + the two triangular-solve kernels
    return {"spi_split_f64": 1, "spi_krige_var_tc": 1, "spi_krige_var_df": 1,
            "spi_krige_cells": 1, "spi_krige_tier": 1}[name]


def make_batch(kind, precision, want_var, n_probe, tensor_cores=True):
    rng = np.random.default_rng(0)
    N, T, C = 12, 5, 40
    data = rng.normal(size=(T, N))
    systems = [(np.arange(N), "0.1 Nug(0.0) + 0.9 Exp(20000)", [0, 1, 2]),
               (np.arange(N - 3), "1.0 Gau(15000)", [3, 4])]
    dom = types.SimpleNamespace(C=C, st=nat.DomainT())
    val_off = np.zeros(T, dtype=np.int64)
    beta = torch.zeros(T * nat.GA, dtype=torch.float64)
    b = steps._KrigeBatch("cpu", dom, kind, systems, [0, 1], data, T, val_off, beta, precision,
                          want_var=want_var, tensor_cores=tensor_cores, n_probe=n_probe)
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
                                 multi=[], pdom=pdom, data_hi=None)
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
