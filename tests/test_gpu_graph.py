"""The small-job machinery: the cell-tile autotuner (InterpPlan.autotune,
spi_krige_cells_tiled) and the job captured in a CUDA graph
(InterpPlan.capture / replay). Both must leave the fields unchanged: the
tiles change only how cells are grouped into CTAs (each cell's sums keep
their order), and a replay reruns the captured kernels on the same
buffers. Checked on the small configuration (150 stations, 24 steps) on a
reduced grid, plain FP64 and mixed, and against the oracle."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import port  # noqa: E402


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotune_and_graph_replay_keep_the_fields(precision):
    import bench
    from spinterps_gb300.steps import InterpPlan, interp_args_for
    w = bench.make_small_workload(nx=60, ny=50)
    iargs = interp_args_for(["OK", ("IDW", 2.0)], est_vars=True)
    kw = dict(est_vars=True, min_vg_val=1e-4, intrp_dtype=np.float64)
    plan = InterpPlan(w["sx"], w["sy"], w["z"], w["cx"], w["cy"], w["vgs"], iargs,
                      precision=precision, **kw)
    plan.execute()
    base = {k: v.clone() for k, v in plan.fields(numpy=False).items()}
    tiles = plan.autotune()
    if precision == "fp64":
        assert tiles and set(tiles.values()) <= {16, 32, 64}
    for v in plan.flds.values():
        v.fill_(float("nan"))
    plan.execute()
    for k, v in plan.fields(numpy=False).items():
        assert torch.equal(v, base[k]), k
    plan.capture()
    for v in plan.flds.values():
        v.fill_(float("nan"))
    plan.replay()
    plan.replay()
    for k, v in plan.fields(numpy=False).items():
        assert torch.equal(v, base[k]), k
    ref, _ = port.interp_steps(w["sx"], w["sy"], w["z"], w["cx"], w["cy"], w["vgs"], iargs,
                               **kw)
    tol = 1e-9 if precision == "fp64" else 1e-5
    for k in ref:
        got = base[k].cpu().numpy()
        assert np.nanmax(np.abs(got - ref[k])) <= tol * np.nanmax(np.abs(ref[k])), k
