"""spinterps_gb300: GB300-native (sm_103a) gridded-interpolation hot path of
spinterps -- ordinary / simple / external-drift kriging, IDW and nearest
neighbour of station time series onto regular grids, with the reference's
driver-level API (station coordinates and values, grid cells, drifts,
variogram strings, per-method estimate and variance fields).

The compute path is CUDA only (``csrc/``, built by ``build.py`` into
``_lib/``), reached through the C ABI of ``include/spinterps_gb300.h``.
"""
from .steps import (  # noqa: F401
    SpInterpSteps, interp_steps, interp_args_for, parse_vg, check_full_nuggetness)
from .legacy import (  # noqa: F401
    OrdinaryKriging, SimpleKriging, ExternalDriftKriging, ExternalDriftKriging_MD,
    OrdinaryIndicatorKriging, SimpleIndicatorKriging)

__all__ = ["SpInterpSteps", "interp_steps", "interp_args_for", "parse_vg",
           "check_full_nuggetness",
           "OrdinaryKriging", "SimpleKriging", "ExternalDriftKriging",
           "ExternalDriftKriging_MD", "OrdinaryIndicatorKriging", "SimpleIndicatorKriging"]
