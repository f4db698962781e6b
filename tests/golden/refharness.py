"""Import the reference's own step engine in this container (fixture making only).

TEST INFRASTRUCTURE. Used by ``make_golden.py`` to run the UNMODIFIED reference
code (``interp/steps.py``, ``interp/grps.py``, ``interp/vgclus.py``,
``misc.py`` and the Cython kernels of ``cyth/interpmthds.pyx``) on small
seeded inputs. The reference tree is read only and is never present where the
GPU tests run; the fixtures it produces are committed under ``tests/golden``.

What is stubbed, and why it does not touch the numeric path:
- ``netCDF4``, ``osgeo``, ``shapefile``, ``cftime``, ``pathos``: imported at
  module level by ``misc.py``/``interp/steps.py`` for I/O only.
- ``pandas``: imported by ``interp/grps.py``/``interp/vgclus.py``; the fixtures
  call ``_get_interp`` and ``SpInterpNeighborGrouping.get_neb_idxs_and_grps``,
  neither of which uses pandas.
- the package ``spinterps`` is registered with ``__path__`` pointing at the
  reference root so that the relative imports resolve without running the
  package ``__init__`` (which pulls in matplotlib and GIS modules).
- ``spinterps.cyth`` is the reference's ``cyth/interpmthds.pyx`` compiled by
  ``oracle/build_ref.py`` (Cython 3, ``cpow=True``).
"""
import importlib
import importlib.util
import sys
import types
from pathlib import Path

REPO = Path(__file__).resolve().parents[2]


def _stub(name, **attrs):
    mod = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(mod, k, v)
    sys.modules[name] = mod
    return mod


def _root(ref_root):
    from oracle import build_ref
    root = build_ref.reference_root(ref_root)
    if root is None:
        raise RuntimeError(f"give the reference tree as an argument or in ${build_ref.ENV}")
    return root


def load_reference(ref_root=None):
    """Return a namespace with the reference's step engine and kernels."""
    sys.path.insert(0, str(REPO))
    ref_root = _root(ref_root)
    sys.path.insert(0, str(REPO))
    from oracle import build_ref

    so_dir = build_ref.build(ref_root)
    if so_dir is None:
        raise RuntimeError("reference tree or Cython not available")

    class _Anything:
        def __getattr__(self, item):
            return _Anything()

        def __call__(self, *a, **k):
            return _Anything()

    _stub("netCDF4", Dataset=None)
    _stub("shapefile")
    osgeo = _stub("osgeo")
    osgeo.ogr = _Anything()
    osgeo.gdal = _Anything()
    sys.modules["osgeo.ogr"] = osgeo.ogr
    sys.modules["osgeo.gdal"] = osgeo.gdal
    _stub("cftime", datetime=None)
    _stub("pathos")
    _stub("pathos.multiprocessing", ProcessPool=None)
    if "pandas" not in sys.modules:
        try:
            import pandas  # noqa: F401
        except ImportError:
            _stub("pandas", DataFrame=object, Series=object, Index=object)

    pkg = types.ModuleType("spinterps")
    pkg.__path__ = [str(ref_root)]
    sys.modules["spinterps"] = pkg
    interp_pkg = types.ModuleType("spinterps.interp")
    interp_pkg.__path__ = [str(ref_root / "interp")]
    sys.modules["spinterps.interp"] = interp_pkg

    spec = importlib.util.spec_from_file_location(
        "spinterps.cyth.interpmthds",
        str(next(Path(so_dir).glob("interpmthds*.so"))))
    cy = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(cy)
    cyth_pkg = types.ModuleType("spinterps.cyth")
    cyth_pkg.__path__ = []
    for name in dir(cy):
        if not name.startswith("__"):
            setattr(cyth_pkg, name, getattr(cy, name))
    sys.modules["spinterps.cyth"] = cyth_pkg
    sys.modules["spinterps.cyth.interpmthds"] = cy

    misc = importlib.import_module("spinterps.misc")
    steps = importlib.import_module("spinterps.interp.steps")
    grps = importlib.import_module("spinterps.interp.grps")
    return types.SimpleNamespace(cy=cy, misc=misc, steps=steps, grps=grps)


def make_steps(ref, *, min_vg_val, est_vars, intrp_dtype="float32",
               min_var_thr=0.0, min_var_cut=None, max_var_cut=None):
    """Build a ``SpInterpSteps`` without its driver (only the attributes the
    step engine reads, ``interp/steps.py:31-58``)."""
    import numpy as np

    obj = ref.steps.SpInterpSteps.__new__(ref.steps.SpInterpSteps)
    obj._vb = False
    obj._min_vg_val = float(min_vg_val)
    obj._interp_flag_est_vars = bool(est_vars)
    obj._intrp_dtype = np.dtype(intrp_dtype)
    obj._min_var_thr = min_var_thr
    obj._min_var_cut = min_var_cut
    obj._max_var_cut = max_var_cut
    return obj


class _Column:
    """Column view of the stand-in DataFrame."""

    def __init__(self, frame, i):
        self._f, self._i = frame, i

    @property
    def values(self):
        return self._f._a[:, self._i]

    def replace(self, old, new, inplace=False):
        col = self._f._a[:, self._i]
        col[col == old] = new


class MiniDataFrame:
    """The few pandas.DataFrame operations variograms/vgs.py performs
    (construction, column views, sort_values with numpy's quicksort as pandas
    does, column assignment, dropna, values, shape), on one float array. The
    in-place replace through a column (vgs.py:654) takes effect, as it did in
    the pandas 1.x releases contemporary with the reference."""

    def __init__(self, data=None, columns=None):
        import numpy as np
        if isinstance(data, dict):
            self._cols = list(data)
            self._a = np.column_stack([np.asarray(data[c], dtype=float) for c in data])
        else:
            self._cols = list(columns)
            self._a = np.array(data, dtype=float).reshape(-1, len(self._cols))

    def __getitem__(self, k):
        return _Column(self, self._cols.index(k))

    def __setitem__(self, k, v):
        self._a[:, self._cols.index(k)] = v

    @property
    def values(self):
        return self._a

    @property
    def shape(self):
        return self._a.shape

    def sort_values(self, by, inplace=False):
        import numpy as np
        order = np.argsort(self._a[:, self._cols.index(by[0])], kind="quicksort")
        self._a = self._a[order]

    def dropna(self, inplace=False):
        import numpy as np
        self._a = self._a[~np.isnan(self._a).any(axis=1)]


class LocFrame:
    """The pandas.DataFrame operations of interp/drift.py:_prepare_stns_drift
    on a float array with row and column labels: construction from a dict of
    columns or from index/columns, ``.index``, ``.values``, column access,
    and ``.loc[row, col]`` / ``.loc[row, [cols]]`` reads and
    ``.loc[row, col] = v`` writes."""

    def __init__(self, data=None, index=None, columns=None, dtype=float):
        import numpy as np
        if isinstance(data, dict):
            self.columns = list(data)
            self._a = np.column_stack([np.asarray(data[c], dtype=float) for c in data])
            n = self._a.shape[0]
            self.index = np.arange(n) if index is None else np.asarray(index)
        else:
            self.index = np.asarray(index)
            self.columns = list(columns)
            self._a = np.full((len(self.index), len(self.columns)), np.nan)
        self._rows = {k: i for i, k in enumerate(self.index.tolist())}
        outer = self

        class _Loc:
            def _ix(self, key):
                r, c = key
                ri = outer._rows[r]
                if isinstance(c, (list, tuple)):
                    return ri, [outer.columns.index(x) for x in c]
                return ri, outer.columns.index(c)

            def __getitem__(self, key):
                ri, ci = self._ix(key)
                return outer._a[ri, ci]

            def __setitem__(self, key, v):
                ri, ci = self._ix(key)
                outer._a[ri, ci] = v

        self.loc = _Loc()

    @property
    def values(self):
        return self._a

    def __getitem__(self, c):
        return self._a[:, self.columns.index(c)]


def load_prepare():
    """The reference's SpInterpPrepare (interp/prepare.py, with KrigingDrift of
    interp/drift.py), pandas replaced by LocFrame; call after
    load_reference()."""
    pd = sys.modules.get("pandas")
    if pd is None or not hasattr(pd, "__version__"):
        pd = _stub("pandas")
    prep = importlib.import_module("spinterps.interp.prepare")
    drift = importlib.import_module("spinterps.interp.drift")
    drift.pd = types.SimpleNamespace(DataFrame=LocFrame)
    return prep


def load_variogram(ref_root=None):
    """The reference's Variogram class (variograms/vgs.py) with the stand-in
    DataFrame in place of pandas."""
    import importlib.util
    sys.path.insert(0, str(REPO))
    ref_root = _root(ref_root)
    pd = sys.modules.get("pandas")
    if pd is None or not hasattr(pd, "__version__"):
        pd = _stub("pandas")
    saved = getattr(pd, "DataFrame", None)
    pd.DataFrame = MiniDataFrame
    try:
        spec = importlib.util.spec_from_file_location(
            "spinterps_variograms_vgs", str(ref_root / "variograms" / "vgs.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
    finally:
        if saved is not None:
            pd.DataFrame = saved
    mod.DataFrame = MiniDataFrame
    return mod
