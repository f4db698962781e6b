"""The single-neighbourhood kriging classes of the reference's Cython module
(cyth/interpmthds.pyx:251-765, exported by the package ``__init__``) on the
GPU: ``OrdinaryKriging``, ``SimpleKriging``, ``ExternalDriftKriging``,
``ExternalDriftKriging_MD``, ``OrdinaryIndicatorKriging`` and
``SimpleIndicatorKriging``.

Same constructors, same ``krige()`` / ``ikrige()`` methods, and the same
arrays left on the object (numpy, float64): ``in_dists``, the kriging matrix
(``in_vars`` / ``in_covars``) and its inverse, ``rhss``, ``lambdas``, the
Lagrange multipliers (``mus``, ``mus_1``/``mus_2``, ``mus_arr``), ``zk`` and
the variances (``est_vars`` / ``est_covars``), ``ik`` and ``ixi``. The
arithmetic runs in ``spi_legacy_system`` and ``spi_legacy_points``
(csrc/spi_legacy.cu); there is no CPU path.

These classes keep the reference's own semantics, which differ from the
step engine's:
- the semivariogram matrix is 0 on its diagonal and a right-hand side is 0
  at distance 0, so a nugget is a discontinuity;
- there is no min_vg_val cut and no sum check;
- ``SimpleKriging``'s matrix is minus the semivariogram matrix, with a zero
  diagonal. The reference's ``__init__`` fills it with the total sill before
  ``krige()`` has summed the sills.

Differences, by design:
- The reference's ``numpy.linalg.pinv`` is replaced by a Gauss-Jordan
  inverse on the GPU. This is the same matrix whenever pinv's cut-off
  (numpy's default rcond: singular values up to 1e-15 times the largest
  are dropped) removes nothing, which is certain while
  ||A||_F ||A^-1||_F <= 1e15.
- Above that bound, for example with duplicated stations, the matrix takes
  a pseudo-inverse from this package's Jacobi eigen-decomposition on the
  GPU (``spi_sym_pinv``, up to 256 rows; above that ``torch.linalg.pinv``),
  dropping the eigenvalues up to m * eps times the largest. An exactly
  singular matrix's null singular values come out of an SVD as rounding
  noise of about eps to 16 eps times the largest, on either side of
  numpy's 1e-15 depending on the LAPACK build; the wider cut-off drops
  them on every platform. ``pinv_route`` on the object records which
  inverse was used.
- ``krige()`` runs once per object. A second call on the reference's
  object appends the components again and adds onto the old matrix, which
  kriges a different system, so here a second call raises RuntimeError.
- No stations raises ``SpiError`` (the reference inverts a 1 x 1 zero
  matrix).

``krige_points`` is the same computation on CUDA tensors (device-resident
inputs and outputs), for callers that keep their data on the GPU.
"""
import ctypes

import numpy as np
import torch

from . import _native as nat
from .steps import _require_cuda

_CODES = {b"Rng": 0, b"Nug": 1, b"Sph": 2, b"Exp": 3, b"Lin": 4, b"Gau": 5, b"Pow": 6,
          b"Hol": 7}
# ||A||_F ||A^-1||_F bound under which numpy.linalg.pinv (rcond 1e-15)
# drops no singular value: the Gauss-Jordan inverse is its matrix
PINV_COND = 1e15


def parse_model(model):
    """Components ``[(name, sill, range)]`` of a model string, by the split
    rules of cyth/interpmthds.pyx:294-304: split on '+', strip, split on ' '
    into exactly the sill and 'Name(range)', then on '(' and ')'; the range
    is clamped to max(1e-5, range). Raises ValueError (wrong token count, a
    bad number) as the reference's parse does, and KeyError for an unknown
    model name (the reference's C++ map lookup inserts a null function there
    and the process crashes on its first call)."""
    if isinstance(model, str):
        model = model.encode("utf-8")
    out = []
    for submodel in model.split(b"+"):
        submodel = submodel.strip()
        sill, vg = submodel.split(b" ")
        vg, rng = vg.split(b"(")
        rng = rng.split(b")")[0]
        if vg not in _CODES:
            raise KeyError(vg)
        out.append((vg, float(sill), max(1e-5, float(rng))))
    return out


def _vg_struct(comps):
    if len(comps) > nat.SPI_MAX_VG_COMP:
        raise ValueError(f"at most {nat.SPI_MAX_VG_COMP} variogram components, got {len(comps)}")
    vg = nat.VgT()
    vg.n_comp = len(comps)
    for c, (name, sill, rng) in enumerate(comps):
        vg.code[c] = _CODES[name]
        vg.sill[c] = sill
        vg.range[c] = rng
    return vg


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _pinv(lhs, st):
    """The pseudo-inverse of the (symmetric) kriging matrix, eigenvalues up
    to m eps times the largest dropped: spi_sym_pinv's Jacobi
    eigen-decomposition up to SPI_PINV_MAX_M rows, torch.linalg.pinv (an
    SVD with the same cut-off) above that or where the sweeps do not
    converge."""
    m = int(lhs.shape[0])
    if m <= nat.SPI_PINV_MAX_M:
        out = torch.empty_like(lhs)
        scratch = torch.empty(2 * m * m, dtype=torch.float64, device=lhs.device)
        status = torch.zeros(1, dtype=torch.int32, device=lhs.device)
        nat.call("spi_sym_pinv", _ptr(lhs), m, m * float(np.finfo(np.float64).eps), _ptr(out),
                 _ptr(scratch), _ptr(status), st)
        if int(status.item()) >= 0:
            return out
    return torch.linalg.pinv(lhs).contiguous()


def krige_points(kind, xi, yi, zi, xk, yk, model, si=None, sk=None, ixi=None, want_est=True):
    """One legacy kriging run on CUDA tensors (float64, contiguous).

    kind: "OK", "SK" or "EDK"; si [k, n] / sk [k, n_out] drift values for EDK;
    ixi [n]: indicator values (the indicator classes' ``ikrige``). Returns a
    dict of device tensors: in_dists, lhs, lhs_inv, rhss, lambdas, mus
    [m - n, n_out] (None for SK), zk, est (None when want_est is false or for
    EDK), ik (None without ixi), and ``route``: "gj" (the Gauss-Jordan
    inverse) or "pinv" (the pseudo-inverse, taken where pinv's cut-off may
    drop a singular value). Runs on the current stream."""
    comps = parse_model(model) if not isinstance(model, list) else model
    vg = _vg_struct(comps)
    code = nat.KIND[kind]
    dev = _require_cuda(xi.device)
    n, n_out = int(xi.shape[0]), int(xk.shape[0])
    n_drift = int(si.shape[0]) if kind == "EDK" else 0
    a = 0 if kind == "SK" else 1 + n_drift
    m = n + a
    f64 = dict(dtype=torch.float64, device=dev)
    st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    in_dists = torch.empty((n, n), **f64)
    lhs = torch.empty((m, m), **f64)
    inv = torch.empty((m, m), **f64)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    cond = torch.zeros(1, **f64)
    nat.call("spi_legacy_system", code, _ptr(xi), _ptr(yi), n, _ptr(si), n_drift,
             ctypes.byref(vg), _ptr(in_dists), _ptr(lhs), _ptr(inv), _ptr(status), _ptr(cond),
             st)
    route = "gj"
    if int(status.item()) or not float(cond.item()) <= PINV_COND:
        inv = _pinv(lhs, st)
        route = "pinv"
    rhss = torch.empty((n_out, m), **f64)
    lambdas = torch.empty((n_out, n), **f64)
    mus = torch.empty((a, n_out), **f64) if a else None
    zk = torch.empty(n_out, **f64)
    est = torch.empty(n_out, **f64) if (want_est and kind != "EDK") or ixi is not None else None
    ik = torch.empty(n_out, **f64) if ixi is not None else None
    nat.call("spi_legacy_points", code, _ptr(xi), _ptr(yi), _ptr(zi), _ptr(ixi), n, _ptr(xk),
             _ptr(yk), _ptr(sk), n_out, n_drift, ctypes.byref(vg), _ptr(inv), _ptr(rhss),
             _ptr(lambdas), _ptr(mus), _ptr(zk), _ptr(est), _ptr(ik), st)
    return dict(in_dists=in_dists, lhs=lhs, lhs_inv=inv, rhss=rhss, lambdas=lambdas, mus=mus,
                zk=zk, est=est, ik=ik, route=route)


def _dev(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def _host(t):
    return t.cpu().numpy()


class _LegacyKriging:
    _kind = "OK"

    def __init__(self, xi, yi, zi, xk, yk, model="1.0 Sph(2)"):
        self.xi = xi
        self.yi = yi
        self.zi = zi
        self.xk = xk
        self.yk = yk
        self.model = bytes(model, "utf-8")
        self.in_count = self.xi.shape[0]
        self.out_count = self.xk.shape[0]
        self.vgs, self.sills, self.ranges = [], [], []
        self.zk = np.zeros(self.out_count)
        self.in_dists = np.zeros((self.in_count, self.in_count))
        self.lambdas = np.zeros((self.out_count, self.in_count))
        self.pinv_route = None
        self._ran = False

    def _run(self, ixi=None, si=None, sk=None):
        if self._ran:
            raise RuntimeError(
                "krige() runs once per object (a second call on the reference's class "
                "kriges a different system); make a new object")
        _require_cuda("cuda")
        comps = parse_model(self.model)
        for name, sill, rng in comps:
            self.vgs.append(name)
            self.sills.append(sill)
            self.ranges.append(rng)
        self._ran = True
        r = krige_points(self._kind, _dev(self.xi), _dev(self.yi), _dev(self.zi),
                         _dev(self.xk), _dev(self.yk), comps,
                         si=None if si is None else _dev(si), sk=None if sk is None else _dev(sk),
                         ixi=None if ixi is None else _dev(ixi))
        torch.cuda.current_stream().synchronize()
        self.pinv_route = r.pop("route")
        return {k: (None if v is None else _host(v)) for k, v in r.items()}


class OrdinaryKriging(_LegacyKriging):
    """cyth/interpmthds.pyx:251-362."""
    _kind = "OK"

    def __init__(self, xi, yi, zi, xk, yk, model="1.0 Sph(2)"):
        super().__init__(xi, yi, zi, xk, yk, model=model)
        self.mus = np.zeros(self.out_count)
        self.est_vars = np.zeros(self.out_count)
        self.in_vars = np.zeros((self.in_count + 1, self.in_count + 1))
        self.in_vars_inv = self.in_vars.copy()
        self.rhss = np.zeros((self.out_count, self.in_count + 1))
        self.out_vars = None

    def _store(self, r):
        self.in_dists, self.in_vars, self.in_vars_inv = r["in_dists"], r["lhs"], r["lhs_inv"]
        self.rhss, self.lambdas, self.zk = r["rhss"], r["lambdas"], r["zk"]
        self.mus = r["mus"][0].copy()
        self.est_vars = r["est"]

    def krige(self):
        self._store(self._run())


class SimpleKriging(_LegacyKriging):
    """cyth/interpmthds.pyx:365-471."""
    _kind = "SK"

    def __init__(self, xi, yi, zi, xk, yk, model="1.0 Sph(2)"):
        super().__init__(xi, yi, zi, xk, yk, model=model)
        self.covar = 0.0
        self.est_covars = np.zeros(self.out_count)
        self.in_covars = np.full((self.in_count, self.in_count), self.covar)
        self.in_covars_inv = self.in_covars.copy()
        self.out_covars = np.zeros((self.out_count, self.in_count))
        self.rhss = np.zeros((self.out_count, self.in_count))

    def _store(self, r):
        for s in self.sills:
            self.covar += s
        self.in_dists, self.in_covars, self.in_covars_inv = r["in_dists"], r["lhs"], r["lhs_inv"]
        self.rhss, self.lambdas, self.zk = r["rhss"], r["lambdas"], r["zk"]
        self.out_covars = r["rhss"].copy()
        self.est_covars = r["est"]

    def krige(self):
        self._store(self._run())


class ExternalDriftKriging(_LegacyKriging):
    """cyth/interpmthds.pyx:474-585 (one drift: si [n], sk [n_out])."""
    _kind = "EDK"

    def __init__(self, xi, yi, zi, si, xk, yk, sk, model="1.0 Sph(2)"):
        super().__init__(xi, yi, zi, xk, yk, model=model)
        self.si = si
        self.sk = sk
        self.mus_1 = np.zeros(self.out_count)
        self.mus_2 = np.zeros(self.out_count)
        self.in_vars = np.zeros((self.in_count + 2, self.in_count + 2))
        self.in_vars_inv = self.in_vars.copy()
        self.rhss = np.zeros((self.out_count, self.in_count + 2))

    def krige(self):
        r = self._run(si=np.reshape(self.si, (1, -1)), sk=np.reshape(self.sk, (1, -1)))
        self.in_dists, self.in_vars, self.in_vars_inv = r["in_dists"], r["lhs"], r["lhs_inv"]
        self.rhss, self.lambdas, self.zk = r["rhss"], r["lambdas"], r["zk"]
        self.mus_1, self.mus_2 = r["mus"][0].copy(), r["mus"][1].copy()


class ExternalDriftKriging_MD(_LegacyKriging):
    """cyth/interpmthds.pyx:588-719 (si [k, n], sk [k, n_out])."""
    _kind = "EDK"

    def __init__(self, xi, yi, zi, si, xk, yk, sk, model="1.0 Sph(2)"):
        assert len(xi.shape) == 1
        assert len(si.shape) == 2
        assert xi.shape[0] == yi.shape[0] == zi.shape[0] == si.shape[1], \
            'Observation points and drift shapes are unequal!'
        assert xk.shape[0] == yk.shape[0] == sk.shape[1], \
            'Resulting points and drifts shapes are unequal!'
        assert si.shape[0] == sk.shape[0], \
            'Observation and reulting drifts have unequal shapes!'
        super().__init__(xi, yi, zi, xk, yk, model=model)
        self.si = si
        self.sk = sk
        self.n_drifts = sk.shape[0]
        self.mus_arr = np.zeros((self.n_drifts + 1, self.out_count))
        m = self.in_count + self.n_drifts + 1
        self.in_vars = np.zeros((m, m))
        self.in_vars_inv = self.in_vars.copy()
        self.rhss = np.zeros((self.out_count, m))

    def krige(self):
        r = self._run(si=self.si, sk=self.sk)
        self.in_dists, self.in_vars, self.in_vars_inv = r["in_dists"], r["lhs"], r["lhs_inv"]
        self.rhss, self.lambdas, self.zk = r["rhss"], r["lambdas"], r["zk"]
        self.mus_arr = r["mus"]


class OrdinaryIndicatorKriging(OrdinaryKriging):
    """cyth/interpmthds.pyx:722-742: ordinary kriging of the indicator
    z <= lim; ``ikrige`` leaves ik = max(0, lambda'ixi) and est_vars =
    max(0, ik (1 - ik))."""

    def __init__(self, xi, yi, zi, xk, yk, lim=1, model="1.0 Sph(2)"):
        super().__init__(xi, yi, zi, xk, yk, model=model)
        self.lim = lim
        self.ixi = np.where(self.zi <= self.lim, 1., 0.)
        self.ik = np.zeros(self.out_count)

    def ikrige(self):
        r = self._run(ixi=self.ixi)
        self._store(r)
        self.ik = r["ik"]


class SimpleIndicatorKriging(SimpleKriging):
    """cyth/interpmthds.pyx:745-765: the simple-kriging counterpart
    (est_covars = max(0, ik (1 - ik)))."""

    def __init__(self, xi, yi, zi, xk, yk, lim=1, model="1.0 Sph(2)"):
        super().__init__(xi, yi, zi, xk, yk, model=model)
        self.lim = lim
        self.ixi = np.where(self.zi <= self.lim, 1., 0.)
        self.ik = np.zeros(self.out_count)

    def ikrige(self):
        r = self._run(ixi=self.ixi)
        self._store(r)
        self.ik = r["ik"]
