"""The interpolated fields as a netCDF file laid out like the reference's
(interp/prepare.py:290-432 _initiate_nc, interp/steps.py:879-969
_write_to_disk).

The file holds:
- dimensions ``dimx``, ``dimy``, ``dimt``;
- the cell-centre coordinates (double) and the time values;
- one variable per interpolation label over (dimt, dimy, dimx), in the
  fields' dtype, with ``units`` and ``standard_name``;
- the run's settings as ``sett_*`` global attributes, plus ``Source``.

The reference writes netCDF-4 (HDF5) with zlib compression and
(1, ny, nx) chunks. HDF5 and the netCDF library are not available here, so
this module writes the netCDF classic binary format from its published
specification. The netCDF libraries and xarray read it as they read the
reference's file, through the same names:
- ``fmt=5`` (CDF-5, the default) keeps the reference's 64-bit integer time
  variable;
- ``fmt=2`` (CDF-2, 64-bit offsets, also readable by
  scipy.io.netcdf_file) stores time as 32-bit integers.

The classic formats have no compression or chunking. Fields are written
uncompressed, after the same rounding to ``nmrl_prcn`` decimals
(``driver.round_fields_`` on the GPU).
"""
import struct

import numpy as np

NC_DIMENSION, NC_VARIABLE, NC_ATTRIBUTE = 10, 11, 12
NC_TYPES = {  # numpy dtype -> (nc_type, big-endian dtype)
    np.dtype(np.int8): (1, ">i1"),
    np.dtype("S1"): (2, "S1"),
    np.dtype(np.int16): (3, ">i2"),
    np.dtype(np.int32): (4, ">i4"),
    np.dtype(np.float32): (5, ">f4"),
    np.dtype(np.float64): (6, ">f8"),
    np.dtype(np.int64): (10, ">i8"),  # CDF-5 only
}


def _pad4(b):
    return b + b"\x00" * ((-len(b)) % 4)


class _Header:
    def __init__(self, fmt):
        assert fmt in (1, 2, 5)
        self.fmt = fmt
        self.parts = []

    def count(self, v):  # nelems, dim lengths, dim ids, vsize
        self.parts.append(struct.pack(">q" if self.fmt == 5 else ">i", v))

    def tag(self, v):
        self.parts.append(struct.pack(">i", v))

    def offset(self, v):
        self.parts.append(struct.pack(">q" if self.fmt != 1 else ">i", v))

    def name(self, s):
        b = s.encode("utf-8")
        self.count(len(b))
        self.parts.append(_pad4(b))

    def attrs(self, attrs):
        if not attrs:
            self.tag(0)
            self.count(0)
            return
        self.tag(NC_ATTRIBUTE)
        self.count(len(attrs))
        for k, v in attrs.items():
            self.name(k)
            if isinstance(v, str):
                b = v.encode("utf-8")
                self.tag(2)
                self.count(len(b))
                self.parts.append(_pad4(b))
            else:
                a = np.atleast_1d(np.asarray(v))
                t, be = NC_TYPES[a.dtype]
                self.tag(t)
                self.count(a.size)
                self.parts.append(_pad4(a.astype(be).tobytes()))

    def bytes(self):
        return b"".join(self.parts)


class Deferred:
    """A variable whose data write_nc leaves to later slab writes
    (write_slab): only its shape and dtype are given; its region of the
    file is reserved (sparse, reading as zeros until written)."""

    def __init__(self, shape, dtype):
        self.shape = tuple(int(v) for v in shape)
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape, dtype=np.int64)) * self.dtype.itemsize


def _meta(arr):
    if isinstance(arr, Deferred):
        return arr.shape, arr.dtype, arr.nbytes
    a = np.asarray(arr)
    return a.shape, a.dtype, a.nbytes


def write_nc(path, dims, variables, global_attrs=None, fmt=5):
    """A netCDF classic file with fixed-size (non-record) variables.

    dims: {name: length}; variables: list of (name, dim names, numpy array
    or Deferred, attrs dict); all arrays are written big-endian, each padded
    to 4 bytes. fmt: 1 (CDF-1), 2 (CDF-2, 64-bit offsets) or 5 (CDF-5,
    64-bit data). Returns the path; the byte offset of every variable's data
    is in ``write_nc.begins`` (name -> offset) after the call."""
    dim_names = list(dims)
    for name, dn, arr, _ in variables:
        shape = tuple(dims[d] for d in dn)
        assert tuple(_meta(arr)[0]) == shape, (name, _meta(arr)[0], shape)
        if fmt != 5:
            assert _meta(arr)[1] != np.int64, f"{name}: int64 needs CDF-5"

    def header(begins):
        h = _Header(fmt)
        h.parts.append(b"CDF" + bytes([fmt]))
        h.count(0)  # numrecs: no record dimension
        if dims:
            h.tag(NC_DIMENSION)
            h.count(len(dims))
            for d in dim_names:
                h.name(d)
                h.count(int(dims[d]))
        else:
            h.tag(0)
            h.count(0)
        h.attrs(global_attrs or {})
        if variables:
            h.tag(NC_VARIABLE)
            h.count(len(variables))
            for (name, dn, arr, attrs), beg in zip(variables, begins):
                _, dt, nb = _meta(arr)
                t, _ = NC_TYPES[dt]
                h.name(name)
                h.count(len(dn))
                for d in dn:
                    h.count(dim_names.index(d))
                h.attrs(attrs or {})
                h.tag(t)
                vsize = nb + ((-nb) % 4)
                if fmt != 5 and vsize > 2**32 - 4:
                    vsize = 2**32 - 1
                h.count(vsize)
                h.offset(beg)
        else:
            h.tag(0)
            h.count(0)
        return h.bytes()

    # offsets depend on the header's length, which does not depend on them
    hlen = len(header([0] * len(variables)))
    begins, pos = [], hlen
    for _, _, arr, _ in variables:
        begins.append(pos)
        n = _meta(arr)[2]
        pos += n + ((-n) % 4)
    with open(path, "wb") as f:
        f.write(header(begins))
        for _, _, arr, _ in variables:
            nb = _meta(arr)[2]
            if isinstance(arr, Deferred):
                f.seek(nb + ((-nb) % 4), 1)
                continue
            a = np.ascontiguousarray(arr)
            be = a.astype(NC_TYPES[a.dtype][1], copy=False)
            f.write(be.tobytes())
            f.write(b"\x00" * ((-a.nbytes) % 4))
        f.truncate(pos)
    write_nc.begins = {v[0]: b for v, b in zip(variables, begins)}
    return path


def write_slab(path, begin, block, first):
    """Write ``block`` (leading axis = the variable's first dimension) into
    a Deferred variable whose data starts at byte ``begin``, from index
    ``first`` of its first dimension on (big-endian, as write_nc)."""
    a = np.ascontiguousarray(block)
    per = int(np.prod(a.shape[1:], dtype=np.int64)) * a.dtype.itemsize
    with open(path, "r+b") as f:
        f.seek(int(begin) + int(first) * per)
        f.write(a.astype(NC_TYPES[a.dtype][1], copy=False).tobytes())


def write_interp_nc(path, x_crds, y_crds, time_vals, fields, interp_args, *, xlab="X",
                    ylab="Y", tlab="time", tunits=None, tcldr=None, vunits="", vlab="",
                    settings=None, fmt=5):
    """The reference's output file: its dimension names (dimx, dimy, dimt)
    and variables, one per interpolation label (interp_args: the reference's
    (type, dir, label[, idw_exp]) tuples), with units and standard_name as
    _initiate_nc sets them (IDW: '{vlab} ({label[:3]}_exp_{exp})').
    fields: label -> [T, ny, nx] array, or a Deferred of that shape whose
    steps come later through write_slab (offsets in write_nc.begins);
    settings: name -> value, written as 'sett_<name>' string attributes;
    Source = the file's path."""
    T, ny, nx = len(time_vals), len(y_crds), len(x_crds)
    dims = {"dimx": nx, "dimy": ny, "dimt": T}
    tv = np.asarray(time_vals)
    tv = tv.astype(np.int64 if fmt == 5 else np.int32)
    tatt = {}
    if tunits is not None:
        tatt["units"] = str(tunits)
    if tcldr is not None:
        tatt["calendar"] = str(tcldr)
    variables = [(xlab, ("dimx",), np.asarray(x_crds, np.float64), {}),
                 (ylab, ("dimy",), np.asarray(y_crds, np.float64), {}),
                 (tlab, ("dimt",), tv, tatt)]
    for a in interp_args:
        lab = a[2]
        std = f"{vlab} ({lab[:3]}_exp_{a[3]})" if a[0] == "IDW" else f"{vlab} ({lab})"
        fl = fields[lab]
        variables.append((lab, ("dimt", "dimy", "dimx"),
                          fl if isinstance(fl, Deferred) else np.asarray(fl),
                          {"units": str(vunits), "standard_name": std}))
    gatt = {f"sett_{k}": str(v) for k, v in (settings or {}).items()}
    gatt["Source"] = str(path)
    return write_nc(path, dims, variables, gatt, fmt=fmt)


def read_nc(path):
    """A reader for the files write_nc makes (classic formats, fixed-size
    variables): returns (dims, {name: (dim names, array, attrs)}, global
    attrs)."""
    buf = open(path, "rb").read()
    assert buf[:3] == b"CDF", "not a netCDF classic file"
    fmt = buf[3]
    pos = [4]

    def take(fmtc, n):
        v = struct.unpack_from(fmtc, buf, pos[0])
        pos[0] += n
        return v[0]

    cnt = (lambda: take(">q", 8)) if fmt == 5 else (lambda: take(">i", 4))
    off = (lambda: take(">i", 4)) if fmt == 1 else (lambda: take(">q", 8))
    tag = lambda: take(">i", 4)  # noqa: E731

    def name():
        n = cnt()
        s = buf[pos[0]:pos[0] + n].decode("utf-8")
        pos[0] += n + ((-n) % 4)
        return s

    inv = {t: be for _, (t, be) in NC_TYPES.items()}

    def attrs():
        t = tag()
        n = cnt()
        out = {}
        for _ in range(n if t == NC_ATTRIBUTE else 0):
            k = name()
            ty = tag()
            m = cnt()
            if ty == 2:
                out[k] = buf[pos[0]:pos[0] + m].decode("utf-8")
                size = m
            else:
                dt = np.dtype(inv[ty])
                size = m * dt.itemsize
                out[k] = np.frombuffer(buf, dt, m, pos[0]).astype(dt.newbyteorder("="))
            pos[0] += size + ((-size) % 4)
        return out

    cnt()  # numrecs
    t = tag()
    nd = cnt()
    dims = {}
    for _ in range(nd if t == NC_DIMENSION else 0):
        k = name()
        dims[k] = cnt()
    dn = list(dims)
    gatt = attrs()
    t = tag()
    nv = cnt()
    out = {}
    for _ in range(nv if t == NC_VARIABLE else 0):
        k = name()
        ids = [cnt() for _ in range(cnt())]
        va = attrs()
        ty = tag()
        cnt()  # vsize
        beg = off()
        dt = np.dtype(inv[ty])
        shape = tuple(dims[dn[i]] for i in ids)
        arr = np.frombuffer(buf, dt, int(np.prod(shape)), beg).reshape(shape)
        out[k] = (tuple(dn[i] for i in ids), arr.astype(dt.newbyteorder("=")), va)
    return dims, out, gatt
