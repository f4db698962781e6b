"""ctypes binding of ``include/spinterps_gb300.h`` (the C ABI).

The structs below mirror the header field by field. Every call checks the
returned ``spi_status`` and raises :class:`SpiError`. There is no fallback:
if the CUDA library cannot be loaded, :func:`lib` raises.
"""
import ctypes
import threading
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_lib" / "libspinterps_gb300.so"

c_i32 = ctypes.c_int32
c_i64 = ctypes.c_int64
c_dbl = ctypes.c_double
c_ptr = ctypes.c_void_p

SPI_MAX_VG_COMP = 4
SPI_MAX_DRIFT = 7
SPI_PINV_MAX_M = 256
SPI_VAR_TC_KC = 8
SPI_VAR_TC_CHUNK_FLOATS = 3 * 256 * SPI_VAR_TC_KC + 4 * SPI_VAR_TC_KC
SPI_IDW_TC_CHUNK_FLOATS = 3 * 64 * 8 + 4 * 8


def idw_tc_pack_floats(n_stns, n_steps):
    """SPI_IDW_TC_PACK_FLOATS of the header."""
    return ((n_steps + 31) // 32) * ((n_stns + 7) // 8) * SPI_IDW_TC_CHUNK_FLOATS
SPI_IR_MAX_ITERS = 12
SPI_PINV_SLOTS = 16
SPI_PINV_SCRATCH_DOUBLES = SPI_PINV_SLOTS * 2 * SPI_PINV_MAX_M * SPI_PINV_MAX_M
GA = SPI_MAX_DRIFT + 1
KIND = {"OK": 0, "SK": 1, "EDK": 2}
# spi_vg_t codes (SPI_VG_*)
VG_CODE = {"Rng": 0, "Nug": 1, "Sph": 2, "Exp": 3, "Lin": 4, "Gau": 5, "Pow": 6, "Hol": 7}
SPI_NOALLOC_MAX_STNS = 512
SPI_NOALLOC_MAX_STEPS = 64

STATUS = {
    0: "SPI_OK",
    1: "SPI_ERR_ARG",
    2: "SPI_ERR_VG",
    3: "SPI_ERR_CUDA",
    4: "SPI_ERR_WORKSPACE",
    5: "SPI_ERR_TOO_LARGE",
}


SPI_ERR_TOO_LARGE = 5


class SpiError(RuntimeError):
    def __init__(self, fn, code, detail=""):
        msg = f"{fn} returned {STATUS.get(code, code)}"
        super().__init__(f"{msg} ({detail})" if detail else msg)
        self.code = code
        self.detail = detail


class VgT(ctypes.Structure):
    _fields_ = [("n_comp", c_i32), ("code", c_i32 * SPI_MAX_VG_COMP),
                ("sill", c_dbl * SPI_MAX_VG_COMP), ("range", c_dbl * SPI_MAX_VG_COMP)]


class DomainT(ctypes.Structure):
    _fields_ = [("n_stns", c_i64), ("stn_x", c_ptr), ("stn_y", c_ptr),
                ("n_cells", c_i64), ("cell_x", c_ptr), ("cell_y", c_ptr),
                ("n_drift", c_i32), ("stn_drift", c_ptr), ("cell_drift", c_ptr),
                ("min_vg_val", c_dbl), ("stn_split", c_ptr), ("cell_split", c_ptr),
                ("split_res", c_dbl)]


class SystemsT(ctypes.Structure):
    _fields_ = [("n_sys", c_i32), ("kind", c_i32), ("stn_off", c_ptr), ("stn_idx", c_ptr),
                ("vg", c_ptr), ("mat_off", c_ptr), ("step_off", c_ptr), ("steps", c_ptr),
                ("val_off", c_ptr), ("out_row", c_ptr), ("max_n", c_i32)]


class KrigeWsT(ctypes.Structure):
    _fields_ = [("l_arena", c_ptr), ("linv_arena", c_ptr), ("status", c_ptr), ("route", c_ptr),
                ("cond", c_ptr), ("shift", c_ptr), ("w_hat", c_ptr), ("beta", c_ptr),
                ("g_cols", c_ptr), ("s_inv", c_ptr), ("g_colsum", c_ptr), ("linv_hi", c_ptr),
                ("linv_lo", c_ptr), ("g_hi", c_ptr), ("g_lo", c_ptr), ("w_hi", c_ptr),
                ("w_lo", c_ptr), ("cell_yy", c_ptr), ("tier", c_ptr), ("var_cells", c_ptr),
                ("pinv_scratch", c_ptr), ("pinv_used", c_ptr), ("l32", c_ptr), ("ir", c_ptr),
                ("ir_iters", c_ptr), ("cond_ir", c_dbl), ("gj_scratch", c_ptr),
                ("linv_tc", c_ptr), ("linv_tc_off", c_ptr)]


class OutT(ctypes.Structure):
    _fields_ = [("out_f64", c_i32), ("est", c_ptr), ("var", c_ptr), ("clip_min_on", c_i32),
                ("clip_max_on", c_i32), ("clip_min", c_dbl), ("clip_max", c_dbl)]


_SIGS = {
    "spi_parse_vg": [ctypes.c_char_p, ctypes.POINTER(VgT)],
    "spi_check_full_nuggetness": [ctypes.c_char_p, c_dbl, ctypes.POINTER(c_i32)],
    "spi_fill_dists_2d_mat": [c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_i64, c_ptr, c_ptr],
    "spi_fill_vg_var_arr": [c_ptr, c_i64, c_i64, c_ptr, c_i32, c_i32, ctypes.POINTER(VgT),
                            c_dbl, c_ptr],
    "spi_copy_2d_arr_at_idxs": [c_ptr, c_i64, c_i64, c_ptr, c_i64, c_ptr, c_i64, c_ptr, c_i64,
                                c_ptr],
    "spi_split_coords": [c_ptr, c_ptr, c_i64, c_dbl, c_dbl, c_dbl, c_ptr, c_ptr],
    "spi_split_f64": [c_ptr, c_ptr, c_ptr, c_i64, c_ptr],
    "spi_krige_factor": [ctypes.POINTER(DomainT), ctypes.POINTER(SystemsT),
                         ctypes.POINTER(KrigeWsT), c_dbl, c_ptr],
    "spi_krige_duals": [ctypes.POINTER(DomainT), ctypes.POINTER(SystemsT), c_ptr,
                        ctypes.POINTER(KrigeWsT), c_ptr],
    "spi_krige_cells": [ctypes.POINTER(DomainT), ctypes.POINTER(SystemsT), c_ptr,
                        ctypes.POINTER(KrigeWsT), c_i32, c_i32, c_i32, c_dbl,
                        ctypes.POINTER(OutT), c_ptr],
    "spi_idw_cells": [ctypes.POINTER(DomainT), c_i32, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
                      c_ptr, c_dbl, c_i32, ctypes.POINTER(OutT), c_ptr],
    "spi_nnb_cells": [ctypes.POINTER(DomainT), c_i32, c_ptr, c_ptr, c_ptr,
                      ctypes.POINTER(OutT), c_ptr],
    "spi_fill_rows": [c_i32, c_ptr, c_ptr, c_ptr, c_i64, ctypes.POINTER(OutT), c_ptr],
    "spi_krige_cells_tiled": [ctypes.POINTER(DomainT), ctypes.POINTER(SystemsT), c_ptr,
                              ctypes.POINTER(KrigeWsT), c_i32, c_i32, c_i32, c_dbl,
                              ctypes.POINTER(OutT), c_i32, c_ptr],
    "spi_krige_tier": [ctypes.POINTER(SystemsT), ctypes.POINTER(KrigeWsT), c_i64, c_ptr, c_ptr,
                       c_ptr, c_ptr, c_ptr, c_dbl, c_dbl, c_dbl, c_dbl, c_ptr, c_ptr, c_ptr,
                       c_ptr],
    "spi_krige_var_tc_pack": [ctypes.POINTER(DomainT), ctypes.POINTER(SystemsT),
                              ctypes.POINTER(KrigeWsT), c_ptr],
    "spi_krige_var_df": [ctypes.POINTER(DomainT), ctypes.POINTER(SystemsT),
                         ctypes.POINTER(KrigeWsT), c_dbl, c_ptr],
    "spi_krige_var_tc": [ctypes.POINTER(DomainT), ctypes.POINTER(SystemsT),
                         ctypes.POINTER(KrigeWsT), c_dbl, c_ptr, c_ptr],
    "spi_krige_loo": [ctypes.POINTER(DomainT), ctypes.POINTER(SystemsT),
                      ctypes.POINTER(KrigeWsT), c_ptr, c_ptr],
    "spi_vg_empirical": [c_i32, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_i64, c_i64,
                         c_i32, c_dbl, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr],
    "spi_vg_de": [c_i32, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_i32, c_dbl, c_ptr, c_ptr, c_ptr,
                  c_ptr],
    "spi_neb_select": [c_i32, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_i32, c_i32, c_i32, c_ptr,
                       c_ptr],
    "spi_vg_refine": [c_i32, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_dbl, c_ptr, c_ptr,
                      c_ptr, c_ptr],
    "spi_vg_features": [c_i32, c_ptr, c_ptr, c_ptr, c_ptr, c_i32, c_ptr, c_ptr],
    "spi_mlp_forward": [c_i32, c_i32, c_i32, c_i32, c_i32, c_ptr, c_ptr, c_i32, c_ptr, c_ptr,
                        c_ptr],
    "spi_mlp_grad": [c_i32, c_i32, c_i32, c_i32, c_i32, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
                     ctypes.c_float, c_i32, c_ptr, c_ptr, c_ptr, c_ptr],
    "spi_mlp_adam": [c_ptr, c_ptr, c_ptr, c_ptr, c_i64, ctypes.c_float, ctypes.c_float,
                     ctypes.c_float, ctypes.c_float, c_i32, c_ptr],
    "spi_krige_ok_noalloc": [ctypes.POINTER(DomainT), c_ptr, c_i32, ctypes.POINTER(VgT), c_ptr,
                             c_i32, c_i32, ctypes.POINTER(OutT), c_ptr, c_ptr],
    "spi_points_in_polygons": [c_ptr, c_ptr, c_i64, c_i32, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
                               c_ptr],
    "spi_field_stats": [c_ptr, c_i32, c_i32, c_i64, c_i64, c_i32, c_ptr, c_i64, c_ptr, c_ptr],
    "spi_round_fields": [c_ptr, c_i32, c_i64, c_i32, c_ptr],
    "spi_local_cells": [ctypes.POINTER(DomainT), c_i32, c_i32, c_ptr, c_i32, c_ptr, c_ptr, c_ptr,
                        c_i64, c_ptr, c_ptr, c_dbl, c_dbl, c_i32, ctypes.POINTER(OutT), c_ptr,
                        c_ptr],
    "spi_peak_fma": [c_i32, c_i64, c_ptr, ctypes.POINTER(c_i64), c_ptr],
    "spi_legacy_system": [c_i32, c_ptr, c_ptr, c_i32, c_ptr, c_i32, ctypes.POINTER(VgT), c_ptr,
                          c_ptr, c_ptr, c_ptr, c_ptr, c_ptr],
    "spi_legacy_points": [c_i32, c_ptr, c_ptr, c_ptr, c_ptr, c_i32, c_ptr, c_ptr, c_ptr, c_i64,
                          c_i32, ctypes.POINTER(VgT), c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
                          c_ptr, c_ptr],
    "spi_sym_pinv": [c_ptr, c_i32, c_dbl, c_ptr, c_ptr, c_ptr, c_ptr],
    "spi_local_groups": [ctypes.POINTER(DomainT), c_i32, c_i32, c_ptr, c_i32, c_ptr, c_ptr,
                         c_i32, c_ptr, c_ptr, c_ptr, c_i64, c_ptr, c_ptr, c_dbl, c_i32,
                         ctypes.POINTER(OutT), c_ptr, c_i64, c_ptr, c_ptr],
    "spi_idw_cells_tc": [ctypes.POINTER(DomainT), c_i32, c_ptr, c_ptr, c_ptr, c_ptr, c_ptr,
                         c_dbl, c_ptr, c_i64, ctypes.POINTER(OutT), c_ptr, c_ptr],
}

# every entry point the header declares (checked by the CPU tests)
EXPORTS = sorted(list(_SIGS) + ["spi_version", "spi_cuda_error", "spi_mlp_n_params",
                                 "spi_local_groups_scratch_bytes"])

_lib = None
_lock = threading.Lock()


def load(path=LIB_PATH):
    """Load the shared library (no GPU needed) and bind the signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not Path(path).exists():
            raise RuntimeError(
                f"spinterps_gb300 CUDA library not built ({path}); run "
                "spinterps_gb300.build.build() first -- there is no CPU fallback")
        lib = ctypes.CDLL(str(path))
        for name, args in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        lib.spi_version.restype = ctypes.c_char_p
        lib.spi_version.argtypes = []
        lib.spi_cuda_error.restype = ctypes.c_char_p
        lib.spi_cuda_error.argtypes = []
        lib.spi_mlp_n_params.restype = c_i64
        lib.spi_mlp_n_params.argtypes = [c_i32, c_i32, c_i32, c_i32]
        lib.spi_local_groups_scratch_bytes.restype = c_i64
        lib.spi_local_groups_scratch_bytes.argtypes = [c_i32, c_i32, c_i32, c_i32, c_i32]
        _lib = lib
        return lib


def lib():
    return load()


def call(name, *args):
    """Call an entry point; raise SpiError on a non-zero status."""
    rc = getattr(lib(), name)(*args)
    if rc != 0:
        detail = ""
        if STATUS.get(rc) == "SPI_ERR_CUDA":
            detail = (lib().spi_cuda_error() or b"").decode(errors="replace")
        raise SpiError(name, rc, detail)
    return rc
