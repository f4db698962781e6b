"""Build the oracle's C restatement (``oracle/vgfill.c``) into ``oracle/_build``.

TEST INFRASTRUCTURE ONLY. ``-ffp-contract=off`` keeps every multiply and add
separately rounded, as in the reference's x86-64 build, on x86 and Arm alike.
"""
import ctypes
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "vgfill.c"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "liboracle.so"


def build(force=False):
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = OUT_DIR / "liboracle.so.tmp"
    subprocess.run(
        ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
         str(SRC), "-o", str(tmp), "-lm"],
        check=True)
    tmp.replace(LIB)
    return LIB


_lib = None


def lib():
    """Load (building on first use) the oracle's C library."""
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build()))
        d = ctypes.c_double
        p = ctypes.c_void_p
        i64 = ctypes.c_int64
        _lib.orc_vg_eval.restype = d
        _lib.orc_vg_eval.argtypes = [ctypes.c_int, d, d, d]
        _lib.orc_fill_dists_2d_mat.restype = None
        _lib.orc_fill_dists_2d_mat.argtypes = [p, p, i64, p, p, i64, p]
        _lib.orc_fill_vg_var_arr.restype = None
        _lib.orc_fill_vg_var_arr.argtypes = [
            p, i64, i64, p, ctypes.c_int, ctypes.c_int, ctypes.c_int, p, p, p, d]
        _lib.orc_copy_2d_arr_at_idxs.restype = None
        _lib.orc_copy_2d_arr_at_idxs.argtypes = [p, i64, p, i64, p, i64, p, i64]
        _lib.orc_fill_wts_and_sum.restype = d
        _lib.orc_fill_wts_and_sum.argtypes = [p, i64, p, d]
        _lib.orc_get_mults_sum.restype = d
        _lib.orc_get_mults_sum.argtypes = [p, p, i64]
        _lib.orc_idw_group.restype = i64
        _lib.orc_idw_group.argtypes = [p, i64, i64, p, i64, p, p, d, p, p]
    return _lib


if __name__ == "__main__":
    print(build(force=True))
