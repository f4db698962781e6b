"""Recipe: compile the reference's Cython kernels into ``oracle/_ref/``.

TEST INFRASTRUCTURE ONLY. Nothing in the product imports this module.

The reference's only native component is ``cyth/interpmthds.pyx`` (built by
the reference through pyximport as C++, ``cyth/interpmthds.pyxbld:3-9``).
This recipe cythonizes that file where it lies (the reference tree is read
only; all outputs go to ``oracle/_ref/``) with ``cpow=True`` so that ``**``
keeps the Cython 0.29 C semantics the reference was written against (with
Cython 3's default ``cpow=False`` a zero distance in IDW raises instead of
producing inf/NaN), then compiles it with g++ against numpy's headers.

Usage (only where the reference tree exists, i.e. not on the GPU host)::

    python oracle/build_ref.py REFERENCE_ROOT

or with the root in the environment variable SPINTERPS_REFERENCE_ROOT
(``build()`` without an argument reads it, and builds nothing when it is
unset).
"""
import os
import subprocess
import sys
import sysconfig
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
ENV = "SPINTERPS_REFERENCE_ROOT"


def reference_root(ref_root=None):
    """The reference tree: the argument, else $SPINTERPS_REFERENCE_ROOT, else
    None."""
    if ref_root is None:
        ref_root = os.environ.get(ENV)
    return Path(ref_root) if ref_root else None


def build(ref_root=None, force=False):
    """Build ``oracle/_ref/interpmthds*.so``; return its directory or None
    (no reference tree given, or Cython absent)."""
    ref_root = reference_root(ref_root)
    if ref_root is None:
        return None
    pyx = ref_root / "cyth" / "interpmthds.pyx"
    if not pyx.exists():
        return None
    try:
        from Cython.Build import cythonize  # noqa: F401
        from Cython.Compiler import Main as cymain
    except ImportError:
        return None
    import numpy as np

    OUT.mkdir(parents=True, exist_ok=True)
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    so_path = OUT / f"interpmthds{suffix}"
    if so_path.exists() and not force:
        return OUT
    cpp_path = OUT / "interpmthds.cpp"
    opts = cymain.CompilationOptions(
        cymain.default_options,
        cplus=True,
        output_file=str(cpp_path),
        language_level=3,
        compiler_directives={"cpow": True},
    )
    res = cymain.compile(str(pyx), opts)
    if res.num_errors:
        raise RuntimeError("cython failed on the reference kernels")
    inc = [sysconfig.get_paths()["include"], np.get_include()]
    cmd = ["g++", "-O2", "-shared", "-fPIC", "-std=c++17", "-w"]
    for i in inc:
        cmd += ["-I", i]
    cmd += [str(cpp_path), "-o", str(so_path)]
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    out = build(sys.argv[1] if len(sys.argv) > 1 else None, force=True)
    print("built" if out else "reference not present", out)
