"""Compile the CUDA sources into ``spinterps_gb300/_lib/libspinterps_gb300.so``.

One ``-gencode`` (sm_103a), translation units compiled in parallel, then
linked into a shared library with the CUDA runtime linked statically, so the
library loads beside any PyTorch build. In-tree output (git-ignored).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libspinterps_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-I", str(ROOT / "include"), "-I", str(CSRC)]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found")
    return cand


def sources():
    return sorted(CSRC.glob("*.cu"))


def _stale():
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + list((ROOT / "include").glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force=False, verbose=False, extra=()):
    """Build the library if a source changed; return its path."""
    if not force and not _stale():
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    nv = nvcc()
    objs = []

    def compile_one(src):
        obj = OUT / (src.stem + ".o")
        cmd = [nv, *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        for obj, err in ex.map(compile_one, sources()):
            objs.append(obj)
            if verbose and err:
                sys.stderr.write(err)
    tmp = OUT / (LIB.name + ".tmp")
    cmd = [nv, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
