"""Build libytgb.so: the sm_103a kernels and the host C++ behind include/ytgb.h.

One nvcc invocation compiles the CUDA translation units for sm_103a only and
the host C++ with ``-ffp-contract=off`` (the host float64 arithmetic must round
like yt's compiled Cython on every host, including aarch64 where GCC would
otherwise fuse multiply-adds).  ``--fmad=false`` keeps the device float64
traversal free of contractions as well; the float32 sampling code spells its
fused multiply-adds explicitly.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUTDIR = PKG / "lib"
LIB = OUTDIR / "libytgb.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["ytgb_render.cu", "ytgb_prep.cu", "ytgb_octree.cu", "ytgb_offaxis.cu"]
CPP_SOURCES = ["ytgb_host.cpp", "ytgb_pack.cpp"]
# the CPython extension that scans a sampler's bricks natively
MARSHAL_SOURCE = CSRC / "ytgb_pymarshal.cpp"
MARSHAL = OUTDIR / ("_ytgb_marshal" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libytgb")


def _sources():
    return [CSRC / s for s in CU_SOURCES + CPP_SOURCES] + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [
        INCLUDE / "ytgb.h"]


def up_to_date() -> bool:
    if not LIB.exists() or not MARSHAL.exists() or MARSHAL.stat().st_mtime < MARSHAL_SOURCE.stat().st_mtime:
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources() if p.exists())


def build_marshal() -> Path:
    """Compile the ``_ytgb_marshal`` CPython extension (plain C API, no
    numpy headers) next to libytgb.so."""
    OUTDIR.mkdir(parents=True, exist_ok=True)
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("a C++ compiler is required to build _ytgb_marshal")
    tmp = MARSHAL.with_suffix(f".{os.getpid()}.tmp")
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", f"-I{sysconfig.get_paths()['include']}",
           str(MARSHAL_SOURCE), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, MARSHAL)
    return MARSHAL


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    objdir = OUTDIR / "_obj"
    objdir.mkdir(parents=True, exist_ok=True)
    inc = [f"-I{INCLUDE}", f"-I{CSRC}"]
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]

    def compile_one(src: Path) -> Path:
        obj = objdir / (src.stem + ".o")
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, "-lineinfo", "--fmad=false", *common, *inc, "-c", str(src), "-o", str(obj)]
            if verbose:
                cmd += ["-Xptxas", "-v"]
        else:
            cmd = [nvcc, *common, *inc, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    srcs = [CSRC / s for s in CU_SOURCES + CPP_SOURCES]
    with ThreadPoolExecutor(max_workers=min(8, len(srcs) + 1)) as ex:
        marshal = ex.submit(build_marshal)
        objs = list(ex.map(compile_one, srcs))
        marshal.result()
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-Xcompiler", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
