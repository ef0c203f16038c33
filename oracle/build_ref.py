"""Build recipe for the reference's own ray-casting sampler -- TEST INFRASTRUCTURE.

This script compiles yt's hot-path Cython/C++ modules (the sampler path of
``yt/utilities/lib``: image_samplers, grid_traversal, partitioned_grid,
lenses, amr_kdtools, interpolators, _octree_raytracing, image_utilities,
fixed_interpolator)
into importable extension modules under ``oracle/_ref/pkg/``.  Nothing it
produces is product code: only tests, ``__graft_entry__.smoke`` and the CPU
baseline of ``bench.py`` load it, as a checker.

Stage 1 (only where the reference checkout exists, i.e. the development
container): ``cythonize`` the reference ``.pyx`` files into C++ under
``oracle/_ref/gen/`` and stage the handful of headers and
``fixed_interpolator.cpp`` they include next to them.  The flags follow the
reference's own build (``setup.py:33-69``, ``setupext.py:406-409``):
``-std=c++14 -fopenmp``, ``language_level=3``, the NumPy API macros.

Stage 2 (anywhere ``oracle/_ref/gen`` exists): compile every generated
``.cpp`` with ``g++`` into ``oracle/_ref/pkg/yt/utilities/lib/*.so`` and
write a minimal ``yt`` package shell (``yt/funcs.py`` provides only
``mylog``, the one Python-level name ``image_samplers.pyx:32`` imports).

Two builds are made: ``pkg`` with ``-ffp-contract=off`` (bit-exact FP64
semantics on every host, the parity oracle) and, with ``--timed``, ``pkg_timed``
with the reference's default flags (the timed CPU baseline; on aarch64 GCC
contracts multiply-adds by default).

Also compiled: ``oracle/ref_trace.pyx``, this repository's own probe that
calls the reference's ``walk_volume`` (``grid_traversal.pyx:26-140``) with a
recording callback, to pin the visited-cell sequence per ray.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
GEN = OUT / "gen"
# the reference checkout: YTGB_REFERENCE_ROOT, else a directory named
# "reference" beside this checkout
REF_ROOT = Path(os.environ.get("YTGB_REFERENCE_ROOT", str(HERE.parent.parent / "reference")))
LIB_REL = Path("yt/utilities/lib")

MODULES = [
    "image_samplers",
    "grid_traversal",
    "partitioned_grid",
    "lenses",
    "amr_kdtools",
    "interpolators",
    "_octree_raytracing",
    "image_utilities",
]
# headers / sources the generated C++ includes, staged so that stage 2 can run
# on a machine without the reference checkout
STAGED = [
    "fixed_interpolator.cpp",
    "fixed_interpolator.hpp",
    "platform_dep.h",
    "platform_dep_math.hpp",
    "_octree_raytracing.hpp",
]
NUMPY_MACROS = ["-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION", "-DNPY_TARGET_VERSION=NPY_1_21_API_VERSION"]


def _cythonize() -> None:
    from Cython.Build import cythonize  # noqa: PLC0415  (dev container only)
    from setuptools import Extension  # noqa: PLC0415

    src_lib = REF_ROOT / LIB_REL
    GEN.mkdir(parents=True, exist_ok=True)
    for name in STAGED:
        shutil.copyfile(src_lib / name, GEN / name)
    exts = []
    for m in MODULES:
        exts.append(
            Extension(
                f"yt.utilities.lib.{m}",
                [str(LIB_REL / f"{m}.pyx")],
                language="c++",
            )
        )
    cwd = os.getcwd()
    os.chdir(REF_ROOT)
    try:
        out = cythonize(
            exts,
            build_dir=str(OUT / "cybuild"),
            compiler_directives={"language_level": 3},
            aliases={
                "LIB_DIR": "yt/utilities/lib/",
                "STD_LIBS": ["m"],
                "OMP_ARGS": ["-fopenmp"],
                "FIXED_INTERP": "fixed_interpolator",
                "CPP14_FLAG": ["-std=c++14"],
            },
            include_path=[str(REF_ROOT)],
            quiet=True,
        )
    finally:
        os.chdir(cwd)
    for ext in out:
        name = ext.name.rsplit(".", 1)[1]
        cpp = Path(ext.sources[0])
        if not cpp.is_absolute():
            cpp = REF_ROOT / cpp
        shutil.copyfile(cpp, GEN / f"{name}.cpp")
    # the trace probe (this repository's own code) cimports the reference
    probe = Extension("ytref_trace", [str(HERE / "ref_trace.pyx")], language="c++")
    out = cythonize(
        [probe],
        build_dir=str(OUT / "cybuild"),
        compiler_directives={"language_level": 3},
        include_path=[str(REF_ROOT)],
        quiet=True,
    )
    cpp = Path(out[0].sources[0])
    shutil.copyfile(cpp, GEN / "ytref_trace.cpp")
    shutil.rmtree(OUT / "cybuild", ignore_errors=True)


def _compile(pkg: Path, fp_contract_off: bool, jobs: int) -> None:
    import numpy  # noqa: PLC0415

    libdir = pkg / LIB_REL
    libdir.mkdir(parents=True, exist_ok=True)
    for d in (pkg / "yt", pkg / "yt/utilities", libdir):
        (d / "__init__.py").touch()
    (pkg / "yt" / "funcs.py").write_text(
        "import logging\n\nmylog = logging.getLogger('ytref')\n"
    )
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    inc = [
        f"-I{sysconfig.get_paths()['include']}",
        f"-I{numpy.get_include()}",
        f"-I{GEN}",
    ]
    flags = ["-O2", "-fPIC", "-std=c++14", "-fopenmp", "-fwrapv", *NUMPY_MACROS]
    if fp_contract_off:
        flags.append("-ffp-contract=off")
    objdir = pkg / "_obj"
    objdir.mkdir(exist_ok=True)
    fobj = objdir / "fixed_interpolator.o"
    subprocess.run(
        ["g++", *flags, *inc, "-c", str(GEN / "fixed_interpolator.cpp"), "-o", str(fobj)],
        check=True,
    )

    def one(name: str) -> None:
        target = (libdir if name != "ytref_trace" else pkg) / f"{name}{suffix}"
        cmd = ["g++", *flags, *inc, "-shared", str(GEN / f"{name}.cpp"), str(fobj),
               "-o", str(target), "-lm"]
        subprocess.run(cmd, check=True)

    names = [*MODULES, "ytref_trace"]
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(one, names))


def build(timed: bool = False, jobs: int | None = None) -> Path | None:
    """Build the reference sampler.  Returns the package path, or None when
    neither the reference checkout nor staged generated sources exist."""
    jobs = jobs or min(8, os.cpu_count() or 1)
    if (REF_ROOT / LIB_REL / "image_samplers.pyx").exists():
        _cythonize()
    if not (GEN / "image_samplers.cpp").exists():
        return None
    _compile(OUT / "pkg", fp_contract_off=True, jobs=jobs)
    if timed:
        _compile(OUT / "pkg_timed", fp_contract_off=False, jobs=jobs)
    return OUT / "pkg"


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--timed", action="store_true")
    args = ap.parse_args()
    p = build(timed=args.timed)
    print("built:", p)
    sys.exit(0 if p is not None else 1)
