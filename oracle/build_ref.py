"""Build recipe for the unmodified reference solver (test infrastructure only).

This script compiles the reference's own ``jyulb`` Cython package so that its
FP64 OpenMP solver can serve as the checker and as the timed CPU baseline. It
never copies reference sources into the repository: the ``.pyx``/``.pxd``
files are translated where they lie, and every output goes to ``oracle/_ref/``
(git-ignored):

* ``oracle/_ref/src/*.cpp``  C++ generated by Cython (only where the reference
  sources and Cython are present);
* ``oracle/_ref/jyulb/*.so`` the compiled modules, importable as ``jyulb.*``
  once ``oracle/_ref`` is first on ``sys.path``.

On a machine without the reference tree or without Cython (e.g. an Arm GPU
host), the generated ``.cpp`` files that travelled with the repository are
compiled directly with ``g++``; no Cython is needed for that step.

Build flags follow the reference's own ``setup.py:23-69`` (``-fopenmp -O3``,
C++), with two Cython directives the reference needs under Cython 3:
``language_level=2`` (implicit relative cimports, ``jyulb/isothermal.pyx:133-146``)
and ``legacy_implicit_noexcept=True`` (otherwise every ``nogil`` ``cdef void``
call re-acquires the GIL and the solver is ~1000x slower).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC_OUT = os.path.join(OUT, "src")
PKG_OUT = os.path.join(OUT, "jyulb")
# the reference's jyulb package: JYULB_REFERENCE_PKG, else the jyulb folder of
# JYULB_REFERENCE_ROOT, else of a directory named "reference" beside this
# repository
REF_PKG = os.environ.get("JYULB_REFERENCE_PKG") or os.path.join(
    os.environ.get("JYULB_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"),
    "jyulb")
MODULES = ["defs", "bcs", "D3Q19", "isothermal", "flow_field"]


def _cythonize() -> bool:
    """Translate the reference .pyx files to C++ into oracle/_ref/src."""
    if not os.path.isdir(REF_PKG):
        return False
    try:
        from Cython.Compiler import Main as cymain  # noqa: F401
    except ImportError:
        return False
    os.makedirs(SRC_OUT, exist_ok=True)
    for mod in MODULES:
        pyx = os.path.join(REF_PKG, mod + ".pyx")
        out = os.path.join(SRC_OUT, mod + ".cpp")
        if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(pyx):
            continue
        cmd = [sys.executable, "-m", "cython", "--cplus", "-2",
               "-X", "legacy_implicit_noexcept=True",
               "-I", REF_PKG, "-o", out, pyx]
        subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return True


def _compile_one(mod: str) -> str:
    import numpy as np

    src = os.path.join(SRC_OUT, mod + ".cpp")
    ext = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    dst = os.path.join(PKG_OUT, mod + ext)
    if os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(src):
        return dst
    inc = sysconfig.get_paths()["include"]
    cmd = ["g++", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c++14",
           "-w", "-I", inc, "-I", np.get_include(), src, "-o", dst + ".tmp",
           "-fopenmp"]
    subprocess.run(cmd, check=True)
    os.replace(dst + ".tmp", dst)
    return dst


def build(verbose: bool = False) -> bool:
    """Build the reference modules; returns False when nothing can be built."""
    _cythonize()
    if not all(os.path.exists(os.path.join(SRC_OUT, m + ".cpp")) for m in MODULES):
        if verbose:
            print("reference sources unavailable: oracle/_ref not built")
        return False
    os.makedirs(PKG_OUT, exist_ok=True)
    init = os.path.join(PKG_OUT, "__init__.py")
    if not os.path.exists(init):
        with open(init, "w") as fh:
            fh.write('"""Reference jyulb package compiled from its own sources."""\n')
    with ThreadPoolExecutor(max_workers=len(MODULES)) as ex:
        outs = list(ex.map(_compile_one, MODULES))
    if verbose:
        for o in outs:
            print("built", os.path.relpath(o, HERE))
    return True


def available() -> bool:
    ext = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    return all(os.path.exists(os.path.join(PKG_OUT, m + ext)) for m in MODULES)


def clean() -> None:
    shutil.rmtree(OUT, ignore_errors=True)


if __name__ == "__main__":
    ok = build(verbose=True)
    sys.exit(0 if ok else 1)
