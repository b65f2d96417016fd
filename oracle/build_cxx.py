"""Build recipe for the reference's C++ executable (test infrastructure only).

Compiles ``jyu_lb_isothermal`` from the reference's own sources where they lie
(``source/isothermal/jyu_lb_isothermal.cpp`` and ``include/*/*.cpp``) with
``g++`` directly -- the reference's makefile is not used -- into
``oracle/_ref/jyu_lb_isothermal`` (git-ignored).  Nothing is copied into the
repository.  The executable is the checker for the engine's C++-kernel
physics option and for the input-script front end: ``tests/golden/
make_cxx_golden.py`` runs it on small seeded cases and commits the outputs.

Flags: ``-std=c++14`` (the sources use dynamic exception specifications,
ill-formed from C++17), ``-O2 -fopenmp`` as the reference's makefile, and
``-ffp-contract=off`` so that no compiler on any architecture fuses its
multiply-adds (the engine's FP64 path is built the same way).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
EXE = os.path.join(OUT, "jyu_lb_isothermal")
# the reference checkout: JYULB_REFERENCE_ROOT, else a directory named
# "reference" beside this repository
REF = os.environ.get("JYULB_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
SOURCES = ["source/isothermal/jyu_lb_isothermal.cpp", "include/common/node.cpp", "include/common/filter.cpp",
           "include/collision/collision.cpp", "include/kernel/kernel.cpp", "include/solver/solver.cpp",
           "include/io/input_parser.cpp", "include/io/raw_io.cpp"]
INCLUDES = ["include/common", "include/dvs", "include/collision", "include/kernel", "include/solver", "include/io"]


def available() -> bool:
    return os.path.exists(EXE)


def build(force: bool = False) -> str | None:
    """Builds the executable when the reference tree is present; returns its
    path, or None when it cannot be built here."""
    srcs = [os.path.join(REF, s) for s in SOURCES]
    if not all(os.path.exists(s) for s in srcs):
        return EXE if available() else None
    if available() and not force and all(os.path.getmtime(EXE) >= os.path.getmtime(s) for s in srcs):
        return EXE
    os.makedirs(OUT, exist_ok=True)
    cmd = ["g++", "-std=c++14", "-O2", "-fopenmp", "-ffp-contract=off", "-w"]
    cmd += ["-I" + os.path.join(REF, i) for i in INCLUDES]
    cmd += srcs + ["-o", EXE]
    subprocess.run(cmd, check=True)
    return EXE


if __name__ == "__main__":
    path = build(force="--force" in sys.argv)
    print(path or "reference C++ sources not found")
