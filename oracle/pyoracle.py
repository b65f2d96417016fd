"""ctypes front end of the C oracle (``oracle/lbm_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg, never by the engine.

``Oracle`` mirrors the reference ``jyulb.isothermal.Solver`` surface that the
tests need (construction, NumPy views of the halo-padded fields, the interior
getters, ``finalize_init`` and ``evolve``) and adds ``populations()``, which
returns the post-collision populations as a ``(19, nx, ny, nz)`` array in the
reference's lattice-vector order (``jyulb/D3Q19.pxd:59-79``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "lbm_oracle.c")
LIB = os.path.join(HERE, "_build", "liblbm_oracle.so")

_lib = None


def build() -> str:
    """Compile the oracle with IEEE-faithful flags (no FMA contraction)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp"
        subprocess.run(["gcc", "-O2", "-std=c99", "-ffp-contract=off", "-fno-fast-math",
                        "-fPIC", "-shared", SRC, "-o", tmp], check=True)
        os.replace(tmp, LIB)
    return LIB


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        lib.orc_create.restype = vp
        lib.orc_create.argtypes = [ctypes.c_int] * 4 + [ctypes.c_double, dp, ip, ctypes.c_double]
        lib.orc_destroy.argtypes = [vp]
        for name, rt in (("orc_phase", ctypes.POINTER(ctypes.c_uint8)), ("orc_den", dp),
                         ("orc_vel", dp), ("orc_acc", dp), ("orc_f", dp)):
            getattr(lib, name).restype = rt
            getattr(lib, name).argtypes = [vp]
        lib.orc_finalize.restype = ctypes.c_long
        lib.orc_finalize.argtypes = [vp]
        lib.orc_evolve.restype = ctypes.c_uint
        lib.orc_evolve.argtypes = [vp, ctypes.c_uint]
        lib.orc_set_gravity.argtypes = [vp, dp]
        lib.orc_prm.restype = ctypes.c_double
        lib.orc_prm.argtypes = [vp, ctypes.c_int]
        lib.orc_nfluid.restype = ctypes.c_long
        lib.orc_nfluid.argtypes = [vp]
        _lib = lib
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """FP64 pull-scheme solver with the reference's semantics."""

    def __init__(self, lat_size, rlx_scheme=0, kvisc=1.0 / 6.0, g=None, bc=None,
                 trt_magic=0.0):
        lib = _load()
        nx, ny, nz = (int(v) for v in lat_size[:3])
        self.nx, self.ny, self.nz = nx, ny, nz
        self.NI, self.NJ, self.NK = nx + 2, ny + 2, nz + 2
        g_arr = np.zeros(3) if g is None else np.ascontiguousarray(g, dtype=np.float64)
        bc_arr = np.full(6, 1, dtype=np.int32) if bc is None else np.ascontiguousarray(bc, dtype=np.int32)
        self._h = lib.orc_create(nx, ny, nz, int(rlx_scheme), float(kvisc), _dptr(g_arr),
                                 bc_arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                 float(trt_magic))
        self._lib = lib
        sh = (self.NI, self.NJ, self.NK)
        ncnt = self.NI * self.NJ * self.NK
        self.phase = np.ctypeslib.as_array(lib.orc_phase(self._h), shape=(ncnt,)).reshape(sh)
        self.den = np.ctypeslib.as_array(lib.orc_den(self._h), shape=(ncnt,)).reshape(sh)
        self.vel = np.ctypeslib.as_array(lib.orc_vel(self._h), shape=(3 * ncnt,)).reshape(sh + (3,))
        self.acc = np.ctypeslib.as_array(lib.orc_acc(self._h), shape=(3 * ncnt,)).reshape(sh + (3,))
        self.rlx_prm = (lib.orc_prm(self._h, 0), lib.orc_prm(self._h, 1))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.orc_destroy(h)
            self._h = None

    # interior views, same slicing as jyulb/isothermal.pyx:1465-1511
    def get_phase(self):
        return self.phase[1:-1, 1:-1, 1:-1]

    def get_den(self):
        return self.den[1:-1, 1:-1, 1:-1]

    def get_vel(self):
        return self.vel[1:-1, 1:-1, 1:-1, :]

    def get_acc(self):
        return self.acc[1:-1, 1:-1, 1:-1, :]

    def set_gravity(self, g):
        self._lib.orc_set_gravity(self._h, _dptr(np.ascontiguousarray(g, dtype=np.float64)))

    def finalize_init(self) -> int:
        return int(self._lib.orc_finalize(self._h))

    def evolve(self, n: int) -> int:
        r = self._lib.orc_evolve(self._h, int(n))
        if r == 0xFFFFFFFF:
            raise RuntimeError("finalize_init must be called before evolve")
        return int(r)

    def populations(self) -> np.ndarray:
        """Post-collision populations, (19, nx, ny, nz), interior only."""
        ncnt = self.NI * self.NJ * self.NK
        f = np.ctypeslib.as_array(self._lib.orc_f(self._h), shape=(19 * ncnt,))
        return f.reshape(19, self.NI, self.NJ, self.NK)[:, 1:-1, 1:-1, 1:-1].copy()
