"""Shared helpers for the parity tests: golden fixtures, oracle runs and
engine runs of the same case."""
from __future__ import annotations

import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["poiseuille_4x34x4", "cavity_trt", "porous_reg", "pdiff_sym", "couette_ladd",
         "random_mix_trt", "random_sym_reg", "z1_fixed_vel", "invel_grav",
         "edge_single_site", "edge_column_sym", "edge_sheet_zou_he", "edge_enclosed_site"]


# 1000-step cases on larger lattices: the fixtures hold SHA-256 digests of the
# reference's arrays (f, den, vel over the fluid sites) instead of the arrays
LARGE_CASES = ["large_cavity_trt", "large_channel_reg", "large_lid_inlet_bgk", "large_zflow_trt"]


def digest(a) -> str:
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def load_case(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    c = json.loads(str(z["meta"]))
    c.update(phase=z["phase"], den0=z["den0"], vel0=z["vel0"],
             acc0=z["acc0"] if z["acc0"].size else None)
    if "sha256" not in c:
        c.update(f=z["f"], den=z["den"], vel=z["vel"])
    # the reference's full halo-padded den / vel and its twelve bc-data face
    # arrays after the last evolve call
    for k in z.files:
        if k in ("den_full", "vel_full") or k.startswith("bcd_"):
            c[k] = z[k]
    return c


def _setup(obj, c):
    obj.get_phase()[:] = c["phase"]
    obj.get_den()[:] = c["den0"]
    obj.get_vel()[:] = c["vel0"]
    if c["acc0"] is not None:
        obj.get_acc()[:] = c["acc0"]


def run_oracle(c, chunks=None):
    from pyoracle import Oracle

    o = Oracle(c["lat"], c["scheme"], c["kvisc"], c["g"], c["bc"], c.get("trt_magic", 0.0) or 0.0)
    _setup(o, c)
    nf = o.finalize_init()
    for n in (chunks or c["chunks"]):
        o.evolve(n)
    return nf, o.populations(), o.get_den().copy(), o.get_vel().copy()


def make_engine(c, precision=0, **extra):
    from jyulb.isothermal import Solver

    kw = {"precision": precision, **extra}
    if c.get("trt_magic"):
        kw["trt_magic"] = c["trt_magic"]
    s = Solver(np.array(c["lat"], dtype=np.int32), c["scheme"], c["kvisc"],
               np.array(c["g"], dtype=np.float64), np.array(c["bc"], dtype=np.int32), **kw)
    _setup(s, c)
    return s


def run_engine(c, precision=0, chunks=None):
    s = make_engine(c, precision)
    nf = s.finalize_init()
    for n in (chunks or c["chunks"]):
        s.evolve(n)
    return nf, s.populations(), np.array(s.get_den()), np.array(s.get_vel())


def rel_err(a, b):
    """max |a-b| / max |b|"""
    a = np.asarray(a)
    b = np.asarray(b)
    d = np.abs(a - b).max() if a.size else 0.0
    s = np.abs(b).max() if b.size else 0.0
    return d / s if s > 0 else d
