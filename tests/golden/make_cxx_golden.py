"""Generates the golden fixtures of the reference C++ executable's collision
model: small seeded cases run by the executable built from the reference's
own sources (oracle/build_cxx.py), one thread, with every input and output
stored in tests/golden/cxx_<case>.npz.

Run where the reference tree is present:
    python tests/golden/make_cxx_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def script(base, size, dr, dt, rden, kvisc, g, ext, flow, coll, steps, period):
    """Input script in the executable parser's layout (no face lines)."""
    lines = ["# base name", base, "# lattice size", " ".join(map(str, size)), "# dr", repr(dr), "# dt", repr(dt),
             "# reference density", repr(rden), "# kinematic viscosity", repr(kvisc), "# gravity",
             " ".join(repr(v) for v in g), "# external forcing", str(ext), "# flow type", str(flow),
             "# collision operator", str(coll), "# time steps", str(steps), "# evolution info interval",
             str(period), "# execution info", "golden case"]
    return "\n".join(lines) + "\n"


def raw_write(path, arr):
    (arr.transpose(2, 1, 0, 3) if arr.ndim == 4 else arr.transpose(2, 1, 0)).tofile(path)


def raw_read(path, size, comps=0, dtype=np.float64):
    nx, ny, nz = size
    d = np.fromfile(path, dtype=dtype)
    if comps:
        return d.reshape(nz, ny, nx, comps).transpose(2, 1, 0, 3).copy()
    return d.reshape(nz, ny, nx).transpose(2, 1, 0).copy()


def cases():
    rng = np.random.default_rng(4242)
    out = {}
    # tube along z, TRT, laminar, gravity along the tube
    nx, ny, nz = 10, 9, 16
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    geom = np.where((X - 4.5) ** 2 + (Y - 4.0) ** 2 <= 12.0, 255, 0).astype(np.uint8)[:, :, None].repeat(nz, 2)
    out["tube_trt"] = dict(size=(nx, ny, nz), geom=geom, dr=1.0, dt=1.0, rden=1.0, kvisc=0.1, g=(0.0, 0.0, 1e-5),
                           ext=0, flow=1, coll=1, steps=60, period=20)
    # channel with an obstacle, BGK, Stokes flow, non-unit dr, dt, ref_den
    nx, ny, nz = 12, 10, 6
    geom = np.full((nx, ny, nz), 255, np.uint8)
    geom[:, 0, :] = 0
    geom[:, -1, :] = 0
    Xg, Yg, Zg = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    geom[(Xg - 5) ** 2 + (Yg - 5) ** 2 + (Zg - 2.5) ** 2 <= 5.0] = 0
    out["channel_bgk_stokes"] = dict(size=(nx, ny, nz), geom=geom, dr=0.5, dt=0.25, rden=2.0, kvisc=0.05,
                                     g=(2e-5, 0.0, 0.0), ext=0, flow=0, coll=0, steps=50, period=25)
    # periodic box with random solids, TRT, laminar, external forcing and
    # initial density / velocity fields
    nx, ny, nz = 8, 8, 8
    geom = np.where(rng.random((nx, ny, nz)) < 0.15, 0, 255).astype(np.uint8)
    den = 1.5 * (1.0 + 0.01 * rng.standard_normal((nx, ny, nz)))
    vel = 0.01 * rng.standard_normal((nx, ny, nz, 3))
    frc = 1e-5 * rng.standard_normal((nx, ny, nz, 3))
    out["box_trt_forced"] = dict(size=(nx, ny, nz), geom=geom, dr=1.0, dt=1.0, rden=1.5, kvisc=0.08,
                                 g=(0.0, 3e-6, 0.0), ext=1, flow=1, coll=1, steps=40, period=10, den=den, vel=vel,
                                 frc=frc)
    # MRT request with turbulent flow type: the executable falls back to TRT
    nx, ny, nz = 6, 7, 5
    geom = np.where(rng.random((nx, ny, nz)) < 0.1, 0, 255).astype(np.uint8)
    out["box_mrt_fallback"] = dict(size=(nx, ny, nz), geom=geom, dr=1.0, dt=1.0, rden=1.0, kvisc=0.2,
                                   g=(1e-6, -2e-6, 5e-7), ext=0, flow=2, coll=2, steps=30, period=15)
    return out


def main():
    import build_cxx

    exe = build_cxx.build()
    if exe is None:
        raise SystemExit("reference C++ sources not found")
    for name, c in cases().items():
        with tempfile.TemporaryDirectory() as td:
            base = os.path.join(td, "case")
            text = script("case", c["size"], c["dr"], c["dt"], c["rden"], c["kvisc"], c["g"], c["ext"], c["flow"],
                          c["coll"], c["steps"], c["period"])
            open(os.path.join(td, "run.in"), "w").write(text)
            raw_write(base + ".geom.in.raw", c["geom"])
            for key, ext in (("den", ".den.in.raw"), ("vel", ".vel.in.raw"), ("frc", ".force.in.raw")):
                if key in c:
                    raw_write(base + ext, c[key])
            env = dict(os.environ, OMP_NUM_THREADS="1")
            r = subprocess.run([exe, "run.in"], cwd=td, env=env, capture_output=True, text=True, check=True)
            evol = np.loadtxt(base + ".evol", comments="#")
            den_out = raw_read(base + ".den.out.raw", c["size"])
            vel_out = raw_read(base + ".vel.out.raw", c["size"], 3)
        arrays = dict(geom=c["geom"], evol=evol, den_out=den_out, vel_out=vel_out,
                      den_in=c.get("den", np.zeros(0)), vel_in=c.get("vel", np.zeros(0)),
                      frc_in=c.get("frc", np.zeros(0)))
        meta = {k: c[k] for k in ("size", "dr", "dt", "rden", "kvisc", "g", "ext", "flow", "coll", "steps", "period")}
        meta["script"] = text
        meta["stdout_tail"] = r.stdout.splitlines()[-12:]
        np.savez_compressed(os.path.join(HERE, f"cxx_{name}.npz"), meta=json.dumps(meta), **arrays)
        print(name, evol.shape, float(np.abs(vel_out).max()))


if __name__ == "__main__":
    main()
