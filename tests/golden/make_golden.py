"""Generates the golden fixtures in tests/golden/*.npz by running the
unmodified reference solver (jyulb, built from its own sources into
oracle/_ref by oracle/build_ref.py) on small seeded cases.

Each fixture stores the case description, the exact inputs (interior phase,
den, vel, acc), the evolve-call chunking, and the reference's outputs after the
last call: post-collision populations decoded from Solver.f1's Bundle-C layout
(jyulb/isothermal.pyx:1532-1704) into (19, nx, ny, nz), the interior den
and vel, the full halo-padded den and vel arrays (den_full, vel_full), and
the twelve readonly bc-data face arrays
(bc_data_den_face_* / bc_data_vel_face_*, jyulb/isothermal.pxd:159-171) as
bcd_den_<face> / bcd_vel_<face>.  Run from the repository root:

    python oracle/build_ref.py && python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))

from jyulb.isothermal import Solver  # noqa: E402  (the reference build)

BGK, TRT, REG = 0, 1, 2
FACES = ("1X", "X1", "1Y", "Y1", "1Z", "Z1")
WALL, PER, FD, FV, SYM = 0, 1, 2, 3, 4


def decode_bundle_c(s) -> np.ndarray:
    f = np.asarray(s.f1)
    N = s.NCNT
    out = np.empty((19, N))
    out[0:5] = f[:5 * N].reshape(N, 5).T
    out[5:14] = f[5 * N:14 * N].reshape(N, 9).T
    out[14:19] = f[14 * N:].reshape(N, 5).T
    return out.reshape(19, s.NI, s.NJ, s.NK)[:, 1:-1, 1:-1, 1:-1]


def spheres(shape, radius, porosity, rng):
    nx, ny, nz = shape
    phase = np.ones(shape, dtype=np.uint8)
    X, Y, Z = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    for _ in range(1000):
        if phase.mean() <= porosity:
            break
        c = rng.uniform(0, 1, 3) * np.array(shape)
        d2 = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2
        phase[d2 <= radius * radius] = 0
    return phase


def cases():
    out = []
    # the 4x34x4 gravity channel with solid rows, at 1000 steps
    nx, ny, nz = 4, 34, 4
    ph = np.ones((nx, ny, nz), np.uint8); ph[:, 0, :] = 0; ph[:, -1, :] = 0
    out.append(dict(name="poiseuille_4x34x4", lat=[nx, ny, nz], scheme=BGK, kvisc=(0.8 - 0.5) / 3.0,
                    g=[1e-6, 0, 0], bc=[PER] * 6, phase=ph, den=np.ones(ph.shape),
                    vel=np.zeros(ph.shape + (3,)), acc=None, chunks=[1000]))
    # lid-driven cavity, TRT, Zou-He lid on Y1
    n = 10
    ph = np.ones((n, n, n), np.uint8)
    vel = np.zeros((n, n, n, 3)); vel[:, -1, :, 0] = 0.05
    out.append(dict(name="cavity_trt", lat=[n, n, n], scheme=TRT, kvisc=0.02, g=[0, 0, 0],
                    bc=[WALL, WALL, WALL, FV, WALL, WALL], phase=ph, den=np.ones(ph.shape), vel=vel,
                    acc=None, chunks=[100, 100]))
    # porous channel, regularized, spheres, periodic x/z, walls in y
    rng = np.random.default_rng(7)
    sh = (12, 10, 10)
    ph = spheres(sh, 2.5, 0.6, rng)
    out.append(dict(name="porous_reg", lat=list(sh), scheme=REG, kvisc=(0.7 - 0.5) / 3.0,
                    g=[5e-6, 0, 0], bc=[PER, PER, WALL, WALL, PER, PER], phase=ph,
                    den=np.ones(sh), vel=np.zeros(sh + (3,)), acc=None, chunks=[150]))
    # pressure-driven channel: Zou-He density in/out, symmetric + wall in y
    sh = (10, 6, 4)
    ph = np.ones(sh, np.uint8)
    den = np.ones(sh); den[0] = 1.01; den[-1] = 0.99
    out.append(dict(name="pdiff_sym", lat=list(sh), scheme=BGK, kvisc=0.1, g=[0, 0, 0],
                    bc=[FD, FD, WALL, SYM, PER, PER], phase=ph, den=den, vel=np.zeros(sh + (3,)),
                    acc=None, chunks=[50, 50]))
    # Couette: moving solid plates (Ladd) inside a periodic box
    sh = (12, 5, 4)
    ph = np.ones(sh, np.uint8); ph[0] = 0; ph[-1] = 0
    vel = np.zeros(sh + (3,)); vel[-1, :, :, 1] = 1e-3; vel[-1, :, :, 2] = 2e-3; vel[0, :, :, 1] = -5e-4
    out.append(dict(name="couette_ladd", lat=list(sh), scheme=BGK, kvisc=0.5 / 6.0, g=[0, 0, 0],
                    bc=[PER] * 6, phase=ph, den=np.ones(sh), vel=vel, acc=None, chunks=[300]))
    # random everything: obstacles, moving solids, acceleration field,
    # Zou-He velocity/density on x, symmetric and wall in y, periodic z
    rng = np.random.default_rng(11)
    sh = (7, 6, 5)
    ph = (rng.random(sh) > 0.25).astype(np.uint8)
    den = 1.0 + 0.01 * rng.standard_normal(sh)
    vel = 0.02 * rng.standard_normal(sh + (3,))
    acc = 1e-4 * rng.standard_normal(sh + (3,))
    out.append(dict(name="random_mix_trt", lat=list(sh), scheme=TRT, kvisc=0.05,
                    g=[1e-5, -2e-5, 3e-6], bc=[FV, FD, SYM, WALL, PER, PER], phase=ph, den=den,
                    vel=vel, acc=acc, chunks=[7, 13]))
    # symmetric faces on every axis plus moving solids, regularized
    rng = np.random.default_rng(12)
    sh = (6, 7, 5)
    ph = (rng.random(sh) > 0.2).astype(np.uint8)
    out.append(dict(name="random_sym_reg", lat=list(sh), scheme=REG, kvisc=0.04, g=[0, 1e-5, 0],
                    bc=[SYM, SYM, SYM, WALL, SYM, SYM], phase=ph,
                    den=1.0 + 0.01 * rng.standard_normal(sh), vel=0.02 * rng.standard_normal(sh + (3,)),
                    acc=None, chunks=[5, 6]))
    # the reference's Z1 bc-data condition: a lone Z1 FIXED_VEL face keeps den=1, vel=0
    sh = (5, 5, 6)
    ph = np.ones(sh, np.uint8)
    vel = np.zeros(sh + (3,)); vel[:, :, -1, 0] = 0.04
    out.append(dict(name="z1_fixed_vel", lat=list(sh), scheme=BGK, kvisc=0.05, g=[0, 0, 0],
                    bc=[PER, PER, PER, PER, WALL, FV], phase=ph, den=np.ones(sh), vel=vel, acc=None,
                    chunks=[20, 20]))
    # gravity + Zou-He velocity inlet / density outlet (acc/2 carried into bc data)
    sh = (8, 6, 3)
    ph = np.ones(sh, np.uint8)
    vel = np.zeros(sh + (3,)); vel[0, :, :, 0] = 0.01
    out.append(dict(name="invel_grav", lat=list(sh), scheme=TRT, kvisc=0.08, g=[2e-5, 0, 0],
                    bc=[FV, FD, WALL, WALL, PER, PER], phase=ph, den=np.ones(sh), vel=vel, acc=None,
                    chunks=[10, 10, 10]))
    # degenerate shapes: one site periodic on every axis (each link wraps
    # onto the site itself)
    rng = np.random.default_rng(21)
    sh = (1, 1, 1)
    out.append(dict(name="edge_single_site", lat=list(sh), scheme=TRT, kvisc=0.07,
                    g=[3e-5, -1e-5, 2e-5], bc=[PER] * 6, phase=np.ones(sh, np.uint8),
                    den=np.full(sh, 1.02), vel=0.01 * rng.standard_normal(sh + (3,)), acc=None,
                    chunks=[3, 4]))
    # a single column along z (nz > 128, not a multiple of 32): symmetric x,
    # periodic y, wall below, Zou-He density on top
    sh = (1, 1, 129)
    den = np.ones(sh); den[:, :, -1] = 0.995
    out.append(dict(name="edge_column_sym", lat=list(sh), scheme=REG, kvisc=0.05, g=[0, 0, -1e-5],
                    bc=[SYM, SYM, PER, PER, WALL, FD], phase=np.ones(sh, np.uint8), den=den,
                    vel=0.005 * rng.standard_normal(sh + (3,)), acc=None, chunks=[9, 8]))
    # a flat sheet (nz = 1): Zou-He velocity / density on the y faces of a
    # 2 x 3 x 1 lattice, periodic x and z
    sh = (2, 3, 1)
    vel = np.zeros(sh + (3,)); vel[:, 0, :, 1] = 0.02
    out.append(dict(name="edge_sheet_zou_he", lat=list(sh), scheme=BGK, kvisc=0.1, g=[1e-5, 0, 0],
                    bc=[PER, PER, FV, FD, PER, PER], phase=np.ones(sh, np.uint8), den=np.ones(sh),
                    vel=vel, acc=None, chunks=[5, 6]))
    # one fluid site enclosed by solids, two of which move (Ladd) with a
    # velocity component along their link to the site
    sh = (3, 3, 3)
    ph = np.zeros(sh, np.uint8); ph[1, 1, 1] = 1
    vel = np.zeros(sh + (3,)); vel[1, 2, 1] = [0.01, 0.01, -0.005]; vel[2, 1, 0] = [0.01, 0.02, -0.01]
    out.append(dict(name="edge_enclosed_site", lat=list(sh), scheme=TRT, kvisc=0.03, g=[0, 0, 0],
                    bc=[WALL] * 6, phase=ph, den=np.ones(sh), vel=vel, acc=None, chunks=[6, 7]))
    return out


def large_cases():
    """1000-step cases on lattices where the engine's size-dependent paths run
    (consecutive-site blocks for nz not a multiple of 32; whole 128-site rows
    for the bulk-copy staged step; boundary-node tables over many blocks).
    Their arrays are stored as SHA-256 digests of the float64 bytes (C
    order, little endian; f, den and vel over the fluid sites only) plus a
    strided sample, not in full."""
    out = []
    # TRT cavity with the reference's fixed magic 3/16, Zou-He lid on Y1,
    # nz = 42
    sh = (40, 48, 42)
    ph = np.ones(sh, np.uint8)
    vel = np.zeros(sh + (3,)); vel[:, -1, :, 0] = 0.05
    out.append(dict(name="large_cavity_trt", lat=list(sh), scheme=TRT, kvisc=0.02, g=[0, 0, 0],
                    bc=[WALL, WALL, WALL, FV, WALL, WALL], phase=ph, den=np.ones(sh), vel=vel, acc=None,
                    chunks=[1000]))
    # regularized channel through seeded spheres (90% fluid), gravity along
    # x, periodic x/z, wall below and symmetric face on top, nz = 128
    rng = np.random.default_rng(31)
    sh = (64, 32, 128)
    ph = spheres(sh, 4.0, 0.9, rng)
    out.append(dict(name="large_channel_reg", lat=list(sh), scheme=REG, kvisc=(0.7 - 0.5) / 3.0,
                    g=[5e-6, 0, 0], bc=[PER, PER, WALL, SYM, PER, PER], phase=ph, den=np.ones(sh),
                    vel=np.zeros(sh + (3,)), acc=None, chunks=[600, 400]))
    # BGK channel with a Zou-He velocity inlet (profile) on 1X and density
    # outlet on X1, a solid lid row moving tangentially across both faces
    # (the corner sites have Zou-He and moving-wall links), seeded obstacles,
    # a symmetric face on 1Z and a wall on Z1; nz = 36, two evolve calls
    rng = np.random.default_rng(47)
    sh = (48, 40, 36)
    ph = spheres(sh, 3.0, 0.96, rng)
    ph[:4] = 1
    ph[-4:] = 1
    ph[:, -1, :] = 0
    vel = np.zeros(sh + (3,))
    vel[:, -1, :, 0] = 0.03
    vel[:, -1, :, 2] = 0.01
    y = (np.arange(sh[1]) + 0.5) / (sh[1] - 1)
    prof = np.clip(4.0 * y * (1.0 - y), 0.0, None)
    vel[0, :-1, :, 0] = 0.02 * prof[:-1, None]
    den = np.ones(sh)
    den[-1] = 0.998
    out.append(dict(name="large_lid_inlet_bgk", lat=list(sh), scheme=BGK, kvisc=0.04, g=[0, 0, 0],
                    bc=[FV, FD, WALL, WALL, SYM, WALL], phase=ph, den=den, vel=vel, acc=None,
                    chunks=[700, 300]))
    # TRT (magic 3/16) flow along z: Zou-He velocity inlet with a profile on
    # 1Z (Z1 is then read too), density outlet on Z1, periodic x, walls in y,
    # seeded obstacles, a small body force along z; nz = 64, two evolve calls
    rng = np.random.default_rng(53)
    sh = (32, 28, 64)
    ph = spheres(sh, 2.5, 0.97, rng)
    ph[:, :, :4] = 1
    ph[:, :, -4:] = 1
    vel = np.zeros(sh + (3,))
    y = (np.arange(sh[1]) + 0.5) / sh[1]
    vel[:, :, 0, 2] = 0.03 * (4.0 * y * (1.0 - y))[None, :]
    vel[:, :, 0, 0] = 0.002 * np.sin(2 * np.pi * np.arange(sh[0]) / sh[0])[:, None]
    den = np.ones(sh)
    den[:, :, -1] = 1.001
    out.append(dict(name="large_zflow_trt", lat=list(sh), scheme=TRT, kvisc=0.03, g=[0, 0, 2e-7],
                    bc=[PER, PER, WALL, WALL, FV, FD], phase=ph, den=den, vel=vel, acc=None,
                    chunks=[500, 500]))
    return out


def digest(a) -> str:
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


SAMPLE_STRIDE = 97  # every 97th value of the flattened arrays goes into the sample


def run(case):
    s = Solver(np.array(case["lat"], dtype=np.int32), case["scheme"], case["kvisc"],
               np.array(case["g"], dtype=np.float64), np.array(case["bc"], dtype=np.int32))
    s.get_phase()[:] = case["phase"]
    s.get_den()[:] = case["den"]
    s.get_vel()[:] = case["vel"]
    if case["acc"] is not None:
        s.get_acc()[:] = case["acc"]
    nf = s.finalize_init()
    for c in case["chunks"]:
        s.evolve(c)
    bcd = {"den_full": np.array(s.den), "vel_full": np.array(s.vel)}
    for face in FACES:
        bcd["bcd_den_" + face] = np.array(getattr(s, "bc_data_den_face_" + face))
        bcd["bcd_vel_" + face] = np.array(getattr(s, "bc_data_vel_face_" + face))
    return nf, decode_bundle_c(s), np.array(s.get_den()), np.array(s.get_vel()), bcd


def main(names=None):
    for case in cases() + large_cases():
        if names and case["name"] not in names:
            continue
        nf, f, den, vel, bcd = run(case)
        meta = {k: case[k] for k in ("name", "lat", "scheme", "kvisc", "g", "bc", "chunks")}
        meta["nfluid"] = int(nf)
        path = os.path.join(HERE, case["name"] + ".npz")
        acc = case["acc"] if case["acc"] is not None else np.zeros(0)
        arrays = dict(f=f, den=den, vel=vel, **bcd)
        if case["name"].startswith("large_"):
            # f, den and vel over the fluid sites (what the solver defines),
            # the halo-padded arrays and bc data whole
            fl = case["phase"] != 0
            arrays.update(f=f[:, fl], den=den[fl], vel=vel[fl])
            meta["sha256"] = {k: digest(a) for k, a in arrays.items()}
            meta["sample_stride"] = SAMPLE_STRIDE
            arrays = {k + "_sample": np.ascontiguousarray(a).reshape(-1)[::SAMPLE_STRIDE]
                      for k, a in (("f", f), ("den", den), ("vel", vel))}
        np.savez_compressed(path, meta=json.dumps(meta), phase=case["phase"], den0=case["den"],
                            vel0=case["vel"], acc0=acc, **arrays)
        print(f"{case['name']:18s} fluid={nf:5d} -> {os.path.relpath(path, ROOT)} "
              f"({os.path.getsize(path) // 1024} KB)")


if __name__ == "__main__":
    # optional case names: write only those fixtures
    main(sys.argv[1:])
