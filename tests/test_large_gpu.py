"""FP64 parity at 1000 steps on lattices where the engine's size-dependent
paths run, against SHA-256 digests of the reference's own arrays
(tests/golden/make_golden.py, large_cases):

* large_cavity_trt, 40x48x42 TRT cavity (magic 3/16) with a Zou-He lid on
  Y1: nz = 42 is not a multiple of 32, so the dense sweep takes blocks of
  128 consecutive sites with (i, j, k) from multiply-shift division;
* large_channel_reg, 64x32x128 regularized channel through spheres (90%
  fluid), gravity, a symmetric face on Y1 (8192 boundary nodes, 64 blocks of
  the boundary-node path): nz = 128 and mostly fluid, so FP32 runs the
  bulk-copy staged local step;
* large_lid_inlet_bgk, 48x40x36 BGK channel with a Zou-He velocity inlet
  (profile) and density outlet, a solid lid row moving tangentially across
  both faces (corner sites with Zou-He and moving-wall links), seeded
  obstacles, symmetric 1Z and wall Z1, two evolve calls: nz = 36 again takes
  the consecutive-site blocks;
* large_zflow_trt, 32x28x64 TRT flow along z from a Zou-He velocity profile
  on 1Z to a density outlet on Z1, through obstacles, periodic x, walls in y,
  two evolve calls: the z faces' Zou-He at size.

The FP64 engine must reproduce the reference's populations, den, vel, the
whole halo-padded den / vel and the twelve bc-data face arrays bit for bit;
FP32 storage must stay within 1e-5 (relative L2 of the velocity) of it."""
import numpy as np
import pytest

from helpers import LARGE_CASES, digest, load_case, make_engine

pytestmark = pytest.mark.gpu

FACES = ("1X", "X1", "1Y", "Y1", "1Z", "Z1")


def _run(c, precision):
    s = make_engine(c, precision)
    nf = s.finalize_init()
    for n in c["chunks"]:
        s.evolve(n)
    return s, nf


@pytest.mark.parametrize("name", LARGE_CASES)
def test_fp64_digests_equal_reference_at_1000_steps(name):
    c = load_case(name)
    s, nf = _run(c, 0)
    assert nf == c["nfluid"]
    fl = c["phase"] != 0
    h = c["sha256"]
    assert digest(s.populations()[:, fl]) == h["f"]
    assert digest(np.asarray(s.get_den())[fl]) == h["den"]
    assert digest(np.asarray(s.get_vel())[fl]) == h["vel"]
    assert digest(s.den) == h["den_full"]
    assert digest(s.vel) == h["vel_full"]
    for face in FACES:
        assert digest(getattr(s, "bc_data_den_face_" + face)) == h["bcd_den_" + face], face
        assert digest(getattr(s, "bc_data_vel_face_" + face)) == h["bcd_vel_" + face], face


@pytest.mark.parametrize("name", LARGE_CASES)
def test_fp32_velocity_within_1e5_of_fp64_at_1000_steps(name):
    c = load_case(name)
    fl = c["phase"] != 0
    s64, _ = _run(c, 0)
    v64 = np.asarray(s64.get_vel())[fl].copy()
    del s64
    s32, _ = _run(c, 1)
    v32 = np.asarray(s32.get_vel())[fl]
    err = np.linalg.norm(v32 - v64) / np.linalg.norm(v64)
    assert err <= 1e-5, err
