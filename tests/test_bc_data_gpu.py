"""The reference's readonly bc-data face arrays and its halo semantics.

Solver.bc_data_den_face_* / bc_data_vel_face_* (jyulb/isothermal.pxd:159-171)
are copies of the first / last interior layer of den and vel, halo rows
included, taken at the start of every evolve call for the faces the reference
refreshes (jyulb/isothermal.pyx:476-502, with its Z1 condition at :500).  The
reference refreshes the periodic / symmetric halo layers of den and vel at the
start of every step, so after evolve(n) they hold the images of step n-1's
moments.  The FP64 engine must give all twelve arrays and the whole
halo-padded den / vel bit for bit as the reference does on every golden case
(the fixtures hold the reference's arrays: tests/golden/make_golden.py)."""
import numpy as np
import pytest

from helpers import CASES, load_case, make_engine

pytestmark = pytest.mark.gpu

FACES = ("1X", "X1", "1Y", "Y1", "1Z", "Z1")


def _check(s, c):
    for face in FACES:
        np.testing.assert_array_equal(getattr(s, "bc_data_den_face_" + face), c["bcd_den_" + face], err_msg=face)
        np.testing.assert_array_equal(getattr(s, "bc_data_vel_face_" + face), c["bcd_vel_" + face], err_msg=face)
    np.testing.assert_array_equal(s.den, c["den_full"])
    np.testing.assert_array_equal(s.vel, c["vel_full"])


@pytest.mark.parametrize("name", CASES)
def test_bc_data_and_halos_equal_reference(name):
    c = load_case(name)
    s = make_engine(c, 0)
    s.finalize_init()
    for n in c["chunks"]:
        s.evolve(n)
    _check(s, c)


@pytest.mark.parametrize("name", ["pdiff_sym", "invel_grav", "random_mix_trt", "random_sym_reg"])
def test_bc_data_and_halos_with_kept_f2(name):
    # Solver(keep_f2=True) runs the last step of each call apart; the arrays
    # must not change
    c = load_case(name)
    s = make_engine(c, 0, keep_f2=True)
    s.finalize_init()
    for n in c["chunks"]:
        s.evolve(n)
    _check(s, c)


def test_bc_data_shapes_defaults_and_readonly():
    c = load_case("pdiff_sym")
    s = make_engine(c, 0)
    NI, NJ, NK = s.NI, s.NJ, s.NK
    shapes = {"1X": (NJ, NK), "X1": (NJ, NK), "1Y": (NI, NK), "Y1": (NI, NK), "1Z": (NI, NJ), "Z1": (NI, NJ)}
    for face, sh in shapes.items():
        d, v = getattr(s, "bc_data_den_face_" + face), getattr(s, "bc_data_vel_face_" + face)
        assert d.shape == sh and v.shape == sh + (3,)
        assert (d == 1.0).all() and (v == 0.0).all()  # before the first evolve call
        with pytest.raises(ValueError):
            d[0, 0] = 2.0


def test_bc_data_copied_before_the_finalize_check():
    # the reference copies the bc data before it checks finalize_init
    # (jyulb/isothermal.pyx:1398-1403), so a failed evolve still refreshes it
    c = load_case("pdiff_sym")
    s = make_engine(c, 0)
    with pytest.raises(RuntimeError, match="Finalize solver initialization"):
        s.evolve(3)
    np.testing.assert_array_equal(s.bc_data_den_face_1X, np.asarray(s.den)[1])
    np.testing.assert_array_equal(s.bc_data_vel_face_X1, np.asarray(s.vel)[-2])
    assert (s.bc_data_den_face_1Y == 1.0).all()  # a wall face is never refreshed
