"""Steady channel flows against their analytic profiles, as the reference's
example scripts measure them (tests/profile_cases.py): the FP64 engine
reproduces the reference's mid-domain profile bit for bit, and with it the
reference's relative L2 error against the analytic steady state.  FP32
storage stays within 1e-4 (of the peak speed) of that profile; measured
1e-6 .. 5e-5, the largest on the pressure-driven half channel, whose slow
diffusive modes integrate rounding over the 10 000 steps.  Its error against
the analytic profile is therefore the reference's to within 5e-5."""
import json
import os

import numpy as np
import pytest

import profile_cases as pc

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "profiles.json")))
NAMES = [c["name"] for c in pc.cases()]


def _run(c, precision):
    from jyulb import flow_field
    from jyulb.isothermal import Solver

    s = Solver(np.array(c["lat"], dtype=np.int32), c["scheme"], c["kvisc"], pc.gravity(c),
               np.array(c["bc"], dtype=np.int32), precision=precision)
    pc.setup(s, c, flow_field)
    nf = s.finalize_init()
    for n in c["chunks"]:
        s.evolve(n)
    prof = pc.profile(np.asarray(s.get_vel()), c)
    return nf, prof, pc.error(prof, c, flow_field)


@pytest.mark.parametrize("name", NAMES)
def test_fp64_profile_and_error_equal_reference(name):
    c = next(c for c in pc.cases() if c["name"] == name)
    g = GOLD[name]
    nf, prof, err = _run(c, 0)
    assert nf == g["nfluid"]
    ref = np.array([[float.fromhex(v) for v in row] for row in g["profile"]])
    np.testing.assert_array_equal(prof, ref)
    assert err == float.fromhex(g["error"])


@pytest.mark.parametrize("name", NAMES)
def test_fp32_profile_close_to_reference(name):
    c = next(c for c in pc.cases() if c["name"] == name)
    _, prof, err = _run(c, 1)
    ref = np.array([[float.fromhex(v) for v in row] for row in GOLD[name]["profile"]])
    assert np.abs(prof - ref).max() <= 1e-4 * np.abs(ref).max()
    assert abs(err - float.fromhex(GOLD[name]["error"])) <= 5e-5, err
