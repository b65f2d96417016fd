"""The C oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the built reference).  The oracle follows the
reference's operation order and is compiled without FMA contraction, so the
match is exact."""
import numpy as np
import pytest

from helpers import CASES, load_case, run_oracle


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_bitwise(name):
    c = load_case(name)
    nf, f, den, vel = run_oracle(c)
    assert nf == c["nfluid"]
    fl = c["phase"] != 0
    np.testing.assert_array_equal(f[:, fl], c["f"][:, fl])
    np.testing.assert_array_equal(den[fl], c["den"][fl])
    np.testing.assert_array_equal(vel[fl], c["vel"][fl])


def test_oracle_conserves_mass_periodic():
    c = load_case("c1_poiseuille")
    nf, f, den, vel = run_oracle(c, chunks=[200])
    fl = c["phase"] != 0
    assert abs(den[fl].sum() - nf) < 1e-10


def test_z1_quirk_is_in_the_fixture():
    # a lone Z1 FIXED_VEL face gets den=1, vel=0 as bc data (reference quirk),
    # so the lid layer does not move at the prescribed 0.04
    c = load_case("z1_fixed_vel")
    assert abs(c["vel"][:, :, -1, 0]).max() < 1e-3


def test_oracle_steady_profiles_match_reference():
    # the steady channel flows of the reference's example scripts: the oracle
    # reproduces the reference's mid-domain profiles bit for bit
    import json
    import os

    from pyoracle import Oracle

    import profile_cases as pc
    from jyulb import flow_field

    gold = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "profiles.json")))
    for c in pc.cases():
        o = Oracle(c["lat"], c["scheme"], c["kvisc"], list(pc.gravity(c)), c["bc"])
        pc.setup(o, c, flow_field)
        assert o.finalize_init() == gold[c["name"]]["nfluid"]
        for n in c["chunks"]:
            o.evolve(n)
        prof = pc.profile(o.get_vel(), c)
        ref = np.array([[float.fromhex(v) for v in row] for row in gold[c["name"]]["profile"]])
        np.testing.assert_array_equal(prof, ref, err_msg=c["name"])
        assert pc.error(prof, c, flow_field) == float.fromhex(gold[c["name"]]["error"])
