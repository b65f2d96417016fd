"""Solver.f2, the reference's second population buffer.  The reference's
evolve swaps f1 and f2 after every step (jyulb/isothermal.pyx:1410-1416), so
f2 holds the post-collision populations of the step before the latest.  With
keep_f2=True the Solver keeps that copy; its den/vel/f1 stay those of a
Solver without it, bit for bit.  FP64 also against the oracle."""
import numpy as np
import pytest

from helpers import load_case, make_engine, run_oracle

pytestmark = pytest.mark.gpu

# Zou-He faces with gravity (whose results depend on where evolve calls
# split), moving walls, symmetric faces, a per-site acceleration field
NAMES = ["invel_grav", "couette_ladd", "random_sym_reg", "random_mix_trt"]
CALLS = [1, 4, 3]


def _replay(c, precision, calls):
    s = make_engine(c, precision)
    s.finalize_init()
    for n in calls:
        if n:
            s.evolve(n)
    return s.populations()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", NAMES)
def test_f2_holds_the_previous_step(name, precision):
    c = load_case(name)
    a = make_engine(c, precision, keep_f2=True)
    b = make_engine(c, precision)
    a.finalize_init()
    b.finalize_init()
    assert a.f2.shape == (19 * a.NCNT,) and not a.f2.any()
    done = []
    for n in CALLS:
        before = b.populations()
        assert a.evolve(n) == b.evolve(n)
        np.testing.assert_array_equal(a.populations(), b.populations())
        np.testing.assert_array_equal(a.get_den(), b.get_den())
        np.testing.assert_array_equal(a.get_vel(), b.get_vel())
        # the same evolve calls, the last one a step short
        expect = before if n == 1 else _replay(c, precision, done + [n - 1])
        np.testing.assert_array_equal(a.f2, a._bundle_c(expect))
        if precision == 0:
            _, fo, _, _ = run_oracle(c, chunks=[m for m in done + [n - 1] if m] or [0])
            np.testing.assert_array_equal(expect, fo)
        done.append(n)
    np.testing.assert_array_equal(a.f1, b.f1)


def test_f2_needs_keep_f2():
    c = load_case("couette_ladd")
    s = make_engine(c)
    s.finalize_init()
    s.evolve(2)
    with pytest.raises(AttributeError, match="keep_f2=True"):
        s.f2
