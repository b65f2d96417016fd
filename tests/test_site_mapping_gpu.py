"""The dense sweep's two site mappings give identical results.  Where row
blocks along k would leave lanes idle (nz not a multiple of 32, or above 128
and not a multiple of 128), a block takes 128 consecutive sites (the
default); JLB_LIN=0 keeps the k-lines of rows that other lattices use.
Lattices with Zou-He, symmetric and periodic faces, solids and moving walls,
in all three storage types; FP64 also against the oracle."""
import numpy as np
import pytest

from helpers import make_engine, run_oracle

pytestmark = pytest.mark.gpu

# (shape, bc, solid fraction)
CASES = [((9, 7, 5), [0, 0, 0, 3, 0, 0], 0.0), ((6, 11, 3), [1, 1, 4, 4, 1, 1], 0.2),
         ((7, 5, 45), [3, 2, 0, 0, 1, 1], 0.1), ((5, 4, 100), [1, 1, 1, 1, 4, 4], 0.15),
         ((4, 34, 4), [1, 1, 0, 0, 1, 1], 0.0),
         # above 128 and not a multiple of 128: row blocks of 128 along k
         # would leave lanes idle in the second block of each row
         ((3, 5, 160), [0, 0, 0, 3, 0, 0], 0.0), ((2, 3, 200), [1, 1, 1, 1, 0, 0], 0.1)]


def _case(shape, bc, solid, seed):
    rng = np.random.default_rng(seed)
    c = dict(lat=list(shape), scheme=int(seed % 3), kvisc=0.05, g=[2e-5, -1e-5, 3e-6], bc=list(bc),
             chunks=[3, 1, 4])
    phase = (rng.random(shape) >= solid).astype(np.uint8)
    c["phase"] = phase
    c["den0"] = 1.0 + 0.004 * rng.standard_normal(shape)
    v = 0.01 * rng.standard_normal(shape + (3,))
    v[phase == 0] = 0.02 * rng.standard_normal((int((phase == 0).sum()), 3))  # moving solids
    if bc[3] == 3:
        v[:, -1, :, :] = [0.03, 0.0, 0.01]
    if bc[0] == 3:
        v[0, :, :, :] = [0.02, 0.0, 0.0]
    c["vel0"] = v
    c["acc0"] = None
    return c


def _run(c, precision):
    s = make_engine(c, precision)
    s.finalize_init()
    out = []
    for n in c["chunks"]:
        s.evolve(n)
        out.append((np.array(s.get_den()), np.array(s.get_vel())))
    return s.populations(), out


@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("ci", range(len(CASES)))
def test_linear_and_row_mappings_agree(ci, precision, monkeypatch):
    shape, bc, solid = CASES[ci]
    c = _case(shape, bc, solid, 70 + ci)
    monkeypatch.delenv("JLB_LIN", raising=False)
    f0, out0 = _run(c, precision)
    monkeypatch.setenv("JLB_LIN", "0")
    f1, out1 = _run(c, precision)
    np.testing.assert_array_equal(f1, f0)
    for (d0, v0), (d1, v1) in zip(out0, out1):
        np.testing.assert_array_equal(d1, d0)
        np.testing.assert_array_equal(v1, v0)
    if precision == 0:
        _, fo, do, vo = run_oracle(c)
        np.testing.assert_array_equal(f0, fo)
        np.testing.assert_array_equal(out0[-1][0], do)
        np.testing.assert_array_equal(out0[-1][1], vo)
