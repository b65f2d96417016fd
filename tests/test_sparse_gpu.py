"""The fluid-only population layout (used for FP32 / FP16 storage when
fewer than 80% of the sites are fluid; JLB_SPARSE=1 forces it) against the
lattice layout (JLB_SPARSE=0).  Both run the same arithmetic on the same
values, so FP32 must agree bit for bit; the cases cover porous geometry,
bounce-back, Zou-He and symmetric faces, moving solids, acceleration
fields, chunked evolve calls and a population save / restore in between."""
import os

import numpy as np
import pytest

from helpers import CASES, load_case, make_engine, run_engine

pytestmark = pytest.mark.gpu


class _env:
    def __init__(self, **kv):
        self.kv = kv

    def __enter__(self):
        self.saved = {k: os.environ.get(k) for k in self.kv}
        os.environ.update(self.kv)

    def __exit__(self, *exc):
        for k, v in self.saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _run(c, precision, sparse):
    with _env(JLB_SPARSE="1" if sparse else "0", JLB_TMA="0"):
        return run_engine(c, precision=precision)


def _check(c, precision):
    _, f1, d1, v1 = _run(c, precision, True)
    _, f0, d0, v0 = _run(c, precision, False)
    fl = c["phase"] != 0
    if precision == 1:
        np.testing.assert_array_equal(f1[:, fl], f0[:, fl])
        np.testing.assert_array_equal(d1[fl], d0[fl])
        np.testing.assert_array_equal(v1[fl], v0[fl])
    else:
        np.testing.assert_allclose(f1[:, fl], f0[:, fl], rtol=0, atol=2e-5)
        np.testing.assert_allclose(v1[fl], v0[fl], rtol=0, atol=2e-5)


@pytest.mark.parametrize("name", CASES)
def test_sparse_equals_lattice_golden(name):
    _check(load_case(name), 1)


def _porous(seed, shape, bc, scheme, porosity=0.6):
    rng = np.random.default_rng(seed)
    c = dict(lat=list(shape), scheme=scheme, kvisc=0.05, g=[2e-5, -1e-5, 3e-5], bc=list(bc), chunks=[5, 4, 1])
    c["phase"] = (rng.random(shape) < porosity).astype(np.uint8)
    c["den0"] = 1.0 + 0.005 * rng.standard_normal(shape)
    v = 0.01 * rng.standard_normal(shape + (3,))
    v[c["phase"] == 0] = 0.0
    c["vel0"] = v
    acc = 1e-5 * rng.standard_normal(shape + (3,)) if seed % 2 else None
    c["acc0"] = acc
    return c


SHAPES = [(6, 5, 20), (5, 7, 131)]
BCS = [[1, 1, 1, 1, 1, 1], [0, 0, 1, 1, 0, 0], [1, 1, 0, 0, 3, 2], [4, 0, 1, 1, 1, 1]]


@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("si", range(len(SHAPES)))
@pytest.mark.parametrize("bi", range(len(BCS)))
def test_sparse_equals_lattice_porous(precision, si, bi):
    _check(_porous(10 * si + bi, SHAPES[si], BCS[bi], (si + bi) % 3), precision)


def test_sparse_save_restore_continues():
    c = _porous(5, (6, 6, 24), [1, 1, 1, 1, 1, 1], 1)
    with _env(JLB_SPARSE="1", JLB_TMA="0"):
        s = make_engine(c, precision=1)
        s.finalize_init()
        s.evolve(7)
        state = s.populations()
        s.evolve(5)
        a = s.populations()
        s.set_populations(state)
        s.evolve(5)
        b = s.populations()
    fl = c["phase"] != 0
    np.testing.assert_array_equal(a[:, fl], b[:, fl])
