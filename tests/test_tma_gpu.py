"""The bulk-copy staged step kernel (FP32 / FP16 on domains with nz >= 128)
against the direct kernel (JLB_TMA=0) and the FP64 oracle.  Both kernels
run the same arithmetic on the same values, so they must agree bit for bit;
the comparison covers periodic wrap in k, bounce-back in k, Zou-He and
symmetric boundary nodes, odd and even step counts."""
import os

import numpy as np
import pytest

from helpers import run_engine, run_oracle

pytestmark = pytest.mark.gpu


def _case(seed, bc, scheme, porosity=0.97):
    rng = np.random.default_rng(seed)
    sh = (6, 5, 256)
    c = dict(lat=list(sh), scheme=scheme, kvisc=0.05, g=[2e-5, -1e-5, 3e-5], bc=list(bc), chunks=[7, 4])
    c["phase"] = (rng.random(sh) < porosity).astype(np.uint8)
    c["den0"] = 1.0 + 0.005 * rng.standard_normal(sh)
    v = 0.01 * rng.standard_normal(sh + (3,))
    v[c["phase"] == 0] = 0.0
    c["vel0"] = v
    c["acc0"] = None
    return c


BCS = [[1, 1, 1, 1, 1, 1], [0, 0, 0, 0, 0, 0], [1, 1, 0, 0, 3, 2], [4, 0, 1, 1, 1, 1], [2, 3, 0, 4, 1, 1]]


def _run(c, precision, tma):
    old = os.environ.get("JLB_TMA")
    os.environ["JLB_TMA"] = tma if isinstance(tma, str) else ("1" if tma else "0")
    try:
        return run_engine(c, precision=precision)
    finally:
        if old is None:
            del os.environ["JLB_TMA"]
        else:
            os.environ["JLB_TMA"] = old


@pytest.mark.parametrize("mode", ["1", "L"])
@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("scheme", [0, 1, 2])
@pytest.mark.parametrize("bi", range(len(BCS)))
def test_staged_equals_direct(mode, precision, scheme, bi):
    c = _case(10 * bi + scheme, BCS[bi], scheme)
    _, f1, d1, v1 = _run(c, precision, mode)
    _, f0, d0, v0 = _run(c, precision, False)
    fl = c["phase"] != 0
    if precision == 1:
        # FP32: identical arithmetic on identical values
        np.testing.assert_array_equal(f1[:, fl], f0[:, fl])
        np.testing.assert_array_equal(d1[fl], d0[fl])
        np.testing.assert_array_equal(v1[fl], v0[fl])
    else:
        # FP16 storage: the compiler may contract FP32 operations differently
        # in the two kernels, and a last-bit FP32 difference can move an FP16
        # rounding; the bound is a few FP16 steps of the stored deviations
        np.testing.assert_allclose(f1[:, fl], f0[:, fl], rtol=0, atol=2e-5)
        np.testing.assert_allclose(v1[fl], v0[fl], rtol=0, atol=2e-5)


@pytest.mark.parametrize("bi", range(len(BCS)))
def test_staged_fp32_close_to_oracle(bi):
    c = _case(77 + bi, BCS[bi], 1)
    _, f, d, v = _run(c, 1, True)
    _, fo, do, vo = run_oracle(c)
    fl = c["phase"] != 0
    assert np.abs(v[fl] - vo[fl]).max() <= 1e-6
    assert np.abs(f[:, fl] - fo[:, fl]).max() <= 1e-6


@pytest.mark.parametrize("bc", [[1, 1, 0, 0, 1, 1], [0, 0, 0, 3, 0, 0], [1, 1, 4, 2, 1, 1]])
def test_fp16_two_sites_per_thread_local_step(bc):
    # FP16 storage with nz = 256: the staged local step takes sites (k, k+1)
    # per thread; 64 x 48 rows = 3072 tiles, several per persistent block, so
    # both buffers are refilled.  Against the one-site staged kernel
    # (JLB_H2=0) and the direct kernel; boundary-node and solid sites in a
    # pair keep their half
    rng = np.random.default_rng(11)
    sh = (64, 48, 256)
    c = dict(lat=list(sh), scheme=1, kvisc=0.04, g=[1e-5, 0.0, 0.0], bc=list(bc), chunks=[9, 4])
    c["phase"] = (rng.random(sh) < 0.97).astype(np.uint8)
    c["den0"] = np.ones(sh)
    v = 0.01 * rng.standard_normal(sh + (3,))
    v[c["phase"] == 0] = 0.0
    if bc[3] == 3:
        v[:, -1, :, 0] = 0.04
    c["vel0"] = v
    c["acc0"] = None
    fl = c["phase"] != 0
    _, f2, _, v2 = _run(c, 2, "L")
    old = os.environ.get("JLB_H2")
    os.environ["JLB_H2"] = "0"
    try:
        _, f1, _, v1 = _run(c, 2, "L")
    finally:
        if old is None:
            del os.environ["JLB_H2"]
        else:
            os.environ["JLB_H2"] = old
    _, f0, _, v0 = _run(c, 2, False)
    for f, v in ((f1, v1), (f0, v0)):
        np.testing.assert_allclose(f2[:, fl], f[:, fl], rtol=0, atol=2e-5)
        np.testing.assert_allclose(v2[fl], v[fl], rtol=0, atol=2e-5)
