"""The three ways evolve returns den/vel to the page-locked host arrays give
identical results: the last step run in slabs with each slab's download
overlapped (default when every interior site is fluid), the copy-engine
download after the whole step (JLB_OVERLAP_DOWNLOAD=0) and the kernel that
stores into host memory (JLB_DMA_DOWNLOAD=0).  Lattices with several slabs,
uneven slab sizes, Zou-He faces and both step parities; FP64 also against
the oracle."""
import numpy as np
import pytest

from helpers import make_engine, run_oracle

pytestmark = pytest.mark.gpu


def _case(shape, bc, scheme, seed):
    rng = np.random.default_rng(seed)
    c = dict(lat=list(shape), scheme=scheme, kvisc=0.04, g=[1e-5, 0.0, -2e-6], bc=list(bc), chunks=[5, 1, 4])
    c["phase"] = np.ones(shape, np.uint8)
    c["den0"] = 1.0 + 0.005 * rng.standard_normal(shape)
    v = 0.01 * rng.standard_normal(shape + (3,))
    c["vel0"] = v
    c["acc0"] = None
    return c


def _run(c, precision, monkeypatch, overlap, dma):
    monkeypatch.setenv("JLB_OVERLAP_DOWNLOAD", "1" if overlap else "0")
    monkeypatch.setenv("JLB_DMA_DOWNLOAD", "1" if dma else "0")
    s = make_engine(c, precision)
    s.finalize_init()
    out = []
    for n in c["chunks"]:
        s.evolve(n)
        out.append((np.array(s.get_den()), np.array(s.get_vel())))
    return s.populations(), out


# (nz = 32: 4 rows per block, ny a multiple of 4) and (nz = 128: 1 row per
# block); nx gives 8 uneven slabs
CASES = [((16, 8, 32), [0, 0, 0, 3, 0, 0]), ((37, 3, 128), [3, 2, 1, 1, 0, 0]), ((9, 12, 32), [1, 1, 4, 3, 1, 1])]


@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("ci", range(len(CASES)))
def test_download_paths_agree(ci, precision, monkeypatch):
    shape, bc = CASES[ci]
    c = _case(shape, bc, 1, 40 + ci)
    if bc[3] == 3:
        c["vel0"][:, -1, :, :] = [0.03, 0.0, 0.0]
    f0, out0 = _run(c, precision, monkeypatch, True, True)
    for overlap, dma in ((False, True), (False, False)):
        f1, out1 = _run(c, precision, monkeypatch, overlap, dma)
        np.testing.assert_array_equal(f1, f0)
        for (d0, v0), (d1, v1) in zip(out0, out1):
            np.testing.assert_array_equal(d1, d0)
            np.testing.assert_array_equal(v1, v0)
    if precision == 0:
        _, fo, do, vo = run_oracle(c)
        np.testing.assert_array_equal(f0, fo)
        np.testing.assert_array_equal(out0[-1][0], do)
        np.testing.assert_array_equal(out0[-1][1], vo)
