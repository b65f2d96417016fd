"""GPU test of jlb_reduce_moments_noalloc, the allocation-free variant of the
moment reduction.

It exists for callers that cannot call cudaMalloc, such as code running under
another framework's memory pool or a host that forbids allocation after
start-up.  Its scratch is a static device array shared by all calls.  The
test feeds it the same moments the solver's own jlb_reduce sums (rebuilt as
caller-owned torch tensors) and compares the two results on two calls in a
row, so the second call runs over scratch the first one left behind.  This
file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from helpers import load_case, make_engine

pytestmark = pytest.mark.gpu

TOL = 1e-12  # same relative bound as the FP64 parity tests


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_noalloc_reduce_matches_jlb_reduce(precision):
    import torch

    from jyulb import _native

    lib = _native.load()
    c = load_case("porous_reg")
    s = make_engine(c, precision)
    s.finalize_init()
    fluid = c["phase"].reshape(-1) != 0
    n_sites = fluid.size
    mask = np.where(fluid, 0, 0x80000000).astype(np.uint32)
    nmask = torch.from_numpy(mask.view(np.int32)).cuda()
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    for call in range(2):
        s.evolve(20 + 7 * call)
        ref = np.zeros(8)
        assert lib.jlb_reduce(s._h, _native.dptr(ref)) == 0
        den = np.asarray(s.get_den()).reshape(-1)
        vel = np.asarray(s.get_vel()).reshape(-1, 3)
        if precision == 0:
            cols = [den, vel[:, 0], vel[:, 1], vel[:, 2]]
            tens = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in cols]
        else:
            # the FP32 and FP16-storage solvers keep den - 1 and u in
            # float32; these conversions recover their device values exactly
            cols = [den - 1.0, vel[:, 0], vel[:, 1], vel[:, 2]]
            tens = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda() for a in cols]
        out.fill_(-1.0)
        torch.cuda.synchronize()
        rc = lib.jlb_reduce_moments_noalloc(_ptr(nmask), *[_ptr(t) for t in tens], n_sites, precision,
                                            _ptr(out), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert got[7] == 0.0 and ref[7] == 0.0
        for k in range(7):
            assert abs(got[k] - ref[k]) <= TOL * max(abs(ref[k]), 1e-30) + 1e-300, (call, k, got[k], ref[k])


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from jyulb import _native

    lib = _native.load()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.jlb_reduce_moments_noalloc(dummy, dummy, dummy, dummy, dummy, (1 << 28) + 1, 0, dummy, None)
    assert rc == _native.JLB_ERR_INVALID_ARG
    rc = lib.jlb_reduce_moments_noalloc(dummy, dummy, dummy, dummy, dummy, 0, 0, dummy, None)
    assert rc == _native.JLB_ERR_INVALID_ARG
