"""Relaxation rates of the FP32 / FP16-storage kernels (float_exact_rates in
lbm_common.h) and the FP32 projection weights (lbm_shifted.cuh).

In FP32 a relaxation step that does not return the conserved moments it was
given, by the same relative amount at every step, drifts: a momentum factor
of 1 - 8.5e-9 per step (the nearest floats to the TRT coefficients at
tau+ = 0.56, magic 1/4) accumulates to ~1e-4 over 10^4 steps.  These checks
restate the kernels' float operations and require the pair relaxation plus
the projection to give back exactly the momentum and mass that went in (as
real sums of the float coefficients), with rates within 1e-6 of the exact
ones (or within 2^-23 where the sum w_e + w_o needs that grid).  The header's helper is compiled with g++."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from test_udiv_cpu import CSRC, _cuda_include

SRC = r"""
#include "lbm_common.h"
#include <cstdio>
using namespace jlb;
int main() {
    const double taus[] = {0.5005, 0.51, 0.55, 0.56, 0.6, 0.7, 0.8, 0.9, 1.0, 1.2, 1.5, 2.0, 3.0, 10.0};
    const double magics[] = {0.0, 0.25, 3.0 / 16.0, 1.0 / 12.0, 1.0 / 6.0, 0.5};
    for (double tau : taus)
        for (double magic : magics)
            for (int trt = 0; trt < 2; ++trt) {
                const double we = 1.0 / tau;
                double wo = we;
                if (trt) wo = magic > 0.0 ? 1.0 / (magic / (tau - 0.5) + 0.5) : 8.0 * (2.0 - we) / (8.0 - we);
                double a, b;
                float_exact_rates(trt != 0, we, wo, a, b);
                std::printf("%d %.17g %.17g %.17g %.17g\n", trt, we, wo, a, b);
            }
    return 0;
}
"""


def _rates(tmp_path):
    gxx = shutil.which("g++")
    inc = _cuda_include()
    if gxx is None or inc is None:
        pytest.skip("g++ or the CUDA headers are missing")
    src = tmp_path / "rates.cpp"
    src.write_text(SRC)
    exe = tmp_path / "rates"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, "-I", inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True)
    return [tuple(float(x) for x in line.split()) for line in out.stdout.splitlines()]


def test_float_rates_conserve_momentum_and_mass(tmp_path):
    f = np.float32
    k6, k12 = float.fromhex("0x1.555554p-3"), float.fromhex("0x1.555556p-4")
    assert f(k6) == k6 and f(k12) == k12
    assert 2 * k6 + 8 * k12 == 1.0  # the projection returns H1 exactly (real sum of the float weights)
    rows = _rates(tmp_path)
    assert len(rows) == 14 * 6 * 2
    for trt, we, wo, a, b in rows:
        assert f(a) == a and f(b) == b
        # a rate moves by at most half the grid 2^-22 that keeps w_e + w_o
        # exact when w_e is near 2 (tau+ near 1/2), otherwise by < 1e-6 of it
        tol = 2.0 ** -23
        assert abs(a - we) <= max(1e-6 * we, tol) and abs(b - wo) <= max(1e-6 * wo, tol), (we, wo, a, b)
        we_f, wo_f = f(a), f(b)
        if trt:
            # the kernel's TRT coefficients, in float arithmetic
            c3 = f(f(1.0) - f(f(0.5) * f(we_f + wo_f)))
            c4 = f(f(0.5) * f(we_f - wo_f))
            assert float(c3) + float(c4) + float(wo_f) == 1.0  # odd (momentum) part
            assert float(c3) - float(c4) + float(we_f) == 1.0  # even pairs (mass)
        r = f(f(1.0) - we_f)
        assert float(r) + float(we_f) == 1.0  # BGK / rest population / regularized c1
