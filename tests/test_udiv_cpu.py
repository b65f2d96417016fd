"""The multiply-shift division of the dense sweep's consecutive-site mapping
(UDiv / make_udiv in lbm_common.h): the host-computed multiplier and shifts
give n / d exactly for every 32-bit n, checked over all divisors below
70 000 and random divisors up to 2^32 - 1 with edge and random dividends.
The quotient formula is restated on the host (mulhi as a 64-bit product) and
the header is compiled with g++."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "jyu-lb_gb300", "csrc")

SRC = r"""
#include "lbm_common.h"
#include <cstdio>
#include <random>
using namespace jlb;
static uint32_t quot(uint32_t n, UDiv d) {
    const uint32_t t = (uint32_t)(((uint64_t)n * d.m) >> 32);
    return (t + ((n - t) >> d.s1)) >> d.s2;
}
int main() {
    std::mt19937_64 rng(7);
    long bad = 0, cnt = 0;
    auto check = [&](uint32_t n, uint32_t d, const UDiv &u) { ++cnt; if (quot(n, u) != n / d) ++bad; };
    for (uint32_t d = 1; d < 70000; ++d) {
        const UDiv u = make_udiv(d);
        for (uint32_t n : {0u, 1u, d - 1, d, d + 1, 2 * d - 1, 0xfffffffeu, 0xffffffffu}) check(n, d, u);
        for (int r = 0; r < 20; ++r) check((uint32_t)rng(), d, u);
    }
    for (int r = 0; r < 200000; ++r) {
        uint32_t d = (uint32_t)rng();
        if (d == 0) d = 1;
        const UDiv u = make_udiv(d);
        check((uint32_t)rng(), d, u);
        check(0xffffffffu, d, u);
        check(d, d, u);
    }
    for (uint32_t d : {0x7fffffffu, 0x80000000u, 0x80000001u, 0xffffffffu}) {
        const UDiv u = make_udiv(d);
        for (uint32_t n : {0u, d - 1, d, 0xffffffffu}) check(n, d, u);
    }
    std::printf("%ld %ld\n", cnt, bad);
    return bad != 0;
}
"""


def _cuda_include():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "include", "cuda_runtime.h")):
            return os.path.join(cand, "include")
    return None


def test_udiv_exact(tmp_path):
    gxx = shutil.which("g++")
    inc = _cuda_include()
    if gxx is None or inc is None:
        pytest.skip("g++ or the CUDA headers are missing")
    src = tmp_path / "udiv.cpp"
    src.write_text(SRC)
    exe = tmp_path / "udiv"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, "-I", inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    cnt, bad = map(int, out.stdout.split())
    assert out.returncode == 0 and bad == 0 and cnt > 2_000_000
