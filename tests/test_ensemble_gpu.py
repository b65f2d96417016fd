"""Batched ensemble (jyulb.ensemble) against single-domain solvers.

Channels of uneven size, relaxation time and body force, half of them with a
moving top wall (Ladd), advance in one launch per step.  Each domain must
match a single-domain FP32-shifted Solver of the same configuration (same
physics in FP32; FMA contraction may differ between the two kernels, so the
bound is a few FP32 ulps of the velocity) and an FP64 Solver to FP32 accuracy.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def channels(n, seed, scale=1):
    rng = np.random.default_rng(seed)
    out = []
    for d in range(n):
        nx = int(rng.integers(8, 24)) * scale
        ny = int(rng.integers(6, 16))
        nz = int(rng.integers(4, 12))
        tau = float(rng.uniform(0.55, 1.5))
        gx = float(rng.uniform(1e-7, 1e-5))
        phase = np.ones((nx, ny, nz), np.uint8)
        phase[:, 0, :] = 0
        phase[:, -1, :] = 0
        vel = np.zeros((nx, ny, nz, 3))
        if d % 2 == 1:
            vel[:, -1, :, 0] = float(rng.uniform(0.01, 0.05))
        out.append(dict(phase=phase, vel=vel, kvisc=(tau - 0.5) / 3.0, g=[gx, 0.0, 0.0]))
    return out


def single(c, scheme, precision, steps):
    from jyulb.isothermal import Solver

    s = Solver(np.array(c["phase"].shape, dtype=np.int32), scheme, c["kvisc"], np.array(c["g"]), None,
               precision=precision)
    s.get_phase()[:] = c["phase"]
    s.get_vel()[:] = c["vel"]
    s.finalize_init()
    s.evolve(steps)
    return s


@pytest.mark.parametrize("scheme", [0, 1, 2])
@pytest.mark.parametrize("steps", [40, 41])
def test_ensemble_matches_single_domain_runs(scheme, steps):
    from jyulb.ensemble import Domain, Ensemble

    cs = channels(6, 100 + scheme)
    ens = Ensemble([Domain(c["phase"], None, c["vel"], c["kvisc"], c["g"]) for c in cs], scheme)
    ens.evolve(steps)
    info = ens.info()
    assert info["block"] in (64, 128, 256)
    for d, c in enumerate(cs):
        fl = c["phase"] != 0
        den, vel = ens.moments(d)
        s32 = single(c, scheme, 1, steps)
        v32 = np.asarray(s32.get_vel())
        vmax = np.abs(v32[fl]).max()
        assert np.abs(vel[fl] - v32[fl]).max() <= 1e-5 * vmax + 1e-12, d
        f = ens.populations(d)
        assert np.abs(f[:, fl] - s32.populations()[:, fl]).max() <= 1e-7
        s64 = single(c, scheme, 0, steps)
        v64 = np.asarray(s64.get_vel())
        err = np.linalg.norm(vel[fl] - v64[fl]) / np.linalg.norm(v64[fl])
        assert err <= 1e-4, (d, err)
        assert abs(den[fl] - np.asarray(s64.get_den())[fl]).max() <= 1e-6


def test_ensemble_rejects_unsupported_faces():
    from jyulb.ensemble import Domain, Ensemble

    ph = np.ones((4, 4, 4), np.uint8)
    with pytest.raises(RuntimeError, match="WALL and PERIODIC"):
        Ensemble([Domain(ph, bc=[3, 2, 1, 1, 1, 1])], 0)
