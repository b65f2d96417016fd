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


def test_ensemble_rejects_invalid_boundary_sets():
    from jyulb.ensemble import Domain, Ensemble

    # the single-domain checks apply: fixed faces only on opposite pairs
    with pytest.raises(ValueError):
        Ensemble([Domain(np.ones((4, 4, 4), np.uint8), bc=[3, 1, 2, 1, 1, 1])], 0)


def _boundary_domains(seed):
    # uneven boundary sets: Zou-He velocity inlet / density outlet, Zou-He
    # pressure difference, symmetric faces, moving solids next to Zou-He
    # faces, and a plain channel with a moving top wall
    from jyulb.defs import FIXED_DEN, FIXED_VEL, PERIODIC, SYMMETRIC, WALL

    rng = np.random.default_rng(seed)
    out = []
    sh = (14, 9, 6)
    ph = np.ones(sh, np.uint8); ph[6:8, 3:6, :] = 0
    vel = np.zeros(sh + (3,)); vel[0, :, :, 0] = 0.02
    out.append(dict(phase=ph, den=None, vel=vel, kvisc=0.05, g=[0.0, 0.0, 0.0],
                    bc=[FIXED_VEL, FIXED_DEN, WALL, WALL, PERIODIC, PERIODIC]))
    sh = (12, 7, 5)
    den = np.ones(sh); den[0] = 1.01; den[-1] = 0.99
    out.append(dict(phase=np.ones(sh, np.uint8), den=den, vel=None, kvisc=0.08, g=[0.0, 0.0, 0.0],
                    bc=[FIXED_DEN, FIXED_DEN, WALL, SYMMETRIC, PERIODIC, PERIODIC]))
    sh = (8, 10, 7)
    out.append(dict(phase=np.ones(sh, np.uint8), den=None, vel=None, kvisc=0.04, g=[0.0, 0.0, 2e-5],
                    bc=[SYMMETRIC, WALL, SYMMETRIC, SYMMETRIC, PERIODIC, PERIODIC]))
    sh = (10, 8, 6)
    ph = np.ones(sh, np.uint8); ph[:, -1, :] = 0
    vel = np.zeros(sh + (3,)); vel[:, -1, :, 2] = 0.03; vel[0, :-1, :, 0] = 0.01
    out.append(dict(phase=ph, den=None, vel=vel, kvisc=0.06, g=[1e-5, 0.0, 0.0],
                    bc=[FIXED_VEL, FIXED_DEN, WALL, WALL, PERIODIC, PERIODIC]))
    sh = (9, 8, 5)
    ph = np.ones(sh, np.uint8); ph[:, 0, :] = 0; ph[:, -1, :] = 0
    vel = np.zeros(sh + (3,)); vel[:, -1, :, 0] = 0.02
    out.append(dict(phase=ph, den=None, vel=vel, kvisc=0.1, g=[float(rng.uniform(1e-6, 1e-5)), 0.0, 0.0],
                    bc=[PERIODIC] * 6))
    # two plates moving at different velocities (Couette): the boundary-node
    # path, as no single wall velocity serves the domain
    sh = (10, 6, 4)
    ph = np.ones(sh, np.uint8); ph[0] = 0; ph[-1] = 0
    vel = np.zeros(sh + (3,)); vel[0, :, :, 1] = -0.01; vel[-1, :, :, 1] = 0.015; vel[-1, :, :, 2] = 0.005
    out.append(dict(phase=ph, den=None, vel=vel, kvisc=0.07, g=[0.0, 0.0, 0.0], bc=[PERIODIC] * 6))
    return out


@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_ensemble_boundary_sets_match_single_domains(scheme):
    from jyulb.ensemble import Domain, Ensemble
    from jyulb.isothermal import Solver

    cs = _boundary_domains(7)
    ens = Ensemble([Domain(c["phase"], c["den"], c["vel"], c["kvisc"], c["g"], c["bc"]) for c in cs], scheme)
    steps = 37
    ens.evolve(steps)
    for d, c in enumerate(cs):
        s = Solver(np.array(c["phase"].shape, dtype=np.int32), scheme, c["kvisc"], np.array(c["g"]),
                   np.array(c["bc"], dtype=np.int32), precision=1)
        s.get_phase()[:] = c["phase"]
        if c["den"] is not None:
            s.get_den()[:] = c["den"]
        if c["vel"] is not None:
            s.get_vel()[:] = c["vel"]
        s.finalize_init()
        s.evolve(steps)  # one call: boundary data read once, as the ensemble does
        fl = c["phase"] != 0
        den, vel = ens.moments(d)
        v32 = np.asarray(s.get_vel())
        vmax = np.abs(v32[fl]).max()
        assert np.abs(vel[fl] - v32[fl]).max() <= 1e-5 * vmax + 1e-12, d
        assert np.abs(den[fl] - np.asarray(s.get_den())[fl]).max() <= 1e-6, d
        f = ens.populations(d)
        assert np.abs(f[:, fl] - s.populations()[:, fl]).max() <= 1e-7, d


@pytest.mark.parametrize("scheme", [1, 2])
def test_ensemble_boundary_data_change_between_calls(scheme):
    # Zou-He data and the previous-step density re-read between calls, as
    # Solver.evolve does: the inlet ramps, the outlet density steps, and the
    # moving top wall next to the Zou-He faces reads the new density
    from jyulb.ensemble import Domain, Ensemble
    from jyulb.isothermal import Solver

    cs = _boundary_domains(9)
    ens = Ensemble([Domain(c["phase"], c["den"], c["vel"], c["kvisc"], c["g"], c["bc"]) for c in cs], scheme)
    sol = []
    for c in cs:
        s = Solver(np.array(c["phase"].shape, dtype=np.int32), scheme, c["kvisc"], np.array(c["g"]),
                   np.array(c["bc"], dtype=np.int32), precision=1)
        s.get_phase()[:] = c["phase"]
        if c["den"] is not None:
            s.get_den()[:] = c["den"]
        if c["vel"] is not None:
            s.get_vel()[:] = c["vel"]
        s.finalize_init()
        sol.append(s)
    for call, n in enumerate((19, 12, 7)):
        if call > 0:
            for d, c in enumerate(cs):
                den, vel = ens.moments(d)
                fl = c["phase"] != 0
                if c["bc"][0] == 3:
                    vel[0, :, :, 0] = np.where(fl[0], 0.02 + 0.005 * call, vel[0, :, :, 0])
                if c["bc"][1] == 2:
                    den[-1] = np.where(fl[-1], 1.0 + 0.002 * call, den[-1])
                ens.set_bc(d, den, vel)
                s = sol[d]
                s.get_den()[fl] = den[fl]
                s.get_vel()[fl] = vel[fl]
        ens.evolve(n)
        for s in sol:
            s.evolve(n)
    for d, c in enumerate(cs):
        fl = c["phase"] != 0
        den, vel = ens.moments(d)
        s = sol[d]
        v32 = np.asarray(s.get_vel())
        vmax = np.abs(v32[fl]).max()
        assert np.abs(vel[fl] - v32[fl]).max() <= 1e-5 * vmax + 1e-12, d
        assert np.abs(den[fl] - np.asarray(s.get_den())[fl]).max() <= 1e-6, d
        f = ens.populations(d)
        assert np.abs(f[:, fl] - s.populations()[:, fl]).max() <= 1e-7, d


@pytest.mark.parametrize("pf", ["3", "40"])
def test_ensemble_prefetch_changes_nothing(pf, monkeypatch):
    # the L2 line prefetch (forced here: these domains fit in L2, where it is
    # off by default) is a hint; results are bit for bit those without it
    from jyulb.ensemble import Domain, Ensemble

    cs = channels(5, 300)
    out = []
    for v in ("0", pf):
        monkeypatch.setenv("JLB_BATCH_PF", v)
        ens = Ensemble([Domain(c["phase"], None, c["vel"], c["kvisc"], c["g"]) for c in cs], 1)
        ens.evolve(23)
        out.append([ens.populations(d) for d in range(len(cs))])
    for f0, f1 in zip(*out):
        np.testing.assert_array_equal(f0, f1)
