"""The C oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the built reference).  The oracle follows the
reference's operation order and is compiled without FMA contraction, so the
match is exact."""
import numpy as np
import pytest

from helpers import CASES, LARGE_CASES, digest, load_case, run_oracle


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_bitwise(name):
    c = load_case(name)
    nf, f, den, vel = run_oracle(c)
    assert nf == c["nfluid"]
    fl = c["phase"] != 0
    np.testing.assert_array_equal(f[:, fl], c["f"][:, fl])
    np.testing.assert_array_equal(den[fl], c["den"][fl])
    np.testing.assert_array_equal(vel[fl], c["vel"][fl])


def test_oracle_conserves_mass_periodic():
    c = load_case("poiseuille_4x34x4")
    nf, f, den, vel = run_oracle(c, chunks=[200])
    fl = c["phase"] != 0
    assert abs(den[fl].sum() - nf) < 1e-10


def test_z1_quirk_is_in_the_fixture():
    # a lone Z1 FIXED_VEL face gets den=1, vel=0 as bc data (reference quirk),
    # so the lid layer does not move at the prescribed 0.04
    c = load_case("z1_fixed_vel")
    assert abs(c["vel"][:, :, -1, 0]).max() < 1e-3


def test_oracle_steady_profiles_match_reference():
    # the steady channel flows of the reference's example scripts: the oracle
    # reproduces the reference's mid-domain profiles bit for bit
    import json
    import os

    from pyoracle import Oracle

    import profile_cases as pc
    from jyulb import flow_field

    gold = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "profiles.json")))
    for c in pc.cases():
        o = Oracle(c["lat"], c["scheme"], c["kvisc"], list(pc.gravity(c)), c["bc"])
        pc.setup(o, c, flow_field)
        assert o.finalize_init() == gold[c["name"]]["nfluid"]
        for n in c["chunks"]:
            o.evolve(n)
        prof = pc.profile(o.get_vel(), c)
        ref = np.array([[float.fromhex(v) for v in row] for row in gold[c["name"]]["profile"]])
        np.testing.assert_array_equal(prof, ref, err_msg=c["name"])
        assert pc.error(prof, c, flow_field) == float.fromhex(gold[c["name"]]["error"])


@pytest.mark.parametrize("zsym", [False, True])
@pytest.mark.parametrize("scheme", ["BGK", "TRT", "REG"])
def test_torch_step_matches_oracle(scheme, zsym):
    # the pure-torch FP64 step that checks the adjoint's gradients reproduces
    # the oracle (and so the reference) on its channel: Zou-He velocity inlet
    # with a per-site u_x, density outlet, walls in y, periodic or symmetric z,
    # a cylinder
    import torch

    from pyoracle import Oracle
    from torch_lbm import run

    rng = np.random.default_rng(4)
    nx, ny, nz = 12, 8, 4
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    phase = np.ones((nx, ny, nz), np.uint8)
    phase[(X - 5) ** 2 + (Y - 4) ** 2 <= 2.0] = 0
    uin = 0.02 + 0.005 * rng.standard_normal((ny, nz))
    tau, g, steps = 0.8, np.array([1e-5, 2e-6, 0.0]), 25
    sch = {"BGK": 0, "TRT": 1, "REG": 2}[scheme]
    if zsym:
        g = np.array([1e-5, 2e-6, 3e-6])
    u = run(phase, torch.tensor(tau, dtype=torch.float64), torch.tensor(g), torch.tensor(uin), steps,
            scheme=scheme, zsym=zsym).numpy()
    o = Oracle([nx, ny, nz], sch, (tau - 0.5) / 3.0, list(g), [3, 2, 0, 0, 4, 4] if zsym else [3, 2, 0, 0, 1, 1])
    o.get_phase()[:] = phase
    o.finalize_init()  # from rest, as the torch step starts
    o.get_vel()[0, :, :, 0] = uin  # inlet data, read at the evolve call
    o.evolve(steps)
    fl = phase != 0
    ref = np.moveaxis(o.get_vel(), -1, 0)[:, fl]
    np.testing.assert_allclose(u[:, fl], ref, rtol=0, atol=1e-13 * np.abs(ref).max())


@pytest.mark.parametrize("name", CASES)
def test_oracle_halo_arrays_match_reference_bitwise(name):
    # the whole halo-padded den / vel after the last evolve call: the
    # periodic / symmetric halos hold the images of the moments of the step
    # before the last (jyulb/isothermal.pyx:1408-1411)
    from pyoracle import Oracle

    c = load_case(name)
    o = Oracle(c["lat"], c["scheme"], c["kvisc"], c["g"], c["bc"], 0.0)
    o.get_phase()[:] = c["phase"]
    o.get_den()[:] = c["den0"]
    o.get_vel()[:] = c["vel0"]
    if c["acc0"] is not None:
        o.get_acc()[:] = c["acc0"]
    o.finalize_init()
    for n in c["chunks"]:
        o.evolve(n)
    np.testing.assert_array_equal(o.den, c["den_full"])
    np.testing.assert_array_equal(o.vel, c["vel_full"])


@pytest.mark.parametrize("name", LARGE_CASES)
def test_oracle_matches_reference_digests_at_1000_steps(name):
    # the 1000-step fixtures on larger lattices: SHA-256 digests of the
    # reference's float64 arrays
    from pyoracle import Oracle

    c = load_case(name)
    o = Oracle(c["lat"], c["scheme"], c["kvisc"], c["g"], c["bc"], 0.0)
    o.get_phase()[:] = c["phase"]
    o.get_den()[:] = c["den0"]
    o.get_vel()[:] = c["vel0"]
    assert o.finalize_init() == c["nfluid"]
    for n in c["chunks"]:
        o.evolve(n)
    fl = c["phase"] != 0
    h = c["sha256"]
    assert digest(o.populations()[:, fl]) == h["f"]
    assert digest(o.get_den()[fl]) == h["den"]
    assert digest(o.get_vel()[fl]) == h["vel"]
    assert digest(o.den) == h["den_full"]
    assert digest(o.vel) == h["vel_full"]


def _field_case(kind, seed=3):
    """phase, bc, den, vel, solid velocity of the general torch step's cases"""
    rng = np.random.default_rng(seed)
    sv = None
    if kind == "y":
        shape, bc = (8, 10, 4), [1, 1, 3, 2, 1, 1]
    elif kind == "z":
        shape, bc = (6, 6, 10), [1, 1, 0, 0, 3, 2]
    elif kind == "x1":
        shape, bc = (12, 6, 4), [2, 3, 0, 0, 1, 1]
    else:  # moving lid with an inlet
        shape, bc = (10, 8, 4), [3, 2, 0, 0, 1, 1]
    nx, ny, nz = shape
    phase = np.ones(shape, np.uint8)
    phase[nx // 2 - 1:nx // 2 + 1, ny // 2 - 1:ny // 2 + 1, :] = 0
    den = np.ones(shape)
    vel = np.zeros(shape + (3,))
    sl = {0: (0, slice(None), slice(None)), 1: (nx - 1, slice(None), slice(None)),
          2: (slice(None), 0, slice(None)), 3: (slice(None), ny - 1, slice(None)),
          4: (slice(None), slice(None), 0), 5: (slice(None), slice(None), nz - 1)}
    for f in range(6):
        if bc[f] == 3:
            v = vel[sl[f]]
            v[..., f >> 1] = (-1 if f & 1 else 1) * (0.02 + 0.004 * rng.standard_normal(v.shape[:-1]))
            v[..., ((f >> 1) + 1) % 3] = 0.002 * rng.standard_normal(v.shape[:-1])
            vel[sl[f]] = v
        elif bc[f] == 2:
            den[sl[f]] = 1.0 + 0.002 * rng.standard_normal(den[sl[f]].shape)
            v = vel[sl[f]]
            v[..., ((f >> 1) + 1) % 3] = 0.001 * rng.standard_normal(v.shape[:-1])
            vel[sl[f]] = v
    if kind == "lid":
        phase[:, -1, :] = 0
        sv = np.zeros(shape + (3,))
        sv[:, -1, :, 0] = 0.05
        sv[:, -1, :, 2] = 0.01
        den[:, -2, :] += 0.001 * rng.standard_normal((nx, nz))  # read by the lid's Ladd term
        vel[0, :-1, :, 0] = 0.01 + 0.002 * rng.standard_normal((ny - 1, nz))
    return phase, bc, den, vel, sv


@pytest.mark.parametrize("kind", ["y", "z", "x1", "lid"])
@pytest.mark.parametrize("scheme", ["TRT", "REG"])
def test_general_torch_step_matches_oracle(kind, scheme):
    # the general pure-torch step (Zou-He on any fixed face from den / vel,
    # moving solids with Ladd's term) reproduces the oracle from rest, with
    # the face data and the previous-step density read at the evolve call
    import torch

    from pyoracle import Oracle
    from torch_lbm import run_fields

    phase, bc, den, vel, sv = _field_case(kind)
    tau, g, steps = 0.8, np.array([2e-6, -1e-6, 1e-6]), 21
    sch = {"TRT": 1, "REG": 2}[scheme]
    o = Oracle(list(phase.shape), sch, (tau - 0.5) / 3.0, list(g), bc, 0.25 if scheme == "TRT" else 0.0)
    o.get_phase()[:] = phase
    if sv is not None:
        o.get_vel()[:] = sv
    o.finalize_init()
    f0 = o.populations()  # rest, except next to the moving solids
    u = run_fields(phase, torch.tensor(tau, dtype=torch.float64), torch.tensor(g), torch.tensor(den),
                   torch.tensor(vel), steps, bc, magic=0.25 if scheme == "TRT" else None, scheme=scheme,
                   solid_vel=sv, f0=f0).numpy()
    fl = phase != 0
    o.get_den()[fl] = den[fl]
    o.get_vel()[fl] = vel[fl]
    o.evolve(steps)
    ref = np.moveaxis(o.get_vel(), -1, 0)[:, fl]
    np.testing.assert_allclose(u[:, fl], ref, rtol=0, atol=1e-13 * np.abs(ref).max())
