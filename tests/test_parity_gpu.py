"""GPU parity of the CUDA engine against the reference (golden fixtures) and
the C oracle.

FP64 path: compiled without FMA contraction and evaluated in the
reference's operation order, so populations, den and vel are expected to be
bit-identical to the reference's x86-64 build; the bar the tests enforce is
the 1e-12 relative bound, with exact equality checked separately.
FP32 / FP16 paths: errors against the FP64 oracle with stated tolerances.
"""
import numpy as np
import pytest

from helpers import CASES, load_case, make_engine, rel_err, run_engine, run_oracle

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


@pytest.mark.parametrize("name", CASES)
def test_fp64_matches_reference_golden(name):
    c = load_case(name)
    nf, f, den, vel = run_engine(c)
    assert nf == c["nfluid"]
    fl = c["phase"] != 0
    assert rel_err(f[:, fl], c["f"][:, fl]) <= TOL64
    assert rel_err(den[fl], c["den"][fl]) <= TOL64
    assert rel_err(vel[fl], c["vel"][fl]) <= TOL64


@pytest.mark.parametrize("name", CASES)
def test_fp64_is_bitwise_reference(name):
    c = load_case(name)
    nf, f, den, vel = run_engine(c)
    fl = c["phase"] != 0
    np.testing.assert_array_equal(f[:, fl], c["f"][:, fl])
    np.testing.assert_array_equal(den[fl], c["den"][fl])
    np.testing.assert_array_equal(vel[fl], c["vel"][fl])


def _random_case(seed, lat, scheme, bc, porosity=0.8, moving=True, acc=True, chunks=(3, 4)):
    rng = np.random.default_rng(seed)
    sh = tuple(lat)
    c = dict(lat=list(lat), scheme=scheme, kvisc=float(rng.uniform(0.02, 0.2)),
             g=list(1e-5 * rng.standard_normal(3)), bc=list(bc), chunks=list(chunks))
    c["phase"] = (rng.random(sh) < porosity).astype(np.uint8)
    c["den0"] = 1.0 + 0.01 * rng.standard_normal(sh)
    v = 0.02 * rng.standard_normal(sh + (3,))
    if not moving:
        v[c["phase"] == 0] = 0.0
    c["vel0"] = v
    c["acc0"] = 1e-4 * rng.standard_normal(sh + (3,)) if acc else None
    return c


BCSETS = [
    [1, 1, 1, 1, 1, 1],
    [0, 0, 0, 0, 0, 0],
    [4, 4, 1, 1, 0, 4],
    [3, 2, 4, 0, 1, 1],
    [0, 4, 2, 3, 4, 0],
    [1, 1, 0, 0, 3, 3],
    [4, 0, 4, 0, 4, 0],
]


@pytest.mark.parametrize("scheme", [0, 1, 2])
@pytest.mark.parametrize("bi", range(len(BCSETS)))
def test_fp64_vs_oracle_random(scheme, bi):
    c = _random_case(100 * bi + scheme, (9, 7, 11), scheme, BCSETS[bi], chunks=(4, 5))
    _, f0, d0, v0 = run_oracle(c)
    _, f1, d1, v1 = run_engine(c)
    fl = c["phase"] != 0
    np.testing.assert_array_equal(f1[:, fl], f0[:, fl])
    np.testing.assert_array_equal(d1[fl], d0[fl])
    np.testing.assert_array_equal(v1[fl], v0[fl])


@pytest.mark.parametrize("odd", [1, 3, 33, 65])
def test_odd_step_counts_and_graph_path(odd):
    # odd totals leave the AA array in its streamed state; long calls replay
    # the captured step graphs
    c = _random_case(7, (6, 10, 40), 1, [1, 1, 0, 0, 1, 1], chunks=(odd, 2))
    _, f0, d0, v0 = run_oracle(c)
    _, f1, d1, v1 = run_engine(c)
    fl = c["phase"] != 0
    np.testing.assert_array_equal(f1[:, fl], f0[:, fl])
    np.testing.assert_array_equal(v1[fl], v0[fl])


def test_moving_walls_change_between_calls():
    # solid velocities are re-read at every evolve call (Ladd's term)
    from pyoracle import Oracle

    c = _random_case(3, (8, 8, 8), 0, [1] * 6, porosity=0.75, moving=False, acc=False, chunks=(5,))
    o = Oracle(c["lat"], c["scheme"], c["kvisc"], c["g"], c["bc"])
    s = make_engine(c)
    for obj in (o, s):
        obj.get_phase()[:] = c["phase"]
        obj.get_den()[:] = c["den0"]
        obj.get_vel()[:] = c["vel0"]
    assert s.finalize_init() == o.finalize_init()
    sol = c["phase"] == 0
    rng = np.random.default_rng(5)
    for it in range(3):
        for obj in (o, s):
            obj.evolve(4 + it)
        w = 0.01 * rng.standard_normal((int(sol.sum()), 3)) if it < 2 else np.zeros((int(sol.sum()), 3))
        for obj in (o, s):
            v = obj.get_vel()
            v[sol] = w
    for obj in (o, s):
        obj.evolve(3)
    fl = ~sol
    np.testing.assert_array_equal(s.populations()[:, fl], o.populations()[:, fl])
    np.testing.assert_array_equal(np.asarray(s.get_vel())[fl], o.get_vel()[fl])


def _walls_case(bc, seed):
    from pyoracle import Oracle

    c = _random_case(seed, (7, 6, 8), 1, bc, porosity=0.8, moving=False, acc=False, chunks=(4,))
    o = Oracle(c["lat"], c["scheme"], c["kvisc"], c["g"], c["bc"])
    s = make_engine(c)
    for obj in (o, s):
        obj.get_phase()[:] = c["phase"]
        obj.get_den()[:] = c["den0"]
        obj.get_vel()[:] = c["vel0"]
    assert s.finalize_init() == o.finalize_init()
    return c, o, s


def test_moving_walls_mixed_faces_static_halo():
    # the Solver's default: halo cells of wall faces are not re-read; interior
    # solids (and their periodic / symmetric halo images) are
    c, o, s = _walls_case([1, 1, 0, 0, 4, 4], 21)
    sol = c["phase"] == 0
    rng = np.random.default_rng(8)
    for it in range(3):
        for obj in (o, s):
            obj.evolve(3 + it)
        w = 0.01 * rng.standard_normal((int(sol.sum()), 3))
        for obj in (o, s):
            obj.get_vel()[sol] = w
    for obj in (o, s):
        obj.evolve(4)
    fl = ~sol
    np.testing.assert_array_equal(s.populations()[:, fl], o.populations()[:, fl])
    np.testing.assert_array_equal(np.asarray(s.get_vel())[fl], o.get_vel()[fl])


def test_halo_wall_velocity_reread_without_static_halo():
    # through the C ABI default (no static-halo promise) a velocity written
    # into the halo of a wall face moves that wall, as in the reference's
    # stream step, which reads the halo solid's velocity (Ladd)
    c, o, s = _walls_case([0, 0, 1, 1, 1, 1], 22)
    assert s._lib.jlb_set_static_halo(s._h, 0) == 0
    for obj in (o, s):
        obj.evolve(3)
    for obj in (o, s):
        obj.vel[0, 1:-1, 1:-1, 1] = 0.02
        obj.vel[-1, 1:-1, 1:-1, 2] = -0.01
    for obj in (o, s):
        obj.evolve(5)
    fl = c["phase"] != 0
    np.testing.assert_array_equal(s.populations()[:, fl], o.populations()[:, fl])
    np.testing.assert_array_equal(np.asarray(s.get_vel())[fl], o.get_vel()[fl])


def test_acc_and_gravity_updates_between_calls():
    from pyoracle import Oracle

    c = _random_case(9, (6, 8, 7), 2, [0, 0, 1, 1, 1, 1], acc=False, chunks=(3,))
    o = Oracle(c["lat"], c["scheme"], c["kvisc"], c["g"], c["bc"])
    s = make_engine(c)
    for obj in (o, s):
        obj.get_phase()[:] = c["phase"]
        obj.get_den()[:] = c["den0"]
        obj.get_vel()[:] = c["vel0"]
    s.finalize_init(); o.finalize_init()
    s.evolve(3); o.evolve(3)
    rng = np.random.default_rng(1)
    a = 1e-4 * rng.standard_normal(tuple(c["lat"]) + (3,))
    s.get_acc()[:] = a; o.get_acc()[:] = a
    s.evolve(4); o.evolve(4)
    s.gravity = [0.0, 2e-5, 0.0]; o.set_gravity(np.array([0.0, 2e-5, 0.0]))
    s.get_acc()[:] = 0.0; o.get_acc()[:] = 0.0
    s.evolve(5); o.evolve(5)
    fl = c["phase"] != 0
    np.testing.assert_array_equal(s.populations()[:, fl], o.populations()[:, fl])
    np.testing.assert_array_equal(np.asarray(s.get_den())[fl], o.get_den()[fl])


def test_chunking_is_irrelevant_without_zou_he():
    c = load_case("poiseuille_4x34x4")
    _, f_a, _, v_a = run_engine(c, chunks=[1000])
    _, f_b, _, v_b = run_engine(c, chunks=[100] * 10)
    np.testing.assert_array_equal(f_a, f_b)
    np.testing.assert_array_equal(v_a, v_b)


def test_save_load_state_continues_identically():
    c = load_case("cavity_trt")
    s = make_engine(c)
    s.finalize_init()
    s.evolve(37)
    st = s.save_state()
    s.evolve(20)
    ref = s.populations()
    s.load_state(st)
    s.evolve(20)
    np.testing.assert_array_equal(s.populations(), ref)


def test_reduce_matches_host_sums():
    c = load_case("porous_reg")
    s = make_engine(c)
    nf = s.finalize_init()
    s.evolve(50)
    r = s.reduce()
    fl = c["phase"] != 0
    den = np.asarray(s.get_den())[fl]
    vel = np.asarray(s.get_vel())[fl]
    assert abs(r["mass"] - den.sum()) <= 1e-12 * nf
    assert np.allclose(r["momentum"], (den[:, None] * vel).sum(0), rtol=1e-12, atol=1e-18)
    assert np.allclose(r["vel_sum"], vel.sum(0), rtol=1e-12, atol=1e-18)


@pytest.mark.parametrize("precision,tol", [(1, 2e-5), (2, 3e-2)])
@pytest.mark.parametrize("name", ["poiseuille_4x34x4", "cavity_trt", "porous_reg", "invel_grav"])
def test_reduced_precision_velocity_error(name, precision, tol):
    # relative L2 velocity error of FP32-shifted (tol 2e-5) and FP16-storage
    # (tol 3e-2) against the FP64 reference outputs
    c = load_case(name)
    _, f, den, vel = run_engine(c, precision=precision)
    fl = c["phase"] != 0
    err = np.linalg.norm(vel[fl] - c["vel"][fl]) / np.linalg.norm(c["vel"][fl])
    assert err <= tol, err
    assert abs(den[fl] - c["den"][fl]).max() <= (1e-6 if precision == 1 else 1e-3)


EDGE = ["edge_single_site", "edge_column_sym", "edge_sheet_zou_he", "edge_enclosed_site"]


@pytest.mark.parametrize("precision,tol", [(1, 1e-4), (2, 5e-2)])
@pytest.mark.parametrize("name", EDGE)
def test_reduced_precision_degenerate_shapes(name, precision, tol):
    # the FP32 / FP16 kernels on 1-site, 1-column, 1-sheet and enclosed
    # lattices (the last on the fluid-only layout) against the reference's
    # FP64 outputs; few sites, so the relative L2 bound is looser than above
    c = load_case(name)
    nf, f, den, vel = run_engine(c, precision=precision)
    assert nf == c["nfluid"]
    fl = c["phase"] != 0
    err = np.linalg.norm(vel[fl] - c["vel"][fl]) / np.linalg.norm(c["vel"][fl])
    assert err <= tol, err
    assert abs(den[fl] - c["den"][fl]).max() <= (1e-6 if precision == 1 else 1e-3)


def test_mass_conserved_large_periodic():
    # size-independent property at a larger size: mass and (force-free)
    # momentum of a periodic box stay constant
    from jyulb.isothermal import Solver

    n = 64
    rng = np.random.default_rng(3)
    s = Solver(np.array([n, n, n], dtype=np.int32), 1, 0.05, None, None)
    s.get_phase()[:] = 1
    s.get_den()[:] = 1.0 + 0.001 * rng.standard_normal((n, n, n))
    s.get_vel()[:] = 0.01 * rng.standard_normal((n, n, n, 3))
    s.finalize_init()
    s.evolve(1)
    r0 = s.reduce()
    s.evolve(200)
    r1 = s.reduce()
    # per-site rounding of ~1e-16 per step over 2.6e5 sites and 200 steps
    assert abs(r1["mass"] - r0["mass"]) <= 1e-12 * r0["mass"]
    assert np.allclose(r1["momentum"], r0["momentum"], rtol=0, atol=1e-12 * r0["mass"])


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("bi", [2, 3, 4, 6])
def test_rows_of_96_sites_with_boundary_nodes(precision, bi):
    # nz = 96 gives the direct kernel row blocks of 96 threads; its
    # boundary-node blocks must be counted in blocks of 96 too (Zou-He,
    # symmetric and moving-wall nodes: several hundred here)
    c = _random_case(400 + bi, (5, 6, 96), 1, BCSETS[bi], chunks=(3, 4))
    _, f0, d0, v0 = run_oracle(c)
    _, f1, d1, v1 = run_engine(c, precision)
    fl = c["phase"] != 0
    if precision == 0:
        np.testing.assert_array_equal(f1[:, fl], f0[:, fl])
        np.testing.assert_array_equal(v1[fl], v0[fl])
    else:
        assert np.abs(f1[:, fl] - f0[:, fl]).max() <= 1e-6
        assert np.abs(v1[fl] - v0[fl]).max() <= 1e-6
