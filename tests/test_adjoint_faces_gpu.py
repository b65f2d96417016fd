"""The adjoint with Zou-He data on any fixed face and with moving solids,
against central differences of the FP64 model.

Zou-He data come from the den / vel fields at the boundary sites
(ChannelProblem.forward_fields), as Solver.evolve reads them; their
gradients cover FIXED_VEL velocities (all three components) and FIXED_DEN
densities and tangential velocities on all six faces.  A moving solid lid
enters through Ladd's term, whose density of the previous step carries its
own adjoint through the reverse sweep.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields(shape, faces, rng, u0=0.02):
    """den, vel with inflow data on the given (face, normal velocity) list"""
    nx, ny, nz = shape
    den = np.ones(shape)
    vel = np.zeros(shape + (3,))
    sl = {0: (0, slice(None), slice(None)), 1: (nx - 1, slice(None), slice(None)),
          2: (slice(None), 0, slice(None)), 3: (slice(None), ny - 1, slice(None)),
          4: (slice(None), slice(None), 0), 5: (slice(None), slice(None), nz - 1)}
    for face, kind in faces:
        idx = sl[face]
        if kind == "vel":
            ax = face >> 1
            sign = -1.0 if face & 1 else 1.0
            v = vel[idx]
            v[..., ax] = sign * (u0 + 0.004 * rng.standard_normal(v.shape[:-1]))
            for t in range(3):
                if t != ax:
                    v[..., t] = 0.002 * rng.standard_normal(v.shape[:-1])
            vel[idx] = v
        else:
            den[idx] = 1.0 + 0.002 * rng.standard_normal(den[idx].shape)
            v = vel[idx]
            v[..., ((face >> 1) + 1) % 3] = 0.001 * rng.standard_normal(v.shape[:-1])
            vel[idx] = v
    return den, vel


def _fd_check(p, ref, tau, g, den, vel, steps, target, probes, tol):
    p.forward_fields(tau, g, den, vel, steps, target)
    dtau, dg, dden, dvel = p.backward_fields()

    def L(tau_=tau, g_=g, den_=den, vel_=vel):
        return ref.forward_fields(tau_, g_, den_, vel_, steps, target)[0]

    h = 1e-5
    fd = (L(tau_=tau + h) - L(tau_=tau - h)) / (2 * h)
    assert abs(dtau - fd) <= tol * abs(fd), ("tau", dtau, fd)
    scale_v = np.abs(dvel).max()
    scale_d = np.abs(dden).max()
    if probes:
        assert scale_v > 0
    for kind, idx in probes:
        hv = 1e-6
        if kind == "den":
            dp, dm = den.copy(), den.copy()
            dp[idx] += hv
            dm[idx] -= hv
            fd = (L(den_=dp) - L(den_=dm)) / (2 * hv)
            got, scale = dden[idx], scale_d
        else:
            vp, vm = vel.copy(), vel.copy()
            vp[idx] += hv
            vm[idx] -= hv
            fd = (L(vel_=vp) - L(vel_=vm)) / (2 * hv)
            got, scale = dvel[idx], scale_v
        assert abs(got - fd) <= tol * max(abs(fd), 1e-3 * scale), (kind, idx, got, fd)
    return dden, dvel


FACE_CASES = [
    # inflow on 1Y, outflow on Y1; periodic x and z
    ([1, 1, 3, 2, 1, 1], [(2, "vel"), (3, "den")],
     [("vel", (5, 0, 1, 1)), ("vel", (7, 0, 2, 0)), ("vel", (3, 0, 0, 2)), ("den", (6, 13, 1)), ("vel", (4, 13, 2, 2))]),
    # inflow on X1 (u_x < 0), outflow on 1X
    ([2, 3, 0, 0, 1, 1], [(1, "vel"), (0, "den")],
     [("vel", (15, 4, 1, 0)), ("vel", (15, 6, 2, 1)), ("den", (0, 5, 1)), ("den", (0, 8, 3))]),
    # inflow on 1Z, outflow on Z1 (Z1 data read because 1Z is FIXED_VEL)
    ([1, 1, 0, 0, 3, 2], [(4, "vel"), (5, "den")],
     [("vel", (3, 4, 0, 2)), ("vel", (5, 6, 0, 0)), ("den", (4, 5, 11)), ("vel", (2, 7, 11, 0))]),
]


@pytest.mark.parametrize("bc,faces,probes", FACE_CASES)
@pytest.mark.parametrize("scheme", [1, 2])
def test_fp64_face_data_gradients_match_central_differences(bc, faces, probes, scheme):
    from jyulb.adjoint import ChannelProblem
    from jyulb.defs import FP64

    rng = np.random.default_rng(sum(bc) + scheme)
    shape = {0: (16, 10, 4), 1: (12, 14, 4), 2: (8, 10, 12)}[faces[0][0] >> 1]
    phase = np.ones(shape, np.uint8)
    phase[shape[0] // 2 - 1:shape[0] // 2 + 1, shape[1] // 2 - 1:shape[1] // 2 + 1, :] = 0
    den, vel = _fields(shape, faces, rng)
    plane = shape[0] // 2 + 2
    target = 0.01 * rng.standard_normal((shape[1], shape[2], 3))
    magic = 0.25 if scheme == 1 else None
    kw = dict(bc=bc, rlx_scheme=scheme, precision=FP64, trt_magic=magic, loss_plane=plane, checkpoint_every=7)
    p = ChannelProblem(phase, **kw)
    ref = ChannelProblem(phase, **kw)
    g = np.array([2e-6, -1e-6, 1e-6])
    _fd_check(p, ref, 0.8, g, den, vel, 30, target, probes, 1e-6)


def test_z1_velocity_face_is_not_read_without_a_1z_velocity_face():
    # bc[Z1] = FIXED_VEL with bc[1Z] = FIXED_DEN: the solver keeps Z1's data
    # at den 1, vel 0 (the reference refreshes Z1 only when bc[Z1] is
    # FIXED_DEN or bc[1Z] is FIXED_VEL), so vel there changes nothing and has
    # no gradient
    from jyulb.adjoint import ChannelProblem
    from jyulb.defs import FP64

    shape = (8, 10, 12)
    rng = np.random.default_rng(5)
    phase = np.ones(shape, np.uint8)
    den, vel = _fields(shape, [(4, "den"), (5, "vel")], rng)
    target = 0.01 * rng.standard_normal((10, 12, 3))
    p = ChannelProblem(phase, bc=[1, 1, 0, 0, 2, 3], rlx_scheme=1, precision=FP64, trt_magic=0.25, loss_plane=4,
                       checkpoint_every=5)
    L1, _ = p.forward_fields(0.8, [1e-6, 0, 0], den, vel, 20, target)
    _, _, dden, dvel = p.backward_fields()
    v0 = vel.copy()
    v0[:, :, -1] = 0.0
    L0, _ = p.forward_fields(0.8, [1e-6, 0, 0], den, v0, 20, target)
    assert L1 == L0
    assert np.all(dvel[:, :, -1] == 0.0)
    assert np.abs(dden[:, :, 0]).max() > 0


@pytest.mark.parametrize("precision", [0, 1])
def test_uin_and_field_forms_agree(precision):
    # forward(uin) is forward_fields with vel[0, :, :, 0] = uin and den 1
    from jyulb.adjoint import ChannelProblem
    from jyulb.defs import FIXED_DEN, FIXED_VEL, PERIODIC, TRT, WALL

    shape = (14, 8, 4)
    rng = np.random.default_rng(7)
    phase = np.ones(shape, np.uint8)
    phase[6:8, 3:5, :] = 0
    uin = 0.02 + 0.004 * rng.standard_normal((8, 4))
    target = 0.01 * rng.standard_normal((8, 4, 3))
    p = ChannelProblem(phase, bc=[FIXED_VEL, FIXED_DEN, WALL, WALL, PERIODIC, PERIODIC], rlx_scheme=TRT,
                       precision=precision, trt_magic=0.25, loss_plane=10, checkpoint_every=6)
    L1, u1 = p.forward(0.75, [1e-6, 0, 0], uin, 25, target)
    dtau1, dg1, duin = p.backward()
    vel = np.zeros(shape + (3,))
    vel[0, :, :, 0] = uin
    L2, u2 = p.forward_fields(0.75, [1e-6, 0, 0], None, vel, 25, target)
    dtau2, dg2, dden, dvel = p.backward_fields()
    assert L1 == L2
    np.testing.assert_array_equal(u1, u2)
    assert dtau1 == dtau2
    np.testing.assert_array_equal(dg1, dg2)
    np.testing.assert_array_equal(duin, dvel[0, :, :, 0])


def test_uin_form_refuses_a_velocity_face_other_than_1x():
    from jyulb.adjoint import ChannelProblem
    from jyulb.defs import FIXED_DEN, FIXED_VEL, FP64, PERIODIC, WALL

    p = ChannelProblem(np.ones((8, 10, 4), np.uint8), bc=[WALL, WALL, FIXED_VEL, FIXED_DEN, PERIODIC, PERIODIC],
                       precision=FP64, loss_plane=4)
    with pytest.raises(RuntimeError, match="forward_fields"):
        p.forward(0.8, [0, 0, 0], np.zeros((10, 4)), 5)


def _lid_case(precision, with_inlet):
    from jyulb.adjoint import ChannelProblem
    from jyulb.defs import FIXED_DEN, FIXED_VEL, FP64, PERIODIC, WALL

    shape = (14, 10, 4)
    rng = np.random.default_rng(11)
    phase = np.ones(shape, np.uint8)
    phase[:, -1, :] = 0          # lid: solid row moving in x
    phase[5:7, 2:4, :] = 0       # immobile obstacle
    sv = np.zeros(shape + (3,))
    sv[:, -1, :, 0] = 0.05
    sv[:, -1, :, 2] = 0.01
    bc = [FIXED_VEL, FIXED_DEN, WALL, WALL, PERIODIC, PERIODIC] if with_inlet else [WALL, WALL, WALL, WALL,
                                                                                   PERIODIC, PERIODIC]
    den, vel = _fields(shape, [(0, "vel"), (1, "den")] if with_inlet else [], rng, u0=0.01)
    target = 0.01 * rng.standard_normal((10, 4, 3))
    kw = dict(bc=bc, rlx_scheme=1, trt_magic=0.25, loss_plane=9, checkpoint_every=6, solid_vel=sv)
    return (ChannelProblem(phase, precision=precision, **kw), ChannelProblem(phase, precision=FP64, **kw),
            den, vel, target)


@pytest.mark.parametrize("with_inlet", [False, True])
@pytest.mark.parametrize("precision,tol", [(0, 1e-6), (1, 1e-4)])
def test_moving_lid_adjoint_matches_central_differences(with_inlet, precision, tol):
    # the lid's Ladd term reads the previous step's density of its
    # neighbours; with the inlet, the corner sites have both a Zou-He face
    # and moving links
    p, ref, den, vel, target = _lid_case(precision, with_inlet)
    g = np.array([3e-6, 1e-6, 0.0])
    probes = [("vel", (0, 4, 1, 0)), ("vel", (0, 8, 2, 0)), ("den", (13, 5, 1)), ("den", (13, 8, 3))] \
        if with_inlet else []
    _fd_check(p, ref, 0.7, g, den, vel, 36, target, probes, tol)
    # the body force
    p.forward_fields(0.7, g, den, vel, 36, target)
    _, dg, _, _ = p.backward_fields()
    hg = 1e-7
    for c in range(2):
        e = np.zeros(3)
        e[c] = hg
        fd = (ref.forward_fields(0.7, g + e, den, vel, 36, target)[0] -
              ref.forward_fields(0.7, g - e, den, vel, 36, target)[0]) / (2 * hg)
        assert abs(dg[c] - fd) <= tol * abs(fd), (c, dg[c], fd)


def test_field_loss_fn_autograd():
    import torch

    from jyulb.adjoint import field_loss_fn

    p, _, den, vel, target = _lid_case(0, True)
    tau = torch.tensor(0.7, dtype=torch.float64, requires_grad=True)
    g = torch.tensor([3e-6, 0.0, 0.0], dtype=torch.float64, requires_grad=True)
    d = torch.tensor(den, requires_grad=True)
    v = torch.tensor(vel, requires_grad=True)
    L = field_loss_fn(p, tau, g, d, v, target, 20)
    L.backward()
    dtau, dg, dden, dvel = p.backward_fields()
    assert float(tau.grad) == pytest.approx(dtau, rel=1e-12)
    np.testing.assert_allclose(v.grad.numpy(), dvel, rtol=1e-12)
    np.testing.assert_allclose(d.grad.numpy(), dden, rtol=1e-12)


@pytest.mark.parametrize("kind,scheme", [("y", "TRT"), ("z", "TRT"), ("x1", "REG"), ("lid", "TRT"), ("lid", "REG")])
def test_fp64_field_adjoint_matches_torch_autograd(kind, scheme):
    # every entry of d/d den and d/d vel, with tau and g, against autograd
    # through the pure-torch FP64 step, which the oracle pins on the CPU
    # (test_general_torch_step_matches_oracle, same cases)
    import torch

    from jyulb.adjoint import ChannelProblem
    from jyulb.defs import FP64
    from pyoracle import Oracle
    from test_oracle_golden import _field_case
    from torch_lbm import run_fields

    phase, bc, den, vel, sv = _field_case(kind)
    nx, ny, nz = phase.shape
    tau, g, steps, plane = 0.8, np.array([2e-6, -1e-6, 1e-6]), 15, nx // 2 + 1
    magic = 0.25 if scheme == "TRT" else None
    sch = {"TRT": 1, "REG": 2}[scheme]
    rng = np.random.default_rng(8)
    target = 0.01 * rng.standard_normal((ny, nz, 3))
    p = ChannelProblem(phase, bc=bc, rlx_scheme=sch, precision=FP64, trt_magic=magic, loss_plane=plane,
                       checkpoint_every=4, solid_vel=sv)
    L, _ = p.forward_fields(tau, g, den, vel, steps, target)
    dtau, dg, dden, dvel = p.backward_fields()

    o = Oracle(list(phase.shape), sch, (tau - 0.5) / 3.0, list(g), bc, magic or 0.0)
    o.get_phase()[:] = phase
    if sv is not None:
        o.get_vel()[:] = sv
    o.finalize_init()
    t_tau = torch.tensor(tau, dtype=torch.float64, requires_grad=True)
    t_g = torch.tensor(g, requires_grad=True)
    t_den = torch.tensor(den, requires_grad=True)
    t_vel = torch.tensor(vel, requires_grad=True)
    u = run_fields(phase, t_tau, t_g, t_den, t_vel, steps, bc, magic=magic, scheme=scheme, solid_vel=sv,
                   f0=o.populations())
    fl = torch.from_numpy(phase[plane] != 0)
    d = u[:, plane].permute(1, 2, 0) - torch.tensor(target)
    Lt = (d[fl] ** 2).sum()
    Lt.backward()
    lt = float(Lt.detach())
    assert abs(L - lt) <= 1e-10 * abs(lt)
    assert abs(dtau - float(t_tau.grad)) <= 1e-8 * abs(float(t_tau.grad))
    np.testing.assert_allclose(dg, t_g.grad.numpy(), rtol=1e-8, atol=1e-10 * np.abs(t_g.grad.numpy()).max())
    gd, gv = t_den.grad.numpy(), t_vel.grad.numpy()
    np.testing.assert_allclose(dden, gd, rtol=1e-7, atol=1e-9 * max(np.abs(gd).max(), np.abs(gv).max()))
    np.testing.assert_allclose(dvel, gv, rtol=1e-7, atol=1e-9 * max(np.abs(gd).max(), np.abs(gv).max()))
    assert np.abs(gd).max() > 0 and np.abs(gv).max() > 0
