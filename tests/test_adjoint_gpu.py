"""The hand-written adjoint (jyulb.adjoint) against torch autograd through a
pure-torch FP64 step and against central finite differences.

Problem: a channel with a cylinder (axis z), Zou-He velocity inlet with a
u_x parameter per inlet site, density outlet, walls in y, periodic z; TRT
(magic 1/4) or BGK with a body force; loss = sum |u - target|^2 on one x
plane after the last step.  Checkpoint intervals that do not divide the step
count exercise partial segments and odd parities.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def setup(seed=0, shape=(16, 10, 6), r=2.0):
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    cyl = (X - nx * 0.4) ** 2 + (Y - ny * 0.5) ** 2 <= r * r
    phase = np.ones(shape, np.uint8)
    phase[cyl] = 0
    uin = 0.02 + 0.005 * rng.standard_normal((ny, nz))
    target = 0.01 * rng.standard_normal((ny, nz, 3))
    return phase, uin, target


def torch_grads(phase, tau, g, uin, target, steps, plane, scheme, magic, zwall=False, zsym=False):
    import torch

    from torch_lbm import run

    t_tau = torch.tensor(tau, dtype=torch.float64, requires_grad=True)
    t_g = torch.tensor(g, dtype=torch.float64, requires_grad=True)
    t_uin = torch.tensor(uin, dtype=torch.float64, requires_grad=True)
    u = run(phase, t_tau, t_g, t_uin, steps, magic=magic, scheme=scheme, periodic=(False, False, not zwall),
            zsym=zsym)
    fl = torch.from_numpy(phase[plane] != 0)
    d = u[:, plane].permute(1, 2, 0) - torch.tensor(target)
    L = (d[fl] ** 2).sum()
    L.backward()
    return float(L.detach()), float(t_tau.grad), t_g.grad.numpy(), t_uin.grad.numpy()


@pytest.mark.parametrize("scheme,zb_name", [("TRT", "periodic"), ("BGK", "periodic"), ("TRT", "wall"),
                                            ("REG", "periodic"), ("REG", "wall"), ("TRT", "symmetric"),
                                            ("REG", "symmetric")])
def test_fp64_adjoint_matches_torch_autograd(scheme, zb_name):
    from jyulb.adjoint import ChannelProblem
    from jyulb.defs import BGK, FIXED_DEN, FIXED_VEL, FP64, PERIODIC, REGULARIZATION, SYMMETRIC, TRT, WALL

    zwall, zsym = zb_name == "wall", zb_name == "symmetric"
    phase, uin, target = setup(1)
    tau, g, steps, plane = 0.8, np.array([1e-5, 2e-6, 1e-6 if (zwall or zsym) else 0.0]), 30, 12
    magic = 0.25 if scheme == "TRT" else None
    zb = WALL if zwall else SYMMETRIC if zsym else PERIODIC
    sch = {"TRT": TRT, "BGK": BGK, "REG": REGULARIZATION}[scheme]
    p = ChannelProblem(phase, bc=[FIXED_VEL, FIXED_DEN, WALL, WALL, zb, zb], rlx_scheme=sch,
                       precision=FP64, trt_magic=magic, loss_plane=plane, checkpoint_every=7)
    L, _ = p.forward(tau, g, uin, steps, target)
    dtau, dg, duin = p.backward()
    Lt, dtau_t, dg_t, duin_t = torch_grads(phase, tau, g, uin, target, steps, plane, scheme, magic, zwall, zsym)
    assert abs(L - Lt) <= 1e-10 * abs(Lt)
    assert abs(dtau - dtau_t) <= 1e-8 * abs(dtau_t)
    nd = 3 if (zwall or zsym) else 2
    np.testing.assert_allclose(dg[:nd], dg_t[:nd], rtol=1e-8)
    np.testing.assert_allclose(duin, duin_t, rtol=1e-7, atol=1e-9 * np.abs(duin_t).max())


def test_fp64_adjoint_rows_of_96_sites():
    # nz = 96: the reverse kernel's row blocks have 96 threads, and its
    # boundary-node blocks (the Zou-He inlet and outlet, 2 x 4 x 96 nodes)
    # must be counted in blocks of 96
    from jyulb.adjoint import ChannelProblem
    from jyulb.defs import FIXED_DEN, FIXED_VEL, FP64, PERIODIC, TRT, WALL

    phase, uin, target = setup(4, shape=(10, 4, 96), r=1.0)
    tau, g, steps, plane = 0.8, np.array([1e-5, 0.0, 0.0]), 14, 7
    p = ChannelProblem(phase, bc=[FIXED_VEL, FIXED_DEN, WALL, WALL, PERIODIC, PERIODIC], rlx_scheme=TRT,
                       precision=FP64, trt_magic=0.25, loss_plane=plane, checkpoint_every=5)
    L, _ = p.forward(tau, g, uin, steps, target)
    dtau, dg, duin = p.backward()
    Lt, dtau_t, dg_t, duin_t = torch_grads(phase, tau, g, uin, target, steps, plane, "TRT", 0.25)
    assert abs(L - Lt) <= 1e-10 * abs(Lt)
    assert abs(dtau - dtau_t) <= 1e-8 * abs(dtau_t)
    np.testing.assert_allclose(duin, duin_t, rtol=1e-7, atol=1e-9 * np.abs(duin_t).max())


@pytest.mark.parametrize("scheme", [1, 2])
# FP32: the adjoint of the FP32 model against differences of the FP64 model,
# so the bound covers both the adjoint and the FP32 model's rounding (measured
# <= 1e-6 here, 4e-5 on a 40x16x8 channel over 300 steps)
@pytest.mark.parametrize("precision,tol", [(0, 1e-6), (1, 1e-4)])
def test_adjoint_matches_central_differences(precision, tol, scheme):
    from jyulb.adjoint import ChannelProblem
    from jyulb.defs import FP64

    phase, uin, target = setup(2, shape=(20, 12, 4))
    tau, g, steps, plane = 0.7, np.array([5e-6, 0.0, 0.0]), 40, 15
    magic = 0.25 if scheme == 1 else None
    p = ChannelProblem(phase, rlx_scheme=scheme, precision=precision, trt_magic=magic, loss_plane=plane,
                       checkpoint_every=8)
    p.forward(tau, g, uin, steps, target)
    dtau, dg, duin = p.backward()
    ref = ChannelProblem(phase, rlx_scheme=scheme, precision=FP64, trt_magic=magic, loss_plane=plane,
                         checkpoint_every=8)

    def L(tau_, g_, uin_):
        return ref.forward(tau_, g_, uin_, steps, target)[0]

    h = 1e-5
    fd_tau = (L(tau + h, g, uin) - L(tau - h, g, uin)) / (2 * h)
    assert abs(dtau - fd_tau) <= tol * abs(fd_tau)
    hg = 1e-7
    e = np.array([hg, 0.0, 0.0])
    fd_gx = (L(tau, g + e, uin) - L(tau, g - e, uin)) / (2 * hg)
    assert abs(dg[0] - fd_gx) <= tol * abs(fd_gx)
    for (j, k) in [(3, 1), (6, 2), (9, 0)]:
        du = np.zeros_like(uin)
        du[j, k] = 1e-6
        fd = (L(tau, g, uin + du) - L(tau, g, uin - du)) / 2e-6
        assert abs(duin[j, k] - fd) <= tol * max(abs(fd), 1e-3 * np.abs(duin).max()), (j, k, duin[j, k], fd)


def test_autograd_function_end_to_end():
    import torch

    from jyulb.adjoint import ChannelProblem, loss_fn
    from jyulb.defs import FP64, TRT

    phase, uin, target = setup(3)
    p = ChannelProblem(phase, rlx_scheme=TRT, precision=FP64, trt_magic=0.25, loss_plane=11, checkpoint_every=5)
    tau = torch.tensor(0.9, dtype=torch.float64, requires_grad=True)
    g = torch.tensor([1e-5, 0.0, 0.0], dtype=torch.float64, requires_grad=True)
    u = torch.tensor(uin, dtype=torch.float64, requires_grad=True)
    L = loss_fn(p, tau, g, u, target, 20)
    L.backward()
    dtau, dg, duin = p.backward()
    assert float(tau.grad) == pytest.approx(dtau, rel=1e-12)
    np.testing.assert_allclose(u.grad.numpy(), duin, rtol=1e-12)
