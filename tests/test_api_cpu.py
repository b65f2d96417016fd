"""Host-side tests that need no GPU: the C ABI loads and exports what the
header declares, argument validation matches the reference's messages, and
the NumPy parts of the package (defs, D3Q19, bcs, flow_field) behave like
the reference's."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _lib():
    from jyulb import _native

    return _native.load()


def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "jyulb_gb300.h")).read()
    declared = sorted(set(re.findall(r"\b(jlb_[a-z_0-9]+)\s*\(", hdr)))
    assert declared, "no declarations found"
    lib = _lib()
    for name in declared:
        assert hasattr(lib, name), name
    from jyulb import _native

    assert sorted(_native.EXPORTED_SYMBOLS) == declared


def test_build_info():
    assert b"sm_103a" in _lib().jlb_build_info()


def _cfg(**kw):
    from jyulb import _native

    c = _native.jlb_config()
    c.lat_size[:] = kw.get("lat", [4, 4, 4])
    c.rlx_scheme = kw.get("scheme", 0)
    c.kvisc = kw.get("kvisc", 0.1)
    c.g[:] = kw.get("g", [0, 0, 0])
    c.bc[:] = kw.get("bc", [1] * 6)
    c.precision = kw.get("precision", 0)
    c.trt_magic = kw.get("magic", 0.0)
    return c


@pytest.mark.parametrize("kw,msg", [
    (dict(lat=[0, 4, 4]), "Invalid lattice size input."),
    (dict(scheme=3), "Invalid relaxation scheme input."),
    (dict(kvisc=0.0), "Invalid kinematic viscosity input."),
    (dict(bc=[5, 0, 1, 1, 1, 1]), "Invalid boundary condition input."),
    (dict(bc=[1, 0, 1, 1, 1, 1]), "Invalid periodic bc setup (in x-dir.)."),
    (dict(bc=[0, 0, 1, 0, 1, 1]), "Invalid periodic bc setup (in y-dir.)."),
    (dict(bc=[0, 0, 0, 0, 4, 1]), "Invalid periodic bc setup (in z-dir.)."),
    (dict(bc=[2, 0, 3, 0, 1, 1]), "Invalid fixed variable bc setup."),
    (dict(bc=[0, 0, 0, 2, 3, 0]), "Invalid fixed variable bc setup."),
    (dict(precision=7), "Invalid precision input."),
    (dict(lat=[46341, 46341, 1]), "Lattice too large: nx * ny must stay below 2^31."),
])
def test_c_abi_validation_messages(kw, msg):
    lib = _lib()
    buf = ctypes.create_string_buffer(256)
    rc = lib.jlb_check_config(ctypes.byref(_cfg(**kw)), buf, 256)
    assert rc == -1
    assert buf.value.decode() == msg


def test_c_abi_accepts_valid_configs():
    lib = _lib()
    for bc in ([1] * 6, [0] * 6, [3, 2, 0, 4, 1, 1], [4, 4, 4, 4, 4, 4], [0, 0, 2, 2, 0, 0]):
        assert lib.jlb_check_config(ctypes.byref(_cfg(bc=bc)), None, 0) == 0


@pytest.mark.parametrize("args,msg", [
    (((0, 4, 4),), "Invalid lattice size input."),
    (((4, 4, 4), 5), "Invalid relaxation scheme input."),
    (((4, 4, 4), 0, -1.0), "Invalid kinematic viscosity input."),
    (((4, 4, 4), 0, 0.1, None, [1, 0, 1, 1, 1, 1]), "Invalid periodic bc setup (in x-dir.)."),
    (((4, 4, 4), 0, 0.1, None, [2, 2, 3, 0, 1, 1]), "Invalid fixed variable bc setup."),
    (((65536, 32768, 1),), "Lattice too large: nx * ny must stay below 2^31."),
])
def test_solver_validation_raises_value_error(args, msg):
    from jyulb.isothermal import Solver

    with pytest.raises(ValueError, match=re.escape(msg)):
        Solver(*args)


def test_with_iflow_shape_mismatch():
    from jyulb.isothermal import Solver

    with pytest.raises(ValueError, match="x-dimension"):
        Solver.with_iflow(np.ones((3, 4, 5), np.uint8), np.ones((4, 4, 5)), np.zeros((3, 4, 5, 3)))


def test_solver_fails_loudly_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from jyulb import _native
    from jyulb.isothermal import Solver

    with pytest.raises(_native.EngineUnavailable):
        Solver(np.array([4, 4, 4], dtype=np.int32))
    assert b"CUDA" in _lib().jlb_last_error(None)


def test_defs_values_match_reference_enums():
    from jyulb import defs

    assert (defs.X, defs.Y, defs.Z) == (0, 1, 2)
    assert [defs.FACE_1X, defs.FACE_X1, defs.FACE_1Y, defs.FACE_Y1, defs.FACE_1Z, defs.FACE_Z1] == list(range(6))
    assert (defs.SOLID, defs.FLUID) == (0, 1)
    assert (defs.BGK, defs.TRT, defs.REGULARIZATION) == (0, 1, 2)
    assert (defs.WALL, defs.PERIODIC, defs.FIXED_DEN, defs.FIXED_VEL, defs.SYMMETRIC) == (0, 1, 2, 3, 4)


def test_flow_field_profiles():
    from jyulb import flow_field

    H = 11
    d = np.zeros(H)
    v = np.zeros(H)
    flow_field.poise_plate_steady_state_pgrad(H, 0.2 / 6.0, -1e-5, d, v)
    assert np.allclose(d, np.arange(H) + 0.5 - H / 2)
    umax = 0.5 * (H / 2) ** 2 * 1e-5 / (0.2 / 6.0)
    assert np.allclose(v, umax * (1 - (d / (H / 2)) ** 2))
    v2 = np.zeros(H)
    flow_field.poise_plate_steady_state_umax(H, umax, d, v2)
    assert np.allclose(v, v2)
    vc = np.zeros((H, 2))
    flow_field.couette_plate_steady_state(H, 0.0, 0.0, 1e-5, 2e-5, d, vc)
    assert np.allclose(vc[:, 0], (np.arange(H) + 0.5) * 1e-5 / H)


def test_d3q19_tables_and_projection():
    from jyulb.D3Q19 import D3Q19_H10

    d = D3Q19_H10()
    assert abs(d.LW.sum() - 1.0) < 1e-15
    assert all(d.OPP_LVEC[l] == 18 - l for l in range(19))
    assert np.allclose(d.LW @ np.stack([d.LX, d.LY, d.LZ]).T, 0)
    rng = np.random.default_rng(0)
    den = 1 + 0.01 * rng.standard_normal(5)
    vel = 0.05 * rng.standard_normal((3, 5))
    feq = d.eq(den, vel)
    h = d.f_to_h(feq)
    assert np.allclose(h, d.den_vel_to_heq(den, vel), atol=1e-14)


@pytest.mark.parametrize("method", ["forw_euler_BGK", "forw_euler_TRT", "forw_euler_regul"])
def test_d3q19_collisions_conserve_mass_and_add_force(method):
    from jyulb.D3Q19 import D3Q19_H10

    d = D3Q19_H10()
    rng = np.random.default_rng(1)
    f = d.eq(1 + 0.01 * rng.standard_normal(7), 0.03 * rng.standard_normal((3, 7)))
    f += 1e-4 * rng.standard_normal(f.shape)
    acc = np.array([1e-4, -2e-4, 3e-5])
    den0, mom0 = d.f_to_den_mom(f)
    den, vel, fp = getattr(d, method)(f.copy(), acc, [0.9, 1.1])
    den1, mom1 = d.f_to_den_mom(fp)
    assert np.allclose(den1, den0, atol=1e-15)
    assert np.allclose(mom1, mom0 + den0 * acc[:, None], atol=1e-14)
    assert np.allclose(vel, mom0 / den0 + 0.5 * acc[:, None], atol=1e-15)


@pytest.mark.parametrize("face", range(6))
def test_bcs_zou_he_enforces_velocity_and_density(face):
    from jyulb import bcs
    from jyulb.D3Q19 import D3Q19_H10

    d = D3Q19_H10()
    rng = np.random.default_rng(face)
    f = d.eq(np.full(4, 1.0), 0.02 * rng.standard_normal((3, 4))) + 1e-4 * rng.standard_normal((19, 4))
    v = np.array([0.03, -0.02, 0.01])
    name = ["1x", "x1", "1y", "y1", "1z", "z1"][face]
    g = getattr(bcs, f"fix_vel_face_{name}_D3Q19")(1.0, v, f.copy())
    den, mom = d.f_to_den_mom(g)
    assert np.allclose(mom / den, v[:, None], atol=1e-14)
    g = getattr(bcs, f"fix_den_face_{name}_D3Q19")(1.02, v, f.copy())
    den, mom = d.f_to_den_mom(g)
    assert np.allclose(den, 1.02, atol=1e-14)
    tang = [a for a in range(3) if a != face >> 1]
    assert np.allclose(mom[tang] / 1.02, v[tang, None], atol=1e-14)


def test_loss_fn_backward_differentiates_its_own_forward_run():
    """Two loss_fn graphs on one problem: each backward pass must return the
    gradients of its own loss, although the problem's backward run only
    knows the latest forward run.  A stand-in problem (no GPU) whose
    gradient is the tau of the forward run it follows shows which run each
    backward pass differentiated."""
    torch = pytest.importorskip("torch")
    from jyulb.adjoint import loss_fn

    class FakeProblem:
        def __init__(self):
            self.run_id = 0
            self.last_tau = None
            self.forwards = 0

        def forward(self, tau, g, uin, steps, target=None, rho_out=1.0):
            self.run_id += 1
            self.forwards += 1
            self.last_tau = tau
            return tau * tau, None

        def backward(self):
            return 2.0 * self.last_tau, np.zeros(3), np.zeros((2, 2))

    p = FakeProblem()
    g, uin = torch.zeros(3, dtype=torch.float64), torch.zeros(2, 2, dtype=torch.float64)
    t1 = torch.tensor(0.6, dtype=torch.float64, requires_grad=True)
    t2 = torch.tensor(0.9, dtype=torch.float64, requires_grad=True)
    l1 = loss_fn(p, t1, g, uin, None, 10)
    l2 = loss_fn(p, t2, g, uin, None, 10)
    l1.backward()  # the problem's latest forward run is l2's
    assert abs(float(t1.grad) - 1.2) < 1e-15
    assert p.forwards == 3  # l1's forward run was repeated once
    l2.backward()
    assert abs(float(t2.grad) - 1.8) < 1e-15
    assert p.forwards == 4


def test_new_entry_points_reject_null_handles_without_a_gpu():
    # argument checks come before any CUDA call
    from jyulb import _native

    lib = _lib()
    inv = _native.JLB_ERR_INVALID_ARG
    g = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    loss = ctypes.c_double()
    assert lib.jlb_adj_forward_fields(None, 0.8, g, None, None, 1, None, ctypes.byref(loss), None) == inv
    assert lib.jlb_adj_backward_fields(None, None, None, None, None) == inv
    assert lib.jlb_adj_backward(None, None, None, None) == inv
    h = ctypes.c_void_p()
    ph = np.ones((4, 4, 4), np.uint8)
    assert lib.jlb_adj_create_moving(ctypes.byref(_cfg()), _native.u8ptr(ph), None, 1, 5, ctypes.byref(h)) == inv
    assert b"solid velocity" in lib.jlb_adj_last_error(None)
    assert lib.jlb_batch_set_bc(None, 0, None, None) == inv


def test_field_loss_fn_backward_differentiates_its_own_forward_run():
    """field_loss_fn follows loss_fn's rule for two graphs on one problem."""
    torch = pytest.importorskip("torch")
    from jyulb.adjoint import field_loss_fn

    class FakeProblem:
        def __init__(self):
            self.run_id = 0
            self.last = None
            self.forwards = 0

        def forward_fields(self, tau, g, den, vel, steps, target=None):
            self.run_id += 1
            self.forwards += 1
            self.last = (tau, den.copy(), vel.copy())
            return tau * float(den.sum()), None

        def backward_fields(self):
            tau, den, vel = self.last
            return float(den.sum()), np.zeros(3), np.full(den.shape, tau), np.zeros(vel.shape)

    p = FakeProblem()
    g = torch.zeros(3, dtype=torch.float64)
    d1 = torch.ones(2, 2, 2, dtype=torch.float64, requires_grad=True)
    d2 = torch.full((2, 2, 2), 2.0, dtype=torch.float64, requires_grad=True)
    v = torch.zeros(2, 2, 2, 3, dtype=torch.float64)
    t1 = torch.tensor(0.6, dtype=torch.float64, requires_grad=True)
    t2 = torch.tensor(0.9, dtype=torch.float64, requires_grad=True)
    l1 = field_loss_fn(p, t1, g, d1, v, None, 10)
    l2 = field_loss_fn(p, t2, g, d2, v, None, 10)
    l1.backward()
    assert abs(float(t1.grad) - 8.0) < 1e-15 and np.allclose(d1.grad.numpy(), 0.6)
    assert p.forwards == 3
    l2.backward()
    assert abs(float(t2.grad) - 16.0) < 1e-15 and np.allclose(d2.grad.numpy(), 0.9)
    assert p.forwards == 4
