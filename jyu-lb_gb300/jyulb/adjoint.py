"""Gradients of a velocity-field loss through the D3Q19 time step.

``ChannelProblem`` is a domain (BGK, TRT or regularized; FP32-shifted or FP64) started from
rest, with immobile or moving solids (``solid_vel``: Ladd's moving bounce-back)
and Zou-He faces.  ``forward`` takes the u_x of each site of a FIXED_VEL inlet
on face 1X as the parameter; ``forward_fields`` takes the den / vel values that
every fixed face reads at its boundary sites, on any of the six faces.  The
forward run advances ``steps`` steps and scores the stored velocity
on the plane x = ``loss_plane``:  L = sum over fluid sites of |u - target|^2.
The backward run is the hand-written discrete adjoint of the fused step
(reverse AA sweep with the transposed collision, Zou-He and bounce-back
maps), with checkpoints every ``checkpoint_every`` steps and recomputation
in between.  ``loss_fn`` wraps both in a ``torch.autograd.Function`` whose
inputs are the relaxation time ``tau``, the body force ``g`` (3,) and the
inlet velocities ``uin`` (ny, nz); ``field_loss_fn`` takes ``den`` (nx, ny, nz)
and ``vel`` (nx, ny, nz, 3) in place of ``uin``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from .defs import FIXED_DEN, FIXED_VEL, FP32, TRT, WALL, PERIODIC


class ChannelProblem:
    def __init__(self, phase, bc=None, rlx_scheme=TRT, precision=FP32, trt_magic=None, loss_plane=None,
                 checkpoint_every=50, stream=None, solid_vel=None):
        self._lib = _native.load()
        self.phase = np.ascontiguousarray(phase, dtype=np.uint8)
        nx, ny, nz = self.phase.shape
        self.shape = (nx, ny, nz)
        self.bc = [FIXED_VEL, FIXED_DEN, WALL, WALL, PERIODIC, PERIODIC] if bc is None else [int(b) for b in bc]
        self.loss_plane = int(nx * 3 // 4 if loss_plane is None else loss_plane)
        cfg = _native.jlb_config()
        cfg.lat_size[:] = [nx, ny, nz]
        cfg.rlx_scheme = int(rlx_scheme)
        cfg.kvisc = 0.1  # replaced by tau at every forward run
        cfg.g[:] = [0.0, 0.0, 0.0]
        cfg.bc[:] = self.bc
        cfg.precision = int(precision)
        cfg.trt_magic = 0.0 if trt_magic is None else float(trt_magic)
        cfg.stream = None if stream is None else int(stream)
        h = ctypes.c_void_p()
        if solid_vel is None:
            rc = self._lib.jlb_adj_create(ctypes.byref(cfg), _native.u8ptr(self.phase), self.loss_plane,
                                          int(checkpoint_every), ctypes.byref(h))
        else:
            sv = np.ascontiguousarray(solid_vel, dtype=np.float64).reshape(nx, ny, nz, 3)
            rc = self._lib.jlb_adj_create_moving(ctypes.byref(cfg), _native.u8ptr(self.phase), _native.dptr(sv),
                                                 self.loss_plane, int(checkpoint_every), ctypes.byref(h))
        if rc != _native.JLB_OK:
            raise (ValueError if rc == _native.JLB_ERR_INVALID_ARG else RuntimeError)(
                self._lib.jlb_adj_last_error(None).decode())
        self._h = h
        self.steps = 0
        self.run_id = 0  # counts forward runs; backward() differentiates the last one

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None:
            self._lib.jlb_adj_destroy(h)
            self._h = None

    def _check(self, rc):
        if rc != _native.JLB_OK:
            raise RuntimeError(self._lib.jlb_adj_last_error(self._h).decode())

    def forward(self, tau, g, uin, steps, target=None, rho_out=1.0):
        """Runs the forward model; returns (loss, u on the loss plane)."""
        _, ny, nz = self.shape
        g = np.ascontiguousarray(g, dtype=np.float64).reshape(3)
        uin = np.ascontiguousarray(uin, dtype=np.float64).reshape(ny, nz)
        tgt = None if target is None else np.ascontiguousarray(target, dtype=np.float64).reshape(ny, nz, 3)
        loss = ctypes.c_double()
        up = np.zeros((ny, nz, 3))
        self._check(self._lib.jlb_adj_forward(self._h, float(tau), _native.dptr(g), _native.dptr(uin),
                                              float(rho_out), int(steps),
                                              _native.dptr(tgt) if tgt is not None else None,
                                              ctypes.byref(loss), _native.dptr(up)))
        self.steps = int(steps)
        self.run_id += 1
        return float(loss.value), up

    def backward(self):
        """Gradients of the last forward run's loss: (dtau, dg (3,), duin (ny,nz))."""
        _, ny, nz = self.shape
        dtau = ctypes.c_double()
        dg = np.zeros(3)
        duin = np.zeros((ny, nz))
        self._check(self._lib.jlb_adj_backward(self._h, ctypes.byref(dtau), _native.dptr(dg), _native.dptr(duin)))
        return float(dtau.value), dg, duin

    def forward_fields(self, tau, g, den, vel, steps, target=None):
        """Forward run that reads den (nx,ny,nz) and vel (nx,ny,nz,3) where
        Solver.evolve reads them: the Zou-He data at the boundary sites of the
        fixed faces, and the first step's previous-step density of the sites
        next to moving solids (None: 1 and 0); returns (loss, u on the loss
        plane)."""
        nx, ny, nz = self.shape
        g = np.ascontiguousarray(g, dtype=np.float64).reshape(3)
        d = None if den is None else np.ascontiguousarray(den, dtype=np.float64).reshape(nx, ny, nz)
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(nx, ny, nz, 3)
        tgt = None if target is None else np.ascontiguousarray(target, dtype=np.float64).reshape(ny, nz, 3)
        loss = ctypes.c_double()
        up = np.zeros((ny, nz, 3))
        self._check(self._lib.jlb_adj_forward_fields(
            self._h, float(tau), _native.dptr(g), _native.dptr(d) if d is not None else None,
            _native.dptr(v) if v is not None else None, int(steps),
            _native.dptr(tgt) if tgt is not None else None, ctypes.byref(loss), _native.dptr(up)))
        self.steps = int(steps)
        self.run_id += 1
        return float(loss.value), up

    def backward_fields(self):
        """Gradients of the last forward run's loss: (dtau, dg (3,), dden
        (nx,ny,nz), dvel (nx,ny,nz,3)), the last two non-zero at the sites of
        the faces whose data are parameters."""
        nx, ny, nz = self.shape
        dtau = ctypes.c_double()
        dg = np.zeros(3)
        dden = np.zeros((nx, ny, nz))
        dvel = np.zeros((nx, ny, nz, 3))
        self._check(self._lib.jlb_adj_backward_fields(self._h, ctypes.byref(dtau), _native.dptr(dg),
                                                      _native.dptr(dden), _native.dptr(dvel)))
        return float(dtau.value), dg, dden, dvel


    def timers(self):
        """Device milliseconds of the last runs: forward, recompute, reverse
        sweep, whole backward."""
        out = np.zeros(4)
        self._check(self._lib.jlb_adj_timers(self._h, _native.dptr(out)))
        return {"forward": out[0], "recompute": out[1], "reverse": out[2], "backward": out[3]}


def loss_fn(problem, tau, g, uin, target, steps, rho_out=1.0):
    """L(tau, g, uin) as a differentiable torch scalar (torch tensors in,
    gradients from the adjoint).

    The problem's backward run differentiates its latest forward run.  When
    another forward run on the same problem came after this node's (two
    loss_fn graphs on one problem), the backward pass first repeats this
    node's forward run with its own inputs, so every node gets the gradients
    of its own loss."""
    import torch

    class _AdjointLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, tau_t, g_t, uin_t):
            args = (float(tau_t.detach().cpu()), g_t.detach().cpu().double().numpy(),
                    uin_t.detach().cpu().double().numpy())
            loss, _ = problem.forward(*args, steps, target, rho_out)
            ctx.dev, ctx.dtype = tau_t.device, tau_t.dtype
            ctx.args = args
            ctx.run_id = problem.run_id
            return torch.tensor(loss, dtype=torch.float64, device=tau_t.device)

        @staticmethod
        def backward(ctx, grad_out):
            if problem.run_id != ctx.run_id:
                problem.forward(*ctx.args, steps, target, rho_out)
                ctx.run_id = problem.run_id
            dtau, dg, duin = problem.backward()
            s = float(grad_out)
            return (torch.tensor(s * dtau, dtype=torch.float64, device=ctx.dev),
                    torch.tensor(s * dg, dtype=torch.float64, device=ctx.dev),
                    torch.tensor(s * duin, dtype=torch.float64, device=ctx.dev))

    return _AdjointLoss.apply(tau, g, uin)


def field_loss_fn(problem, tau, g, den, vel, target, steps):
    """L(tau, g, den, vel) as a differentiable torch scalar: ``loss_fn`` with
    the Zou-He data of every fixed face taken from den (nx, ny, nz) and vel
    (nx, ny, nz, 3) at its boundary sites (``ChannelProblem.forward_fields``).
    The same rule for repeated forward runs on one problem applies."""
    import torch

    class _AdjointFieldLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, tau_t, g_t, den_t, vel_t):
            args = (float(tau_t.detach().cpu()), g_t.detach().cpu().double().numpy(),
                    den_t.detach().cpu().double().numpy(), vel_t.detach().cpu().double().numpy())
            loss, _ = problem.forward_fields(*args, steps, target)
            ctx.dev = tau_t.device
            ctx.args = args
            ctx.run_id = problem.run_id
            return torch.tensor(loss, dtype=torch.float64, device=tau_t.device)

        @staticmethod
        def backward(ctx, grad_out):
            if problem.run_id != ctx.run_id:
                problem.forward_fields(*ctx.args, steps, target)
                ctx.run_id = problem.run_id
            dtau, dg, dden, dvel = problem.backward_fields()
            s = float(grad_out)
            return tuple(torch.tensor(s * np.asarray(x), dtype=torch.float64, device=ctx.dev)
                         for x in (dtau, dg, dden, dvel))

    return _AdjointFieldLoss.apply(tau, g, den, vel)
