"""Lattice-Boltzmann solver for isothermal single-phase flows, D3Q19, on one
GB300 GPU.

Drop-in for ``jyulb.isothermal.Solver`` (jyulb/isothermal.pyx,
jyulb/isothermal.pxd:38-114): same constructors, properties, update methods,
getters and error behaviour; the time-step loop runs as fused AA-pattern CUDA
kernels (libjyulb_gb300.so) instead of the reference's OpenMP pull loop.

The solver owns halo-padded host arrays with the reference's layout --
``phase`` (NI,NJ,NK) uint8, ``den`` (NI,NJ,NK), ``vel``/``acc`` (NI,NJ,NK,3)
float64, k fastest -- and the getters return writable views of their
interior.  They are page-locked when CUDA is present, so the GPU reads and
writes them in place.  As in the reference:

* ``phase`` is read by ``finalize_init``;
* ``den``/``vel`` are the initial field, and ``evolve`` overwrites them on
  fluid sites with the pre-collision density and u = j/den + a/2;
* ``vel`` of solid sites are wall velocities (Ladd's moving bounce-back) and
  ``den``/``vel`` of the Zou-He face layers are the boundary data; both are
  re-read at every ``evolve`` call;
* ``acc`` is added to gravity at every step (read at every ``evolve`` call
  once a view of it has been handed out);
* the halo cells of wall and Zou-He faces, which the reference's getters do
  not reach, keep the values they had at ``finalize_init``.

Additions of this engine (keyword-only): ``precision`` (defs.FP64 / FP32 /
FP16 / FP64_FAST), ``trt_magic`` (TRT magic parameter; None keeps the reference's 3/16) and
``stream`` (a cudaStream_t handle as int to run on; default: the engine's own),
plus ``populations``, ``set_populations``, ``reduce``, ``save_state`` and
``load_state``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from .D3Q19 import D3Q19_H10, LVECS
from .defs import (BGK, FACE_1X, FACE_1Y, FACE_1Z, FACE_X1, FACE_Y1, FACE_Z1, FIXED_DEN,
                   FIXED_VEL, FP16, FP32, FP64, FP64_FAST, PERIODIC, REGULARIZATION, SOLID, SYMMETRIC,
                   TRT, WALL, X, Y, Z)

_ERRS = {
    _native.JLB_ERR_INVALID_ARG: ValueError,
    _native.JLB_ERR_STATE: RuntimeError,
    _native.JLB_ERR_NUMERIC: FloatingPointError,
}


def _host_array(shape, dtype, fill):
    """Page-locked (GPU-addressable) array when CUDA is usable, else plain."""
    try:
        import torch
        if torch.cuda.is_available():
            t = torch.empty(int(np.prod(shape)), dtype={np.uint8: torch.uint8, np.float64: torch.float64}[dtype],
                            pin_memory=True)
            a = t.numpy().reshape(shape)
            a[...] = fill
            return a
    except Exception:
        pass
    return np.full(shape, fill, dtype=dtype)


def check_bc(bc):
    """Boundary-condition validation of the reference (jyulb/isothermal.pyx:378-426);
    raises ValueError with the reference's messages."""
    valid = (WALL, PERIODIC, FIXED_DEN, FIXED_VEL, SYMMETRIC)
    fixed = (FIXED_DEN, FIXED_VEL)
    for s in range(6):
        if bc[s] not in valid:
            raise ValueError('Invalid boundary condition input.')
    for ax, name in ((0, 'x'), (1, 'y'), (2, 'z')):
        a, b = bc[2 * ax], bc[2 * ax + 1]
        if (a == PERIODIC or b == PERIODIC) and a != b:
            raise ValueError(f'Invalid periodic bc setup (in {name}-dir.).')
    fx = [bc[2 * ax] in fixed or bc[2 * ax + 1] in fixed for ax in range(3)]
    for ax in range(3):
        if fx[ax] and any(fx[o] for o in range(3) if o != ax):
            raise ValueError('Invalid fixed variable bc setup.')


class Solver:
    """D3Q19 isothermal lattice-Boltzmann solver (see the module docstring)."""

    def __init__(self, lat_size, rlx_scheme=BGK, kvisc=1.0 / 6.0, g=None, bc=None, *,
                 precision=FP64, trt_magic=None, stream=None, kernel='jyulb', stokes=False,
                 second_order_forcing=False, keep_f2=False):
        self.error_msg = ''
        # the reference's second population buffer is kept only on request
        # (one population download per evolve call; see the f2 property)
        self._keep_f2 = bool(keep_f2)
        self._f2 = None
        lat = [int(v) for v in np.asarray(lat_size).reshape(-1)[:3]]
        # argument checks of jyulb/isothermal.pyx:196-230
        if len(lat) < 3 or lat[X] < 1 or lat[Y] < 1 or lat[Z] < 1:
            self.error_msg = 'Invalid lattice size input.'
            raise ValueError(self.error_msg)
        if lat[X] * lat[Y] >= 2 ** 31:
            # the step kernels index rows of k-lines with 32-bit integers
            self.error_msg = 'Lattice too large: nx * ny must stay below 2^31.'
            raise ValueError(self.error_msg)
        if rlx_scheme not in (BGK, TRT, REGULARIZATION):
            self.error_msg = 'Invalid relaxation scheme input.'
            raise ValueError(self.error_msg)
        if not kvisc > 0.0:
            self.error_msg = 'Invalid kinematic viscosity input.'
            raise ValueError(self.error_msg)
        if precision not in (FP64, FP32, FP16, FP64_FAST):
            raise ValueError('Invalid precision input.')
        self._g = np.zeros(3) if g is None else np.array([g[X], g[Y], g[Z]], dtype=np.float64)
        if bc is None:
            self._bc = [PERIODIC] * 6
        else:
            bcl = [int(b) for b in bc[:6]]
            try:
                check_bc(bcl)
            except ValueError as e:
                self.error_msg = str(e)
                raise
            self._bc = bcl
        self.NI, self.NJ, self.NK = lat[X] + 2, lat[Y] + 2, lat[Z] + 2
        self.NCNT = self.NI * self.NJ * self.NK
        self.kvisc = float(kvisc)
        self.rlx_scheme = int(rlx_scheme)
        self.precision = int(precision)
        self.trt_magic = None if trt_magic is None else float(trt_magic)
        # collision model: 'jyulb' (this package's reference) or 'cxx' (the
        # reference C++ executable's, include/kernel/kernel.cpp:410-550, with
        # its linear "Stokes" equilibrium and second-order forcing switches;
        # kvisc and g are then its dimensionless values and acc holds a
        # force density)
        if kernel not in ('jyulb', 'cxx'):
            raise ValueError('Invalid collision kernel input.')
        self.kernel = kernel
        self.kernel_opts = 0
        if kernel == 'cxx':
            self.kernel_opts = ((_native.JLB_CXX_LINEAR_EQ if stokes else 0) |
                                (_native.JLB_CXX_FORCE2 if second_order_forcing else 0))
        elif stokes or second_order_forcing:
            raise ValueError('Invalid kernel options input.')
        self._stream = stream
        self.tot_tsteps = 0
        self.init_done = 0
        self.dvs = D3Q19_H10()
        sh = (self.NI, self.NJ, self.NK)
        self.phase = _host_array(sh, np.uint8, SOLID)
        self.den = _host_array(sh, np.float64, 1.0)
        self.vel = _host_array(sh + (3,), np.float64, 0.0)
        self._acc = _host_array(sh + (3,), np.float64, 0.0)
        self._acc_exposed = False
        self.fluid_lsite_domain = None
        # relaxation parameters (jyulb/isothermal.pyx:274-287)
        tau_e = 0.5 + self.dvs.AS2 * self.kvisc
        self.rlx_prm = np.zeros(LVECS)
        self.rlx_prm[0] = 1.0 / tau_e
        if rlx_scheme == TRT:
            w = self.rlx_prm[0]
            if self.trt_magic is None:
                self.rlx_prm[1] = 8.0 * (2.0 - w) / (8.0 - w)
            else:
                self.rlx_prm[1] = 1.0 / (self.trt_magic / (tau_e - 0.5) + 0.5)
        self.njump = np.array([(li * self.NJ + lj) * self.NK + lk for li, lj, lk in
                               zip(self.dvs.LI, self.dvs.LJ, self.dvs.LK)], dtype=np.int32)
        self._h = None
        self._lib = None
        self._create_engine()

    # -- construction --------------------------------------------------------
    def _create_engine(self):
        try:
            lib = _native.load()
        except OSError as e:
            raise _native.EngineUnavailable(f'cannot load the CUDA engine: {e}') from e
        cfg = _native.jlb_config()
        cfg.lat_size[:] = [self.NI - 2, self.NJ - 2, self.NK - 2]
        cfg.rlx_scheme = self.rlx_scheme
        cfg.kvisc = self.kvisc
        cfg.g[:] = list(self._g)
        cfg.bc[:] = self._bc
        cfg.precision = self.precision
        cfg.trt_magic = 0.0 if self.trt_magic is None else self.trt_magic
        cfg.kernel = _native.JLB_KERNEL_CXX if self.kernel == 'cxx' else _native.JLB_KERNEL_JYULB
        cfg.kernel_opts = self.kernel_opts
        cfg.stream = None if self._stream is None else int(self._stream)
        h = ctypes.c_void_p()
        rc = lib.jlb_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != _native.JLB_OK:
            msg = lib.jlb_last_error(None).decode()
            if rc == _native.JLB_ERR_INVALID_ARG:
                raise ValueError(msg)
            raise _native.EngineUnavailable(f'CUDA engine unavailable: {msg}')
        self._lib = lib
        self._h = h
        # the getters reach the interior only, as the reference's do, so the
        # halo cells of wall and Zou-He faces keep their initial values and
        # evolve need not re-read their solid velocities
        lib.jlb_set_static_halo(h, 1)

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and self._lib is not None:
            self._lib.jlb_destroy(h)
            self._h = None

    @classmethod
    def with_iflow(cls, phase, iden, ivel, rlx_scheme=BGK, kvisc=1.0 / 6.0, g=None, bc=None, **kw):
        """Solver with the initial flow field prescribed (jyulb/isothermal.pyx:301-360)."""
        phase = np.asarray(phase)
        iden = np.asarray(iden)
        ivel = np.asarray(ivel)
        for ax, name in ((X, 'x'), (Y, 'y'), (Z, 'z')):
            if iden.shape[ax] != phase.shape[ax] or ivel.shape[ax] != phase.shape[ax]:
                raise ValueError('Invalid input for the initial flow field: '
                                 f'array sizes do not match ({name}-dimension)!')
        s = cls(np.array(phase.shape, dtype=np.int32), rlx_scheme, kvisc, g, bc, **kw)
        s.phase[1:-1, 1:-1, 1:-1] = phase
        s.den[1:-1, 1:-1, 1:-1] = iden
        s.vel[1:-1, 1:-1, 1:-1, :] = ivel
        return s

    def _raise(self, rc):
        msg = self._lib.jlb_last_error(self._h).decode()
        raise _ERRS.get(rc, RuntimeError)(msg)

    # -- properties ------------------------------------------------------------
    @property
    def gravity(self):
        return self._g.copy()

    @gravity.setter
    def gravity(self, g):
        self._g[:] = [g[X], g[Y], g[Z]]

    @property
    def g(self):
        return self._g.copy()

    @property
    def bc(self):
        return list(self._bc)

    def _bundle_c(self, f):
        """(19, nx, ny, nz) populations in the reference's Bundle-C layout
        (NCNT*19 values, jyulb/isothermal.pyx:1532-1704), halo entries 0."""
        NI, NJ, NK, N = self.NI, self.NJ, self.NK, self.NCNT
        full = np.zeros((LVECS, NI, NJ, NK))
        full[:, 1:-1, 1:-1, 1:-1] = f
        full = full.reshape(LVECS, N)
        out = np.empty(LVECS * N)
        out[:5 * N].reshape(N, 5)[:] = full[0:5].T
        out[5 * N:14 * N].reshape(N, 9)[:] = full[5:14].T
        out[14 * N:].reshape(N, 5)[:] = full[14:19].T
        return out

    @property
    def f1(self):
        """Post-collision populations of the latest step in the reference's
        Bundle-C layout (NCNT*19 values, jyulb/isothermal.pyx:1532-1704);
        halo entries are 0."""
        return self._bundle_c(self.populations())

    @property
    def f2(self):
        """The reference's second population buffer.  Its evolve swaps f1
        and f2 after every step (jyulb/isothermal.pyx:1410-1416), so f2 holds
        the post-collision populations of the step before the latest one
        (zeros before the first step), in Bundle-C layout; halo entries are 0
        here.  The in-place AA pattern keeps a single lattice, so a Solver
        keeps this copy only when built with keep_f2=True: evolve(n) then
        runs n-1 steps, downloads the populations and runs the last step."""
        if not self._keep_f2:
            raise AttributeError('f2 is kept only by a Solver built with keep_f2=True '
                                 '(the in-place AA pattern has no second lattice)')
        if self._f2 is None:
            return np.zeros(LVECS * self.NCNT)
        return self._bundle_c(self._f2)

    # -- update methods --------------------------------------------------------
    def finalize_init(self):
        """Finish the set-up; returns the number of fluid sites
        (jyulb/isothermal.pyx:1333-1365)."""
        if self.error_occured():
            raise RuntimeError('Invalid solver setup: finalization aborted!')
        if self._acc_exposed and self.kernel == 'cxx':
            # the C++ executable's initial state includes the forcing term
            rc = self._lib.jlb_set_acc(self._h, _native.dptr(self._acc))
            if rc != _native.JLB_OK:
                self._raise(rc)
        n = ctypes.c_uint64()
        rc = self._lib.jlb_finalize_init(self._h, _native.u8ptr(self.phase), _native.dptr(self.den),
                                         _native.dptr(self.vel), ctypes.byref(n))
        if rc != _native.JLB_OK:
            self._raise(rc)
        interior = self.phase[1:-1, 1:-1, 1:-1]
        if n.value >= 1:
            self.fluid_lsite_domain = np.array(np.nonzero(interior), dtype=np.uint32)
        self.init_done = 1
        return int(n.value)

    def evolve(self, tsteps):
        """Advance ``tsteps`` time steps; returns the total step count
        (jyulb/isothermal.pyx:1370-1418)."""
        if self.error_occured():
            raise RuntimeError('Invalid solver setup: evolve aborted!')
        acc = _native.dptr(self._acc) if self._acc_exposed else None
        tsteps = int(tsteps)
        # the engine copies the bc data first, as the reference does before
        # its own checks (jyulb/isothermal.pyx:1398), then raises the
        # reference's RuntimeError if finalize_init has not been called, and
        # returns the step count unchanged on a lattice without fluid sites
        if self.init_done == 0 or self.fluid_lsite_domain is None or not (self._keep_f2 and tsteps > 0):
            self.tot_tsteps = self._jlb_evolve(tsteps, acc)
            return self.tot_tsteps
        if tsteps == 1:
            prev = self.populations()
            self.tot_tsteps = self._jlb_evolve(1, acc)
        else:
            # n-1 steps, a copy of the populations, then the last step on the
            # device with the inputs this call read, as inside one evolve(n)
            self._jlb_evolve(tsteps - 1, acc)
            # the last step's halo rules read step n-1's moments, which the
            # host arrays now hold (jyulb/isothermal.pyx:1408-1411)
            self._enforce_den_vel_per_sym_bc()
            prev = self.populations()
            rc = self._lib.jlb_step(self._h, 1, 1)
            if rc == _native.JLB_OK:
                rc = self._lib.jlb_download_moments(self._h, _native.dptr(self.den), _native.dptr(self.vel))
            if rc != _native.JLB_OK:
                self._raise(rc)
            self.tot_tsteps = int(self._lib.jlb_tot_tsteps(self._h))
        self._f2 = prev
        return self.tot_tsteps

    def _enforce_den_vel_per_sym_bc(self):
        """Periodic copy / symmetric mirror of den and vel into the halo layers
        of the host arrays, face by face in the reference's order and index
        coverage (jyulb/isothermal.pyx:582-686): x faces cover the interior
        (j, k), y faces all i and interior k, z faces all (i, j); a symmetric
        face flips the normal velocity component."""
        for face in range(6):
            b = self._bc[face]
            if b not in (PERIODIC, SYMMETRIC):
                continue
            ax, side = face // 2, face % 2
            n = (self.NI, self.NJ, self.NK)[ax]
            per = b == PERIODIC
            rd, wr = (1, n - 1 if per else 0) if side == 0 else (n - 2, 0 if per else n - 1)
            inner_j, inner_k = slice(1, self.NJ - 1), slice(1, self.NK - 1)
            if ax == 0:
                r, w = (rd, inner_j, inner_k), (wr, inner_j, inner_k)
            elif ax == 1:
                r, w = (slice(None), rd, inner_k), (slice(None), wr, inner_k)
            else:
                r, w = (slice(None), slice(None), rd), (slice(None), slice(None), wr)
            self.den[w] = self.den[r]
            v = self.vel[r].copy()
            if not per:
                v[..., ax] = -v[..., ax]
            self.vel[w] = v

    def _jlb_evolve(self, tsteps, acc):
        tot = ctypes.c_uint32()
        rc = self._lib.jlb_evolve(self._h, tsteps, _native.dptr(self._g), _native.dptr(self.den),
                                  _native.dptr(self.vel), acc, ctypes.byref(tot))
        if rc != _native.JLB_OK:
            self._raise(rc)
        return int(tot.value)

    # -- status ------------------------------------------------------------------
    def error_occured(self):
        return len(self.error_msg)

    # -- equation of state (jyulb/isothermal.pyx:1431-1458) --------------------
    def eos_den2p(self, den):
        return self.dvs.INV_AS2 * den

    def eos_p2den(self, p):
        return self.dvs.AS2 * p

    # -- getters (jyulb/isothermal.pyx:1465-1527) ------------------------------
    def get_phase(self):
        return self.phase[1:-1, 1:-1, 1:-1]

    @property
    def acc(self):
        """Halo-padded acceleration field; once handed out it is re-read at
        every evolve call."""
        self._acc_exposed = True
        return self._acc

    def get_acc(self):
        self._acc_exposed = True
        return self._acc[1:-1, 1:-1, 1:-1, :]

    def get_vel(self):
        return self.vel[1:-1, 1:-1, 1:-1, :]

    def get_den(self):
        return self.den[1:-1, 1:-1, 1:-1]

    def get_fluid_lat_sites(self):
        return self.fluid_lsite_domain

    # -- engine additions --------------------------------------------------------
    def populations(self):
        """Post-collision populations of the latest step, (19, nx, ny, nz) FP64,
        lattice vectors in the reference's order."""
        self._need_init()
        f = np.empty((LVECS, self.NI - 2, self.NJ - 2, self.NK - 2))
        rc = self._lib.jlb_get_populations(self._h, _native.dptr(f))
        if rc != _native.JLB_OK:
            self._raise(rc)
        return f

    def set_populations(self, f):
        """Overwrite the populations with post-collision values (same layout)."""
        self._need_init()
        f = np.ascontiguousarray(f, dtype=np.float64)
        if f.shape != (LVECS, self.NI - 2, self.NJ - 2, self.NK - 2):
            raise ValueError('populations must have shape (19, nx, ny, nz)')
        rc = self._lib.jlb_set_populations(self._h, _native.dptr(f))
        if rc != _native.JLB_OK:
            self._raise(rc)

    def save_state(self):
        """Snapshot for restart: populations, den/vel and the step count."""
        return {'f': self.populations(), 'den': self.den.copy(), 'vel': self.vel.copy(),
                'tot_tsteps': self.tot_tsteps}

    def load_state(self, state):
        self.set_populations(state['f'])
        self.den[...] = state['den']
        self.vel[...] = state['vel']
        self.tot_tsteps = int(state['tot_tsteps'])

    def reduce(self):
        """FP64 sums over fluid sites of the last stored moments: mass,
        momentum (den*u) and velocity."""
        self._need_init()
        out = np.zeros(8)
        rc = self._lib.jlb_reduce(self._h, _native.dptr(out))
        if rc != _native.JLB_OK:
            self._raise(rc)
        return {'mass': out[0], 'momentum': out[1:4].copy(), 'vel_sum': out[4:7].copy()}

    def residual(self):
        """Steady-state convergence residual ||u - u_prev|| / ||u|| over fluid
        sites, u_prev being the velocity at the previous call (zero before
        the first); FP64 sums on the GPU."""
        self._need_init()
        out = np.zeros(1)
        rc = self._lib.jlb_residual(self._h, _native.dptr(out))
        if rc != _native.JLB_OK:
            self._raise(rc)
        return float(out[0])

    FLOW_INFO_KEYS = ('tot_den', 'tot_jx', 'tot_jy', 'tot_jz', 'tot_j2', 'ave_ux', 'ave_uy', 'ave_uz', 'ave_u2',
                      'max_u2', 'max_den', 'min_den')

    def flow_info(self, ref_den=1.0):
        """Flow information of the last step, as the C++ executable's
        IsothermalSolver::calc_flow_info (include/solver/solver.cpp:64-129):
        sums of den, den*u and den*|u|, means of u and |u|, max |u| and the
        density extremes over fluid sites (``*_u2`` are speeds |u|, as
        there).  Computed in FP64 on the GPU."""
        self._need_init()
        out = np.zeros(12)
        rc = self._lib.jlb_flow_info(self._h, float(ref_den), _native.dptr(out))
        if rc != _native.JLB_OK:
            self._raise(rc)
        return dict(zip(self.FLOW_INFO_KEYS, (float(v) for v in out)))

    # bc_data_den_face_* / bc_data_vel_face_* (jyulb/isothermal.pxd:159-171):
    # the face layers of den and vel that the last evolve call read
    def _bc_data(self, face):
        ax = face // 2
        na = self.NJ if ax == 0 else self.NI
        nb = self.NJ if ax == 2 else self.NK
        den = np.empty((na, nb))
        vel = np.empty((na, nb, 3))
        rc = self._lib.jlb_bc_data(self._h, face, _native.dptr(den), _native.dptr(vel))
        if rc != _native.JLB_OK:
            self._raise(rc)
        den.flags.writeable = False
        vel.flags.writeable = False
        return den, vel

    @property
    def kernel_launches(self):
        return int(self._lib.jlb_kernel_launches(self._h))

    @property
    def transfer_bytes(self):
        """(host-to-device, device-to-host) bytes moved by the engine so far."""
        out = (ctypes.c_uint64 * 2)()
        self._lib.jlb_transfer_bytes(self._h, out)
        return int(out[0]), int(out[1])

    def _need_init(self):
        if not self.init_done:
            raise RuntimeError('finalize_init has not been called')


def _bc_data_property(face, which):
    def get(self):
        return self._bc_data(face)[which]
    name = ("den", "vel")[which]
    get.__doc__ = (f"Readonly copy of the {name} face layer of face {_FACE_NAMES[face]} read by the last "
                   "evolve call (den = 1, vel = 0 before the first and on faces the reference does not refresh).")
    return property(get)


_FACE_NAMES = ("1X", "X1", "1Y", "Y1", "1Z", "Z1")
for _face, _name in enumerate(_FACE_NAMES):
    setattr(Solver, f"bc_data_den_face_{_name}", _bc_data_property(_face, 0))
    setattr(Solver, f"bc_data_vel_face_{_name}", _bc_data_property(_face, 1))
del _face, _name
