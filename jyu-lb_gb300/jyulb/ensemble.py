"""Batched ensembles: many independent D3Q19 domains of uneven size,
relaxation time, body force and boundary set advanced together on one GPU.

The reference advances one ``Solver`` at a time (jyulb/isothermal.pyx:
1370-1418); an ensemble there is a Python loop over Solver objects.  Here all
domains share one packed node index, one FP32-shifted population array and one
kernel launch per time step (graph-replayed), with the block size chosen by a
timing autotuner at set-up.

Each domain is described like a Solver: interior ``phase``, ``den`` and
``vel`` arrays (k fastest), ``kvisc``, gravity ``g`` and per-face ``bc``
(WALL, PERIODIC, FIXED_DEN, FIXED_VEL or SYMMETRIC).  ``vel`` on solid sites
gives moving walls (Ladd's term).  Zou-He faces take their data from ``den``
and ``vel`` once, at set-up (a Solver re-reads them at every evolve call).
The boundary nodes of domains with Zou-He or symmetric faces, or with
moving solids of more than one velocity, run the single-domain
boundary-node path in a second launch per step.  The relaxation scheme is
common to the ensemble.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from .defs import BGK, PERIODIC


class Domain:
    def __init__(self, phase, den=None, vel=None, kvisc=1.0 / 6.0, g=None, bc=None, trt_magic=None):
        self.phase = np.ascontiguousarray(phase, dtype=np.uint8)
        if self.phase.ndim != 3:
            raise ValueError('phase must be a 3-D array')
        sh = self.phase.shape
        self.den = None if den is None else np.ascontiguousarray(den, dtype=np.float64)
        self.vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64)
        if self.den is not None and self.den.shape != sh:
            raise ValueError('den must match phase')
        if self.vel is not None and self.vel.shape != sh + (3,):
            raise ValueError('vel must have shape phase.shape + (3,)')
        self.kvisc = float(kvisc)
        self.g = np.zeros(3) if g is None else np.asarray(g, dtype=np.float64)
        self.bc = [PERIODIC] * 6 if bc is None else [int(b) for b in bc]
        self.trt_magic = trt_magic


class Ensemble:
    """All domains advance together: ``Ensemble(domains, rlx_scheme).evolve(n)``."""

    def __init__(self, domains, rlx_scheme=BGK, stream=None):
        self._lib = _native.load()
        self.domains = list(domains)
        self.rlx_scheme = int(rlx_scheme)
        n = len(self.domains)
        arr = (_native.jlb_domain * n)()
        for i, d in enumerate(self.domains):
            c = arr[i]
            c.lat_size[:] = list(d.phase.shape)
            c.kvisc = d.kvisc
            c.g[:] = list(d.g)
            c.bc[:] = d.bc
            c.trt_magic = 0.0 if d.trt_magic is None else float(d.trt_magic)
            c.phase = _native.u8ptr(d.phase)
            c.den = _native.dptr(d.den) if d.den is not None else None
            c.vel = _native.dptr(d.vel) if d.vel is not None else None
        h = ctypes.c_void_p()
        rc = self._lib.jlb_batch_create(self.rlx_scheme, arr, n, None if stream is None else int(stream),
                                        ctypes.byref(h))
        if rc != _native.JLB_OK:
            msg = self._lib.jlb_batch_last_error(None).decode()
            raise (ValueError if rc == _native.JLB_ERR_INVALID_ARG else RuntimeError)(msg)
        self._h = h
        self.tot_tsteps = 0

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None:
            self._lib.jlb_batch_destroy(h)
            self._h = None

    def _check(self, rc):
        if rc != _native.JLB_OK:
            raise RuntimeError(self._lib.jlb_batch_last_error(self._h).decode())

    def evolve(self, tsteps):
        self._check(self._lib.jlb_batch_step(self._h, int(tsteps)))
        self.tot_tsteps += int(tsteps)
        return self.tot_tsteps

    def set_bc(self, d, den=None, vel=None):
        """Zou-He data of domain d from den (nx,ny,nz) / vel (nx,ny,nz,3) at
        its boundary sites, as Solver.evolve re-reads them at every call; den
        also becomes the sites' previous-step density (moving solids' Ladd
        term).  None keeps that field's current values."""
        sh = self.domains[d].phase.shape
        dd = None if den is None else np.ascontiguousarray(den, dtype=np.float64).reshape(sh)
        vv = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(sh + (3,))
        self._check(self._lib.jlb_batch_set_bc(self._h, d, _native.dptr(dd) if dd is not None else None,
                                               _native.dptr(vv) if vv is not None else None))

    def moments(self, d):
        """(den, vel) of domain d after the last step; solid sites keep the
        domain's input values."""
        dom = self.domains[d]
        sh = dom.phase.shape
        den = np.ones(sh) if dom.den is None else dom.den.copy()
        vel = np.zeros(sh + (3,)) if dom.vel is None else dom.vel.copy()
        self._check(self._lib.jlb_batch_moments(self._h, d, _native.dptr(den), _native.dptr(vel)))
        return den, vel

    def populations(self, d):
        sh = self.domains[d].phase.shape
        f = np.empty((19,) + sh)
        self._check(self._lib.jlb_batch_populations(self._h, d, _native.dptr(f)))
        return f

    def info(self):
        out = (ctypes.c_int64 * 8)()
        self._check(self._lib.jlb_batch_info(self._h, out))
        return {'sites': out[0], 'fluid_sites': out[1], 'block': out[2], 'tiles': out[3],
                'launches': out[4], 'tune_us_per_step': {64: out[5], 128: out[6], 256: out[7]}}

    def fluid_sites(self, d):
        return int(self._lib.jlb_batch_domain_fluid(self._h, d))
