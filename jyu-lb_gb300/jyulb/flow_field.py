"""Analytic steady flow profiles used to check the solver
(jyulb/flow_field.pyx:20-123).  Plates sit half a lattice spacing outside the
first and last lattice site.  Outputs are written into the caller's arrays.
"""
from __future__ import annotations

import numpy as np


def poise_plate_steady_state_pgrad(H, dvisc, pgrad, centrel_dist, ana_vel):
    """Plane Poiseuille flow driven by the pressure gradient ``pgrad``
    (jyulb/flow_field.pyx:20-49)."""
    H = int(H)
    ch = 0.5 * H
    umax = -0.5 * ch * ch * pgrad / dvisc
    x = np.arange(H, dtype=np.float64)
    d = (0.5 + x) - ch
    centrel_dist[:H] = d
    r = d / ch
    ana_vel[:H] = umax * (1.0 - r * r)


def poise_plate_steady_state_umax(H, umax, centrel_dist, ana_vel):
    """Plane Poiseuille flow with centre-line velocity ``umax``
    (jyulb/flow_field.pyx:55-81)."""
    H = int(H)
    ch = 0.5 * H
    x = np.arange(H, dtype=np.float64)
    d = (0.5 + x) - ch
    centrel_dist[:H] = d
    r = d / ch
    ana_vel[:H] = umax * (1.0 - r * r)


def couette_plate_steady_state(H, low_v1, low_v2, upp_v1, upp_v2, centrel_dist, ana_vel):
    """Plane Couette flow between plates moving tangentially
    (jyulb/flow_field.pyx:87-123); ``ana_vel`` has shape (>= H, 2)."""
    H = int(H)
    ch = 0.5 * H
    g1 = (upp_v1 - low_v1) / float(H)
    g2 = (upp_v2 - low_v2) / float(H)
    x = np.arange(H, dtype=np.float64)
    dl = 0.5 + x
    centrel_dist[:H] = dl - ch
    ana_vel[:H, 0] = low_v1 + dl * g1
    ana_vel[:H, 1] = low_v2 + dl * g2
