"""Zou-He fixed density / fixed velocity boundary maps for D3Q19
(jyulb/bcs.pyx:31-716), as NumPy functions.

Each ``fix_{den,vel}_face_<f>_D3Q19(den, vel, f)`` takes post-streaming
populations ``f`` of shape (19, ...) at nodes of face <f> and overwrites the
five unknown populations in place, exactly as the reference's C-level
functions do for one node.  ``den`` may be a scalar or an array over the
trailing node shape; ``vel`` has shape (3, ...).  The GPU time step applies
the same maps inside its boundary-node path.
"""
from __future__ import annotations

import numpy as np

# populations with zero normal component and leaving through each face,
# per face 1X, X1, 1Y, Y1, 1Z, Z1
_ZERO = [(5, 6, 7, 8, 9, 10, 11, 12, 13)] * 2 + [(1, 2, 3, 8, 9, 10, 15, 16, 17)] * 2 + \
        [(0, 2, 4, 6, 9, 12, 14, 16, 18)] * 2
_OUT = [(0, 1, 2, 3, 4), (14, 15, 16, 17, 18), (0, 5, 6, 7, 14), (4, 11, 12, 13, 18),
        (1, 5, 8, 11, 15), (3, 7, 10, 13, 17)]


def _assign(face, jx, jy, jz, f):
    """Unknown populations of the Zou-He scheme (jyulb/bcs.pyx:487-716)."""
    s6, s3 = 1.0 / 6.0, 1.0 / 3.0
    if face == 0:
        t = f[11] + f[12] + f[13] - f[5] - f[6] - f[7]
        u = f[7] + f[10] + f[13] - f[5] - f[8] - f[11]
        f[14] = f[4] + s6 * jx + 0.5 * t - 0.5 * jy
        f[18] = f[0] + s6 * jx - 0.5 * t + 0.5 * jy
        f[15] = f[3] + s6 * jx + 0.5 * u - 0.5 * jz
        f[17] = f[1] + s6 * jx - 0.5 * u + 0.5 * jz
        f[16] = f[2] + s3 * jx
    elif face == 1:
        t = f[11] + f[12] + f[13] - f[5] - f[6] - f[7]
        u = f[7] + f[10] + f[13] - f[5] - f[8] - f[11]
        f[0] = f[18] - s6 * jx + 0.5 * t - 0.5 * jy
        f[4] = f[14] - s6 * jx - 0.5 * t + 0.5 * jy
        f[1] = f[17] - s6 * jx + 0.5 * u - 0.5 * jz
        f[3] = f[15] - s6 * jx - 0.5 * u + 0.5 * jz
        f[2] = f[16] - s3 * jx
    elif face == 2:
        t = f[15] + f[16] + f[17] - f[1] - f[2] - f[3]
        u = f[17] + f[10] + f[3] - f[15] - f[8] - f[1]
        f[4] = f[14] + s6 * jy + 0.5 * t - 0.5 * jx
        f[18] = f[0] + s6 * jy - 0.5 * t + 0.5 * jx
        f[11] = f[7] + s6 * jy + 0.5 * u - 0.5 * jz
        f[13] = f[5] + s6 * jy - 0.5 * u + 0.5 * jz
        f[12] = f[6] + s3 * jy
    elif face == 3:
        t = f[15] + f[16] + f[17] - f[1] - f[2] - f[3]
        u = f[17] + f[10] + f[3] - f[15] - f[8] - f[1]
        f[0] = f[18] - s6 * jy + 0.5 * t - 0.5 * jx
        f[14] = f[4] - s6 * jy - 0.5 * t + 0.5 * jx
        f[5] = f[13] - s6 * jy + 0.5 * u - 0.5 * jz
        f[7] = f[11] - s6 * jy - 0.5 * u + 0.5 * jz
        f[6] = f[12] - s3 * jy
    elif face == 4:
        t = f[18] + f[16] + f[14] - f[4] - f[2] - f[0]
        u = f[18] + f[12] + f[4] - f[14] - f[6] - f[0]
        f[3] = f[15] + s6 * jz + 0.5 * t - 0.5 * jx
        f[17] = f[1] + s6 * jz - 0.5 * t + 0.5 * jx
        f[7] = f[11] + s6 * jz + 0.5 * u - 0.5 * jy
        f[13] = f[5] + s6 * jz - 0.5 * u + 0.5 * jy
        f[10] = f[8] + s3 * jz
    else:
        t = f[18] + f[16] + f[14] - f[4] - f[2] - f[0]
        u = f[18] + f[12] + f[4] - f[14] - f[6] - f[0]
        f[1] = f[17] - s6 * jz + 0.5 * t - 0.5 * jx
        f[15] = f[3] - s6 * jz - 0.5 * t + 0.5 * jx
        f[5] = f[13] - s6 * jz + 0.5 * u - 0.5 * jy
        f[11] = f[7] - s6 * jz - 0.5 * u + 0.5 * jy
        f[8] = f[10] - s3 * jz
    return f


def _fix_den(face, den, vel, f):
    ax, high = face >> 1, face & 1
    kn = sum(f[q] for q in _ZERO[face]) + sum(f[q] for q in _OUT[face])
    out = sum(f[q] for q in _OUT[face])
    j = [den * vel[0], den * vel[1], den * vel[2]]
    j[ax] = (out - (den - kn)) if high else ((den - kn) - out)
    return _assign(face, j[0], j[1], j[2], f)


def _fix_vel(face, den, vel, f):
    ax, high = face >> 1, face & 1
    kn = sum(f[q] for q in _ZERO[face]) + sum(f[q] for q in _OUT[face])
    out = sum(f[q] for q in _OUT[face])
    dbc = (kn + out) / ((1.0 + vel[ax]) if high else (1.0 - vel[ax]))
    return _assign(face, dbc * vel[0], dbc * vel[1], dbc * vel[2], f)


def fix_den_face_1x_D3Q19(den, vel, f): return _fix_den(0, den, vel, f)
def fix_den_face_x1_D3Q19(den, vel, f): return _fix_den(1, den, vel, f)
def fix_den_face_1y_D3Q19(den, vel, f): return _fix_den(2, den, vel, f)
def fix_den_face_y1_D3Q19(den, vel, f): return _fix_den(3, den, vel, f)
def fix_den_face_1z_D3Q19(den, vel, f): return _fix_den(4, den, vel, f)
def fix_den_face_z1_D3Q19(den, vel, f): return _fix_den(5, den, vel, f)
def fix_vel_face_1x_D3Q19(den, vel, f): return _fix_vel(0, den, vel, f)
def fix_vel_face_x1_D3Q19(den, vel, f): return _fix_vel(1, den, vel, f)
def fix_vel_face_1y_D3Q19(den, vel, f): return _fix_vel(2, den, vel, f)
def fix_vel_face_y1_D3Q19(den, vel, f): return _fix_vel(3, den, vel, f)
def fix_vel_face_1z_D3Q19(den, vel, f): return _fix_vel(4, den, vel, f)
def fix_vel_face_z1_D3Q19(den, vel, f): return _fix_vel(5, den, vel, f)
