"""Raw lattice files of the reference's C++ executable
(include/io/raw_io.cpp:23-275, include/io/raw_io.h).

File names are ``<base><ext>``: geometry ``.geom.in.raw`` / ``.geom.out.raw``
(one byte per site, 255 = fluid, 0 = solid), density ``.den.in.raw`` /
``.den.out.raw`` (one float64 per site), velocity ``.vel.in.raw`` /
``.vel.out.raw`` and force ``.force.in.raw`` / ``.force.out.raw`` (three
float64 per site, components innermost).  Sites are ordered with i fastest:
element (i, j, k) sits at k*nx*ny + j*nx + i (raw_io.cpp:245-258).  Arrays in
this module use the package's (nx, ny, nz[, 3]) order, k fastest.

Field readers set fluid sites only and leave solid sites untouched; writers
store the fluid values and fill solid sites with the given initial value, as
the reference does.  A file that cannot be opened gives the reference's
warning and a False return.
"""
from __future__ import annotations

import numpy as np

FLUID_NODE = 255  # include/common/const.h:13-14
SOLID_NODE = 0


def _open(base, ext, mode):
    fname = str(base) + ext
    try:
        return open(fname, mode)
    except OSError:
        print(f"Warning: cannot open file {fname}!")
        return None


def _read(base, ext, count, dtype):
    fh = _open(base, ext, "rb")
    if fh is None:
        return None
    with fh:
        data = np.fromfile(fh, dtype=dtype, count=count)
    if data.size != count:
        raise ValueError(f"{base}{ext}: expected {count} values, found {data.size}")
    return data


def _to_ijk(flat, size, comps=0):
    nx, ny, nz = size
    if comps:
        return np.ascontiguousarray(flat.reshape(nz, ny, nx, comps).transpose(2, 1, 0, 3))
    return np.ascontiguousarray(flat.reshape(nz, ny, nx).transpose(2, 1, 0))


def _to_raw(arr):
    if arr.ndim == 4:
        return np.ascontiguousarray(arr.transpose(2, 1, 0, 3)).ravel()
    return np.ascontiguousarray(arr.transpose(2, 1, 0)).ravel()


def read_geom(base, size):
    """(nx, ny, nz) uint8 raw geometry (255 fluid, 0 solid) from
    ``<base>.geom.in.raw``, or None if the file cannot be opened."""
    size = tuple(int(s) for s in size)
    data = _read(base, ".geom.in.raw", size[0] * size[1] * size[2], np.uint8)
    return None if data is None else _to_ijk(data, size)


def write_geom(base, geom):
    """Writes ``<base>.geom.out.raw`` from (nx, ny, nz) raw geometry."""
    fh = _open(base, ".geom.out.raw", "wb")
    if fh is None:
        return False
    with fh:
        _to_raw(np.asarray(geom, dtype=np.uint8)).tofile(fh)
    return True


def geom_to_phase(geom):
    """Raw geometry -> jyulb phase (FLUID = 1 where the byte is 255)."""
    return (np.asarray(geom) == FLUID_NODE).astype(np.uint8)


def phase_to_geom(phase):
    """jyulb phase -> raw geometry bytes (255 fluid, 0 solid)."""
    return np.where(np.asarray(phase) != 0, FLUID_NODE, SOLID_NODE).astype(np.uint8)


def _read_field(base, ext, fluid, out, comps):
    size = fluid.shape
    count = size[0] * size[1] * size[2] * max(comps, 1)
    data = _read(base, ext, count, np.float64)
    if data is None:
        return False
    vals = _to_ijk(data, size, comps)
    out[fluid] = vals[fluid]
    return True


def _write_field(base, ext, field, fluid, init, comps):
    fh = _open(base, ext, "wb")
    if fh is None:
        return False
    shape = fluid.shape + ((comps,) if comps else ())
    buf = np.empty(shape, np.float64)
    buf[...] = init
    buf[fluid] = np.asarray(field)[fluid]
    with fh:
        _to_raw(buf).tofile(fh)
    return True


def read_den(base, fluid, den):
    """Density of the fluid sites (boolean mask ``fluid``) from
    ``<base>.den.in.raw`` into ``den`` (nx, ny, nz)."""
    return _read_field(base, ".den.in.raw", np.asarray(fluid, bool), den, 0)


def write_den(base, den, fluid, iden):
    """``<base>.den.out.raw``: fluid densities, ``iden`` on solid sites."""
    return _write_field(base, ".den.out.raw", den, np.asarray(fluid, bool), iden, 0)


def read_vel(base, fluid, vel):
    """Velocity of the fluid sites from ``<base>.vel.in.raw`` into ``vel``
    (nx, ny, nz, 3)."""
    return _read_field(base, ".vel.in.raw", np.asarray(fluid, bool), vel, 3)


def write_vel(base, vel, fluid, ivel=(0.0, 0.0, 0.0)):
    """``<base>.vel.out.raw``: fluid velocities, ``ivel`` on solid sites."""
    return _write_field(base, ".vel.out.raw", vel, np.asarray(fluid, bool), np.asarray(ivel, np.float64), 3)


def read_frc(base, fluid, frc):
    """Force density of the fluid sites from ``<base>.force.in.raw``."""
    return _read_field(base, ".force.in.raw", np.asarray(fluid, bool), frc, 3)


def write_frc(base, frc, fluid, ifrc=(0.0, 0.0, 0.0)):
    """``<base>.force.out.raw``: fluid force densities, ``ifrc`` elsewhere."""
    return _write_field(base, ".force.out.raw", frc, np.asarray(fluid, bool), np.asarray(ifrc, np.float64), 3)
