"""Input-script front end: the reference C++ executable's driver
(source/isothermal/jyu_lb_isothermal.cpp:60-170) and input parser
(include/io/input_parser.cpp:56-139) in front of the GPU engine.

    python -m jyulb.cli run.in

The script lists, one per line and in this order, with '#' comment lines
anywhere between them: the base name of the raw files, the lattice size
(nx ny nz), lattice spacing dr, time step dt, reference density, kinematic
viscosity, gravity (gx gy gz), external forcing (0/1), flow type (Stokes 0,
laminar 1, turbulent 2), collision operator (BGK 0, TRT 1, MRT 2, regularized
3), then -- as the shipped example scripts have them (tube.in) -- one line
per domain face (-x, +x, -y, +y, -z, +z) with a boundary code (periodic 0,
fixed wall 1, shear wall 2, fixed density 3, fixed velocity 4) and its data,
then the number of time steps, the flow-information interval and a free-text
execution note.  The reference's parser has no face lines and would read the
first face code as the step count; `parse_input_script(..., face_lines=False)`
reads that shorter layout.

The run reads ``<base>.geom.in.raw`` and, when present, ``.den.in.raw``,
``.vel.in.raw`` (and ``.force.in.raw`` with external forcing), advances the
steps on the GPU with flow information every interval into ``<base>.evol``,
and writes ``<base>.den.out.raw`` and ``<base>.vel.out.raw``.  Physical
units convert as the executable's kernel does (include/kernel/kernel.cpp:
410-465): c_r = dr/dt, density / ref_den, velocity / c_r, viscosity
dt/dr^2, gravity dt^2/dr, force density / (ref_den c_r / dt).

By default the run uses the executable's own collision model on the GPU
(``physics="cxx"``: linear equilibrium for Stokes flow, quadratic otherwise;
first-order forcing, second-order with external forcing; BGK or TRT, other
operators fall back to TRT with the executable's warning) and reproduces its
output files.  ``physics="jyulb"`` runs this package's reference collision
(BGK, TRT, regularized) instead and admits the Zou-He faces of the face lines.
"""
from __future__ import annotations

import math
import sys
import time

import numpy as np

from . import raw_io
from .defs import BGK, FIXED_DEN, FIXED_VEL, PERIODIC, REGULARIZATION, TRT, WALL

STOKES_FLOW, LAMINAR_FLOW, TURBULENT_FLOW = 0, 1, 2
CPP_BGK, CPP_TRT, CPP_MRT, CPP_REG = 0, 1, 2, 3
FACE_PERIODIC, FACE_WALL, FACE_SHEAR, FACE_DEN, FACE_VEL = 0, 1, 2, 3, 4
FACE_DATA = {FACE_PERIODIC: 0, FACE_WALL: 0, FACE_SHEAR: 2, FACE_DEN: 3, FACE_VEL: 3}


class InputScript:
    """Parameters of one run, defaults as in IsothermalInputParser
    (include/io/input_parser.cpp:13-36)."""

    def __init__(self):
        self.base = "jyu_lb_isothermal"
        self.size = [1, 1, 1]
        self.dr = 1.0
        self.dt = 1.0
        self.ref_den = 1.0
        self.kvisc = 1.0 / 6.0
        self.g = [0.0, 0.0, 0.0]
        self.external_forcing = False
        self.flow_type = STOKES_FLOW
        self.collision_operator = CPP_BGK
        self.faces = [(FACE_PERIODIC, ())] * 6
        self.tsteps = 1000
        self.evol_period = 100
        self.exec_info = ""


class _Lines:
    """Line-oriented reader with the parser's comment rule: lines that start
    with '#' where a value is expected are skipped."""

    def __init__(self, text):
        self.lines = text.splitlines()
        self.pos = 0

    def next_line(self):
        while self.pos < len(self.lines) and self.lines[self.pos].startswith("#"):
            self.pos += 1
        if self.pos >= len(self.lines):
            return None
        line = self.lines[self.pos]
        self.pos += 1
        return line

    def values(self, n, conv):
        line = self.next_line()
        if line is None:
            return None
        tok = line.split()
        if len(tok) < n:
            raise ValueError(f"input script line {self.pos}: expected {n} value(s), found {line!r}")
        return [conv(t) for t in tok[:n]], tok[n:]


def _warn(msg, default):
    print(f"Warning: {msg}!Warning: using default {default}!")


def parse_input_script(text, face_lines=None):
    """InputScript from the text of an input script.  face_lines: True for
    the layout with six face lines (tube.in), False for the executable
    parser's layout without them, None to tell them apart by the number of
    value lines after the collision operator (nine or eight with face lines,
    three or two without)."""
    p = InputScript()
    rd = _Lines(text)
    line = rd.next_line()
    if line is None:
        return p
    p.base = line.strip().split()[0] if line.strip() else ""
    (sz, _) = rd.values(3, int)
    for a, v in enumerate(sz):
        if v < 1:
            _warn("invalid lattice size argument", "lattice size")
        else:
            p.size[a] = v

    def positive(name, attr, msg):
        (v,), _ = rd.values(1, float)
        if v <= 0.0:
            _warn(f"{msg} must be positive", msg)
        else:
            setattr(p, attr, v)

    positive("dr", "dr", "lattice spacing")
    positive("dt", "dt", "discrete time step")
    positive("ref_den", "ref_den", "reference density")
    positive("kvisc", "kvisc", "kinematic viscosity")
    (p.g, _) = rd.values(3, float)
    (ef,), _ = rd.values(1, int)
    if ef not in (0, 1):
        _warn("invalid external forcing option argument", "external forcing option")
    else:
        p.external_forcing = ef == 1
    (ft,), _ = rd.values(1, int)
    if ft not in (STOKES_FLOW, LAMINAR_FLOW, TURBULENT_FLOW):
        _warn("invalid flow type argument", "flow type")
    else:
        p.flow_type = ft
    (co,), _ = rd.values(1, int)
    if co not in (CPP_BGK, CPP_TRT, CPP_MRT, CPP_REG):
        _warn("invalid collision operator argument", "collision operator")
    else:
        p.collision_operator = co
    if face_lines is None:
        rest = [l for l in rd.lines[rd.pos:] if not l.startswith("#")]
        face_lines = len(rest) >= 8
    if face_lines:
        faces = []
        for f in range(6):
            (code,), rest = rd.values(1, int)
            if code not in FACE_DATA:
                raise ValueError(f"face {f}: unknown boundary code {code}")
            need = FACE_DATA[code]
            if len(rest) < need:
                raise ValueError(f"face {f}: boundary code {code} needs {need} value(s)")
            faces.append((code, tuple(float(t) for t in rest[:need])))
        p.faces = faces
    (p.tsteps,), _ = rd.values(1, int)
    (p.evol_period,), _ = rd.values(1, int)
    line = rd.next_line()
    p.exec_info = "" if line is None else line.strip("\t\v\n\r").split("\t")[0]
    return p


EVOL_HEADER = ("#1. Tstep \t 2. t \t 3. Tot.den \t"
               "4. Tot.jx \t 5. Tot.jy \t 6. Tot.jz \t 7. Tot.j2 \t"
               "8. Ave.ux \t 9. Ave.uy \t 10. Ave.uz \t 11. Ave.u2 \t"
               "12. Max.u2 \t 13. Max.den \t 14. Min.den")


def evol_row(step_col, time_col, info):
    """One .evol line: the integer first column, then 13 values in %.12e
    (jyu_lb_isothermal.cpp:21-56; the executable passes the step count to the
    time column and dt*step to the step column, which coincide for dt = 1)."""
    vals = [time_col] + [info[k] for k in ("tot_den", "tot_jx", "tot_jy", "tot_jz", "tot_j2", "ave_ux",
                                           "ave_uy", "ave_uz", "ave_u2", "max_u2", "max_den", "min_den")]
    return f"{int(step_col)}\t" + "\t".join(f"{v:.12e}" for v in vals)


def scaled_info(solver, p):
    """Flow information of the solver (lattice units) in the script's
    physical units."""
    cr = units(p)["cr"]
    fi = solver.flow_info(1.0)
    out = dict(fi)
    for k in ("tot_den", "max_den", "min_den"):
        out[k] = fi[k] * p.ref_den
    for k in ("tot_jx", "tot_jy", "tot_jz", "tot_j2"):
        out[k] = fi[k] * p.ref_den * cr
    for k in ("ave_ux", "ave_uy", "ave_uz", "ave_u2", "max_u2"):
        out[k] = fi[k] * cr
    return out


def units(p):
    """The executable's unit conversions in its own evaluation order
    (include/kernel/kernel.cpp:414-419, 457-465): lattice speed c_r = dr/dt,
    body-force unit ref_den c_r / dt, viscosity / (dr c_r), gravity dt / c_r."""
    inv_dt = 1.0 / p.dt
    cr = p.dr * inv_dt
    inv_cr = 1.0 / cr
    bf_unit = p.ref_den * inv_dt * cr
    return dict(cr=cr, inv_cr=inv_cr, inv_dr=1.0 / p.dr, inv_ref_den=1.0 / p.ref_den, inv_bf_unit=1.0 / bf_unit,
                kvisc=(1.0 / p.dr) * inv_cr * p.kvisc, g=[p.dt * inv_cr * gv for gv in p.g])


def build_solver(p, precision=0, stream=None, physics="cxx"):
    """A jyulb Solver set up from the script and its raw input files.

    physics="cxx" runs the executable's own collision model (linear or
    quadratic equilibrium from the flow type, first- or second-order forcing
    from the external-forcing switch; periodic and wall faces only) and
    reproduces its output; physics="jyulb" runs this package's reference
    collision and also accepts Zou-He faces."""
    from .isothermal import Solver

    u = units(p)
    inv_cr = u["inv_cr"]
    if physics == "cxx":
        scheme = {CPP_BGK: BGK, CPP_TRT: TRT}.get(p.collision_operator)
    else:
        scheme = {CPP_BGK: BGK, CPP_TRT: TRT, CPP_REG: REGULARIZATION}.get(p.collision_operator)
        if p.flow_type == STOKES_FLOW:
            print("Warning: the linear (Stokes) equilibrium needs physics='cxx'; using the quadratic equilibrium")
    if scheme is None:
        print("Warning: using default collision operator (TRT)")
        scheme = TRT
    bc = []
    for code, _ in p.faces:
        if code == FACE_SHEAR:
            raise ValueError("shear-wall faces are not supported")
        if physics == "cxx" and code not in (FACE_PERIODIC, FACE_WALL):
            raise ValueError("the executable's collision model has no Zou-He faces; use physics='jyulb'")
        bc.append({FACE_PERIODIC: PERIODIC, FACE_WALL: WALL, FACE_DEN: FIXED_DEN, FACE_VEL: FIXED_VEL}[code])
    geom = raw_io.read_geom(p.base, p.size)
    if geom is None:
        raise FileNotFoundError(f"{p.base}.geom.in.raw")
    phase = raw_io.geom_to_phase(geom)
    fluid = phase != 0
    kw = {}
    if physics == "cxx":
        kw = dict(kernel="cxx", stokes=p.flow_type == STOKES_FLOW, second_order_forcing=bool(p.external_forcing))
    s = Solver(np.array(p.size, dtype=np.int32), scheme, u["kvisc"], np.array(u["g"], dtype=np.float64),
               np.array(bc, dtype=np.int32), precision=precision, stream=stream, **kw)
    s.get_phase()[:] = phase
    # dimensional fields with the executable's defaults, then scaled by the
    # same multiplications (kernel.cpp:335-337)
    den_in = np.full(tuple(p.size), p.ref_den)
    if not raw_io.read_den(p.base, fluid, den_in):
        print("No input file for density: using default initial density.")
        print("--------------------------------------------------------------")
    vel_in = np.zeros(tuple(p.size) + (3,))
    if not raw_io.read_vel(p.base, fluid, vel_in):
        print("No input file for velocity: using default initial velocity.")
        print("--------------------------------------------------------------")
    den = den_in * u["inv_ref_den"]
    vel = vel_in * inv_cr
    # Zou-He face data sit on the face layers of den / vel
    for f, (code, data) in enumerate(p.faces):
        ax, hi = f // 2, f % 2
        sl = [slice(None)] * 3
        sl[ax] = -1 if hi else 0
        sl = tuple(sl)
        if code == FACE_DEN:
            den[sl] = data[0] * u["inv_ref_den"]
            t = [a for a in range(3) if a != ax]
            vel[sl + (t[0],)] = data[1] * inv_cr
            vel[sl + (t[1],)] = data[2] * inv_cr
            vel[sl + (ax,)] = 0.0
        elif code == FACE_VEL:
            for a in range(3):
                vel[sl + (a,)] = data[a] * inv_cr
    s.get_den()[:] = den
    s.get_vel()[:] = vel
    if p.external_forcing:
        frc = np.zeros(tuple(p.size) + (3,))
        if raw_io.read_frc(p.base, fluid, frc):
            acc = s.get_acc()
            acc[:] = 0.0
            if physics == "cxx":
                acc[fluid] = frc[fluid] * u["inv_bf_unit"]  # force density, as the executable uses it
            else:
                # force density -> per-site acceleration with the initial density
                acc[fluid] = (frc[fluid] * u["inv_bf_unit"]) / den[fluid][:, None]
    return s, fluid


def run(p, precision=0, out=None, physics="cxx"):
    """The executable's main loop on the GPU; returns the solver."""
    out = sys.stdout if out is None else out
    s, fluid = build_solver(p, precision, physics=physics)
    cr = units(p)["cr"]
    nf = s.finalize_init()
    evol = open(p.base + ".evol", "w")
    evol.write(EVOL_HEADER + "\n")
    info = scaled_info(s, p)  # moments of the initial state
    print(f"tstep {0}, tot.mass = {info['tot_den']:e}, max.u2 = {info['max_u2']:e}", file=out)
    evol.write(evol_row(0, 0.0, info) + "\n")
    period = p.evol_period if p.evol_period > 0 else max(p.tsteps, 1)
    t0 = time.perf_counter()
    done = 0
    while done < p.tsteps:
        n = min(period, p.tsteps - done)
        s.evolve(n)
        done += n
        info = scaled_info(s, p)
        print(f"tstep {done}, tot.mass = {info['tot_den']:e}, max.u2 = {info['max_u2']:e}", file=out)
        evol.write(evol_row(int(p.dt * done), float(done), info) + "\n")
    ms = int((time.perf_counter() - t0) * 1000.0 + 0.5)
    evol.close()
    print("==============================================================", file=out)
    print(f"Computational time: {ms} milliseconds", file=out)
    print("--------------------------------------------------------------", file=out)
    mflups = (nf * p.tsteps / 1e3) / ms if ms > 0 else math.inf
    print(f"MFLUPS: {mflups:f}", file=out)
    print("==============================================================", file=out)
    den = np.array(s.get_den()) * p.ref_den
    vel = np.array(s.get_vel()) * cr
    # solid sites: the executable writes its node data's initial density,
    # a member its constructor never sets (include/common/data.h:75-87); it
    # reads 0 in practice, and 0 is written here
    raw_io.write_den(p.base, den, fluid, 0.0)
    raw_io.write_vel(p.base, vel, fluid)
    return s


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    physics = "cxx"
    if "--physics" in argv:
        i = argv.index("--physics")
        physics = argv[i + 1]
        argv = argv[:i] + argv[i + 2:]
    if not argv:
        print("Warning: not enough input arguments!")
        print("Warning: using default simulation parameters!")
        p = InputScript()
    else:
        try:
            text = open(argv[0]).read()
        except OSError:
            print("Warning: unable to open input script!Warning: using default simulation parameters!")
            text = None
        p = parse_input_script(text) if text is not None else InputScript()
    run(p, physics=physics)
    return 0


if __name__ == "__main__":
    sys.exit(main())
