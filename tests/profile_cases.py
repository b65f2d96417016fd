"""Steady channel flows with analytic profiles: the configurations of the
reference's example scripts (examples/poiseuille_*.py, examples/couette.py,
as shipped: sizes, viscosities, schemes, boundary sets, 20 calls of 500
steps) and the 4x34x4 gravity channel of 20000 steps.  Each case sets up any
solver with the reference's Solver interface (get_phase / get_den / get_vel)
and measures the relative L2 error of the mid-domain profile against the
analytic steady state from a `flow_field` module, as the scripts do
(examples/poiseuille_grav.py:160-203, examples/couette.py).

TEST INFRASTRUCTURE: imported by tests/golden/make_profiles.py (with the
reference's own Solver and flow_field) and by tests/test_profiles_gpu.py.
"""
from __future__ import annotations

import numpy as np

X, Y, Z = 0, 1, 2
FACES = {"1X": 0, "X1": 1, "1Y": 2, "Y1": 3, "1Z": 4, "Z1": 5}
WALL, PERIODIC, FIXED_DEN, FIXED_VEL, SYMMETRIC = 0, 1, 2, 3, 4
BGK, TRT = 0, 1


def _lat(plate, flow, dummy, H, L, W):
    lat = [0, 0, 0]
    lat[plate], lat[flow], lat[dummy] = H, L, W
    return lat


def _bc(**faces):
    bc = [PERIODIC] * 6
    for f, kind in faces.items():
        bc[FACES[f]] = kind
    return bc


def _mid(lat, plate, h):
    c = [n // 2 for n in lat]
    c[plate] = h
    return tuple(c)


def cases():
    out = []
    # gravity-driven channel between two walls (poiseuille_grav.py)
    out.append(dict(name="poiseuille_grav", scheme=BGK, kvisc=0.2 / 6.0, plate=X, flow=Y, dummy=Z,
                    lat=_lat(X, Y, Z, 11, 10, 5), bc=_bc(**{"1X": WALL, "X1": WALL}), grav=1e-5,
                    kind="grav", H=11, half=False))
    # half channel: wall and symmetric centre line (poiseuille_grav_sym.py)
    out.append(dict(name="poiseuille_grav_sym", scheme=TRT, kvisc=0.2 / 6.0, plate=X, flow=Z, dummy=Y,
                    lat=_lat(X, Z, Y, 6, 10, 4), bc=_bc(**{"1X": WALL, "X1": SYMMETRIC}), grav=1e-5,
                    kind="grav", H=6, half=True))
    # Zou-He velocity inlet (parabolic) and density outlet (poiseuille_invel.py)
    out.append(dict(name="poiseuille_invel", scheme=BGK, kvisc=2.0 / 6.0, plate=Y, flow=Z, dummy=X,
                    lat=_lat(Y, Z, X, 11, 10, 5),
                    bc=_bc(**{"1Z": FIXED_VEL, "Z1": FIXED_DEN, "1Y": WALL, "Y1": WALL}),
                    kind="invel", umax=1e-3, H=11, half=False))
    out.append(dict(name="poiseuille_invel_sym", scheme=TRT, kvisc=0.2 / 6.0, plate=Y, flow=Z, dummy=X,
                    lat=_lat(Y, Z, X, 6, 10, 5),
                    bc=_bc(**{"1Z": FIXED_VEL, "Z1": FIXED_DEN, "1Y": WALL, "Y1": SYMMETRIC}),
                    kind="invel", umax=1e-3, H=6, half=True))
    # Zou-He density inlet and outlet (poiseuille_pdiff.py)
    out.append(dict(name="poiseuille_pdiff", scheme=BGK, kvisc=2.0 / 6.0, plate=Y, flow=Z, dummy=X,
                    lat=_lat(Y, Z, X, 11, 10, 5),
                    bc=_bc(**{"1Z": FIXED_DEN, "Z1": FIXED_DEN, "1Y": WALL, "Y1": WALL}),
                    kind="pdiff", kpgrad=-1e-5, H=11, half=False))
    out.append(dict(name="poiseuille_pdiff_sym", scheme=TRT, kvisc=0.2 / 6.0, plate=Y, flow=Z, dummy=X,
                    lat=_lat(Y, Z, X, 6, 10, 5),
                    bc=_bc(**{"1Z": FIXED_DEN, "Z1": FIXED_DEN, "1Y": WALL, "Y1": SYMMETRIC}),
                    kind="pdiff", kpgrad=-1e-5, H=6, half=True))
    # moving solid plates, Ladd's bounce-back (couette.py)
    out.append(dict(name="couette", scheme=BGK, kvisc=0.5 / 6.0, plate=X, flow=Y, dummy=Z,
                    lat=[12, 5, 4], bc=[PERIODIC] * 6, kind="couette", H=10,
                    plates=((0.0, 0.0), (1e-5, 2e-5))))
    # the 4x34x4 gravity channel with solid rows, 20000 steps
    out.append(dict(name="channel_4x34x4", scheme=BGK, kvisc=(0.8 - 0.5) / 3.0, plate=Y, flow=X, dummy=Z,
                    lat=[4, 34, 4], bc=[PERIODIC] * 6, grav=1e-6, kind="grav_rows", H=32, half=False,
                    chunks=[20000]))
    for c in out:
        c.setdefault("chunks", [500] * 20)
    return out


def gravity(c):
    g = np.zeros(3)
    if c["kind"] in ("grav", "grav_rows"):
        g[c["flow"]] = c["grav"]
    return g


def analytic(c, flow_field):
    H = c["H"]
    n = 2 * H if c.get("half") else H
    dist, ana = np.zeros(n), np.zeros(n)
    if c["kind"] in ("grav", "grav_rows"):
        flow_field.poise_plate_steady_state_pgrad(n, c["kvisc"], -c["grav"], dist, ana)
    elif c["kind"] == "invel":
        flow_field.poise_plate_steady_state_umax(n, c["umax"], dist, ana)
    elif c["kind"] == "pdiff":
        flow_field.poise_plate_steady_state_pgrad(n, c["kvisc"], c["kpgrad"], dist, ana)
    else:
        a2 = np.zeros((H, 2))
        (l1, l2), (u1, u2) = c["plates"]
        flow_field.couette_plate_steady_state(H, l1, l2, u1, u2, dist, a2)
        return a2
    return ana


def setup(obj, c, flow_field):
    """Writes the case's phase, den and vel through the getters' views."""
    lat, plate, flow, dummy = c["lat"], c["plate"], c["flow"], c["dummy"]
    phase, den, vel = obj.get_phase(), obj.get_den(), obj.get_vel()
    phase[...] = 1
    if c["kind"] == "grav_rows":
        sl = [slice(None)] * 3
        for row in (0, lat[plate] - 1):
            sl[plate] = row
            phase[tuple(sl)] = 0
    elif c["kind"] == "invel":
        ana = analytic(c, flow_field)
        for w in range(lat[dummy]):
            for h in range(lat[plate]):
                idx = [0, 0, 0]
                idx[dummy], idx[plate], idx[flow] = w, h, 0
                vel[tuple(idx) + (flow,)] = ana[h]
    elif c["kind"] == "pdiff":
        pgrad = c["kpgrad"]
        pdiff = (lat[flow] - 1.0) * pgrad
        pin = 1.0 / 3.0 - 0.5 * pdiff
        for l in range(lat[flow]):
            sl = [slice(None)] * 3
            sl[flow] = l
            den[tuple(sl)] = 3.0 * (pin + l * pgrad)
    elif c["kind"] == "couette":
        (l1, l2), (u1, u2) = c["plates"]
        for row, (v1, v2) in ((0, (l1, l2)), (c["H"] + 1, (u1, u2))):
            sl = [slice(None)] * 3
            sl[plate] = row
            phase[tuple(sl)] = 0
            vel[tuple(sl) + (flow,)] = v1
            vel[tuple(sl) + (dummy,)] = v2


def profile(vel, c):
    """Velocity vectors on the mid-domain line across the plates."""
    lat, plate = c["lat"], c["plate"]
    if c["kind"] == "couette":
        rows = range(1, c["H"] + 1)
    elif c["kind"] == "grav_rows":
        rows = range(1, lat[plate] - 1)
    else:
        rows = range(c["H"])
    return np.array([vel[_mid(lat, plate, h)] for h in rows])


def error(prof, c, flow_field):
    """The scripts' relative L2 error of the profile against the analytic one."""
    ana = analytic(c, flow_field)
    if c["kind"] == "couette":
        # speed of the in-plane velocity against the analytic speed
        sim = np.sqrt((prof ** 2).sum(axis=1))
        a = np.sqrt((ana ** 2).sum(axis=1))
    else:
        sim = prof[:, c["flow"]]
        a = ana[: len(sim)]
    num = den = 0.0
    for s_, a_ in zip(sim, a):
        num += (s_ - a_) * (s_ - a_)
        den += a_ * a_
    return float(np.sqrt(num / den))
