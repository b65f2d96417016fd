"""Runs the unmodified reference solver (built into oracle/_ref by
oracle/build_ref.py) on the steady channel flows of tests/profile_cases.py
and records, per case, the mid-domain velocity profile (exact, as float
hex strings) and the relative L2 error against the analytic steady state
computed with the reference's own flow_field.  Run from the repository root:

    python oracle/build_ref.py && python tests/golden/make_profiles.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
sys.path.insert(0, os.path.dirname(HERE))

from jyulb import flow_field  # noqa: E402  (the reference build)
from jyulb.isothermal import Solver  # noqa: E402

import profile_cases as pc  # noqa: E402


def main():
    out = {}
    for c in pc.cases():
        s = Solver(np.array(c["lat"], dtype=np.int32), c["scheme"], c["kvisc"], pc.gravity(c),
                   np.array(c["bc"], dtype=np.int32))
        pc.setup(s, c, flow_field)
        nf = s.finalize_init()
        for n in c["chunks"]:
            s.evolve(n)
        prof = pc.profile(np.asarray(s.get_vel()), c)
        err = pc.error(prof, c, flow_field)
        out[c["name"]] = {"nfluid": int(nf), "error": err.hex(),
                          "profile": [[float(v).hex() for v in row] for row in prof]}
        print(f"{c['name']:22s} fluid={nf:5d} rel L2 error vs analytic = {err:.4e}")
    with open(os.path.join(HERE, "profiles.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
