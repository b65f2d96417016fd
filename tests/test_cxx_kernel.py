"""The reference C++ executable's collision model (kernel="cxx") and the
input-script front end against the executable's own outputs (golden
fixtures made by tests/golden/make_cxx_golden.py from the executable built
from the reference's sources)."""
import io
import json
import os
import subprocess
import sys

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ORACLE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle")
CASES = ["tube_trt", "channel_bgk_stokes", "box_trt_forced", "box_mrt_fallback"]


def load(name):
    z = np.load(os.path.join(GOLDEN, f"cxx_{name}.npz"))
    meta = json.loads(str(z["meta"]))
    return meta, {k: z[k] for k in z.files if k != "meta"}


def write_inputs(tmp_path, arr):
    base = str(tmp_path / "case")
    arr["geom"].transpose(2, 1, 0).tofile(base + ".geom.in.raw")
    for key, ext in (("den_in", ".den.in.raw"), ("vel_in", ".vel.in.raw"), ("frc_in", ".force.in.raw")):
        a = arr[key]
        if a.size:
            (a.transpose(2, 1, 0, 3) if a.ndim == 4 else a.transpose(2, 1, 0)).tofile(base + ext)
    return base


def read_out(base, size):
    nx, ny, nz = size
    den = np.fromfile(base + ".den.out.raw").reshape(nz, ny, nx).transpose(2, 1, 0)
    vel = np.fromfile(base + ".vel.out.raw").reshape(nz, ny, nx, 3).transpose(2, 1, 0, 3)
    return den, vel


@pytest.mark.parametrize("name", CASES)
def test_script_parses_like_the_executable(name):
    from jyulb.cli import parse_input_script

    meta, _ = load(name)
    p = parse_input_script(meta["script"])
    assert list(p.size) == list(meta["size"])
    assert (p.dr, p.dt, p.ref_den, p.kvisc) == (meta["dr"], meta["dt"], meta["rden"], meta["kvisc"])
    assert (p.tsteps, p.evol_period, p.flow_type, p.collision_operator) == (
        meta["steps"], meta["period"], meta["flow"], meta["coll"])
    assert p.external_forcing == bool(meta["ext"])


def test_fixture_matches_a_fresh_executable_run(tmp_path):
    """Pins a committed fixture to the reference executable where it can be
    built (the reference tree is not present everywhere)."""
    sys.path.insert(0, ORACLE)
    import build_cxx

    exe = build_cxx.build()
    if exe is None:
        pytest.skip("reference C++ sources not present")
    meta, arr = load("box_trt_forced")
    base = write_inputs(tmp_path, arr)
    open(str(tmp_path / "run.in"), "w").write(meta["script"])
    subprocess.run([exe, "run.in"], cwd=str(tmp_path), env=dict(os.environ, OMP_NUM_THREADS="1"),
                   capture_output=True, check=True)
    den, vel = read_out(base, meta["size"])
    assert np.array_equal(den, arr["den_out"]) and np.array_equal(vel, arr["vel_out"])


def test_cxx_kernel_options_validated():
    from jyulb.defs import FIXED_VEL, REGULARIZATION, TRT, WALL
    from jyulb.isothermal import Solver

    with pytest.raises(ValueError):
        Solver([4, 4, 4], REGULARIZATION, 0.1, kernel="cxx")
    with pytest.raises(ValueError):
        Solver([4, 4, 4], TRT, 0.1, None, [FIXED_VEL, WALL, WALL, WALL, WALL, WALL], kernel="cxx")
    with pytest.raises(ValueError):
        Solver([4, 4, 4], TRT, 0.1, precision=1, kernel="cxx")
    with pytest.raises(ValueError):
        Solver([4, 4, 4], TRT, 0.1, stokes=True)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_cxx_kernel_reproduces_the_executable(name, tmp_path):
    from jyulb import cli

    meta, arr = load(name)
    base = write_inputs(tmp_path, arr)
    p = cli.parse_input_script(meta["script"])
    p.base = base
    cli.run(p, out=io.StringIO(), physics="cxx")
    den, vel = read_out(base, meta["size"])
    # FP64 with the executable's evaluation order: bit for bit
    np.testing.assert_array_equal(den, arr["den_out"])
    np.testing.assert_array_equal(vel, arr["vel_out"])
    evol = np.loadtxt(base + ".evol", comments="#")
    ref = arr["evol"]
    assert evol.shape == ref.shape
    np.testing.assert_array_equal(evol[:, :2], ref[:, :2])
    # sums over the fluid sites in another order: compare each column with
    # the size of its terms (sum |j| bounds the j sums, mean |u| the mean u)
    scale = np.abs(ref).max(axis=0)
    scale[3:7] = np.abs(ref[:, 6]).max()
    scale[7:11] = np.abs(ref[:, 10]).max()
    err = np.abs(evol - ref) / np.maximum(scale, 1e-300)
    assert (err <= 1e-12).all(), err.max(axis=0)
