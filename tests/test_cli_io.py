"""The input-script front end, the raw-file I/O and the .evol format of the
reference's C++ executable (no GPU needed), and a GPU run of the front end
checked against the Solver it drives."""
import os

import numpy as np
import pytest

SCRIPT = """# base name
pipe_case
# size
6 5 9
# dr
0.5
# dt
0.25
# reference density
2.0
# viscosity
0.01
# gravity
0.0 0.0 2.0e-6
# external forcing
0
# flow type
1
# collision operator
1
# faces -x +x -y +y -z +z
1
1
0
0
3 2.0 0.0 0.0
4 0.0 0.0 0.01
# steps
40
# info interval
15
# note
small pipe run
"""


def test_parse_script_with_face_lines():
    from jyulb.cli import FACE_DEN, FACE_VEL, FACE_WALL, parse_input_script

    p = parse_input_script(SCRIPT)
    assert p.base == "pipe_case"
    assert p.size == [6, 5, 9]
    assert (p.dr, p.dt, p.ref_den, p.kvisc) == (0.5, 0.25, 2.0, 0.01)
    assert p.g == [0.0, 0.0, 2.0e-6]
    assert (p.external_forcing, p.flow_type, p.collision_operator) == (False, 1, 1)
    assert p.faces[0] == (FACE_WALL, ())
    assert p.faces[4] == (FACE_DEN, (2.0, 0.0, 0.0))
    assert p.faces[5] == (FACE_VEL, (0.0, 0.0, 0.01))
    assert (p.tsteps, p.evol_period, p.exec_info) == (40, 15, "small pipe run")


def test_parse_script_without_face_lines_and_defaults(capsys):
    from jyulb.cli import parse_input_script

    lines = [l for l in SCRIPT.splitlines()]
    i = lines.index("# faces -x +x -y +y -z +z")
    short = "\n".join(lines[:i] + lines[i + 7:])
    p = parse_input_script(short, face_lines=False)
    assert (p.tsteps, p.evol_period) == (40, 15)
    bad = short.replace("\n0.01\n", "\n-1\n")
    q = parse_input_script(bad, face_lines=False)
    assert q.kvisc == pytest.approx(1.0 / 6.0)
    assert "kinematic viscosity must be positive" in capsys.readouterr().out


def test_raw_files_are_i_fastest(tmp_path):
    from jyulb import raw_io

    base = str(tmp_path / "case")
    nx, ny, nz = 4, 3, 2
    geom = np.zeros((nx, ny, nz), np.uint8)
    geom[1, 2, 1] = 255
    raw_io.write_geom(base, geom)
    data = np.fromfile(base + ".geom.out.raw", np.uint8)
    assert data.size == nx * ny * nz and data[1 * nx * ny + 2 * nx + 1] == 255 and data.sum() == 255
    os.rename(base + ".geom.out.raw", base + ".geom.in.raw")
    back = raw_io.read_geom(base, (nx, ny, nz))
    assert np.array_equal(back, geom)
    fluid = raw_io.geom_to_phase(back) != 0
    vel = np.random.default_rng(0).standard_normal((nx, ny, nz, 3))
    assert raw_io.write_vel(base, vel, fluid, (9.0, 8.0, 7.0))
    v = np.fromfile(base + ".vel.out.raw", np.float64)
    k, j, i = 1, 2, 1
    assert np.array_equal(v[3 * (k * nx * ny + j * nx + i):][:3], vel[i, j, k])
    assert np.array_equal(v[:3], [9.0, 8.0, 7.0])
    os.rename(base + ".vel.out.raw", base + ".vel.in.raw")
    got = np.zeros((nx, ny, nz, 3))
    assert raw_io.read_vel(base, fluid, got)
    assert np.array_equal(got[fluid], vel[fluid]) and not got[~fluid].any()
    assert raw_io.read_den(base, fluid, np.zeros((nx, ny, nz))) is False


def test_evol_row_format():
    from jyulb.cli import EVOL_HEADER, evol_row

    info = dict(tot_den=512.0, tot_jx=1e-3, tot_jy=0.0, tot_jz=-2.5e-7, tot_j2=3.0, ave_ux=1.0, ave_uy=2.0,
                ave_uz=3.0, ave_u2=4.0, max_u2=5.0, max_den=1.0, min_den=0.5)
    row = evol_row(1000, 1000.0, info)
    cols = row.split("\t")
    assert cols[0] == "1000" and cols[1] == "1.000000000000e+03" and cols[2] == "5.120000000000e+02"
    assert len(cols) == 14 and EVOL_HEADER.startswith("#1. Tstep")


@pytest.mark.gpu
def test_cli_run_matches_solver(tmp_path, capsys):
    from jyulb import cli, raw_io

    p = cli.parse_input_script(SCRIPT)
    p.base = str(tmp_path / "pipe")
    nx, ny, nz = p.size
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    geom = np.where((X - 2.5) ** 2 + (Y - 2.0) ** 2 <= 4.0, 255, 0).astype(np.uint8)[:, :, None].repeat(nz, 2)
    raw_io.write_geom(p.base, geom)
    os.rename(p.base + ".geom.out.raw", p.base + ".geom.in.raw")
    s = cli.run(p, physics="jyulb")
    out = capsys.readouterr().out
    assert "tstep 40, tot.mass" in out and "MFLUPS" in out
    rows = [l.split("\t") for l in open(p.base + ".evol").read().splitlines()[1:]]
    assert [r[0] for r in rows] == ["0", "3", "7", "10"]  # dt * step with dt = 0.25
    # the same run through the Solver API
    ref, fluid = cli.build_solver(p, physics="jyulb")
    ref.finalize_init()
    for n in (15, 15, 10):
        ref.evolve(n)
    cr = p.dr / p.dt
    den = np.array(ref.get_den()) * p.ref_den
    vel = np.array(ref.get_vel()) * cr
    d_out = np.zeros((nx, ny, nz))
    v_out = np.zeros((nx, ny, nz, 3))
    assert raw_io._read_field(p.base, ".den.out.raw", fluid, d_out, 0)
    assert raw_io._read_field(p.base, ".vel.out.raw", fluid, v_out, 3)
    assert np.array_equal(d_out[fluid], den[fluid]) and np.array_equal(v_out[fluid], vel[fluid])
    # last .evol row against NumPy flow information of the same fields
    last = [float(x) for x in rows[-1][2:]]
    dd, vv = den[fluid], vel[fluid]
    um = np.sqrt((vv ** 2).sum(1))
    want = [dd.sum(), *(dd[:, None] * vv).sum(0), (dd * um).sum(), *vv.mean(0), um.mean(), max(um.max(), 0.0),
            max(dd.max(), p.ref_den), min(dd.min(), p.ref_den)]
    np.testing.assert_allclose(last, want, rtol=1e-11, atol=1e-18)
