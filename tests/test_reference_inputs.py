"""The reference's own case inputs (grid file, plot3d surface, job sheet)
read into a case: the readers on a small set of inputs written here, the
shipped cylinder inputs (copied into tests/fixtures), and on the GPU solves
of cases built from such inputs, the shipped one included, against the
oracle."""
import os

import numpy as np
import pytest

from code_mge_gb300 import _abi as A
from code_mge_gb300 import reference_inputs as R

# the reference's shipped cylinder inputs (tests/fixtures/copy_reference_inputs.py)
REF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fixtures", "cylinder")


def write_inputs(d, n=(32, 2, 32), nlevel=2):
    """A .pin with one grid per level (each level halves the cell size over
    half the extent), a plot3d cylinder of radius 0.5 (side, 2 span rows) and
    a job sheet: Euler, JST, M = 0.5."""
    lines = ["BEGIN GRID DATA", " "]
    ext, hy = 4.0, 0.25
    for L in range(1, nlevel + 1):
        f = 2 ** (L - 1)
        pts = (n[0] + 1, n[1] * f + 1, n[2] + 1)
        e = ext / f
        lines += ["GRID.NAME = %d" % (100 * L + 1), "! level %d" % L,
                  "POINTS %d %d %d" % pts, "ORIGIN %.5f 0.0 %.5f" % (-e, -e),
                  "LENGTH %.5f %.5f %.5f" % (2 * e, n[1] * hy, 2 * e), ""]
    lines.append("END GRID DATA")
    open(os.path.join(d, "case.pin"), "w").write("\n".join(lines) + "\n")
    th = np.linspace(0.0, 2.0 * np.pi, 65)
    x, z = 0.5 * np.cos(th), 0.5 * np.sin(th)
    with open(os.path.join(d, "case.p3d"), "w") as fh:
        fh.write("1\n%d %d 1\n" % (len(th), 2))
        for arr in (np.concatenate([x, x]), np.concatenate([np.zeros_like(x), np.full_like(x, 0.5)]),
                    np.concatenate([z, z])):
            for q in range(0, len(arr), 5):
                fh.write(" ".join("%16.10E" % v for v in arr[q:q + 5]) + "\n")
    js = """ CONTROL
  {
  mcyc = 2:6
  }
 FLOW
  {
  mach = 0.5
  gamma = 1.40
  alphad = 0.0,
  }
 NUMERICS
  {
  cflf = -2.8,
  vis2 = 0.5,
  vis4 = 0.5,
  smoo = 0.6,
  mgtype = 1,
  cstp = 0.25:0.16667:0.375:0.5:1.0
  cdis = 1.0:0.0:0.56:0.0:0.44
  eqntype = 'e'
  distype = 'c'
  }
 DOMAIN
  {
  xbound = ( -4.00, 4.00 )  bc_type = ( -20, -20)
  ybound = (  0.00, 0.50 )  bc_type = ( -60, -60)
!  zbound = ( -1.00, 1.00 )  bc_type = ( -50, -50)
  zbound = ( -4.00, 4.00 )  bc_type = ( -20, -20)
  }
"""
    open(os.path.join(d, "jobsheet"), "w").write(js)
    return [os.path.join(d, f) for f in ("case.pin", "case.p3d", "jobsheet")]


def test_readers_on_written_inputs(tmp_path):
    pin, p3d, js = write_inputs(str(tmp_path))
    grids = R.read_pin(pin)
    assert [g["name"] for g in grids] == [101, 201]
    assert grids[1]["points"] == (33, 5, 33) and grids[1]["origin"] == (-2.0, 0.0, -2.0)
    zones = R.read_plot3d(p3d)
    assert zones[0][0].shape == (1, 2, 65)
    poly = R.section_polygon(zones)
    assert poly.shape == (64, 2) and np.allclose(np.hypot(poly[:, 0], poly[:, 1]), 0.5)
    sheet = R.read_jobsheet(js)
    assert sheet["FLOW"]["mach"] == "0.5" and sheet["NUMERICS"]["eqntype"] == "e"
    assert R.domain_bctypes(js) == (-20, -60, -20, -20, -60, -20)   # the commented line is skipped


def test_case_from_written_inputs(tmp_path):
    case = R.case_from_reference(*write_inputs(str(tmp_path)))
    assert case.prm.nlevel == 2 and abs(case.prm.rm - 0.5) < 1e-15 and case.prm.vt == 0
    coarse, fine = case.levels[0][0], case.levels[1][0]
    assert coarse.n == (32, 2, 32) and fine.n == (32, 4, 32)
    assert fine.parent == 1 and fine.ratio == (2, 2, 2) and fine.offset == (8, 0, 8)
    assert fine.bctype == (0, 0, 0, 0, 0, 0) and coarse.bctype == (-20, -60, -20, -20, -60, -20)
    # the body: about pi r^2 / h^2 solid cells in every span plane of the fine grid
    solid = np.sum(fine.arrays["blank"].reshape(fine.dims[::-1])[2:-2, 2:-2, 2:-2] == 0)
    per_plane = solid / fine.n[1]
    assert abs(per_plane - np.pi * 0.25 / (0.125 * 0.125)) < 12
    assert fine.arrays["nmir"] > 0


def test_oracle_solves_a_case_from_written_inputs(tmp_path):
    from oracle.oracle import OracleCycle
    case = R.case_from_reference(*write_inputs(str(tmp_path)))
    o = OracleCycle(case)
    hist, n, f = o.solve()
    assert n == 6 and hist[-1] < hist[0] and np.isfinite(f.cd)   # mcyc = 2:6


def test_shipped_cylinder_inputs():
    pin, p3d, js = (os.path.join(REF, f) for f in ("cylinder05_1.pin", "cylinder.p3d", "jobsheet"))
    assert [g["name"] for g in R.read_pin(os.path.join(REF, "cylinder05_11122.pin"))] == \
        [101, 201, 301, 401, 402, 501, 502]
    multi = R.case_from_reference(os.path.join(REF, "cylinder05_11122.pin"), p3d, js)
    assert [len(row) for row in multi.levels] == [1, 1, 1, 2, 2]
    assert [s.parent for s in multi.levels[4]] == [1, 2]   # 501 in 401, 502 in 402
    case = R.case_from_reference(pin, p3d, js)
    sp = case.levels[0][0]
    assert sp.n == (448, 8, 256) and case.prm.eqntype == A.MGE_EQN_NS and case.prm.vt == 0
    assert abs(case.prm.cfl - 2.0) < 1e-15 and abs(case.prm.vis4 - 2.0 / 32.0) < 1e-15
    assert sp.bctype == (-20, -60, -20, -20, -60, -20)
    assert sp.arrays["nmir"] > 0


@pytest.mark.gpu
def test_gpu_solves_a_case_from_written_inputs(gpulib, tmp_path):
    from parity import compare, pair
    case = R.case_from_reference(*write_inputs(str(tmp_path)))
    g, o = pair(case)
    hg, ng, fg = g.solve(use_graph=1)
    ho, no, fo = o.solve()
    assert ng == no
    assert np.max(np.abs(hg - ho) / np.abs(ho)) <= 1e-11
    compare(g, o, "w", 2, rtol=1e-11, phys_only=False)
    assert abs(fg.cd - fo.cd) <= 1e-9 * max(1.0, abs(fo.cd))


@pytest.mark.gpu
def test_gpu_solves_the_shipped_cylinder_case(gpulib):
    """cylinder05_1.pin + cylinder.p3d + jobsheet: Navier-Stokes (Re 500 as
    input_param.f90:111-114 sets it), JST central, 448x8x256, three cycles
    against the oracle on every host thread."""
    from oracle import oracle as O
    from parity import compare, pair
    case = R.case_from_reference(*(os.path.join(REF, f) for f in ("cylinder05_1.pin", "cylinder.p3d", "jobsheet")))
    assert case.prm.nlevel == 1
    case.prm.mcyc[0] = 3
    before = O.load().mgeo_get_threads()
    O.set_threads(os.cpu_count() or 1)
    try:
        g, o = pair(case)
        hg, ng, fg = g.solve(use_graph=1)
        ho, no, fo = o.solve()
    finally:
        O.set_threads(before)
    assert ng == no == 3
    assert np.max(np.abs(hg - ho) / np.abs(ho)) <= 1e-11
    compare(g, o, "w", 1, rtol=1e-11, phys_only=False)
    assert abs(fg.cd - fo.cd) <= 1e-9 * max(1.0, abs(fo.cd))
    g.close()
    o.close()


@pytest.mark.gpu
def test_gpu_solves_the_shipped_multiblock_case(gpulib):
    """cylinder05_11122.pin: five levels, two overlapping blocks on each of
    the two finest (bc_overlap), Navier-Stokes, JST central; the FMG
    sequence with one cycle per coarse level and two on the finest, against
    the oracle on every host thread."""
    from oracle import oracle as O
    from parity import pair
    case = R.case_from_reference(*(os.path.join(REF, f) for f in ("cylinder05_11122.pin", "cylinder.p3d",
                                                                  "jobsheet")))
    for q in range(case.prm.nlevel):
        case.prm.mcyc[q] = 1
    case.prm.mcyc[case.prm.nlevel - 1] = 2
    before = O.load().mgeo_get_threads()
    O.set_threads(os.cpu_count() or 1)
    try:
        g, o = pair(case)
        hg, ng, fg = g.solve(use_graph=1)
        ho, no, fo = o.solve()
    finally:
        O.set_threads(before)
    assert ng == no == 2
    assert np.max(np.abs(hg - ho) / np.abs(ho)) <= 1e-11
    L = case.prm.nlevel
    for s in (1, 2):
        a, b = g.field("w", L, serial=s), o.field("w", L, serial=s)
        assert np.max(np.abs(a - b)) <= 1e-11 * np.max(np.abs(b))
    g.close()
    o.close()
