"""Readers for the reference's own case inputs, so that its shipped cases can
be built and run through this library.

- ``read_pin``: the MGAERO-style grid file (``*.pin``: ``GRID.NAME``,
  ``POINTS``, ``ORIGIN``, ``LENGTH`` per uniform block; ``!`` and ``#`` start
  comments).  GRID.NAME = 100*level + serial (101, 201, ..., 401, 402).
- ``read_plot3d``: an ASCII multi-zone plot3d surface (``nzones``, the
  dimensions of every zone, then x, y, z of each zone in Fortran order).
- ``read_jobsheet``: the job sheet's sections ``NAME { key = value ... }``;
  keys are case-insensitive, ``!`` starts a comment, a line may hold several
  assignments.
- ``case_from_reference``: a ``cases.Case`` from a .pin, a .p3d and a job
  sheet: the grids of the grid file (one per level), the body of the
  surface's first zone (its section, extruded along the span axis), and the
  flow, numerics and domain boundary types of the job sheet, turned into
  parameters as input_param.f90:17-114 does.

The cut-cell records are this library's own (trilinear or multiquadric
radial-basis clouds): the reference's ``solid_ipolcoef`` belongs to its fcode
library, which is not part of the reference tree.
"""
import re

import numpy as np

from . import _abi as A
from . import cases as K


# ------------------------------------------------------------------ grid file
def read_pin(path):
    """The grids of a .pin file: list of dict(name, level, serial, points,
    origin, length)."""
    grids, cur, inside = [], None, False
    for raw in open(path):
        line = raw.split("!")[0].strip()
        if not line or line.startswith("#"):
            continue
        up = line.upper()
        if up.startswith("BEGIN GRID DATA"):
            inside = True
            continue
        if up.startswith("END GRID DATA"):
            break
        if not inside:
            continue
        if up.startswith("GRID.NAME"):
            cur = {"name": int(line.split("=")[1].split()[0])}
            cur["level"], cur["serial"] = cur["name"] // 100, cur["name"] % 100
            grids.append(cur)
        elif cur is not None:
            key, *vals = line.split()
            key = key.upper()
            if key == "POINTS":
                cur["points"] = tuple(int(v) for v in vals[:3])
            elif key == "ORIGIN":
                cur["origin"] = tuple(float(v) for v in vals[:3])
            elif key == "LENGTH":
                cur["length"] = tuple(float(v) for v in vals[:3])
    for g in grids:
        for k in ("points", "origin", "length"):
            if k not in g:
                raise ValueError("grid %d: no %s" % (g["name"], k))
    return grids


# ------------------------------------------------------------------ surface
def _num(v):
    return float(v.replace("D", "E").replace("d", "e"))


def read_plot3d(path):
    """Zones of an ASCII plot3d file: list of (x, y, z) arrays shaped
    (nk, nj, ni), i fastest as in the file."""
    tok = open(path).read().split()
    nz = int(tok[0])
    dims = [tuple(int(v) for v in tok[1 + 3 * q: 4 + 3 * q]) for q in range(nz)]
    pos = 1 + 3 * nz
    zones = []
    for ni, nj, nk in dims:
        n = ni * nj * nk
        xyz = []
        for _ in range(3):
            xyz.append(np.array([_num(v) for v in tok[pos: pos + n]]).reshape(nk, nj, ni))
            pos += n
        zones.append(tuple(xyz))
    return zones


def section_polygon(zones, span_axis=1):
    """The body's section: the first row (j = 0) of the first zone, in the two
    coordinates across the span axis (closing point dropped)."""
    x, y, z = zones[0]
    pts = np.stack([x[0, 0, :], y[0, 0, :], z[0, 0, :]], axis=1)
    poly = pts[:, [a for a in range(3) if a != span_axis]]
    if np.allclose(poly[0], poly[-1]):
        poly = poly[:-1]
    return np.ascontiguousarray(poly)


# ------------------------------------------------------------------ job sheet
_ASSIGN = re.compile(r"([A-Za-z_][\w.]*)\s*=\s*(\([^)]*\)|\"[^\"]*\"|'[^']*'|[^=,\s]+)")


def read_jobsheet(path):
    """{SECTION: {key: value string}}."""
    out, sec, pend = {}, None, None
    for raw in open(path):
        s = raw.split("!")[0].strip()
        if not s:
            continue
        if s == "{":
            sec = pend
            out.setdefault(sec, {})
            continue
        if s.startswith("}"):
            sec = None
            continue
        if sec is None:
            pend = s.split()[0].upper()
            if s.endswith("{"):
                sec = pend
                out.setdefault(sec, {})
            continue
        for key, val in _ASSIGN.findall(s):
            out[sec].setdefault(key.lower(), val.strip().strip("'\""))
    return out


def domain_bctypes(path):
    """bc_type of the six domain faces from the DOMAIN section's
    ``xbound = (lo, hi) bc_type = (a, b)`` lines (face order -x,-y,-z,+x,+y,+z);
    the far field where a line is missing."""
    raw = open(path).read()
    bct = [-20] * 6
    for q, ax in enumerate("xyz"):
        m = re.search(r"^[ \t]*%sbound\s*=\s*\([^)]*\)\s*bc_type\s*=\s*\(\s*(-?\d+)\s*,\s*(-?\d+)\s*\)" % ax,
                      raw, re.I | re.M)
        if m:
            bct[q], bct[q + 3] = int(m.group(1)), int(m.group(2))
    return tuple(bct)


def _list(v):
    return [_num(p) for p in re.split(r"[:,]", v.strip("() ")) if p.strip()]


# ------------------------------------------------------------------ the case
def case_from_reference(pin_path, p3d_path, jobsheet_path, span_axis=1, nlevel=None, mcyc=None, cloud="trilinear",
                        **overrides):
    """A Case from the reference's inputs: the grids of the grid file (the
    grids of one level, in name order, are that level's blocks; each takes
    as parent the block of the level above that holds it, and blocks of a
    level exchange ghost cells where they overlap, bc_overlap), the extruded
    body of the plot3d surface, and the job sheet's flow, numerics and domain
    boundary types.  ``cloud`` picks the records' interpolation clouds
    ("trilinear" or "rbf").  Keyword overrides go to ``cases.params``."""
    js = read_jobsheet(jobsheet_path)
    flow, num, ctl = js.get("FLOW", {}), js.get("NUMERICS", {}), js.get("CONTROL", {})
    grids = sorted(read_pin(pin_path), key=lambda g: g["name"])
    levels = sorted({g["level"] for g in grids})
    if nlevel is not None:
        levels = levels[:nlevel]
    poly = section_polygon(read_plot3d(p3d_path), span_axis)
    body = K.Body("polygon", poly=poly, span_axis=span_axis, cloud=cloud)
    bct = domain_bctypes(jobsheet_path)
    specs = []
    for li, L in enumerate(levels):
        row = []
        for g in [x for x in grids if x["level"] == L]:
            n = tuple(p - 1 for p in g["points"])
            h = tuple(g["length"][a] / n[a] for a in range(3))
            # the grid's first point is the lower corner of its first cell
            spec = K.BlockSpec(n=n, h=h, origin=tuple(g["origin"]), bctype=bct)
            if li > 0:
                parent = _parent_of(spec, specs[-1])
                pb = specs[-1][parent - 1]
                ratio = tuple(int(round(pb.h[a] / h[a])) for a in range(3))
                off = tuple(int(round((g["origin"][a] - pb.origin[a]) / pb.h[a])) for a in range(3))
                spec.parent, spec.ratio, spec.offset = parent, ratio, off
                # embedded grids take their ghost cells from the parent (bc_embed),
                # except across a periodic span they share with it
                spec.bctype = tuple(b if b == -60 and ratio[q % 3] == 1 else 0 for q, b in enumerate(bct))
            row.append(K.make_block_arrays(spec, body))
        specs.append(row)
    eqn = A.MGE_EQN_NS if num.get("eqntype", "e").lower().startswith("n") else A.MGE_EQN_EULER
    dist = {"c": A.MGE_DIS_CENTRAL, "r1": A.MGE_DIS_ROE1, "r2": A.MGE_DIS_ROE2}[num.get("distype", "c").lower()]
    kw = dict(
        mach=_num(flow.get("mach", "0.5")),
        alpha_deg=_num(flow.get("alphad", "0")), beta_deg=_num(flow.get("betad", "0")),
        gamma=_num(flow.get("gamma", "1.4")),
        cfl=_num(num.get("cflf", "-2.8")), vis2=_num(num.get("vis2", "0.5")), vis4_in=_num(num.get("vis4", "0.5")),
        smoo=_num(num.get("smoo", "0")), mgtype=int(_num(num.get("mgtype", "1"))),
        cstp=tuple(_list(num["cstp"])) if "cstp" in num else (0.25, 1.0 / 6.0, 0.375, 0.5, 1.0),
        cdis=tuple(_list(num["cdis"])) if "cdis" in num else (1.0, 0.0, 0.56, 0.0, 0.44),
        eqntype=eqn, distype=dist,
        dissip=A.MGE_DISSIP_MATRIX if num.get("dissip", "scalar").lower().startswith("m") else A.MGE_DISSIP_SCALAR,
        limfac=_num(num.get("limfac", "5")), epsentr=_num(num.get("epsentr", "0.05")),
        prandtl=_num(flow.get("prlmean", "0.72")),
        nlevel=len(specs),
    )
    # the job sheet's reynolds is not used: for NS the reference sets
    # Re = 500 (input_param.f90:111-114), which params() does by default
    if mcyc is None and "mcyc" in ctl:
        mcyc = [int(v) for v in _list(ctl["mcyc"])][: len(specs)]
        mcyc += [mcyc[-1]] * (len(specs) - len(mcyc))
    kw["mcyc"] = mcyc
    kw.update(overrides)
    prm = K.params(**kw)
    span = specs[-1][0].n[span_axis] * specs[-1][0].h[span_axis]
    chord = float(np.ptp(poly[:, 0]))
    name = "reference_" + pin_path.replace("\\", "/").rsplit("/", 1)[-1].rsplit(".", 1)[0]
    return K.Case(name, prm, specs, body, ref_area=chord * span)


def _parent_of(spec, row):
    """Serial of the block of the level above whose physical box holds the
    block's (to a thousandth of the coarse cell)."""
    lo = spec.origin
    hi = tuple(spec.origin[a] + spec.n[a] * spec.h[a] for a in range(3))
    for q, pb in enumerate(row):
        tol = [1e-3 * pb.h[a] for a in range(3)]
        plo = pb.origin
        phi = tuple(pb.origin[a] + pb.n[a] * pb.h[a] for a in range(3))
        if all(lo[a] >= plo[a] - tol[a] and hi[a] <= phi[a] + tol[a] for a in range(3)):
            return q + 1
    raise ValueError("grid at %s lies in no grid of the level above" % (lo,))
