"""Synthetic cases for the multigrid Runge-Kutta cycle.

The reference takes its grids, blanking and cut-cell records from a
preprocessor that is not part of its source tree (make_fsijob and
solid_ipolcoef, called at srcf90/main.f90:44,57).  This module is this
library's own preprocessor for analytic bodies:

* a level hierarchy of uniform Cartesian blocks, level 1 coarsest, each a
  2:1 coarsening of the next (per axis: ratio 2, or 1 for an uncoarsened
  span), either covering the same domain or embedded with doubled extent;
* ``blank`` from the cell-centre inside test, ghosts copied from the adjacent
  physical layer (init_metric.f90:183-218);
* one mirror record per (fluid cell, solid face neighbour) pair, in Fortran
  cell order then face order, with ``faceid`` 1..6 for a solid neighbour at
  -i,-j,-k,+i,+j,+k (efluxb.f90:70-110), the wall normal, and an
  interpolation cloud for the solid cell centre reflected about the wall
  (bc_cutcell.f90:78-97 consumes ``ijkdex``/``coef``).  Two cloud forms:
  ``trilinear`` (default): the 2x2x2 cell-centre stencil around the
  reflected point with solid and zero-weight cells dropped and the weights
  renormalised; ``rbf``: the eight fluid cell centres nearest the reflected
  point, weighted by multiquadric radial-basis interpolation with a constant
  term (the kind of cloud the reference's solid_ipolcoef builds through the
  rbf_nodal / rbfmq_basis interfaces of inc/rbfit.h and inc/rbasis.h; their
  implementation is not in the reference tree, so the node choice and the
  shape parameter here are this module's own).

All geometry is computed in float64 numpy; the same arrays feed the GPU
library and the CPU oracle.
"""
import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A


# --------------------------------------------------------------------- bodies
@dataclass
class Body:
    kind: str                      # "cylinder" (axis z), "sphere", "ellipsoid", "polygon", "none"
    center: tuple = (0.0, 0.0, 0.0)
    radius: float = 0.5
    semi: tuple = (0.5, 0.5, 0.5)  # ellipsoid semi-axes
    poly: object = None            # polygon: (m, 2) section vertices across the span axis
    span_axis: int = 1             # polygon: the axis it is extruded along
    # velocity of the wall, in units of the free-stream speed (the records'
    # qb, bc_cutcell.f90:47-55): a function of the (m, 3) wall points
    # returning (m, 3) velocities; None for a wall at rest
    wall_velocity: object = None
    cloud: str = "trilinear"       # interpolation clouds of the records: "trilinear" or "rbf"

    def _across(self, a, b, c):
        """The two coordinates across the span axis."""
        return [v for q, v in enumerate((a, b, c)) if q != self.span_axis]

    def inside(self, x, y, z):
        if self.kind == "polygon":  # even-odd rule on the section
            u, v = self._across(x, y, z)
            u, v = np.broadcast_arrays(u, v)
            res = np.zeros(u.shape, dtype=bool)
            P = np.asarray(self.poly, dtype=np.float64)
            for q in range(len(P)):
                (u1, v1), (u2, v2) = P[q], P[(q + 1) % len(P)]
                crosses = (v1 > v) != (v2 > v)
                with np.errstate(divide="ignore", invalid="ignore"):
                    ux = u1 + (v - v1) * (u2 - u1) / (v2 - v1)
                res ^= crosses & (u < ux)
            return res
        cx, cy, cz = self.center
        if self.kind == "cylinder":
            return (x - cx) ** 2 + (y - cy) ** 2 < self.radius ** 2
        if self.kind == "sphere":
            return (x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 < self.radius ** 2
        if self.kind == "ellipsoid":
            a, b, c = self.semi
            return ((x - cx) / a) ** 2 + ((y - cy) / b) ** 2 + ((z - cz) / c) ** 2 < 1.0
        return np.zeros(np.broadcast(x, y, z).shape, dtype=bool)

    def project(self, p):
        """Wall point and outward unit normal for points p (n,3) inside the body."""
        c = np.asarray(self.center, dtype=np.float64)
        q = p - c
        if self.kind == "cylinder":
            r = np.hypot(q[:, 0], q[:, 1])
            r = np.where(r == 0.0, 1e-300, r)
            n = np.stack([q[:, 0] / r, q[:, 1] / r, np.zeros_like(r)], axis=1)
            xw = np.stack([c[0] + self.radius * n[:, 0], c[1] + self.radius * n[:, 1], p[:, 2]], axis=1)
            return xw, n
        if self.kind == "sphere":
            r = np.linalg.norm(q, axis=1)
            r = np.where(r == 0.0, 1e-300, r)
            n = q / r[:, None]
            return c + self.radius * n, n
        if self.kind == "ellipsoid":
            s = np.asarray(self.semi, dtype=np.float64)
            # closest point on the ellipsoid: Newton on t for x_i = q_i a_i^2/(a_i^2+t)
            t = np.zeros(len(q))
            for _ in range(40):
                d = s ** 2 + t[:, None]
                g = np.sum((s * q / d) ** 2, axis=1) - 1.0
                dg = -2.0 * np.sum((s * q) ** 2 / d ** 3, axis=1)
                t = t - g / np.where(dg == 0.0, -1e-300, dg)
                t = np.maximum(t, -np.min(s) ** 2 + 1e-12)
            xw = q * s ** 2 / (s ** 2 + t[:, None])
            n = xw / s ** 2
            n = n / np.linalg.norm(n, axis=1)[:, None]
            return c + xw, n
        if self.kind == "polygon":
            # the nearest point of the section's edges; the outward normal
            # points from the (inside) point to it, or along the edge normal
            # for a point on the edge
            keep = [a for a in range(3) if a != self.span_axis]
            P = np.asarray(self.poly, dtype=np.float64)
            A2, B2 = P, np.roll(P, -1, axis=0)
            q2 = p[:, keep]
            d = B2 - A2
            t = np.einsum("mnk,nk->mn", q2[:, None, :] - A2[None], d) / np.maximum(np.sum(d * d, axis=1), 1e-300)
            t = np.clip(t, 0.0, 1.0)
            near = A2[None] + t[..., None] * d[None]
            dist = np.linalg.norm(near - q2[:, None, :], axis=2)
            e = np.argmin(dist, axis=1)
            w2 = near[np.arange(len(p)), e]
            g = w2 - q2
            gl = np.linalg.norm(g, axis=1)
            de = d[e]
            en = np.stack([de[:, 1], -de[:, 0]], axis=1)
            en = en / np.maximum(np.linalg.norm(en, axis=1), 1e-300)[:, None]
            n2 = np.where(gl[:, None] > 1e-14, g / np.maximum(gl, 1e-300)[:, None], en)
            xw = p.copy()
            n = np.zeros_like(p)
            xw[:, keep] = w2
            n[:, keep] = n2
            return xw, n
        raise ValueError(self.kind)


# --------------------------------------------------------------------- blocks
@dataclass
class BlockSpec:
    n: tuple                 # physical cells (nx, ny, nz)
    h: tuple                 # cell sizes
    origin: tuple            # lower corner of cell (2,2,2)
    bctype: tuple            # 6 face codes
    parent: int = -1
    ratio: tuple = (1, 1, 1)
    offset: tuple = (0, 0, 0)
    arrays: dict = field(default_factory=dict)

    @property
    def dims(self):
        return tuple(v + 4 for v in self.n)   # (ib+1, jb+1, kb+1)

    @property
    def ncells(self):
        return self.n[0] * self.n[1] * self.n[2]


FACE_NORMALS = ((-1.0, 0.0, 0.0), (0.0, -1.0, 0.0), (0.0, 0.0, -1.0),
                (1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0))


def make_block_arrays(spec: BlockSpec, body: Body):
    """blank (Fortran order) and cut-cell records of one block."""
    nx, ny, nz = spec.n
    ox, oy, oz = spec.origin
    hx, hy, hz = spec.h
    P = (nx + 4, ny + 4, nz + 4)
    ii = np.arange(P[0], dtype=np.float64)
    jj = np.arange(P[1], dtype=np.float64)
    kk = np.arange(P[2], dtype=np.float64)
    xc = ox + (ii - 1.5) * hx
    yc = oy + (jj - 1.5) * hy
    zc = oz + (kk - 1.5) * hz
    # array indexed [k, j, i] so that ravel() is the Fortran order i-fastest
    solid = body.inside(xc[None, None, :], yc[None, :, None], zc[:, None, None])
    solid = np.broadcast_to(solid, (P[2], P[1], P[0])).copy()
    blank = np.ones((P[2], P[1], P[0]), dtype=np.int32)
    phys = (slice(2, nz + 2), slice(2, ny + 2), slice(2, nx + 2))
    blank[phys] = np.where(solid[phys], 0, 1)
    # ghost layers copied from the adjacent physical layer (init_metric.f90:207-218)
    il, jl, kl = nx + 1, ny + 1, nz + 1
    blank[:, :, 0] = blank[:, :, 2]
    blank[:, :, 1] = blank[:, :, 2]
    blank[:, :, il + 1] = blank[:, :, il]
    blank[:, :, il + 2] = blank[:, :, il]
    blank[:, 0, :] = blank[:, 2, :]
    blank[:, 1, :] = blank[:, 2, :]
    blank[:, jl + 1, :] = blank[:, jl, :]
    blank[:, jl + 2, :] = blank[:, jl, :]
    blank[0, :, :] = blank[2, :, :]
    blank[1, :, :] = blank[2, :, :]
    blank[kl + 1, :, :] = blank[kl, :, :]
    blank[kl + 2, :, :] = blank[kl, :, :]

    recs = []  # (linear cell, faceid, ccid, scid, zz)
    fl = (blank[phys] == 1)
    kcs, jcs, ics = np.nonzero(fl)
    ics = ics + 2
    jcs = jcs + 2
    kcs = kcs + 2
    offs = ((-1, 0, 0, 1), (0, -1, 0, 2), (0, 0, -1, 3), (1, 0, 0, 4), (0, 1, 0, 5), (0, 0, 1, 6))
    cand = []
    for di, dj, dk, fid in offs:
        si_, sj_, sk_ = ics + di, jcs + dj, kcs + dk
        inphys = (si_ >= 2) & (si_ <= il) & (sj_ >= 2) & (sj_ <= jl) & (sk_ >= 2) & (sk_ <= kl)
        sol = np.zeros_like(inphys)
        sol[inphys] = blank[sk_[inphys], sj_[inphys], si_[inphys]] == 0
        sel = np.nonzero(sol)[0]
        for q in sel:
            cand.append((ics[q] + P[0] * (jcs[q] + P[1] * kcs[q]), fid, ics[q], jcs[q], kcs[q], si_[q], sj_[q], sk_[q]))
    cand.sort(key=lambda t: (t[0], t[1]))
    nm = len(cand)
    ccid = np.zeros((nm, 3), dtype=np.int32)
    scid = np.zeros((nm, 3), dtype=np.int32)
    faceid = np.zeros(nm, dtype=np.int32)
    zz = np.zeros(nm, dtype=np.int32)
    for m, t in enumerate(cand):
        ccid[m] = t[2:5]
        scid[m] = t[5:8]
        faceid[m] = t[1]
        zz[m] = (t[1] - 1) % 3 + 1
    npoint = np.zeros(nm, dtype=np.int32)
    ijkdex = np.zeros((nm, A.MGE_MAX_CLOUD, 3), dtype=np.int32)
    coef = np.zeros((nm, A.MGE_MAX_CLOUD), dtype=np.float64)
    nvec = np.zeros((nm, 3), dtype=np.float64)
    if nm:
        xs = np.stack([ox + (scid[:, 0] - 1.5) * hx, oy + (scid[:, 1] - 1.5) * hy, oz + (scid[:, 2] - 1.5) * hz], axis=1)
        xw, n = body.project(xs)
        d = np.sum((xw - xs) * n, axis=1)
        xr = xs + 2.0 * d[:, None] * n
        if body.kind == "cylinder":
            xr[:, 2] = xs[:, 2]
        nvec[:] = n
        g = (xr - np.array([ox, oy, oz])) / np.array([hx, hy, hz]) + 1.5
        q0 = np.floor(g).astype(np.int64)
        fr = g - q0
        lim = np.array([P[0] - 2, P[1] - 2, P[2] - 2])
        q0 = np.clip(q0, 0, lim)
        if body.cloud == "rbf":
            for m in range(nm):
                pts, wts = rbf_cloud(xr[m], q0[m], blank, (ox, oy, oz), (hx, hy, hz), tuple(ccid[m]))
                npoint[m] = len(pts)
                for q, (pt, wgt) in enumerate(zip(pts, wts)):
                    ijkdex[m, q] = pt
                    coef[m, q] = wgt
        for m in (range(nm) if body.cloud != "rbf" else ()):
            pts, wts = [], []
            for dk in (0, 1):
                for dj in (0, 1):
                    for di in (0, 1):
                        wx = fr[m, 0] if di else 1.0 - fr[m, 0]
                        wy = fr[m, 1] if dj else 1.0 - fr[m, 1]
                        wz = fr[m, 2] if dk else 1.0 - fr[m, 2]
                        wgt = wx * wy * wz
                        ci, cj, ck = q0[m, 0] + di, q0[m, 1] + dj, q0[m, 2] + dk
                        if wgt <= 1e-14 or blank[ck, cj, ci] == 0:
                            continue
                        pts.append((ci, cj, ck))
                        wts.append(wgt)
            if not pts:
                pts, wts = [tuple(ccid[m])], [1.0]
            s = sum(wts)
            npoint[m] = len(pts)
            for q, (pt, wgt) in enumerate(zip(pts, wts)):
                ijkdex[m, q] = pt
                coef[m, q] = wgt / s
    area = np.zeros(nm, dtype=np.float64)
    for m in range(nm):
        ax = zz[m] - 1
        area[m] = [hy * hz, hx * hz, hx * hy][ax]
    spec.arrays = dict(blank=np.ascontiguousarray(blank.ravel()), nmir=nm, ccid=ccid, scid=scid,
                       faceid=faceid, zz=zz, npoint=npoint, ijkdex=ijkdex, coef=coef, nvec=nvec,
                       qb=(np.ascontiguousarray(body.wall_velocity(xw), dtype=np.float64)
                           if (nm and body.wall_velocity is not None) else np.zeros((nm, 3))), area=area,
                       psurf=np.ascontiguousarray(xw, dtype=np.float64) if nm else np.zeros((0, 3)))
    return spec


def mq_weights(nodes, x, csq):
    """Multiquadric radial-basis weights w with f(x) ~ sum w_i f(nodes_i):
    the interpolant sum_j a_j sqrt(|y - n_j|^2 + csq) + b through the nodes,
    with sum_j a_j = 0, evaluated at x.  The weights sum to 1, so constants
    are reproduced exactly."""
    nodes = np.asarray(nodes, dtype=np.float64)
    n = len(nodes)
    d2 = np.sum((nodes[:, None, :] - nodes[None, :, :]) ** 2, axis=2)
    M = np.ones((n + 1, n + 1))
    M[:n, :n] = np.sqrt(d2 + csq)
    M[n, n] = 0.0
    rhs = np.ones(n + 1)
    rhs[:n] = np.sqrt(np.sum((nodes - np.asarray(x)) ** 2, axis=1) + csq)
    return np.linalg.solve(M, rhs)[:n]


def rbf_cloud(x, q0, blank, origin, h, fallback):
    """The (at most MGE_MAX_CLOUD) fluid cell centres nearest the point x
    among the 4x4x4 cells around it, and their multiquadric weights; the
    shape parameter is the cloud's mean distance from its centroid."""
    P = blank.shape[::-1]  # (Pi, Pj, Pk); blank is indexed [k, j, i]
    cand = []
    for dk in range(-1, 3):
        for dj in range(-1, 3):
            for di in range(-1, 3):
                ci, cj, ck = q0[0] + di, q0[1] + dj, q0[2] + dk
                if not (0 <= ci < P[0] and 0 <= cj < P[1] and 0 <= ck < P[2]) or blank[ck, cj, ci] == 0:
                    continue
                c = np.array([origin[0] + (ci - 1.5) * h[0], origin[1] + (cj - 1.5) * h[1],
                              origin[2] + (ck - 1.5) * h[2]])
                cand.append((float(np.sum((c - x) ** 2)), (ci, cj, ck), c))
    if not cand:
        return [fallback], [1.0]
    cand.sort(key=lambda t: (t[0], t[1][2], t[1][1], t[1][0]))
    cand = cand[:A.MGE_MAX_CLOUD]
    nodes = np.array([t[2] for t in cand])
    if len(nodes) == 1:
        return [cand[0][1]], [1.0]
    lref = float(np.mean(np.sqrt(np.sum((nodes - nodes.mean(axis=0)) ** 2, axis=1))))
    w = mq_weights(nodes, x, lref * lref)
    return [t[1] for t in cand], [float(v) for v in w]


def _ptr(a, ctype):
    return a.ctypes.data_as(A.C.POINTER(ctype))


def block_desc(spec: BlockSpec):
    """ctypes descriptor pointing into spec.arrays (keep spec alive)."""
    d = A.MgeBlockDesc()
    d.nx, d.ny, d.nz = spec.n
    hx, hy, hz = spec.h
    d.h[:] = spec.h
    d.origin[:] = spec.origin
    d.cellvolume = hx * hy * hz
    d.si[:] = (-(hy * hz), 0.0, 0.0)
    d.sj[:] = (0.0, -(hx * hz), 0.0)
    d.sk[:] = (0.0, 0.0, -(hx * hy))
    d.bctype[:] = spec.bctype
    for f in range(6):
        d.facenvec[f][:] = FACE_NORMALS[f]
    a = spec.arrays
    d.blank = _ptr(a["blank"], A.C.c_int32)
    d.nmir = a["nmir"]
    for key in ("ccid", "scid", "faceid", "zz", "npoint", "ijkdex"):
        a[key] = np.ascontiguousarray(a[key], dtype=np.int32)
        setattr(d, key, _ptr(a[key], A.C.c_int32))
    for key in ("coef", "nvec", "qb", "area"):
        a[key] = np.ascontiguousarray(a[key], dtype=np.float64)
        setattr(d, key, _ptr(a[key], A.C.c_double))
    d.parent = spec.parent
    d.ratio[:] = spec.ratio
    d.offset[:] = spec.offset
    if a.get("psurf") is not None:
        a["psurf"] = np.ascontiguousarray(a["psurf"], dtype=np.float64)
        d.psurf = _ptr(a["psurf"], A.C.c_double)
    return d


# --------------------------------------------------------------------- params
def params(mach, alpha_deg=0.0, beta_deg=0.0, gamma=1.4, cfl=-2.8, vis2=0.5, vis4_in=0.5, smoo=0.6,
           cstp=(0.25, 1.0 / 6.0, 0.375, 0.5, 1.0), cdis=(1.0, 0.0, 0.56, 0.0, 0.44), mgtype=1,
           nlevel=3, mcyc=None, eqntype=A.MGE_EQN_EULER, distype=A.MGE_DIS_CENTRAL,
           dissip=A.MGE_DISSIP_SCALAR, precision=A.MGE_PREC_FP64, irs_variant=0, conv_drop=1.0e6,
           reynolds=None, prandtl=0.72, limfac=5.0, epsentr=0.05, execmode=0, dtstep=None):
    """mge_params as input_param.f90:17-114 derives them from a job sheet."""
    p = A.MgeParams()
    p.mstage = len(cstp)
    for q, v in enumerate(cstp):
        p.cstp[q] = v
    for q, v in enumerate(cdis):
        p.cdis[q] = v
    p.vt = 0 if cfl < 0.0 else 1          # input_param.f90:37-39
    p.cfl = abs(cfl)
    p.vis2 = vis2
    p.vis4 = vis4_in / 32.0               # input_param.f90:40
    p.smoo = smoo
    p.mgtype = mgtype
    p.eqntype = eqntype
    p.distype = distype
    p.dissip = dissip
    p.gamma = gamma
    p.rm = mach
    p.alpha = math.radians(alpha_deg)
    p.beta = math.radians(beta_deg)
    # non-dimensionalisation, input_param.f90:61-69
    p.rho0 = 1.0
    p.p0 = 1.0 / (gamma * mach ** 2.0)
    p.c0 = math.sqrt(gamma * p.p0 / p.rho0)
    p.ei0 = p.p0 / ((gamma - 1.0) * p.rho0)
    p.u0 = mach * p.c0 * math.cos(p.beta) * math.cos(p.alpha)
    p.v0 = mach * p.c0 * math.cos(p.beta) * math.sin(p.alpha)
    p.w0 = mach * p.c0 * math.sin(p.beta)
    p.h0 = gamma * p.ei0 + 0.5 * (p.u0 * p.u0 + p.v0 * p.v0 + p.w0 * p.w0)
    ref_leng = 1.0
    re = reynolds if reynolds is not None else 500.0   # the reference forces Re=500 (input_param.f90:111-114)
    p.viscl = p.rho0 * p.u0 * ref_leng / re if p.u0 != 0.0 else 0.0
    p.prlmean = prandtl
    # temperature scale: p = rho R T with T0 = 1
    p.gas_const = p.p0 / p.rho0
    p.limfac = limfac
    p.epsentr = epsentr
    p.wall_adiabatic = 1
    p.irs_variant = irs_variant
    p.precision = precision
    p.nlevel = nlevel
    mc = list(mcyc) if mcyc is not None else [10] * nlevel
    for q in range(nlevel):
        p.mcyc[q] = int(mc[q])
    p.conv_drop = conv_drop
    # unsteady dual time stepping: dtstep non-dimensional; the reference's
    # default for NS is u0/ref_leng/5 (input_param.f90:93-96)
    p.execmode = execmode
    p.dtstep = dtstep if dtstep is not None else (p.u0 / ref_leng / 5.0 if execmode == 1 else 0.0)
    return p


# --------------------------------------------------------------------- cases
@dataclass
class Case:
    name: str
    prm: A.MgeParams
    levels: list            # levels[l] = [BlockSpec, ...], l = 0 coarsest
    body: Body
    ref_area: float = 1.0

    def descs(self):
        return [[block_desc(s) for s in L] for L in self.levels]

    @property
    def finest_cells(self):
        return sum(s.ncells for s in self.levels[-1])

    def cells_per_level(self):
        return [sum(s.ncells for s in L) for L in self.levels]


def same_domain_hierarchy(body, lo, hi, n_fine, nlevel, coarsen=(True, True, True), bctype=(-20,) * 6):
    """Levels covering one domain, each a 2:1 coarsening of the next."""
    levels = []
    for L in range(nlevel):
        f = nlevel - 1 - L
        n = tuple(int(n_fine[d] // (2 ** f if coarsen[d] else 1)) for d in range(3))
        h = tuple((hi[d] - lo[d]) / n[d] for d in range(3))
        spec = BlockSpec(n=n, h=h, origin=tuple(lo), bctype=tuple(bctype),
                         parent=(1 if L > 0 else -1),
                         ratio=tuple(2 if (coarsen[d] and L > 0) else 1 for d in range(3)),
                         offset=(0, 0, 0))
        levels.append([make_block_arrays(spec, body)])
    return levels


def embedded_hierarchy(body, center, h_fine, n, nlevel, coarsen=(True, True, False), span=None):
    """Levels of equal cell count; each coarser level doubles h and extent."""
    levels = []
    for L in range(nlevel):
        f = nlevel - 1 - L
        h = tuple(h_fine[d] * (2 ** f if coarsen[d] else 1) for d in range(3))
        lo = tuple(center[d] - 0.5 * n[d] * h[d] for d in range(3))
        if L == 0:
            bct = (-20, -20, -60, -20, -20, -60) if not coarsen[2] else (-20,) * 6
        else:
            bct = (0, 0, -60, 0, 0, -60) if not coarsen[2] else (0,) * 6
        off = tuple((n[d] - n[d] // 2) // 2 if (coarsen[d] and L > 0) else 0 for d in range(3))
        spec = BlockSpec(n=tuple(n), h=h, origin=lo, bctype=bct, parent=(1 if L > 0 else -1),
                         ratio=tuple(2 if (coarsen[d] and L > 0) else 1 for d in range(3)), offset=off)
        levels.append([make_block_arrays(spec, body)])
    return levels


def cylinder_split(n=32, span=2, mach=0.3, overlap=4, mcyc_fine=4, **kw):
    """Flow past a D=1 cylinder on two levels: an n x n x span slab over
    [-4,4]^2 (h = 8/n), and embedded in it two fine blocks side by side in x
    (h/2), x in [-2, overlap*h/2] and [0, 2], y in [-2, 2], that share
    `overlap` fine cells around x = 0 and exchange ghost cells there
    (bc_overlap).  The body is cut in both fine blocks."""
    body = Body("cylinder", radius=0.5)
    hc = 8.0 / n
    hf = 0.5 * hc
    lo = (-4.0, -4.0, -0.5 * span * hc)
    coarse = BlockSpec(n=(n, n, span), h=(hc, hc, hc), origin=lo, bctype=(-20, -20, -60, -20, -20, -60))
    row = []
    for x0, x1 in ((-2.0, overlap * hf), (0.0, 2.0)):
        nxf = int(round((x1 - x0) / hf))
        off = (int(round((x0 - lo[0]) / hc)), int(round((-2.0 - lo[1]) / hc)), 0)
        spec = BlockSpec(n=(nxf, int(round(4.0 / hf)), span), h=(hf, hf, hc), origin=(x0, -2.0, lo[2]),
                         bctype=(0, 0, -60, 0, 0, -60), parent=1, ratio=(2, 2, 1), offset=off)
        row.append(make_block_arrays(spec, body))
    levels = [[make_block_arrays(coarse, body)], row]
    prm = params(mach, nlevel=2, mcyc=[1, mcyc_fine], mgtype=1, **kw)
    return Case("cylinder_split_%d" % n, prm, levels, body, ref_area=1.0 * span * hc)


def rotating(omega, center=(0.0, 0.0, 0.0)):
    """Wall velocity of a body turning at omega about the z axis through
    center: (-omega*(y-cy), omega*(x-cx), 0)."""
    def vel(xw):
        xw = np.asarray(xw, dtype=np.float64)
        out = np.zeros_like(xw)
        out[:, 0] = -omega * (xw[:, 1] - center[1])
        out[:, 1] = omega * (xw[:, 0] - center[0])
        return out
    return vel


def cylinder_slab(n=256, span=2, nlevel=3, extent=20.0, mach=0.3, mcyc_fine=500, smoo=0.6, omega=0.0,
                  cloud="trilinear", **kw):
    """Flow past a D=1 cylinder cut into an n x n x span slab over
    [-extent, extent]^2, periodic span, characteristic far field; omega != 0
    turns the wall about the cylinder axis (in free-stream speed per unit
    length)."""
    body = Body("cylinder", radius=0.5, wall_velocity=rotating(omega) if omega else None, cloud=cloud)
    h = 2.0 * extent / n
    lo = (-extent, -extent, -0.5 * span * h)
    hi = (extent, extent, 0.5 * span * h)
    levels = same_domain_hierarchy(body, lo, hi, (n, n, span), nlevel, coarsen=(True, True, False),
                                   bctype=(-20, -20, -60, -20, -20, -60))
    mcyc = [max(1, mcyc_fine // 5)] * (nlevel - 1) + [mcyc_fine]
    prm = params(mach, nlevel=nlevel, mcyc=mcyc, mgtype=1, smoo=smoo, **kw)
    return Case("cylinder_slab_%dx%dx%d" % (n, n, span), prm, levels, body, ref_area=1.0 * span * h)


def sphere_box(n=192, nlevel=4, extent=10.0, mach=0.5, mgtype=2, mcyc_fine=400, smoo=0.6, radius=0.5,
               cloud="trilinear", bctype=(-20,) * 6, **kw):
    """3-D inviscid flow past a D=1 sphere in an n^3 box [-extent, extent]^3.
    bctype: the six faces' boundary conditions (bcond.f90:16-42), far field
    by default."""
    body = Body("sphere", radius=radius, cloud=cloud)
    lo, hi = (-extent,) * 3, (extent,) * 3
    levels = same_domain_hierarchy(body, lo, hi, (n, n, n), nlevel, bctype=bctype)
    mcyc = [max(1, mcyc_fine // 8)] * (nlevel - 1) + [mcyc_fine]
    prm = params(mach, nlevel=nlevel, mcyc=mcyc, mgtype=mgtype, smoo=smoo, **kw)
    return Case("sphere_%d^3" % n, prm, levels, body, ref_area=math.pi * radius ** 2)


def ellipsoid_box(n=64, semi=(1.0, 0.7, 0.5), nlevel=3, extent=None, mach=0.5, alpha_deg=0.0, mgtype=2,
                  mcyc_fine=200, smoo=0.6, **kw):
    """3-D inviscid flow past an ellipsoid in an n^3 box."""
    body = Body("ellipsoid", semi=tuple(semi))
    ext = extent if extent is not None else 6.0 * max(semi)
    lo, hi = (-ext,) * 3, (ext,) * 3
    levels = same_domain_hierarchy(body, lo, hi, (n, n, n), nlevel)
    mcyc = [max(1, mcyc_fine // 8)] * (nlevel - 1) + [mcyc_fine]
    prm = params(mach, alpha_deg=alpha_deg, nlevel=nlevel, mcyc=mcyc, mgtype=mgtype, smoo=smoo, **kw)
    return Case("ellipsoid_%d^3" % n, prm, levels, body, ref_area=math.pi * semi[1] * semi[2])


def cylinder_embedded(n=512, span=2, nlevel=4, h_fine=1.0 / 96.0, mach=0.2, mcyc_fine=200, **kw):
    """Slab cylinder with embedded levels: each coarser level doubles h and extent."""
    body = Body("cylinder", radius=0.5)
    levels = embedded_hierarchy(body, (0.0, 0.0, 0.0), (h_fine, h_fine, h_fine), (n, n, span), nlevel)
    mcyc = [max(1, mcyc_fine // 5)] * (nlevel - 1) + [mcyc_fine]
    prm = params(mach, nlevel=nlevel, mcyc=mcyc, mgtype=1, **kw)
    return Case("cylinder_embedded_%dx%dx%d" % (n, n, span), prm, levels, body, ref_area=span * h_fine)


def recirculation_length(levels, radius=0.5):
    """Length of the closed wake behind a cylinder whose axis is z, with the
    free stream along +x: from the rear of the body (x = radius) along y = 0
    to the first point where the span-averaged u = (rho u)/rho turns from
    negative to non-negative, linear between cell centres.

    ``levels`` lists (w, spec) pairs, finest first, with w shaped (5, k, j, i)
    over the block's cells with their two ghost layers (as ``Cycle.field``
    returns it).  Each x takes the finest level whose physical cells cover it.
    Returns 0.0 when u is not negative just behind the body, and None when the
    wake is still open at the last cell."""
    xs, us, covered = [], [], -np.inf
    for w, sp in levels:
        nx, ny, nz = sp.n
        hx, hy = sp.h[0], sp.h[1]
        ox, oy = sp.origin[0], sp.origin[1]
        yc = oy + (np.arange(ny) + 0.5) * hy
        # the rows straddling y = 0 (one row when a cell centre lies on it)
        jlo = int(np.searchsorted(yc, 0.0, side="right")) - 1
        rows = [jlo] if abs(yc[jlo]) <= 1e-12 * hy else [jlo, jlo + 1]
        ph = w[:, 2:nz + 2, 2:ny + 2, 2:nx + 2]
        u = np.mean([ph[1, :, j, :] / ph[0, :, j, :] for j in rows], axis=0).mean(axis=0)
        xc = ox + (np.arange(nx) + 0.5) * hx
        keep = (xc > radius) & (xc > covered)
        xs.append(xc[keep])
        us.append(u[keep])
        covered = max(covered, ox + nx * hx)
    x, u = np.concatenate(xs), np.concatenate(us)
    order = np.argsort(x)
    x, u = x[order], u[order]
    if len(x) == 0 or u[0] >= 0.0:
        return 0.0
    pos = np.nonzero(u >= 0.0)[0]
    if len(pos) == 0:
        return None
    i = pos[0]
    x0 = x[i - 1] + (0.0 - u[i - 1]) * (x[i] - x[i - 1]) / (u[i] - u[i - 1])
    return float(x0 - radius)


def free_stream_box(n=(12, 10, 8), nlevel=2, mach=0.5, bctype=(-20,) * 6, **kw):
    """No body: free-stream preservation case."""
    body = Body("none")
    lo, hi = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)
    levels = same_domain_hierarchy(body, lo, hi, n, nlevel, bctype=bctype)
    prm = params(mach, nlevel=nlevel, **kw)
    return Case("free_stream", prm, levels, body)
