"""ORACLE / TEST INFRASTRUCTURE ONLY -- a numpy restatement of the reference's SIMPLE
hot path, used to check the GPU implementation where the compiled reference
(oracle/_ref) is not available.  It is never imported by the product.

Every function cites the reference source it restates.  Loops over faces are
vectorised with numpy (scatter-adds via np.add.at); the arithmetic inside each formula
keeps the reference's expression order, so geometry is bit-identical to the compiled
reference and the fields agree to rounding.  Pinned against the compiled reference by
the golden fixtures of tests/golden (tests/test_cpu_oracle.py).

Scope: steady, density model 0, laminar or k-epsilon, energy with the fluid/solid
conjugate coupling, limiters no/Barth/MLP/WENO; linear solves with the restated
CG and BiCGSTAB (Jacobi preconditioner), matching the GMRES->BiCGSTAB and
SSOR->Jacobi remap the configurations ask for.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Dict, List, Optional

import numpy as np

SMALL = 1.e-16  # BasicType.h:15


# --------------------------------------------------------------------------------
# param.in -- readparamfile.cpp:10-260
@dataclasses.dataclass
class Region:
    type1: int = -1
    type2: int = -1
    fixed: float = 2147483647.0
    init: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(10))


@dataclasses.dataclass
class Params:
    gridfile: str = ""
    steady: bool = True
    max_step: int = 10000
    residual_steady: float = 1e-6
    solve_energy: bool = False
    heat_conduction: bool = False
    tur_model: int = 0
    density_model: int = 0
    gravity: tuple = (0.0, 0.0, 0.0)
    pref: float = 1.01325e5
    cell_pref: int = 0
    urf: List[float] = dataclasses.field(default_factory=lambda: [0.6, 0.6, 0.6, 0.5, 0.8, 0.8, 0.8, 0.8])
    limiter: int = 0
    regions: Dict[int, Region] = dataclasses.field(default_factory=dict)
    cp: float = 1006.0
    prl: float = 0.72
    prte: float = 0.9


def parse_params(path: str) -> Params:
    p = Params()
    raw = open(path, "rb").read().decode()
    lines = raw.split("\n")
    if lines and lines[-1] == "":  # std::getline yields no line after a final newline
        lines.pop()
    for line in lines:
        if line.startswith("//") or len(line) == 1:
            continue
        kw = [t.strip() for t in line.split(",")]
        ikey = len(kw) - 1
        kw += [""] * (20 - len(kw))
        k = kw[0]
        f = lambda s: float(s) if s else 0.0  # noqa: E731  (atof of "" is 0)
        if k == "gridfile":
            p.gridfile = kw[1]
        elif k == "steady":
            p.steady, p.max_step, p.residual_steady = True, int(kw[1]), f(kw[2])
        elif k == "energy":
            p.solve_energy = kw[1] == "on"
        elif k == "density":
            p.density_model = int(kw[1])
        elif k == "turbulence":
            p.tur_model = 1 if kw[1] == "ke" else 0
        elif k == "gravity":
            p.gravity = (f(kw[1]), f(kw[2]), f(kw[3]))
        elif k == "PressureRef":
            p.pref = f(kw[1])
            if kw[2]:
                p.cell_pref = int(kw[2]) - 1
        elif k == "relaxation":
            p.urf[0] = p.urf[1] = p.urf[2] = f(kw[1])
            p.urf[3], p.urf[4] = f(kw[2]), f(kw[3])
        elif k == "limiter":
            p.limiter = {"no": 0, "Barth": 1, "MLP": 2, "WENO": 3}[kw[1]]
        elif k == "bound":
            bid = int(kw[1])
            r = Region()
            t = kw[2]
            if t == "Twall":
                r.type1, r.type2, r.fixed = 1, 0, f(kw[3])
            elif t == "Hwall":
                r.type1, r.type2, r.fixed = 1, 1, f(kw[3])
            elif t == "sym":
                r.type1, r.type2, r.fixed = 4, 0, 0.0
            elif t == "inlet":
                r.type1, r.type2 = 2, 0
                for i in range(6):
                    r.init[i] = f(kw[3 + i])
                if p.tur_model == 1:
                    r.init[6], r.init[7] = f(kw[9]), f(kw[10])
            elif t == "outlet":
                r.type1, r.type2, r.fixed = 3, 0, f(kw[3])
            else:
                raise ValueError("unknown boundry type in bound")
            p.regions[bid] = r
        elif k == "volumn":
            bid = int(kw[1])
            r = Region(type1=5, type2=0 if kw[2] == "fluid" else 1)
            for i in range(4, ikey + 1):
                r.init[i - 4] = f(kw[i])
            p.regions[bid] = r
        elif k == "output":
            pass
        elif k == "3dheatconduction":
            p.heat_conduction = True
        else:
            raise ValueError("no such command: " + k)
    return p


# --------------------------------------------------------------------------------
# mesh -- Preprocessor.cpp:13-146 (reader), :181-299 (faces), :308-438 (split)
def read_msh(path: str):
    tok = open(path).read().split()
    pos = 6
    nv = int(tok[pos]); pos += 1
    vert = np.array(tok[pos:pos + 4 * nv], dtype=np.float64).reshape(nv, 4)[:, 1:]
    pos += 4 * nv + 2
    ne = int(tok[pos]); pos += 1
    nn = {2: 3, 3: 4, 4: 4, 5: 8}
    cells, crid, bnd, brid = [], [], [], []
    for _ in range(ne):
        et, nt = int(tok[pos + 1]), int(tok[pos + 2])
        tags = tok[pos + 3:pos + 3 + nt]
        v = [int(x) - 1 for x in tok[pos + 3 + nt:pos + 3 + nt + nn[et]]]
        pos += 3 + nt + nn[et]
        if et == 2:
            bnd.append([v[0], v[1], v[2], v[2]]); brid.append(int(tags[0]))
        elif et == 3:
            bnd.append(v); brid.append(int(tags[0]))
        elif et == 4:
            cells.append([v[0], v[1], v[2], v[2], v[3], v[3], v[3], v[3]]); crid.append(int(tags[0]))
        else:
            cells.append(v); crid.append(int(tags[0]))
    return vert, np.array(cells, np.int64), np.array(crid), np.array(bnd, np.int64).reshape(-1, 4), np.array(brid)


_LOCAL_FACES = ((0, 1, 2, 3), (4, 5, 6, 7), (0, 1, 5, 4), (1, 2, 6, 5), (3, 2, 6, 7), (0, 3, 7, 4))


@dataclasses.dataclass
class Mesh:
    vert: np.ndarray
    cells: np.ndarray       # (nc, 8)
    crid: np.ndarray
    cface: List[List[int]]  # reference Cell[i].face
    fvert: np.ndarray       # (nf, 4)
    c1: np.ndarray
    c2: np.ndarray
    fbnd: np.ndarray
    bface: np.ndarray
    brid: np.ndarray
    ncb: int


def create_faces(vert, cells, crid, bnd, brid) -> Mesh:
    fv, c1, c2, fb = [], [], [], []
    table = {}
    for i, b in enumerate(bnd):
        table[frozenset(b.tolist())] = len(fv)
        fv.append(list(b)); fb.append(i); c1.append(-10); c2.append(-10)
    cface = []
    for ic, cv in enumerate(cells):
        cf = []
        for q in _LOCAL_FACES:
            n1, n2, n3, n4 = (int(cv[k]) for k in q)
            rep = int(n1 in (n2, n3, n4)) + int(n2 in (n3, n4)) + int(n3 == n4)
            if rep > 1:
                continue
            key = frozenset((n1, n2, n3, n4))
            fid = table.get(key)
            if fid is None:
                fid = len(fv)
                table[key] = fid
                fv.append([n1, n2, n3, n4]); c1.append(ic); c2.append(-20); fb.append(-10)
            elif fb[fid] >= 0:
                if c1[fid] == -10:
                    c1[fid] = ic
                else:
                    c2[fid] = ic
            else:
                c2[fid] = ic
            cf.append(fid)
        cface.append(cf)
    return Mesh(vert, cells, crid, cface, np.array(fv, np.int64), np.array(c1), np.array(c2), np.array(fb),
                np.arange(len(bnd)), np.array(brid), len(bnd))


def extract(m: Mesh, new2old, coupled_rid) -> Mesh:
    o2nv, verts = {}, []
    cells = np.zeros((len(new2old), 8), np.int64)
    for i, o in enumerate(new2old):
        for j in range(8):
            iv = int(m.cells[o, j])
            if iv not in o2nv:
                o2nv[iv] = len(verts); verts.append(m.vert[iv])
            cells[i, j] = o2nv[iv]
    o2nf, fv, c1, c2, fb, cface = {}, [], [], [], [], []
    for i, o in enumerate(new2old):
        cf = []
        for of in m.cface[o]:
            if of in o2nf:
                c2[o2nf[of]] = i
            else:
                o2nf[of] = len(fv)
                fv.append([o2nv[int(v)] for v in m.fvert[of]]); c1.append(i); c2.append(-10); fb.append(int(m.fbnd[of]))
            cf.append(o2nf[of])
        cface.append(cf)
    bface, brid = [], []
    for f in range(len(fv)):
        if c2[f] < 0 and fb[f] >= 0:
            brid.append(int(m.brid[fb[f]])); bface.append(f); fb[f] = len(bface) - 1
    ncb = len(bface)
    for f in range(len(fv)):
        if c2[f] < 0 and fb[f] < 0:
            brid.append(coupled_rid); bface.append(f); fb[f] = len(bface) - 1
    return Mesh(np.array(verts), cells, m.crid[np.array(new2old)], cface, np.array(fv, np.int64), np.array(c1),
                np.array(c2), np.array(fb), np.array(bface), np.array(brid), ncb)


# --------------------------------------------------------------------------------
# geometry -- BasicSolver.cpp:296-512 (same expression order, vectorised)
def _dot3(a, b):
    return ((0. + a[..., 0] * b[..., 0]) + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def _cross(b, c):
    return np.stack([b[..., 1] * c[..., 2] - b[..., 2] * c[..., 1], -b[..., 0] * c[..., 2] + b[..., 2] * c[..., 0],
                     b[..., 0] * c[..., 1] - b[..., 1] * c[..., 0]], axis=-1)


def _tri_area(x1, x2, x3):
    a = _cross(x2 - x1, x3 - x1)
    return 0.5 * np.sqrt(a[..., 0] * a[..., 0] + a[..., 1] * a[..., 1] + a[..., 2] * a[..., 2])


def _tet_vol(x1, x2, x3, x4):
    return 1. / 6. * np.abs(_dot3(_cross(x2 - x1, x3 - x1), x4 - x1))


@dataclasses.dataclass
class Geom:
    vol: np.ndarray
    cx: np.ndarray
    fx: np.ndarray
    fn: np.ndarray
    area: np.ndarray
    lam: np.ndarray
    rl: np.ndarray
    xpac: np.ndarray
    xnac: np.ndarray
    bdist: np.ndarray


def geometry(m: Mesh) -> Geom:
    V = m.vert
    cv = V[m.cells]
    cx = 1. / 8. * (((((((cv[:, 0] + cv[:, 1]) + cv[:, 2]) + cv[:, 3]) + cv[:, 4]) + cv[:, 5]) + cv[:, 6]) + cv[:, 7])
    p1, p2, p3, p4 = (V[m.fvert[:, k]] for k in range(4))
    a1, a2 = _tri_area(p1, p2, p4), _tri_area(p2, p3, p4)
    xc1 = 1. / 3 * ((p1 + p2) + p4)
    xc2 = 1. / 3 * ((p2 + p3) + p4)
    fx = (a1[:, None] * xc1 + a2[:, None] * xc2) / (a1 + a2)[:, None]
    fn = 0.5 * _cross(p1 - p3, p2 - p4)
    flip = _dot3(fn, fx - cx[m.c1]) < 0.
    fn[flip] = -fn[flip]
    area = np.sqrt(_dot3(fn, fn))
    inner = m.c2 >= 0
    lam = np.ones(len(fn))
    c2s = np.where(inner, m.c2, 0)
    r1 = np.sqrt(_dot3(fx - cx[m.c1], fx - cx[m.c1]))
    r2 = np.sqrt(_dot3(fx - cx[c2s], fx - cx[c2s]))
    lam[inner] = (r2 / (r1 + r2))[inner]
    x = [cv[:, k] for k in range(8)]
    Vs = [_tet_vol(x[0], x[1], x[3], x[5]), _tet_vol(x[0], x[4], x[3], x[5]), _tet_vol(x[3], x[4], x[7], x[5]),
          _tet_vol(x[1], x[2], x[3], x[6]), _tet_vol(x[1], x[5], x[3], x[6]), _tet_vol(x[7], x[3], x[5], x[6])]
    vol = ((((Vs[0] + Vs[1]) + Vs[2]) + Vs[3]) + Vs[4]) + Vs[5]
    cs = [0.25 * (((x[0] + x[1]) + x[3]) + x[5]), 0.25 * (((x[0] + x[4]) + x[3]) + x[5]),
          0.25 * (((x[3] + x[4]) + x[7]) + x[5]), 0.25 * (((x[1] + x[2]) + x[3]) + x[6]),
          0.25 * (((x[1] + x[5]) + x[3]) + x[6]), 0.25 * (((x[7] + x[3]) + x[5]) + x[6])]
    num = Vs[0][:, None] * cs[0]
    for k in range(1, 6):
        num = num + Vs[k][:, None] * cs[k]
    cx = (1. / vol)[:, None] * num
    bf = m.bface
    bdist = _dot3(fx[bf] - cx[m.c1[bf]], fn[bf]) / area[bf]
    d = np.where(inner[:, None], cx[c2s], fx) - cx[m.c1]
    rl = area / (_dot3(d, fn) / area)
    xpac = np.zeros_like(fx)
    xnac = np.zeros_like(fx)
    ss = _dot3(fx - cx[m.c1], fn) / area
    xpac[inner] = (fx - (ss[:, None] * fn) / area[:, None])[inner]
    ss = _dot3(fx - cx[c2s], fn) / area
    xnac[inner] = (fx - (ss[:, None] * fn) / area[:, None])[inner]
    return Geom(vol, cx, fx, fn, area, lam, rl, xpac, xnac, bdist)


# --------------------------------------------------------------------------------
# Krylov -- the LASPack call sites (tools.cpp:56-64) with the restated algorithms
def _csr_mv(rp, cl, vl, x):
    """y = A x, each row summed over its entries in storage order (reduceat over the
    non-empty rows; an empty row gives 0)."""
    y = np.zeros(len(rp) - 1)
    prod = vl[:rp[-1]] * x[cl[:rp[-1]]]
    nz = np.flatnonzero(np.diff(rp))
    if nz.size:
        y[nz] = np.add.reduceat(prod, np.asarray(rp)[nz])
    return y


def cg(A, b, x, maxit, eps, omega):
    """Jacobi-PCG (Templates Fig. 2.5); returns x, iterations, relative residual."""
    rp, cl, vl, d = A
    bn = np.linalg.norm(b) or 1.0
    r = b - _csr_mv(rp, cl, vl, x)
    res = np.linalg.norm(r) / bn
    it, rho_prev, p = 0, 1.0, None
    while not (res < eps) and it < maxit:
        it += 1
        z = omega * r / d
        rho = r @ z
        p = z.copy() if it == 1 else z + (rho / rho_prev) * p
        q = _csr_mv(rp, cl, vl, p)
        pq = p @ q
        if pq == 0.0:
            break
        a = rho / pq
        x = x + a * p
        r = r - a * q
        res = np.linalg.norm(r) / bn
        rho_prev = rho
    return x, it, res


def bicgstab(A, b, x, maxit, eps, omega):
    """Right-preconditioned BiCGSTAB (Templates Fig. 2.10), Jacobi M = D/omega."""
    rp, cl, vl, d = A
    bn = np.linalg.norm(b) or 1.0
    r = b - _csr_mv(rp, cl, vl, x)
    rt = r.copy()
    res = np.linalg.norm(r) / bn
    it, rho_prev, alpha, om = 0, 1.0, 1.0, 1.0
    p = v = None
    while not (res < eps) and it < maxit:
        rho = rt @ r
        if rho == 0.0:
            break
        it += 1
        p = r.copy() if it == 1 else r + (rho / rho_prev) * (alpha / om) * (p - om * v)
        ph = omega * p / d
        v = _csr_mv(rp, cl, vl, ph)
        rtv = rt @ v
        if rtv == 0.0:
            break
        alpha = rho / rtv
        s = r - alpha * v
        sn = np.linalg.norm(s) / bn
        if sn < eps:
            x = x + alpha * ph
            res = sn
            break
        sh = omega * s / d
        t = _csr_mv(rp, cl, vl, sh)
        tt = t @ t
        om = (t @ s) / tt if tt != 0.0 else 0.0
        x = x + (alpha * ph + om * sh)
        r = s - om * t
        res = np.linalg.norm(r) / bn
        rho_prev = rho
        if om == 0.0:
            break
    return x, it, res


# --------------------------------------------------------------------------------
class Domain:
    """Mesh + geometry + the per-cell face lists of one domain."""

    def __init__(self, m: Mesh, p: Params):
        self.m = m
        self.g = geometry(m)
        self.nc, self.nf, self.nb = len(m.cells), len(m.c1), len(m.bface)
        self.ncb = m.ncb
        self.inner = np.where(m.c2 >= 0)[0]
        self.bc1 = m.c1[m.bface]
        self.t1 = np.array([p.regions[r].type1 for r in m.brid])
        self.t2 = np.array([p.regions[r].type2 for r in m.brid])
        self.binit = np.array([p.regions[r].init for r in m.brid]).reshape(-1, 10)
        self.bfixed = np.array([p.regions[r].fixed for r in m.brid])
        # CSR pattern: row i = [i, interior neighbours in Cell[i].face order]
        rows, cols, self.slot_face, self.slot_row = [0], [], [], []
        for i, cf in enumerate(m.cface):
            cols.append(i)
            for f in cf:
                if m.c2[f] >= 0:
                    cols.append(int(m.c2[f] if m.c1[f] == i else m.c1[f]))
                    self.slot_face.append(f)
                    self.slot_row.append(i)
            rows.append(len(cols))
        self.rp = np.array(rows)
        self.cl = np.array(cols)
        self.diagpos = self.rp[:-1]
        off = np.ones(len(cols), bool)
        off[self.diagpos] = False
        self.offpos = np.where(off)[0]
        self.slot_face = np.array(self.slot_face, np.int64)
        self.slot_row = np.array(self.slot_row, np.int64)
        # wall records per cell, in record order (navier_bc.cpp:478-518)
        self.walls = [b for b in range(self.nb) if self.t1[b] == 1]

    # Gradient + limiter, BasicSolver.cpp:29-288
    def gradient(self, phi, bphi, limiter):
        m, g = self.m, self.g
        gr = np.zeros((self.nc, 3))
        inn = self.inner
        pf = g.lam[inn] * phi[m.c1[inn]] + (1. - g.lam[inn]) * phi[m.c2[inn]]
        np.add.at(gr, m.c1[inn], pf[:, None] * g.fn[inn])
        np.add.at(gr, m.c2[inn], -(pf[:, None] * g.fn[inn]))
        bf = m.bface
        np.add.at(gr, m.c1[bf], bphi[:, None] * g.fn[bf])
        gr = gr / g.vol[:, None]
        if limiter == 3:
            w = 1. / (_dot3(gr, gr) + 1.e-16)
            ss = w.copy()
            t = w[:, None] * gr
            np.add.at(ss, m.c1[inn], w[m.c2[inn]])
            np.add.at(ss, m.c2[inn], w[m.c1[inn]])
            np.add.at(t, m.c1[inn], w[m.c2[inn], None] * gr[m.c2[inn]])
            np.add.at(t, m.c2[inn], w[m.c1[inn], None] * gr[m.c1[inn]])
            gr = t / ss[:, None]
        elif limiter in (1, 2):
            if limiter == 1:
                umax, umin = phi.copy(), phi.copy()
                np.maximum.at(umax, m.c1[inn], phi[m.c2[inn]])
                np.maximum.at(umax, m.c2[inn], phi[m.c1[inn]])
                np.minimum.at(umin, m.c1[inn], phi[m.c2[inn]])
                np.minimum.at(umin, m.c2[inn], phi[m.c1[inn]])
                umax, umin = (umax - phi)[:, None], (umin - phi)[:, None]
            else:
                vmax = np.full(len(m.vert), -1.e8)
                vmin = np.full(len(m.vert), 1.e8)
                np.maximum.at(vmax, m.cells.ravel(), np.repeat(phi, 8))
                np.minimum.at(vmin, m.cells.ravel(), np.repeat(phi, 8))
                umax = vmax[m.cells] - phi[:, None]
                umin = vmin[m.cells] - phi[:, None]
            dx = m.vert[m.cells] - g.cx[:, None, :]
            us = _dot3(np.broadcast_to(gr[:, None, :], dx.shape), dx)
            with np.errstate(divide="ignore", invalid="ignore"):
                f = np.where(us > 1.0e-10, np.minimum(1., umax / us),
                             np.where(us < -1.0e-10, np.minimum(1., umin / us), 1.))
            fi = np.minimum(10., f.min(axis=1))
            gr = fi[:, None] * gr
        return gr


    # Least-squares gradient -- not the reference's (it has Green-Gauss only,
    # BasicSolver.cpp:29-77): the GPU implementation's option "gradient" 1, restated
    # here as its CPU check.  grad phi_c solves sum_j w_j d_j d_j^T g = sum_j w_j d_j
    # (phi_j - phi_c) over the cell's faces, d_j from the cell centroid to the
    # neighbour's centroid (interior face) or to the face centroid (boundary face,
    # phi_j the boundary value), w_j = 1 / |d_j|^2.
    def gradient_lsq(self, phi, bphi):
        m, g = self.m, self.g
        M = np.zeros((self.nc, 3, 3))
        rhs = np.zeros((self.nc, 3))
        inn = self.inner
        for c, o in ((m.c1[inn], m.c2[inn]), (m.c2[inn], m.c1[inn])):
            d = g.cx[o] - g.cx[c]
            w = 1. / _dot3(d, d)
            np.add.at(M, c, w[:, None, None] * d[:, :, None] * d[:, None, :])
            np.add.at(rhs, c, (w * (phi[o] - phi[c]))[:, None] * d)
        bf = m.bface
        c = m.c1[bf]
        d = g.fx[bf] - g.cx[c]
        w = 1. / _dot3(d, d)
        np.add.at(M, c, w[:, None, None] * d[:, :, None] * d[:, None, :])
        np.add.at(rhs, c, (w * (bphi - phi[c]))[:, None] * d)
        return np.linalg.solve(M, rhs[:, :, None])[:, :, 0]


class SimpleNP:
    """The reference's NavierStokesSolver + HeatConductionSolver, restated."""

    def __init__(self, param_path: str, rtc: Optional[float] = None):
        self.p = p = parse_params(param_path)
        grid = p.gridfile
        if not os.path.isabs(grid):
            grid = os.path.join(os.path.dirname(param_path), grid)
        vert, cells, crid, bnd, brid = read_msh(grid)
        gm = create_faces(vert, cells, crid, bnd, brid)
        self.solid = None
        if p.heat_conduction:
            crid_ = next(i for i in range(len(p.regions) + 1) if i not in p.regions)
            p.regions[crid_] = Region(1, 2, 2147483647.0)
            fl = [i for i in range(len(cells)) if p.regions[int(crid[i])].type2 == 0]
            so = [i for i in range(len(cells)) if p.regions[int(crid[i])].type2 == 1]
            self.d = Domain(extract(gm, fl, crid_), p)
            self.solid = Domain(extract(gm, so, crid_), p)
        else:
            self.d = Domain(gm, p)
        self.eps = {"mom": 1e-8, "p": 1e-6, "ke": 1e-8, "t": 1e-8, "ts": 1e-8}
        if rtc is not None:
            self.eps = {k: rtc for k in self.eps}
        self.Residual = np.zeros(10)
        # convection of momentum and the fluid scalars: False the reference's scheme;
        # True the hybrid scheme of the GPU implementation's option "convection" 1
        # (not in the reference)
        self.hybrid = False
        self.init_flow_field()

    # navier.cpp:113-188, HeatConductionSolver.cpp:334-369
    def init_flow_field(self):
        d, p = self.d, self.p
        iv = np.array([p.regions[int(r)].init for r in d.m.crid])
        self.U, self.V, self.W, self.R, self.T = (iv[:, k].copy() for k in range(5))
        self.P = np.zeros(d.nc)
        self.VisLam = iv[:, 5].copy()
        self.VisTur = np.zeros(d.nc)
        self.TE = np.zeros(d.nc)
        self.ED = np.zeros(d.nc)
        if p.tur_model == 1:
            self.TE, self.ED = iv[:, 6].copy(), iv[:, 7].copy()
            self.VisTur = self.R * 0.09 * self.TE * self.TE / (self.ED + SMALL)
        nb = d.nb
        self.BTem = np.zeros(nb)
        self.Bq = np.zeros(nb)
        for b in range(nb):
            t1, t2 = d.t1[b], d.t2[b]
            if t1 == 1:
                if t2 == 0:
                    self.BTem[b] = d.bfixed[b]
                elif t2 == 1:
                    self.Bq[b] = d.bfixed[b]
            elif t1 == 2:
                self.BTem[b] = d.binit[b, 5]
        self.RUFace = np.zeros(d.nf)
        self.BTE = np.zeros(nb)
        self.BED = np.zeros(nb)
        if self.solid is not None:
            s = self.solid
            iv = np.array([p.regions[int(r)].init for r in s.m.crid])
            self.sT, self.sR, self.sK = iv[:, 0].copy(), iv[:, 1].copy(), iv[:, 2].copy()
            self.sBTem = np.zeros(s.nb)
            self.sBq = np.zeros(s.nb)
            for b in range(s.nb):
                if s.t1[b] == 1 and s.t2[b] == 0:
                    self.sBTem[b] = s.bfixed[b]
                elif s.t1[b] == 1 and s.t2[b] == 1:
                    self.sBq[b] = s.bfixed[b]
            self._solid_bc()
            self.sdPhi = s.gradient(self.sT, self.sBTem, p.limiter)

    # SetBCVelocity, navier_bc.cpp:8-108
    def bc_velocity(self):
        d = self.d
        ic = d.bc1
        g = d.g
        bf = d.m.bface
        BR, BU, BV, BW = self.R[ic].copy(), np.zeros(d.nb), np.zeros(d.nb), np.zeros(d.nb)
        t = d.t1
        m = t == 2
        BR[m], BU[m], BV[m], BW[m] = d.binit[m, 4], d.binit[m, 0], d.binit[m, 1], d.binit[m, 2]
        m = t == 3
        BU[m], BV[m], BW[m] = self.U[ic][m], self.V[ic][m], self.W[ic][m]
        m = t == 4
        s = g.fn[bf][m] / g.area[bf][m, None]
        un = (self.U[ic][m] * s[:, 0] + self.V[ic][m] * s[:, 1]) + self.W[ic][m] * s[:, 2]
        BU[m] = self.U[ic][m] - un * s[:, 0]
        BV[m] = self.V[ic][m] - un * s[:, 1]
        BW[m] = self.W[ic][m] - un * s[:, 2]
        if np.any(t == 3):
            fl = BR * ((BU * g.fn[bf, 0] + BV * g.fn[bf, 1]) + BW * g.fn[bf, 2])
            mi, mo = fl[t == 2].sum(), fl[t == 3].sum()
            m = t == 3
            if abs(mo) > SMALL:
                rate = -mi / mo
                BU[m] *= rate; BV[m] *= rate; BW[m] *= rate
            else:
                ao = (BR[m] * g.area[np.arange(d.nb)][m]).sum()  # navier_bc.cpp:72 indexes Face[i]
                rate = (-mi - mo) / ao
                BU[m] += rate * g.fn[bf][m, 0] / g.area[bf][m]
                BV[m] += rate * g.fn[bf][m, 1] / g.area[bf][m]
                BW[m] += rate * g.fn[bf][m, 2] / g.area[bf][m]
        self.BRo, self.BU, self.BV, self.BW = BR, BU, BV, BW

    def _assemble(self, d, app, su, offd):
        """Matrix (CSR, diag first) from per-cell app and per-slot off-diagonals."""
        val = np.zeros(len(d.cl))
        val[d.diagpos] = app
        val[d.offpos] = offd
        return (d.rp, d.cl, val, app)

    def _slot_terms(self, d, face_val_c1side, sign_flip):
        """Per-slot value: the face value from the slot's cell side."""
        f = d.slot_face
        first = d.m.c1[f] == d.slot_row
        v = face_val_c1side[f]
        return np.where(first, v, -v) if sign_flip else v, first

    # BuildVelocityMatrix + CalculateVelocity, navier_velocity.cpp:12-357
    def calculate_velocity(self):
        d, p, g, m = self.d, self.p, self.d.g, self.d.m
        self.Residual[:] = 0.
        self.bc_velocity()
        self.BPre = self.P[d.bc1].copy()
        self.dU = d.gradient(self.U, self.BU, p.limiter)
        self.dV = d.gradient(self.V, self.BV, p.limiter)
        self.dW = d.gradient(self.W, self.BW, p.limiter)
        self.dP = d.gradient(self.P, self.BPre, p.limiter)
        mu = self.VisLam + self.VisTur
        inn = d.inner
        c1, c2 = m.c1[inn], m.c2[inn]
        lam = g.lam[inn][:, None]
        lam2 = 1. - lam
        S = g.fn[inn]
        RU = self.RUFace[inn]
        Visc = (g.lam[inn] * mu[c1] + (1. - g.lam[inn]) * mu[c2])
        G = [lam * gr[c1] + lam2 * gr[c2] for gr in (self.dU, self.dV, self.dW)]
        D = Visc * g.rl[inn]
        up = np.where(RU > 0., c1, c2)
        dx = g.fx[inn] - g.cx[up]
        phis = (self.U, self.V, self.W)
        grs = (self.dU, self.dV, self.dW)
        fcs = [RU * ((ph[up] + _dot3(gr[up], dx)) - ph[up]) for ph, gr in zip(phis, grs)]
        if self.hybrid:  # option of the GPU implementation: no deferred correction
            fcs = [np.zeros_like(RU) for _ in range(3)]
        du, dv, dw = G
        fde = [((du[:, 0] + du[:, 0]) * S[:, 0] + (du[:, 1] + dv[:, 0]) * S[:, 1] + (du[:, 2] + dw[:, 0]) * S[:, 2]) * Visc,
               ((dv[:, 0] + du[:, 1]) * S[:, 0] + (dv[:, 1] + dv[:, 1]) * S[:, 1] + (dv[:, 2] + dw[:, 1]) * S[:, 2]) * Visc,
               ((dw[:, 0] + du[:, 2]) * S[:, 0] + (dw[:, 1] + dv[:, 2]) * S[:, 1] + (dw[:, 2] + dw[:, 2]) * S[:, 2]) * Visc]
        dxc = g.cx[c2] - g.cx[c1]
        fdi = [D * _dot3(Gk, dxc) for Gk in G]
        E = np.zeros((d.nf, 3))
        E[inn] = np.stack([fde[k] - fdi[k] - fcs[k] for k in range(3)], 1)
        Df = np.zeros(d.nf); Df[inn] = D
        # cell gather
        app = np.zeros(d.nc)
        src = np.zeros((d.nc, 3))
        f = d.slot_face
        first = m.c1[f] == d.slot_row
        RUn = np.where(first, self.RUFace[f], -self.RUFace[f])
        if self.hybrid:  # hybrid (Spalding): a_nb = max(-F, D - F/2, 0)
            anb = np.maximum(np.maximum(-RUn, Df[f] - 0.5 * RUn), 0.)
            offd = -anb
            np.add.at(app, d.slot_row, anb)
        else:
            conv = np.minimum(RUn, 0.)
            offd = conv - Df[f]
            np.add.at(app, d.slot_row, -conv + Df[f])
        np.add.at(src, d.slot_row, np.where(first[:, None], E[f], -E[f]))
        # boundary faces (:126-223)
        bf = m.bface
        ic = d.bc1
        t = d.t1
        Vb = mu[ic]
        VAL = Vb * g.rl[bf]
        bapp = VAL.copy()
        Sb = g.fn[bf]
        dxb = g.fx[bf] - g.cx[ic]
        bsrc = np.zeros((d.nb, 3))
        gu, gv, gw = self.dU[ic], self.dV[ic], self.dW[ic]
        fde_b = [((gu[:, 0] + gu[:, 0]) * Sb[:, 0] + (gu[:, 1] + gv[:, 0]) * Sb[:, 1] + (gu[:, 2] + gw[:, 0]) * Sb[:, 2]) * Vb,
                 ((gv[:, 0] + gu[:, 1]) * Sb[:, 0] + (gv[:, 1] + gv[:, 1]) * Sb[:, 1] + (gv[:, 2] + gw[:, 1]) * Sb[:, 2]) * Vb,
                 ((gw[:, 0] + gu[:, 2]) * Sb[:, 0] + (gw[:, 1] + gv[:, 2]) * Sb[:, 1] + (gw[:, 2] + gw[:, 2]) * Sb[:, 2]) * Vb]
        Bs = (self.BU, self.BV, self.BW)
        for k, gk in enumerate((gu, gv, gw)):
            fdi_b = VAL * (_dot3(gk, dxb) - Bs[k])
            bsrc[:, k] = np.where(t == 1, 0., fde_b[k] - fdi_b)
        RUb = self.RUFace[bf]
        fl = np.where((t == 2) | (t == 3), np.minimum(RUb, 0.), 0.)
        bapp = bapp - fl
        for k in range(3):
            bsrc[:, k] -= fl * Bs[k]
        np.add.at(app, ic, bapp)
        np.add.at(src, ic, bsrc)
        urf = p.urf[0]
        app = app / urf
        self.Apr = 1. / app
        A = self._assemble(d, app, None, offd)
        vol = g.vol
        b = [src[:, k] + (1. - urf) * app * ph + (-self.dP[:, k] + self.R * p.gravity[k]) * vol
             for k, ph in enumerate(phis)]
        self.mom_b = b
        self.mom_A = A
        for k, name in enumerate("UVW"):
            old = getattr(self, name)
            x, it, res = bicgstab(A, b[k], old.copy(), 500, self.eps["mom"], 1.2)
            self.Residual[k] = (np.abs(old - x) * vol).sum()
            setattr(self, name, x)

    # CalRUFace2, navier_velocity.cpp:389-442 + coefficient of navier_pressure.cpp:150-153
    def rhie_chow(self):
        d, g, m = self.d, self.d.g, self.d.m
        RU = np.zeros(d.nf)
        bf = m.bface
        RU[bf] = (self.BU * self.BRo) * g.fn[bf, 0] + (self.BV * self.BRo) * g.fn[bf, 1] + (self.BW * self.BRo) * g.fn[bf, 2]
        inn = d.inner
        c1, c2 = m.c1[inn], m.c2[inn]
        lam = g.lam[inn]
        lam2 = 1. - lam
        R1, R2 = self.R[c1], self.R[c2]
        rf = lam * R1 + lam2 * R2
        ruf = lam * R1 * self.U[c1] + lam2 * R2 * self.U[c2]
        rvf = lam * R1 * self.V[c1] + lam2 * R2 * self.V[c2]
        rwf = lam * R1 * self.W[c1] + lam2 * R2 * self.W[c2]
        S = g.fn[inn]
        ru = ruf * S[:, 0] + rvf * S[:, 1] + rwf * S[:, 2]
        P1 = self.P[c1] + _dot3(self.dP[c1], g.xpac[inn] - g.cx[c1])
        P2 = self.P[c2] + _dot3(self.dP[c2], g.xnac[inn] - g.cx[c2])
        dx = g.xnac[inn] - g.xpac[inn]
        d12 = np.sqrt(_dot3(dx, dx))
        aprf = lam * self.Apr[c1] + lam2 * self.Apr[c2]
        volf = lam * g.vol[c1] + lam2 * g.vol[c2]
        dpg = lam[:, None] * self.dP[c1] + lam2[:, None] * self.dP[c2]
        dpn = _dot3(dpg, dx)
        ru = ru - rf * g.area[inn] * aprf / d12 * volf * ((P2 - P1) - dpn)
        RU[inn] = ru
        self.RUFace = RU
        coef = np.zeros(d.nf)
        coef[inn] = (R1 * self.Apr[c1] * lam + R2 * self.Apr[c2] * lam2) * (g.vol[c1] * lam + g.vol[c2] * lam2) * g.rl[inn]
        self.fcoef = coef

    # CalculatePressure + BuildPressureMatrix + CorrectRUFace2, navier_pressure.cpp:9-261
    def calculate_pressure(self):
        d, p, g, m = self.d, self.p, self.d.g, self.d.m
        self.bc_velocity()
        self.rhie_chow()
        bp = np.zeros(d.nc)
        np.add.at(bp, m.c1, self.RUFace)
        inn = d.inner
        np.add.at(bp, m.c2[inn], -self.RUFace[inn])
        f = d.slot_face
        offd = self.fcoef[f]
        app = np.zeros(d.nc)
        np.add.at(app, d.slot_row, -offd)
        A = self._assemble(d, app, None, offd)
        self.p_A, self.p_b = A, bp
        dp, it, res = cg(A, bp, np.zeros(d.nc), 1000, self.eps["p"], 1.3)
        self.p_iters = it
        self.dp = dp
        self.BPre = dp[d.bc1]
        self.dP = d.gradient(dp, self.BPre, p.limiter)
        ref = dp[p.cell_pref]
        self.Residual[3] = (np.abs(dp - ref) * g.vol).sum()
        self.P = self.P + p.urf[3] * (dp - ref)
        coef = g.vol * self.Apr
        self.U = self.U - coef * self.dP[:, 0]
        self.V = self.V - coef * self.dP[:, 1]
        self.W = self.W - coef * self.dP[:, 2]
        self.bc_velocity()
        bf = m.bface
        self.RUFace[bf] = (self.BU * self.BRo) * g.fn[bf, 0] + (self.BV * self.BRo) * g.fn[bf, 1] + (self.BW * self.BRo) * g.fn[bf, 2]
        c1, c2 = m.c1[inn], m.c2[inn]
        dp1 = dp[c1] + p.urf[3] * _dot3(self.dP[c1], g.xpac[inn] - g.cx[c1])
        dp2 = dp[c2] + p.urf[3] * _dot3(self.dP[c2], g.xnac[inn] - g.cx[c2])
        self.RUFace[inn] = self.RUFace[inn] + (-self.fcoef[inn] * (dp2 - dp1))

    # BuildScalarMatrix, navier_scalar.cpp:466-647 / HeatConductionSolver.cpp:175-288
    def scalar_matrix(self, d, phi, bphi, diff, src, app0, grad, RUFace, bq, urf, mode):
        g, m = d.g, d.m
        inn = d.inner
        c1, c2 = m.c1[inn], m.c2[inn]
        lam = g.lam[inn]
        Visc = lam * diff[c1] + (1. - lam) * diff[c2]
        gf = lam[:, None] * grad[c1] + (1. - lam)[:, None] * grad[c2]
        D = Visc * g.rl[inn]
        fcs = np.zeros(len(inn))
        if mode != "solid" and not self.hybrid:
            RU = RUFace[inn]
            up = np.where(RU > 0., c1, c2)
            fcs = RU * ((phi[up] + _dot3(grad[up], g.fx[inn] - g.cx[up])) - phi[up])
        fde = Visc * _dot3(gf, g.fn[inn])
        fdi = D * _dot3(gf, g.cx[c2] - g.cx[c1])
        E = np.zeros(d.nf); E[inn] = fde - fdi - fcs
        Df = np.zeros(d.nf); Df[inn] = D
        f = d.slot_face
        first = m.c1[f] == d.slot_row
        app = app0.copy()
        sphi = src.copy()
        if mode != "solid" and self.hybrid:  # hybrid (option of the GPU implementation)
            RUn = np.where(first, RUFace[f], -RUFace[f])
            anb = np.maximum(np.maximum(-RUn, Df[f] - 0.5 * RUn), 0.)
            offd = -anb
            np.add.at(app, d.slot_row, anb)
        else:
            if mode != "solid":
                RUn = np.where(first, RUFace[f], -RUFace[f])
                conv = np.minimum(RUn, 0.)
            else:
                conv = np.zeros(len(f))
            offd = conv - Df[f]
            np.add.at(app, d.slot_row, -conv + Df[f])
        np.add.at(sphi, d.slot_row, np.where(first, E[f], -E[f]))
        bf = m.bface
        ic = d.bc1
        t1, t2 = d.t1, d.t2
        Vb = diff[ic]
        gb = grad[ic]
        dirich = np.zeros(d.nb, bool)
        fde_b = np.zeros(d.nb)
        if mode == "solid":
            dirich = (t1 == 1) & (t2 == 0)
            flux = ((t1 == 1) | (t1 == 4)) & ~dirich
            fde_b[flux] = 0. - bq[flux] * g.area[bf][flux]
        elif mode == "energy":
            flux = (t1 == 1) & (t2 == 1)
            fde_b[flux] = 0. - bq[flux] * g.area[bf][flux]
            dirich = ~flux & (t1 != 4)
        else:
            dirich = (t1 >= 1) & (t1 <= 4)
        VAL = Vb * g.rl[bf]
        bapp = np.where(dirich, VAL, 0.)
        fde_b = np.where(dirich, Vb * _dot3(gb, g.fn[bf]), fde_b)
        fdi_b = np.where(dirich, VAL * (_dot3(gb, g.fx[bf] - g.cx[ic]) - bphi), 0.)
        fcs_b = np.zeros(d.nb)
        if mode != "solid":
            io = (t1 == 2) | (t1 == 3)
            if np.any((t1 == 2) & (RUFace[bf] > 0)):
                raise RuntimeError("reverse flow get out of inlet. stop!")
            fl = np.where(io, np.minimum(RUFace[bf], 0.), 0.)
            bapp = bapp - fl
            fcs_b = fl * bphi
        np.add.at(app, ic, bapp)
        np.add.at(sphi, ic, fde_b - fdi_b - fcs_b)
        app = app / urf
        A = self._assemble(d, app, None, offd)
        b = sphi + (1. - urf) * app * phi
        return A, b

    # UpdateTurKEpsilon, navier_scalar.cpp:14-172 + SetBCKEpsilon navier_bc.cpp:209-296
    def update_ke(self):
        d, p, g, m = self.d, self.p, self.d.g, self.d.m
        kap, Cmu, C1, C2, sk, se = 0.419, 0.09, 1.44, 1.92, 1.0, 1.3
        vol = g.vol
        VisTE = self.VisLam + self.VisTur / sk
        VisED = self.VisLam + self.VisTur / se
        du, dv, dw = self.dU, self.dV, self.dW
        s1 = ((du[:, 0] + du[:, 0]) * du[:, 0] + (du[:, 1] + dv[:, 0]) * du[:, 1]) + (du[:, 2] + dw[:, 0]) * du[:, 2]
        s2 = ((dv[:, 0] + du[:, 1]) * dv[:, 0] + (dv[:, 1] + dv[:, 1]) * dv[:, 1]) + (dv[:, 2] + dw[:, 1]) * dv[:, 2]
        s3 = ((dw[:, 0] + du[:, 2]) * dw[:, 0] + (dw[:, 1] + dv[:, 2]) * dw[:, 1]) + (dw[:, 2] + dw[:, 2]) * dw[:, 2]
        Prod = self.VisTur * ((s1 + s2) + s3)
        TES = Prod * vol
        ApTE = self.R * self.ED / self.TE * vol
        ApED = np.zeros(d.nc)
        ED = self.ED
        for b in d.walls:
            ic = d.bc1[b]
            f = m.bface[b]
            self.BTE[b] = self.TE[ic]
            self.BED[b] = ED[ic]
            sav = g.fn[f] / (g.area[f] + 1.e-16)
            vn = (self.U[ic] * sav[0] + self.V[ic] * sav[1]) + self.W[ic] * sav[2]
            vt = np.array([self.U[ic], self.V[ic], self.W[ic]]) - vn * sav
            vel = math.sqrt((vt[0] * vt[0] + vt[1] * vt[1]) + vt[2] * vt[2])
            dist = g.bdist[b]
            c25 = Cmu ** 0.25
            utau = c25 * math.sqrt(self.TE[ic])
            yplus = dist * utau * self.R[ic] / (self.VisLam[ic] + SMALL)
            tauw = self.VisLam[ic] * vel / dist
            utau = math.sqrt(tauw / self.R[ic]) if yplus < 11. else c25 * math.sqrt(self.TE[ic])
            Prod[ic] = tauw * utau / (kap * dist)
            eps = Cmu ** 0.75 * self.TE[ic] ** 1.5 / (kap * dist)
            TES[ic] = Prod[ic] * vol[ic]
            ApTE[ic] -= self.R[ic] * ED[ic] / self.TE[ic] * vol[ic]
            ApTE[ic] += self.R[ic] * eps / self.TE[ic] * vol[ic]
            ED[ic] = eps
            self.BED[b] = eps
        for b in range(d.nb):
            rid, ic = int(d.m.brid[b]), d.bc1[b]
            if rid == 2:
                self.BTE[b], self.BED[b] = d.binit[b, 6], d.binit[b, 7]
            elif rid in (3, 4):
                self.BTE[b], self.BED[b] = self.TE[ic], ED[ic]
        grad = d.gradient(self.TE, self.BTE, p.limiter)
        A, b = self.scalar_matrix(d, self.TE, self.BTE, VisTE, TES, ApTE, grad, self.RUFace, None, p.urf[5], "plain")
        x, _, _ = bicgstab(A, b, self.TE.copy(), 500, self.eps["ke"], 1.3)
        self.TE = np.where(1.e-9 > x, 1.e-9, x)
        fact = ED / (self.TE + SMALL) * vol
        EDS = C1 * fact * Prod
        ApED = ApED + C2 * fact * self.R
        grad = d.gradient(ED, self.BED, p.limiter)
        A, b = self.scalar_matrix(d, ED, self.BED, VisED, EDS, ApED, grad, self.RUFace, None, p.urf[5], "plain")
        rp, cl, val, dg = A
        val = val.copy(); dg = dg.copy()
        for bb in d.walls:
            ic = d.bc1[bb]
            val[rp[ic]:rp[ic + 1]] = 0.
            val[rp[ic]] = 1.
            dg[ic] = 1.
            b[ic] = ED[ic]
        x, _, _ = bicgstab((rp, cl, val, dg), b, ED.copy(), 500, self.eps["ke"], 1.3)
        self.ED = np.where(1.e-12 > x, 1.e-12, x)
        self.VisTur = np.where(self.ED > 1.e-12, Cmu * self.R * self.TE * self.TE / (self.ED + SMALL), 0.)

    def _solid_bc(self):
        s = self.solid
        ic = s.bc1
        f = s.m.bface
        t1, t2 = s.t1, s.t2
        m = (t1 == 1) & (t2 == 1)
        self.sBTem[m] = self.sT[ic][m] - self.sBq[m] / (self.sK[ic][m] * s.g.rl[f][m])
        m = ((t1 == 1) & (t2 == 2)) | (t1 == 4)
        self.sBTem[m] = self.sT[ic][m]

    # UpdateEnergy (fluid) navier_scalar.cpp:257-397 and the solid solve HeatConductionSolver.cpp:47-106
    def update_energy(self):
        d, p, g = self.d, self.p, self.d.g
        kc = p.cp * (self.VisLam / p.prl + self.VisTur / p.prte) / p.cp
        kc = kc * 100
        ic = d.bc1
        m = ((d.t1 == 1) & (d.t2 == 1)) | (d.t1 == 3) | (d.t1 == 4)
        self.BTem[m] = self.T[ic][m]
        if self.solid is not None:
            s = self.solid
            k = np.arange(s.nb - s.ncb)
            sb = s.ncb + k
            scell = s.bc1[sb]
            dtdr = _dot3(self.sdPhi[scell], s.g.fx[s.m.bface[sb]] - s.g.cx[scell])
            self.BTem[d.ncb + k] = self.sT[scell] + dtdr
        grad = d.gradient(self.T, self.BTem, p.limiter)
        z = np.zeros(d.nc)
        A, b = self.scalar_matrix(d, self.T, self.BTem, kc, z, z, grad, self.RUFace, self.Bq, p.urf[5], "energy")
        x, _, _ = bicgstab(A, b, self.T.copy(), 500, self.eps["t"], 1.3)
        self.T = x
        if self.solid is not None:
            s = self.solid
            k = np.arange(d.nb - d.ncb)
            fb = d.ncb + k
            fc = d.bc1[fb]
            ff = d.m.bface[fb]
            dtdn = _dot3(grad[fc], g.fn[ff]) / g.area[ff]
            q = 0. - dtdn * kc[fc]
            self.Bq[fb] = q
            self.sBq[s.ncb + k] = 0. - q

    def solid_solve(self, source: float = 0.0):
        s, p = self.solid, self.p
        self._solid_bc()
        self.sdPhi = s.gradient(self.sT, self.sBTem, p.limiter)
        z = np.zeros(s.nc)
        A, b = self.scalar_matrix(s, self.sT, self.sBTem, self.sK, source * s.g.vol, z, self.sdPhi, None, self.sBq,
                                  1.0, "solid")
        x, _, _ = cg(A, b, self.sT.copy(), 500, self.eps["ts"], 1.3)
        self.sT = x

    def outer_iteration(self):
        """navier.cpp:36-53"""
        self.calculate_velocity()
        self.calculate_pressure()
        if self.p.tur_model == 1:
            self.update_ke()
        if self.p.solve_energy:
            self.update_energy()
            if self.solid is not None:
                self.solid_solve()

    def iterate(self, n: int) -> int:
        for k in range(n):
            self.outer_iteration()
            if self.p.steady and max(0.0, self.Residual.max()) < self.p.residual_steady:
                return k + 1
        return n
