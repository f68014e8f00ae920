"""Synthetic inputs in the reference's own formats: Gmsh MSH 2.2 ASCII meshes and
CRLF ``param.in`` files.

The reference ships no mesh (its ``param.in:2`` names an absent ``untitled.msh``),
so every case is generated here.  The MSH layout follows what the reference reader
accepts (``Preprocessor.cpp:13-146``):

* ``$MeshFormat``/``$EndMeshFormat``/``$Nodes`` come first, because the reader skips
  exactly six tokens before the node count (``Preprocessor.cpp:26-31``); there is no
  ``$PhysicalNames`` block;
* elements are of type 2/3 (boundary triangle/quad) and 4/5 (tet/hex), each with two
  tags, the first being the physical id that becomes ``rid``
  (``Preprocessor.cpp:67-71,97``);
* coordinates are written with 17 significant digits so that both readers see the
  same binary doubles.

Boundary ids follow the reference's k-epsilon quirk (``navier_bc.cpp:261,274,286``
compare the *rid* with 2/3/4): inlet 2, outlet 3, symmetry 4, walls 1 or >= 7.

``param.in`` files are written with CRLF line ends and no blank lines, because the
reference parser only skips lines of length 1 (``readparamfile.cpp:27-28``).
"""
from __future__ import annotations

import dataclasses
import os
from typing import Dict, List, Optional, Sequence

import numpy as np

# Physical ids used by the generated cases.
WALL_ID = 1
INLET_ID = 2
OUTLET_ID = 3
SYM_ID = 4
FLUID_ID = 5
SOLID_ID = 6
TWALL_ID = 7

DEFAULT_SEED = 20261203


@dataclasses.dataclass
class Mesh:
    """Vertices plus element blocks, 0-based node indices."""

    nodes: np.ndarray                      # (Nv, 3) float64
    hexes: np.ndarray                      # (Nh, 8) int64
    hex_ids: np.ndarray                    # (Nh,) physical id
    tets: np.ndarray                       # (Nt, 4)
    tet_ids: np.ndarray
    quads: np.ndarray                      # (Nq, 4) boundary quads
    quad_ids: np.ndarray
    tris: np.ndarray                       # (Nr, 3) boundary triangles
    tri_ids: np.ndarray

    @property
    def n_cells(self) -> int:
        return int(len(self.hexes) + len(self.tets))

    @property
    def n_bnd(self) -> int:
        return int(len(self.quads) + len(self.tris))


def _empty(n: int) -> np.ndarray:
    return np.zeros((0, n), dtype=np.int64)


def splitmix64_uniform(seed: int, counter: np.ndarray) -> np.ndarray:
    """Uniform [0,1) doubles from the splitmix64 mix of ``seed + (counter+1)*golden``.

    A counter-based generator: the value for a given (seed, counter) does not depend
    on how many values are drawn, so meshes are identical on every machine.
    """
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) + (counter.astype(np.uint64) + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _grid_nodes(xs: np.ndarray, ys: np.ndarray, zs: np.ndarray) -> np.ndarray:
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    # node index = i + (nx+1)*(j + (ny+1)*k): x fastest
    return np.stack([X.transpose(2, 1, 0).ravel(), Y.transpose(2, 1, 0).ravel(),
                     Z.transpose(2, 1, 0).ravel()], axis=1)


def _hex_corners(nx: int, ny: int, nz: int) -> np.ndarray:
    """(nx*ny*nz, 8) corner node ids in Gmsh hexahedron order, cells x-fastest."""
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i = i.transpose(2, 1, 0).ravel()
    j = j.transpose(2, 1, 0).ravel()
    k = k.transpose(2, 1, 0).ravel()
    sx, sy = nx + 1, (nx + 1) * (ny + 1)

    def nid(a, b, c):
        return (i + a) + sx * (j + b) + sy * (k + c)

    return np.stack([nid(0, 0, 0), nid(1, 0, 0), nid(1, 1, 0), nid(0, 1, 0),
                     nid(0, 0, 1), nid(1, 0, 1), nid(1, 1, 1), nid(0, 1, 1)], axis=1)


def _side_quads(nx: int, ny: int, nz: int, side: str) -> np.ndarray:
    """Boundary quads of one side of the node block, as (m, p, M, q) corner tuples.

    m is the corner with the smallest index, M the opposite one; the Kuhn split
    used for tets cuts every quad along m-M, which keeps the mesh conforming.
    """
    sx, sy = nx + 1, (nx + 1) * (ny + 1)
    if side in ("x0", "x1"):
        i0 = 0 if side == "x0" else nx
        j, k = np.meshgrid(np.arange(ny), np.arange(nz), indexing="ij")
        j, k = j.T.ravel(), k.T.ravel()
        base = i0 + sx * j + sy * k
        return np.stack([base, base + sx, base + sx + sy, base + sy], axis=1)
    if side in ("y0", "y1"):
        j0 = 0 if side == "y0" else ny
        i, k = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
        i, k = i.T.ravel(), k.T.ravel()
        base = i + sx * j0 + sy * k
        return np.stack([base, base + 1, base + 1 + sy, base + sy], axis=1)
    if side in ("z0", "z1"):
        k0 = 0 if side == "z0" else nz
        i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        i, j = i.T.ravel(), j.T.ravel()
        base = i + sx * j + sy * k0
        return np.stack([base, base + 1, base + 1 + sx, base + sx], axis=1)
    raise ValueError(side)


def box_hex(nx: int, ny: int, nz: int, lengths=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0),
            side_ids: Optional[Dict[str, int]] = None, volume_id: int = FLUID_ID) -> Mesh:
    """Uniform hexahedral box.  ``side_ids`` maps x0/x1/y0/y1/z0/z1 to physical ids."""
    side_ids = side_ids or {}
    xs = origin[0] + lengths[0] * np.arange(nx + 1) / nx
    ys = origin[1] + lengths[1] * np.arange(ny + 1) / ny
    zs = origin[2] + lengths[2] * np.arange(nz + 1) / nz
    nodes = _grid_nodes(xs, ys, zs)
    hexes = _hex_corners(nx, ny, nz)
    quads, qids = [], []
    for side in ("x0", "x1", "y0", "y1", "z0", "z1"):
        q = _side_quads(nx, ny, nz, side)
        quads.append(q)
        qids.append(np.full(len(q), side_ids.get(side, WALL_ID), dtype=np.int64))
    return Mesh(nodes, hexes, np.full(len(hexes), volume_id, dtype=np.int64), _empty(4),
                np.zeros(0, np.int64), np.concatenate(quads), np.concatenate(qids), _empty(3),
                np.zeros(0, np.int64))


def lid_cavity_hex(n: int, lid_id: int = INLET_ID, wall_id: int = WALL_ID) -> Mesh:
    """Unit cube of n^3 hexes; the lid (y = 1) carries ``lid_id``, the rest ``wall_id``."""
    ids = {s: wall_id for s in ("x0", "x1", "y0", "z0", "z1")}
    ids["y1"] = lid_id
    return box_hex(n, n, n, side_ids=ids)


# Kuhn split of the unit hexahedron into 6 tets along the diagonal c000 -> c111.
# Corner c(a,b,c) has Gmsh hex index: (0,0,0)0 (1,0,0)1 (1,1,0)2 (0,1,0)3 (0,0,1)4 ...
_C = {(0, 0, 0): 0, (1, 0, 0): 1, (1, 1, 0): 2, (0, 1, 0): 3, (0, 0, 1): 4, (1, 0, 1): 5,
      (1, 1, 1): 6, (0, 1, 1): 7}


def _kuhn_tets() -> List[List[int]]:
    tets = []
    for perm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        p = [0, 0, 0]
        path = [_C[tuple(p)]]
        for ax in perm:
            p[ax] = 1
            path.append(_C[tuple(p)])
        tets.append(path)
    return tets


def box_tet6(nx: int, ny: int, nz: int, jitter: float = 0.0, seed: int = DEFAULT_SEED,
             side_ids: Optional[Dict[str, int]] = None, volume_id: int = FLUID_ID) -> Mesh:
    """Unit box of nx*ny*nz hexes, each cut into 6 tets (Kuhn split).

    Interior nodes move by U(-jitter, +jitter) * h per axis (h = that axis's spacing),
    drawn from the counter-based splitmix64 stream of ``seed``.
    """
    side_ids = side_ids or {}
    base = box_hex(nx, ny, nz, side_ids=side_ids, volume_id=volume_id)
    nodes = base.nodes.copy()
    if jitter > 0.0:
        nid = np.arange(len(nodes))
        i = nid % (nx + 1)
        j = (nid // (nx + 1)) % (ny + 1)
        k = nid // ((nx + 1) * (ny + 1))
        interior = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
        h = np.array([1.0 / nx, 1.0 / ny, 1.0 / nz])
        for ax in range(3):
            u = splitmix64_uniform(seed, nid * 3 + ax)
            d = (2.0 * u - 1.0) * jitter * h[ax]
            nodes[:, ax] = np.where(interior, nodes[:, ax] + d, nodes[:, ax])
    pattern = np.array(_kuhn_tets(), dtype=np.int64)            # (6, 4) local corners
    tets = base.hexes[:, pattern].reshape(-1, 4)                 # cell order: hex-major
    q = base.quads                                               # (m, p, M, q)
    tris = np.concatenate([np.stack([q[:, 0], q[:, 1], q[:, 2]], 1)[:, None, :],
                           np.stack([q[:, 0], q[:, 3], q[:, 2]], 1)[:, None, :]], axis=1).reshape(-1, 3)
    tri_ids = np.repeat(base.quad_ids, 2)
    return Mesh(nodes, _empty(8), np.zeros(0, np.int64), tets,
                np.full(len(tets), volume_id, dtype=np.int64), _empty(4), np.zeros(0, np.int64),
                tris, tri_ids)


def lid_cavity_tet(nx: int, ny: int, nz: int, jitter: float = 0.2, seed: int = DEFAULT_SEED) -> Mesh:
    ids = {s: WALL_ID for s in ("x0", "x1", "y0", "z0", "z1")}
    ids["y1"] = INLET_ID
    return box_tet6(nx, ny, nz, jitter=jitter, seed=seed, side_ids=ids)


def cht_channel(nx: int, ny_fluid: int, ny_solid: int, nz: int, lx: float = 2.0, ly_fluid: float = 0.5,
                ly_solid: float = 0.1, lz: float = 0.5) -> Mesh:
    """Fluid channel bonded to a solid slab below it (conjugate heat transfer).

    One node block spans y in [-ly_solid, ly_fluid]; cells in the ``ny_solid`` lowest
    layers are solid (id 6), the rest fluid (id 5).  Cells are numbered x fastest,
    then y, then z, so the fluid and solid interface faces come out in the same order
    in both sub-meshes -- the reference pairs them by enumeration order
    (``HeatConductionSolver.cpp:377-393,404-425``).

    Boundaries: fluid inlet x=0 id 2, outlet x=lx id 3, fluid top wall id 1,
    fluid z-sides symmetry id 4; solid bottom fixed-temperature wall id 7, solid
    x- and z-sides adiabatic wall id 1.
    """
    ny = ny_fluid + ny_solid
    xs = lx * np.arange(nx + 1) / nx
    ys = np.concatenate([-ly_solid + ly_solid * np.arange(ny_solid) / ny_solid,
                         ly_fluid * np.arange(ny_fluid + 1) / ny_fluid])
    zs = lz * np.arange(nz + 1) / nz
    nodes = _grid_nodes(xs, ys, zs)
    hexes = _hex_corners(nx, ny, nz)
    jcell = (np.arange(len(hexes)) // nx) % ny
    hex_ids = np.where(jcell < ny_solid, SOLID_ID, FLUID_ID).astype(np.int64)
    quads, qids = [], []

    def add(side, ids_of_j):
        q = _side_quads(nx, ny, nz, side)
        quads.append(q)
        qids.append(ids_of_j(q))

    sx = nx + 1
    sy = (nx + 1) * (ny + 1)

    def node_j(q):
        return (q[:, 0] % sy) // sx

    # x sides: layer index of the quad = min node j
    add("x0", lambda q: np.where(node_j(q) < ny_solid, WALL_ID, INLET_ID))
    add("x1", lambda q: np.where(node_j(q) < ny_solid, WALL_ID, OUTLET_ID))
    add("y0", lambda q: np.full(len(q), TWALL_ID))
    add("y1", lambda q: np.full(len(q), WALL_ID))
    add("z0", lambda q: np.where(node_j(q) < ny_solid, WALL_ID, SYM_ID))
    add("z1", lambda q: np.where(node_j(q) < ny_solid, WALL_ID, SYM_ID))
    return Mesh(nodes, hexes, hex_ids, _empty(4), np.zeros(0, np.int64), np.concatenate(quads),
                np.concatenate(qids).astype(np.int64), _empty(3), np.zeros(0, np.int64))


def _format_block(fmt_row: str, arr: np.ndarray) -> str:
    n = arr.shape[0]
    if n == 0:
        return ""
    return (fmt_row * n) % tuple(arr.ravel().tolist())


def write_msh(path: str, mesh: Mesh) -> None:
    """Write Gmsh MSH 2.2 ASCII (boundary elements first, then volume elements)."""
    nv = len(mesh.nodes)
    parts: List[str] = ["$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % nv]
    idx = np.arange(1, nv + 1, dtype=np.float64)[:, None]
    parts.append(_format_block("%d %.17g %.17g %.17g\n", np.concatenate([idx, mesh.nodes], axis=1)))
    parts.append("$EndNodes\n$Elements\n")
    blocks = []
    eid = 1
    for etype, conn, ids in ((2, mesh.tris, mesh.tri_ids), (3, mesh.quads, mesh.quad_ids),
                             (4, mesh.tets, mesh.tet_ids), (5, mesh.hexes, mesh.hex_ids)):
        if len(conn) == 0:
            continue
        m = len(conn)
        cols = [np.arange(eid, eid + m), np.full(m, etype), np.full(m, 2), ids, ids]
        arr = np.concatenate([np.stack(cols, axis=1), conn + 1], axis=1).astype(np.int64)
        blocks.append(_format_block(" ".join(["%d"] * arr.shape[1]) + "\n", arr))
        eid += m
    parts.append("%d\n" % (eid - 1))
    parts.extend(blocks)
    parts.append("$EndElements\n")
    with open(path, "w") as f:
        f.write("".join(parts))


# ----------------------------------------------------------------------------------
# param.in writer (grammar of readparamfile.cpp:59-251)

def _fmt(x) -> str:
    if isinstance(x, (int, np.integer)):
        return str(int(x))
    return repr(float(x))


def write_param(path: str, lines: Sequence[Sequence]) -> None:
    """Write a CRLF ``param.in`` from keyword rows, e.g. ``[("steady", 301, 1e-300), ...]``."""
    out = []
    for row in lines:
        out.append(", ".join([str(row[0])] + [_fmt(v) if not isinstance(v, str) else v for v in row[1:]]))
    with open(path, "wb") as f:
        f.write(("\r\n".join(out) + "\r\n").encode())


def cavity_param(gridfile: str, iters: int, mu: float, rho: float = 1.0, urf=(0.7, 0.3, 0.8),
                 limiter: str = "no", lid_u: float = 1.0, res: float = 1e-300) -> List[tuple]:
    """Laminar lid-driven cavity: lid = inlet region with tangential velocity."""
    return [
        ("gridfile", gridfile),
        ("steady", iters + 1, res),           # "steady, N" runs N-1 outer iterations
        ("energy", "off"),
        ("density", 0),
        ("turbulence", "no"),
        ("PressureRef", 0.0, 1),
        ("relaxation",) + tuple(urf),
        ("limiter", limiter),
        ("bound", WALL_ID, "Hwall", 0.0),
        ("bound", INLET_ID, "inlet", lid_u, 0.0, 0.0, 0.0, rho, 0.0),
        ("volumn", FLUID_ID, "fluid", "fluid", 0.0, 0.0, 0.0, rho, 0.0, mu, 0.0, 0.0),
        ("output", 1000000),
    ]


def batch_cavities(n_cases: int = 48, lmin: int = 12, lmax: int = 64, re_min: float = 50.0,
                   re_max: float = 1000.0, seed: int = DEFAULT_SEED) -> List[tuple]:
    """(edge cells L, Reynolds number) of the many-cavity batch: L uniform on
    {lmin..lmax}, Re uniform on [re_min, re_max], from the counter-based generator
    (draw 2k for L, 2k+1 for Re of case k)."""
    u = splitmix64_uniform(seed, np.arange(2 * n_cases))
    out = []
    for k in range(n_cases):
        L = lmin + min(int(u[2 * k] * (lmax - lmin + 1)), lmax - lmin)
        out.append((L, float(re_min + u[2 * k + 1] * (re_max - re_min))))
    return out


def cht_param(gridfile: str, iters: int, u_in: float = 1.0, nu: float = 1e-5, rho: float = 1.0,
              t_in: float = 300.0, t_wall: float = 400.0, k_solid: float = 15.0, rho_solid: float = 1.0,
              turb: bool = True, urf=(0.7, 0.3, 0.8), limiter: str = "no", intensity: float = 0.05,
              mixing_length: float = 0.05, res: float = 1e-300) -> List[tuple]:
    """Conjugate-heat-transfer channel (k-epsilon optional).

    Inlet k = 1.5 (I U)^2 and eps = Cmu^0.75 k^1.5 / l.  ``turbulence, ke`` precedes the
    ``bound`` rows, because the parser only reads inlet k/eps once the model is on
    (``readparamfile.cpp:187-190``).
    """
    k_in = 1.5 * (intensity * u_in) ** 2 if turb else 0.0
    e_in = 0.09 ** 0.75 * k_in ** 1.5 / mixing_length if turb else 0.0
    rows = [
        ("gridfile", gridfile),
        ("3dheatconduction",),
        ("steady", iters + 1, res),
        ("energy", "on"),
        ("density", 0),
        ("turbulence", "ke" if turb else "no"),
        ("PressureRef", 0.0, 1),
        ("relaxation",) + tuple(urf),
        ("limiter", limiter),
        ("bound", INLET_ID, "inlet", u_in, 0.0, 0.0, 0.0, rho, t_in) + ((k_in, e_in) if turb else ()),
        ("bound", OUTLET_ID, "outlet", 0.0),
        ("bound", WALL_ID, "Hwall", 0.0),
        ("bound", SYM_ID, "sym"),
        ("bound", TWALL_ID, "Twall", t_wall),
        ("volumn", FLUID_ID, "fluid", "fluid", u_in, 0.0, 0.0, rho, t_in, nu * rho, k_in, e_in),
        ("volumn", SOLID_ID, "solid", "slab", t_in, rho_solid, k_solid),
        ("output", 1000000),
    ]
    return rows


def write_case(directory: str, mesh: Mesh, param_rows: Sequence[Sequence], msh_name: str = "mesh.msh",
               param_name: str = "param.in") -> str:
    """Write mesh + param into ``directory``; returns the param path.

    The param's gridfile is the bare mesh file name: the reference keeps it in a
    ``char[100]`` and each keyword token in a ``char[30]`` (``PreProcessor.h:15``,
    ``readparamfile.cpp:17-18``) and opens it relative to the working directory, so
    cases are run from inside ``directory``."""
    os.makedirs(directory, exist_ok=True)
    msh = os.path.join(directory, msh_name)
    write_msh(msh, mesh)
    rows = [tuple(r) for r in param_rows]
    rows = [("gridfile", msh_name) if r[0] == "gridfile" else r for r in rows]
    pp = os.path.join(directory, param_name)
    write_param(pp, rows)
    return pp
