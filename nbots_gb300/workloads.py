"""Seeded synthetic FEM problems in nbots' own input form.

A problem is a 2D mesh (node coordinates, element connectivity, edges, the
model's input vertices and input segments as node sequences), one boundary
condition list in nbots' bc-atom form, and per-element material data.  It
mirrors what nbots carries in ``struct nb_mshquad_s`` / ``struct nb_msh3trg_s``
(sources/nb/geometric_bot/mesh/mesh2D/elements2D/mshquad_struct.h:6-26,
msh3trg_struct.h:6-23) and ``bc_atom_t`` (pde_bot/boundary_conditions/
bc_atom.h:7-12), so the same arrays feed the reference, the oracle and the
CUDA path.

All randomness comes from numpy's PCG64 with a fixed seed.  nbots' own
generator (``nb_statistics_runif``, sources/nb/statistics_bot.c:36-53) is not
used: it drifts out of range for 64-bit seeds.

Node numbering of the structured Q4 grid is row-major ``j*(nx+1)+i`` and each
element lists its nodes counter-clockwise ``n0, n0+1, n0+nx+2, n0+nx+1``,
which matches the Gauss-point order of nbots' Q4 tables
(pde_bot/finite_element/element.c:75-121).
"""
from __future__ import annotations

import dataclasses
from typing import List, Optional

import numpy as np

# bc-atom kinds, in nbots' enum order (pde_bot/boundary_conditions/bcond.h:7-15)
DIRICHLET, NEUMANN = 0, 1
ON_POINT, ON_SEGMENT = 0, 1


@dataclasses.dataclass
class BC:
    """One nbots bc atom: ``nb_bcond_push(bcond, kind, where, id, mask, val)``.

    ``node_vals`` (optional) holds a function-valued condition already
    evaluated at the nodes it touches: for a segment, one (2,) row per node of
    the segment in order; for a vertex, one row.  nbots evaluates the callback
    at exactly those node coordinates (set_bconditions.c:63-131, 192-216).
    """
    kind: int
    where: int
    id: int
    mask: tuple
    val: tuple = (0.0, 0.0)
    node_vals: Optional[np.ndarray] = None


@dataclasses.dataclass
class Problem:
    name: str
    elem: str                      # "q4" or "t3"
    nod: np.ndarray                # (N_nod, 2) float64
    conn: np.ndarray               # (N_elem, nen) uint32
    edges: np.ndarray              # (N_edg, 2) uint32
    vtx: np.ndarray                # (N_vtx,) uint32 node id of each input vertex
    sgm: List[np.ndarray]          # node sequence of each input segment
    bcs: List[BC]
    E: np.ndarray                  # (N_elem,) float64 Young's modulus per element
    nu: float = 0.3
    thickness: float = 1.0
    density: float = 0.0
    self_weight: bool = False
    gravity: tuple = (0.0, -9.81)
    enabled: Optional[np.ndarray] = None   # (N_elem,) bool, None = all
    meta: dict = dataclasses.field(default_factory=dict)

    @property
    def n_nodes(self) -> int:
        return int(self.nod.shape[0])

    @property
    def n_elems(self) -> int:
        return int(self.conn.shape[0])

    @property
    def n_dof(self) -> int:
        return 2 * self.n_nodes


def q4_grid(nx: int, ny: int, lx: float = 2.0, ly: float = 1.0,
            jitter: float = 0.0, seed: int = 0):
    """Structured nx*ny Q4 grid on [0,lx]x[0,ly].

    Interior nodes move by U(-jitter*h, jitter*h) per coordinate (h = lx/nx);
    boundary nodes stay on the boundary so the model segments stay straight.
    Returns (nod, conn, edges).
    """
    hx = lx / nx
    hy = ly / ny
    i = np.arange(nx + 1, dtype=np.float64)
    j = np.arange(ny + 1, dtype=np.float64)
    X, Y = np.meshgrid(i * hx, j * hy)               # (ny+1, nx+1)
    nod = np.stack([X.ravel(), Y.ravel()], axis=1).astype(np.float64)
    if jitter > 0.0:
        rng = np.random.Generator(np.random.PCG64(seed))
        d = rng.uniform(-jitter * hx, jitter * hx, size=((ny - 1) * (nx - 1), 2))
        interior = (np.arange(1, ny)[:, None] * (nx + 1) + np.arange(1, nx)[None, :]).ravel()
        nod[interior] += d
    ii, jj = np.meshgrid(np.arange(nx), np.arange(ny))
    n0 = (jj * (nx + 1) + ii).ravel().astype(np.uint32)
    conn = np.stack([n0, n0 + 1, n0 + nx + 2, n0 + nx + 1], axis=1).astype(np.uint32)
    # unique element edges: horizontal then vertical
    hi, hj = np.meshgrid(np.arange(nx), np.arange(ny + 1))
    h0 = (hj * (nx + 1) + hi).ravel()
    vi, vj = np.meshgrid(np.arange(nx + 1), np.arange(ny))
    v0 = (vj * (nx + 1) + vi).ravel()
    edges = np.concatenate([np.stack([h0, h0 + 1], 1),
                            np.stack([v0, v0 + nx + 1], 1)]).astype(np.uint32)
    return nod, conn, edges


def cantilever_q4(nx: int, ny: int, *, jitter: float = 0.0, seed: int = 0,
                  E=1.0, nu: float = 0.3, thickness: float = 1.0,
                  point_load: float = -1.0, top_traction: float = 0.0,
                  name: str = "") -> Problem:
    """Plane-stress cantilever on [0,2]x[0,1]: left edge clamped, point load at
    the right-edge midpoint, optional uniform downward traction on the top edge.

    The model has 5 input vertices (0,0),(2,0),(2,0.5),(2,1),(0,1) and 5 input
    segments bottom, right-low, right-high, top, left.  nbots spreads a
    constant segment load as a TOTAL force over the segment by sub-segment
    length (set_bconditions.c:133-168), so a traction t on the top edge of
    length 2 is passed as the total 2*t.
    """
    assert ny % 2 == 0, "the point load sits on the node at ny/2"
    nod, conn, edges = q4_grid(nx, ny, jitter=jitter, seed=seed)
    w = nx + 1
    vtx = np.array([0, nx, (ny // 2) * w + nx, ny * w + nx, ny * w], dtype=np.uint32)
    sgm = [
        np.arange(0, nx + 1, dtype=np.uint32),                          # bottom
        (np.arange(0, ny // 2 + 1) * w + nx).astype(np.uint32),          # right low
        (np.arange(ny // 2, ny + 1) * w + nx).astype(np.uint32),         # right high
        (ny * w + np.arange(nx, -1, -1)).astype(np.uint32),              # top (2,1)->(0,1)
        (np.arange(ny, -1, -1) * w).astype(np.uint32),                   # left (0,1)->(0,0)
    ]
    bcs = [BC(DIRICHLET, ON_SEGMENT, 4, (1, 1), (0.0, 0.0)),
           BC(NEUMANN, ON_POINT, 2, (0, 1), (0.0, point_load))]
    if top_traction != 0.0:
        bcs.insert(0, BC(NEUMANN, ON_SEGMENT, 3, (0, 1), (0.0, -top_traction * 2.0)))
    ne = conn.shape[0]
    Ev = np.full(ne, float(E)) if np.isscalar(E) else np.asarray(E, np.float64)
    return Problem(name or f"q4_{nx}x{ny}", "q4", nod, conn, edges, vtx, sgm,
                   bcs, Ev, nu=nu, thickness=thickness,
                   meta=dict(nx=nx, ny=ny, jitter=jitter, seed=seed))


def lognormal_E(n: int, sigma: float, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.exp(rng.normal(0.0, sigma, size=n))


def simp_E(rho: np.ndarray, p: float = 3.0, E0: float = 1.0, Emin: float = 1e-9) -> np.ndarray:
    """SIMP interpolation E(rho) = Emin + rho^p (E0 - Emin)."""
    return Emin + np.power(rho, p) * (E0 - Emin)


# ---------------------------------------------------------------- configs
def config_c1(seed: int = 1) -> Problem:
    """64x32 Q4 cantilever (4,290 DOF), interior jitter U(-0.2h,0.2h), E=1."""
    return cantilever_q4(64, 32, jitter=0.2, seed=seed, name="c1_q4_64x32")


def config_c2(seed: int = 2, nx: int = 1024, ny: int = 512) -> Problem:
    """1024x512 Q4 cantilever (1,051,650 DOF), lognormal E (sigma 0.5),
    point load plus uniform top traction 0.01."""
    p = cantilever_q4(nx, ny, top_traction=0.01, name=f"c2_q4_{nx}x{ny}")
    p.E = lognormal_E(p.n_elems, 0.5, seed)
    p.meta.update(E="lognormal(0,0.5)", seed=seed)
    return p


def config_c4(seed: int = 4, nx: int = 512, ny: int = 256):
    """512x256 SIMP problem: rho ~ U(0.3,0.7), p=3, Emin=1e-9, E0=1."""
    p = cantilever_q4(nx, ny, name=f"c4_simp_{nx}x{ny}")
    rng = np.random.Generator(np.random.PCG64(seed))
    rho = rng.uniform(0.3, 0.7, size=p.n_elems)
    p.E = simp_E(rho)
    p.meta.update(rho=rho, penal=3.0, E0=1.0, Emin=1e-9, seed=seed)
    return p


C5_SIZES = ((64, 32), (128, 64), (256, 128), (512, 256))


def config_c5(n_inst: int = 96, seed: int = 5, sizes=C5_SIZES):
    """Batch of independent Q4 cantilevers of uneven size, each with its own
    SIMP density rho ~ U(0.2,1.0) and 1-4 random point loads on the right or
    top boundary nodes."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for k in range(n_inst):
        nx, ny = sizes[int(rng.integers(0, len(sizes)))]
        p = cantilever_q4(nx, ny, name=f"c5_{k}_{nx}x{ny}", point_load=0.0)
        p.bcs = [p.bcs[0]]  # keep the clamp
        nl = int(rng.integers(1, 5))
        w = nx + 1
        cand = np.concatenate([np.arange(0, ny + 1) * w + nx, ny * w + np.arange(1, nx)])
        picks = rng.choice(cand, size=nl, replace=False)
        # point loads on arbitrary boundary nodes: add them as extra input vertices
        base = len(p.vtx)
        p.vtx = np.concatenate([p.vtx, picks.astype(np.uint32)])
        for q in range(nl):
            fx, fy = rng.uniform(-1.0, 1.0, size=2)
            p.bcs.append(BC(NEUMANN, ON_POINT, base + q, (1, 1), (float(fx), float(fy))))
        rho = rng.uniform(0.2, 1.0, size=p.n_elems)
        p.E = simp_E(rho)
        p.meta.update(rho=rho, penal=3.0, E0=1.0, Emin=1e-9)
        out.append(p)
    return out


# L-shaped domain [0,2]^2 minus (1,2]x(1,2]: model vertices counter-clockwise
# and the six model segments between them.
L_SHAPE = np.array([[0.0, 0.0], [2.0, 0.0], [2.0, 1.0], [1.0, 1.0], [1.0, 2.0], [0.0, 2.0]])


def _zorder(xy: np.ndarray, bits: int = 16) -> np.ndarray:
    """Morton (Z-order) keys of points in [0,2]^2 on a 2^bits grid."""
    q = np.minimum((xy / 2.0 * (1 << bits)).astype(np.uint64), (1 << bits) - 1)

    def spread(v):
        v = v & np.uint64(0xFFFF)
        v = (v | (v << np.uint64(8))) & np.uint64(0x00FF00FF)
        v = (v | (v << np.uint64(4))) & np.uint64(0x0F0F0F0F)
        v = (v | (v << np.uint64(2))) & np.uint64(0x33333333)
        v = (v | (v << np.uint64(1))) & np.uint64(0x55555555)
        return v
    return spread(q[:, 0]) | (spread(q[:, 1]) << np.uint64(1))


def t3_lshape(n_points: int, seed: int = 3, E: float = 1.0, nu: float = 0.25,
              traction: float = 1.0, name: str = "") -> Problem:
    """T3 mesh of the L-shaped domain from n_points seeded uniform interior
    points: Delaunay triangulation of those points plus boundary points at
    the mean interior spacing, triangles of the notch removed, every
    boundary edge checked to be a mesh edge (boundary recovery).  Nodes are
    numbered along a Z-order curve, as a mesher that keeps neighbours close
    in memory would.  Bottom edge clamped; a +x traction of total `traction`
    on the segment x = 1, y in [1, 2] (nbots spreads a constant segment load
    as a total force, set_bconditions.c:133-168)."""
    from scipy.spatial import Delaunay
    rng = np.random.Generator(np.random.PCG64(seed))
    h = np.sqrt(3.0 / n_points)                       # mean spacing (area 3)
    pts = np.empty((0, 2))
    while pts.shape[0] < n_points:
        c = rng.uniform(0.0, 2.0, size=(int(1.4 * (n_points - pts.shape[0])) + 16, 2))
        keep = ~((c[:, 0] > 1.0) & (c[:, 1] > 1.0))
        pts = np.concatenate([pts, c[keep]])
    pts = pts[:n_points]
    # drop interior points closer than h/2 to the boundary (no slivers there)
    x, y = pts[:, 0], pts[:, 1]
    d = np.minimum.reduce([x, y, 2.0 - x, 2.0 - y,
                           np.where(y > 1.0, np.abs(x - 1.0), np.inf),
                           np.where(x > 1.0, np.abs(y - 1.0), np.inf)])
    pts = pts[d > 0.5 * h]
    # boundary points, segment by segment (each segment's nodes in order)
    seg_xy = []
    for s in range(6):
        a, b = L_SHAPE[s], L_SHAPE[(s + 1) % 6]
        m = max(1, int(np.ceil(np.linalg.norm(b - a) / h)))
        t = np.arange(m) / m                          # start vertex, no end vertex
        seg_xy.append(a[None, :] + t[:, None] * (b - a)[None, :])
    bnd = np.concatenate(seg_xy)
    nb = bnd.shape[0]
    allp = np.concatenate([bnd, pts])
    order = np.argsort(_zorder(allp), kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    nod = allp[order].astype(np.float64)
    tri = Delaunay(nod, qhull_options="Qbb Qc Qz Q12").simplices.astype(np.int64)
    cen = nod[tri].mean(axis=1)
    tri = tri[~((cen[:, 0] > 1.0) & (cen[:, 1] > 1.0))]
    # counter-clockwise
    p0, p1, p2 = nod[tri[:, 0]], nod[tri[:, 1]], nod[tri[:, 2]]
    area2 = (p1[:, 0] - p0[:, 0]) * (p2[:, 1] - p0[:, 1]) - (p1[:, 1] - p0[:, 1]) * (p2[:, 0] - p0[:, 0])
    if np.any(area2 == 0.0):
        raise ValueError("degenerate triangle")
    flip = area2 < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    # unique edges
    e = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]])
    e.sort(axis=1)
    key = e[:, 0] * nod.shape[0] + e[:, 1]
    ukey = np.unique(key)
    edges = np.stack([ukey // nod.shape[0], ukey % nod.shape[0]], axis=1)
    # model vertices and segments as node sequences; check boundary recovery
    starts = np.cumsum([0] + [s.shape[0] for s in seg_xy])
    vtx = rank[starts[:6]].astype(np.uint32)
    sgm = []
    for s in range(6):
        ids = list(range(starts[s], starts[s + 1])) + [starts[(s + 1) % 6]]
        seq = rank[np.array(ids)].astype(np.uint32)
        a, b = np.minimum(seq[:-1], seq[1:]), np.maximum(seq[:-1], seq[1:])
        if not np.all(np.isin(a.astype(np.int64) * nod.shape[0] + b, ukey)):
            raise ValueError(f"boundary segment {s} not recovered by the triangulation")
        sgm.append(seq)
    bcs = [BC(NEUMANN, ON_SEGMENT, 3, (1, 0), (traction, 0.0)),
           BC(DIRICHLET, ON_SEGMENT, 0, (1, 1), (0.0, 0.0))]
    Ev = np.full(tri.shape[0], float(E))
    return Problem(name or f"t3_lshape_{n_points}", "t3", nod, tri.astype(np.uint32),
                   edges.astype(np.uint32), vtx, sgm, bcs, Ev, nu=nu, thickness=1.0,
                   meta=dict(n_points=n_points, seed=seed, n_boundary=nb))


def config_c3(seed: int = 3, n_points: int = 2_000_000) -> Problem:
    """T3 L-shape from 2M seeded uniform points (about 4M DOF), E=1, nu=0.25,
    bottom edge clamped, unit +x traction on x=1, y in [1,2]."""
    return t3_lshape(n_points, seed=seed, name=f"c3_t3_lshape_{n_points}")
