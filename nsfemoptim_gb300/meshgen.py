"""Seeded synthetic triangle meshes written as gmsh MSH 4.1 ASCII files.

The reference reads its meshes from gmsh files (``cpp/libs/Mesh/src/gmsh.cpp:451-499``,
``cpp/libs/Mesh/src/io.cpp:65-208``) and needs the physical curve groups ``Left``, ``Right``,
``Top``, ``Bottom`` and ``Circle`` for the channel problem (``cpp/execs/NavierStokes/src/
buildContext.cpp:24-52``).  gmsh itself is not available here, so these generators build
meshes of the same geometry and size:

* ``dfg_channel``: the DFG benchmark channel [0, 2.2] x [0, 0.41] with a cylinder of radius
  0.05 centred at (0.2, 0.2) (``cpp/assets/h_0.01.geo:6-30``).  Structured blocks around an
  O-grid ring at the cylinder, quads split into triangles, interior nodes jittered from a seed.
  The cell size is scaled so the triangle count matches a gmsh mesh of characteristic length
  ``h`` (equilateral triangles of side h), e.g. ~83k triangles at h = 0.005.
* ``jittered_square``: the unit square with ``n x n`` nodes, interior nodes jittered by
  U(+-0.2 h), one diagonal per cell (the standalone pressure-Poisson workload).

Physical group order (and so group ids) follows the reference channel files:
Right=1, Top=2, Left=3, Bottom=4, Circle=5, Interior=6.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

GROUPS = ["Right", "Top", "Left", "Bottom", "Circle", "Interior"]


@dataclass
class TriMesh:
    """Corner-node triangle mesh with named border edges (mirrors ``mesh::TriangleMesh``)."""

    nodes: np.ndarray                      # (V, 2) float64
    triangles: np.ndarray                  # (T, 3) int64, counter-clockwise
    border: dict = field(default_factory=dict)   # group name -> (E, 2) int64 directed edges
    groups: list = field(default_factory=lambda: list(GROUPS))

    @property
    def num_nodes(self) -> int:
        return int(self.nodes.shape[0])

    @property
    def num_triangles(self) -> int:
        return int(self.triangles.shape[0])


def _segment(a: float, b: float, n: int) -> np.ndarray:
    return np.linspace(a, b, n + 1)


def _graded(n: int, first: float, total: float) -> np.ndarray:
    """n+1 points in [0, total] with geometric spacing whose first step is about ``first``."""
    if first * n >= total:
        return np.linspace(0.0, total, n + 1)
    lo, hi = 1.0, 2.0
    while (first * (hi ** n - 1) / (hi - 1)) < total:
        hi *= 2
    for _ in range(200):
        q = 0.5 * (lo + hi)
        s = first * (q ** n - 1) / (q - 1)
        if s < total:
            lo = q
        else:
            hi = q
    q = 0.5 * (lo + hi)
    steps = first * q ** np.arange(n)
    pts = np.concatenate([[0.0], np.cumsum(steps)])
    return pts * (total / pts[-1])


class _Builder:
    """Collects points (deduplicated on a fine lattice) and quads."""

    def __init__(self, tol: float):
        self.tol = tol
        self.key2id: dict = {}
        self.pts: list = []
        self.tris: list = []

    def pid(self, x: float, y: float) -> int:
        k = (int(round(x / self.tol)), int(round(y / self.tol)))
        i = self.key2id.get(k)
        if i is None:
            i = len(self.pts)
            self.key2id[k] = i
            self.pts.append((x, y))
        return i

    def grid(self, X: np.ndarray, Y: np.ndarray, shorter_diagonal: bool) -> None:
        """X, Y: (nu+1, nv+1) point grids; every cell becomes two triangles."""
        nu, nv = X.shape[0] - 1, X.shape[1] - 1
        ids = np.empty(X.shape, dtype=np.int64)
        for i in range(nu + 1):
            for j in range(nv + 1):
                ids[i, j] = self.pid(float(X[i, j]), float(Y[i, j]))
        for i in range(nu):
            for j in range(nv):
                a, b, c, d = ids[i, j], ids[i + 1, j], ids[i + 1, j + 1], ids[i, j + 1]
                if shorter_diagonal:
                    pa, pc = np.array(self.pts[a]), np.array(self.pts[c])
                    pb, pd = np.array(self.pts[b]), np.array(self.pts[d])
                    split_ac = np.sum((pa - pc) ** 2) <= np.sum((pb - pd) ** 2)
                else:
                    split_ac = ((i + j) % 2) == 0
                if split_ac:
                    self.tris.append((a, b, c))
                    self.tris.append((a, c, d))
                else:
                    self.tris.append((a, b, d))
                    self.tris.append((b, c, d))


def dfg_channel(h: float, seed: int = 0, jitter: float = 0.12) -> TriMesh:
    """DFG channel with cylinder: unstructured, near-equilateral triangles of side ~``h`` everywhere
    (as gmsh meshes the reference's ``.geo`` files with lc = clc = h).

    Points: a hexagonal lattice of spacing h jittered by U(+-jitter*h) from ``seed``, kept at least
    0.5 h away from the walls and the cylinder, plus points every ~h along the four walls and the
    cylinder; Delaunay triangulation (scipy) with the triangles inside the cylinder removed.  Every
    cylinder chord is checked to be a mesh edge.
    """
    from scipy.spatial import Delaunay

    L, H = 2.2, 0.41
    cx, cy, r = 0.2, 0.2, 0.05
    rng = np.random.Generator(np.random.PCG64(seed))
    dy = h * math.sqrt(3.0) / 2.0
    rows = []
    for j in range(int(H / dy) + 2):
        y = j * dy
        off = 0.5 * h if (j % 2) else 0.0
        xs = np.arange(off, L + h, h)
        rows.append(np.stack([xs, np.full_like(xs, y)], axis=1))
    lat = np.concatenate(rows)
    lat += rng.uniform(-jitter * h, jitter * h, size=lat.shape)
    d_wall = np.minimum.reduce([lat[:, 0], L - lat[:, 0], lat[:, 1], H - lat[:, 1]])
    d_cyl = np.hypot(lat[:, 0] - cx, lat[:, 1] - cy) - r
    lat = lat[(d_wall > 0.5 * h) & (d_cyl > 0.55 * h)]

    def seg(p0, p1):
        n = max(1, int(round(np.hypot(p1[0] - p0[0], p1[1] - p0[1]) / h)))
        t = np.linspace(0.0, 1.0, n + 1)[:-1]
        return np.stack([p0[0] + t * (p1[0] - p0[0]), p0[1] + t * (p1[1] - p0[1])], axis=1)

    walls = np.concatenate([seg((0, 0), (L, 0)), seg((L, 0), (L, H)), seg((L, H), (0, H)), seg((0, H), (0, 0))])
    nc = max(8, int(round(2 * math.pi * r / h)))
    ang = np.linspace(0.0, 2 * math.pi, nc + 1)[:-1]
    circ = np.stack([cx + r * np.cos(ang), cy + r * np.sin(ang)], axis=1)
    pts = np.concatenate([walls, circ, lat])
    tri = Delaunay(pts).simplices.astype(np.int64)
    cen = pts[tri].mean(axis=1)
    tri = tri[np.hypot(cen[:, 0] - cx, cen[:, 1] - cy) > r]
    # every cylinder chord must be an edge of the triangulation
    c0 = len(walls)
    ed = np.sort(np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]]), axis=1)
    edset = set(map(tuple, ed.tolist()))
    for k in range(nc):
        a, b = c0 + k, c0 + (k + 1) % nc
        if (min(a, b), max(a, b)) not in edset:
            raise RuntimeError("cylinder chord missing from the triangulation; try another seed")
    return _finish(pts, tri, _channel_border(pts, tri, L, H, cx, cy, r))


def dfg_channel_ogrid(h: float, seed: int = 0, jitter: float = 0.15) -> TriMesh:
    """Structured variant: blocks around an O-grid ring at the cylinder (finer cells at the wall)."""
    L, H = 2.2, 0.41
    cx, cy, r = 0.2, 0.2, 0.05
    # equal area: right-isoceles cells s^2/2 == equilateral sqrt(3)/4 h^2
    s = h * math.sqrt(math.sqrt(3.0) / 2.0)
    nx1 = max(2, round(0.1 / s))
    nb = max(4, round(0.2 / s))
    nx3 = max(4, round(1.9 / s))
    ny1 = max(2, round(0.1 / s))
    ny3 = max(2, round(0.11 / s))
    xs1, xs2, xs3 = _segment(0.0, 0.1, nx1), _segment(0.1, 0.3, nb), _segment(0.3, L, nx3)
    ys1, ys2, ys3 = _segment(0.0, 0.1, ny1), _segment(0.1, 0.3, nb), _segment(0.3, H, ny3)
    ys_all = np.concatenate([ys1, ys2[1:], ys3[1:]])

    b = _Builder(tol=1e-9)
    # outer structured blocks
    X, Y = np.meshgrid(xs1, ys_all, indexing="ij")
    b.grid(X, Y, False)
    X, Y = np.meshgrid(xs3, ys_all, indexing="ij")
    b.grid(X, Y, False)
    X, Y = np.meshgrid(xs2, ys1, indexing="ij")
    b.grid(X, Y, False)
    X, Y = np.meshgrid(xs2, ys3, indexing="ij")
    b.grid(X, Y, False)

    # O-grid ring between the cylinder and the square [0.1, 0.3]^2; radial grading so the
    # first radial step matches the circumferential step on the cylinder
    arc_step = (0.5 * math.pi * r) / nb
    nr = max(2, round(0.05 / s) + 3)
    t = _graded(nr, arc_step / 0.05, 1.0)  # fraction of the way from circle to square
    u = np.linspace(0.0, 1.0, nb + 1)
    # four sides: (start corner, end corner, start angle, end angle), counter-clockwise
    sides = [
        ((0.1, 0.1), (0.3, 0.1), 1.25 * math.pi, 1.75 * math.pi),
        ((0.3, 0.1), (0.3, 0.3), 1.75 * math.pi, 2.25 * math.pi),
        ((0.3, 0.3), (0.1, 0.3), 0.25 * math.pi, 0.75 * math.pi),
        ((0.1, 0.3), (0.1, 0.1), 0.75 * math.pi, 1.25 * math.pi),
    ]
    for (p0, p1, a0, a1) in sides:
        sq = np.array(p0)[None, :] * (1 - u[:, None]) + np.array(p1)[None, :] * u[:, None]
        ang = a0 + (a1 - a0) * u
        ci = np.stack([cx + r * np.cos(ang), cy + r * np.sin(ang)], axis=1)
        Xg = ci[:, 0][:, None] * (1 - t[None, :]) + sq[:, 0][:, None] * t[None, :]
        Yg = ci[:, 1][:, None] * (1 - t[None, :]) + sq[:, 1][:, None] * t[None, :]
        # orientation: u runs counter-clockwise around the cylinder, t outward -> the
        # (u, t) frame is clockwise; reverse t so cells come out counter-clockwise
        b.grid(Xg[:, ::-1], Yg[:, ::-1], True)

    pts = np.array(b.pts, dtype=np.float64)
    tris = np.array(b.tris, dtype=np.int64)

    # seeded jitter of interior nodes outside the box around the cylinder
    rng = np.random.Generator(np.random.PCG64(seed))
    eps = 1e-9
    on_border = (np.abs(pts[:, 0]) < eps) | (np.abs(pts[:, 0] - L) < eps) | \
                (np.abs(pts[:, 1]) < eps) | (np.abs(pts[:, 1] - H) < eps)
    in_box = (pts[:, 0] > 0.1 - eps) & (pts[:, 0] < 0.3 + eps) & \
             (pts[:, 1] > 0.1 - eps) & (pts[:, 1] < 0.3 + eps)
    movable = ~(on_border | in_box)
    d = rng.uniform(-jitter * s, jitter * s, size=pts.shape)
    pts[movable] += d[movable]

    return _finish(pts, tris, _channel_border(pts, tris, L, H, cx, cy, r))


def _channel_border(pts, tris, L, H, cx, cy, r):
    """Classify boundary edges (edges used by one triangle) into the five channel groups."""
    edges = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]])
    key = np.sort(edges, axis=1)
    uniq, idx, cnt = np.unique(key, axis=0, return_index=True, return_counts=True)
    bnd = edges[idx[cnt == 1]]  # keep the triangle's (counter-clockwise) direction
    mid = 0.5 * (pts[bnd[:, 0]] + pts[bnd[:, 1]])
    eps = 1e-9
    out = {}
    masks = {
        "Right": np.abs(mid[:, 0] - L) < eps,
        "Top": np.abs(mid[:, 1] - H) < eps,
        "Left": np.abs(mid[:, 0]) < eps,
        "Bottom": np.abs(mid[:, 1]) < eps,
        "Circle": np.hypot(mid[:, 0] - cx, mid[:, 1] - cy) < r + 1e-3,
    }
    total = 0
    for g, m in masks.items():
        e = bnd[m]
        total += len(e)
        out[g] = _order_chain(e, pts, g)
    if total != len(bnd):
        raise RuntimeError("unclassified boundary edges in generated channel mesh")
    return out


def _order_chain(e: np.ndarray, pts: np.ndarray, group: str) -> np.ndarray:
    """Sort border edges along their curve (as gmsh lists them)."""
    mid = 0.5 * (pts[e[:, 0]] + pts[e[:, 1]])
    if group in ("Right", "Left"):
        o = np.argsort(mid[:, 1])
    elif group in ("Top", "Bottom"):
        o = np.argsort(mid[:, 0])
    else:
        o = np.argsort(np.arctan2(mid[:, 1] - 0.2, mid[:, 0] - 0.2))
    return e[o]


def _finish(pts, tris, border) -> TriMesh:
    """Renumber nodes in a column sweep (x, then y) and triangles by centroid; orient CCW."""
    order = np.lexsort((np.round(pts[:, 1], 12), np.round(pts[:, 0], 12)))
    new_id = np.empty(len(pts), dtype=np.int64)
    new_id[order] = np.arange(len(pts))
    pts = pts[order]
    tris = new_id[tris]
    p = pts[tris]
    det = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - \
          (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])
    if np.any(det == 0):
        raise RuntimeError("degenerate triangle in generated mesh")
    neg = det < 0
    tris[neg] = tris[neg][:, [0, 2, 1]]
    c = pts[tris].mean(axis=1)
    to = np.lexsort((c[:, 1], c[:, 0]))
    tris = tris[to]
    border = {g: new_id[e] for g, e in border.items()}
    return TriMesh(nodes=pts, triangles=tris, border=border)


def p1_stiffness(nodes, triangles):
    """P1 Laplacian (stiffness) of a triangle mesh as a CSR (rowStart, col, val): FP64, columns
    sorted, duplicates summed.  K_ij = sum over triangles of area * grad(phi_i) . grad(phi_j), the
    operator the channel context assembles as the pressure stiffness, built here without the P2
    operators for pressure-only workloads."""
    import scipy.sparse as sp

    x = np.asarray(nodes, dtype=np.float64)[np.asarray(triangles)]  # T x 3 x 2
    det = ((x[:, 1, 0] - x[:, 0, 0]) * (x[:, 2, 1] - x[:, 0, 1]) -
           (x[:, 2, 0] - x[:, 0, 0]) * (x[:, 1, 1] - x[:, 0, 1]))
    area = 0.5 * np.abs(det)
    # gradients of the barycentric coordinates: grad(l_i) = (y_j - y_k, x_k - x_j) / det
    g = np.empty((len(x), 3, 2))
    for i, j, k in ((0, 1, 2), (1, 2, 0), (2, 0, 1)):
        g[:, i, 0] = (x[:, j, 1] - x[:, k, 1]) / det
        g[:, i, 1] = (x[:, k, 0] - x[:, j, 0]) / det
    ke = area[:, None, None] * np.einsum("tik,tjk->tij", g, g)
    t = np.asarray(triangles)
    rows = np.repeat(t, 3, axis=1).ravel()
    cols = np.tile(t, (1, 3)).ravel()
    n = len(nodes)
    a = sp.coo_matrix((ke.ravel(), (rows, cols)), shape=(n, n)).tocsr()
    a.sum_duplicates()
    a.sort_indices()
    return a.indptr.astype(np.int32), a.indices.astype(np.int32), a.data


def jittered_square(n: int, seed: int = 0, jitter: float = 0.2) -> TriMesh:
    """Unit square, n x n nodes, interior nodes moved by U(+-jitter*h), one diagonal per cell.

    Border groups: the four sides are written as Bottom/Right/Top/Left (no cylinder).
    """
    hstep = 1.0 / (n - 1)
    g = np.linspace(0.0, 1.0, n)
    X, Y = np.meshgrid(g, g, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel()], axis=1)
    rng = np.random.Generator(np.random.PCG64(seed))
    d = rng.uniform(-jitter * hstep, jitter * hstep, size=pts.shape)
    interior = (X.ravel() > 0) & (X.ravel() < 1) & (Y.ravel() > 0) & (Y.ravel() < 1)
    pts[interior] += d[interior]
    i, j = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="ij")
    a = (i * n + j).ravel()
    bq = ((i + 1) * n + j).ravel()
    c = ((i + 1) * n + j + 1).ravel()
    dq = (i * n + j + 1).ravel()
    tris = np.concatenate([np.stack([a, bq, c], 1), np.stack([a, c, dq], 1)])
    tris = tris.reshape(2, -1, 3).transpose(1, 0, 2).reshape(-1, 3)
    k = np.arange(n - 1)
    border = {
        "Bottom": np.stack([k * n, (k + 1) * n], 1),
        "Right": np.stack([(n - 1) * n + k, (n - 1) * n + k + 1], 1),
        "Top": np.stack([(k + 1) * n + n - 1, k * n + n - 1], 1),
        "Left": np.stack([k + 1, k], 1),
        "Circle": np.zeros((0, 2), dtype=np.int64),
    }
    return TriMesh(nodes=pts, triangles=tris.astype(np.int64), border=border)


def write_gmsh41(path: str, m: TriMesh) -> None:
    """Write ``m`` as gmsh MSH 4.1 ASCII: one curve entity per border group, one surface."""
    groups = [g for g in GROUPS[:5] if len(m.border.get(g, ())) > 0]
    V = m.num_nodes
    nb = sum(len(m.border[g]) for g in groups)
    T = m.num_triangles
    lines = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$PhysicalNames", str(len(GROUPS))]
    for k, g in enumerate(GROUPS[:5]):
        lines.append(f'1 {k + 1} "{g}"')
    lines.append(f'2 6 "{GROUPS[5]}"')
    lines += ["$EndPhysicalNames", "$Entities", f"0 {len(groups)} 1 0"]
    xmin, ymin = m.nodes.min(axis=0).tolist()
    xmax, ymax = m.nodes.max(axis=0).tolist()
    for g in groups:
        tag = GROUPS.index(g) + 1
        e = m.border[g]
        p = m.nodes[np.unique(e)]
        lo, hi = p.min(axis=0).tolist(), p.max(axis=0).tolist()
        lines.append(f"{tag} {lo[0]!r} {lo[1]!r} 0 {hi[0]!r} {hi[1]!r} 0 1 {tag} 0")
    curve_tags = " ".join(str(GROUPS.index(g) + 1) for g in groups)
    lines.append(f"1 {xmin!r} {ymin!r} 0 {xmax!r} {ymax!r} 0 1 6 {len(groups)} {curve_tags}")
    lines += ["$EndEntities", "$Nodes", f"1 {V} 1 {V}", f"2 1 0 {V}"]
    lines += [str(i + 1) for i in range(V)]
    lines += [f"{x!r} {y!r} 0" for x, y in m.nodes.tolist()]
    lines += ["$EndNodes", "$Elements", f"{len(groups) + 1} {nb + T} 1 {nb + T}"]
    tag = 1
    for g in groups:
        e = m.border[g]
        lines.append(f"1 {GROUPS.index(g) + 1} 1 {len(e)}")
        for a, b in e.tolist():
            lines.append(f"{tag} {a + 1} {b + 1}")
            tag += 1
    lines.append(f"2 1 2 {T}")
    for a, b, c in m.triangles.tolist():
        lines.append(f"{tag} {a + 1} {b + 1} {c + 1}")
        tag += 1
    lines.append("$EndElements")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
