"""Seeded synthetic meshes for the benchmark workloads, written as gmsh 2.2 ASCII or
handed over as arrays.

The reference ships no generator (its meshes come from gmsh, not installed here).
These follow the reader's constraints (source/io.d:689-990): sequential node and
element numbers, line elements (type 1) carrying the physical tag as the first tag,
tags 1..N in PhysicalNames order, triangles type 2, quads type 3.

* ``wedge``: [0,3]x[0,1] minus the 15-degree ramp from x=0.5; triangles from a
  seeded Delaunay triangulation of Poisson-disk points whose spacing is graded 2x
  finer toward the ramp.  Tags: Inflow (x=0), Top (y=1), Symmetry (y=0, x<0.5), Ramp,
  Outflow (x=3).
* ``bump_channel``: [0,3]x[0,1] with a bump y = h sin^2(pi (x-1)) on 1<=x<=2;
  Delaunay triangles of Poisson-disk points.  Tags: Inflow, Outflow, Wall.
* ``flat_plate``: [-0.5,2]x[0,0.5]; anisotropic quads in a wall layer (first cell
  1e-4, growth 1.05) and Delaunay triangles above.  Tags: Inflow, Top, Outflow,
  Symmetry (y=0, x<0), Wall (y=0, x>=0).
* ``cylinder``: circle of radius 0.5 at the origin in the 40 x 20 box
  [-10,30]x[-10,10]; Delaunay triangles on rings whose spacing grows linearly with
  the distance from the wall.  Tags: Inflow, Outflow, Top, Bottom, Cylinder.
* ``uniform_quads``: n x n quads on [0,1]^2 with one tag (Freestream).
"""
import math

import numpy as np
from scipy.spatial import Delaunay


class MeshArrays:
    def __init__(self, nodes, elements, b_nodes, b_group_start, tags):
        self.nodes = np.asarray(nodes, dtype=np.float64)
        self.elements = elements  # (M,3) / (M,4) int arrays (1-based) or list of lists
        self.b_nodes = np.asarray(b_nodes, dtype=np.int64).reshape(-1, 2)
        self.b_group_start = list(b_group_start)
        self.tags = list(tags)

    @property
    def n_cells(self):
        return sum(len(e) for e in self.elements) if isinstance(self.elements, list) else len(self.elements)

    def element_list(self):
        if isinstance(self.elements, list):
            out = []
            for e in self.elements:
                out.extend(np.asarray(e).tolist())
            return out
        return self.elements.tolist()

    def as_reader_dict(self):
        """The dict shape the oracle's gmsh restatement returns."""
        return {"nodes": self.nodes, "elements": self.element_list(), "bNodes": self.b_nodes,
                "bGroupStart": self.b_group_start, "bTags": self.tags}

    def to_solver_mesh(self):
        from .solver import Mesh
        els = self.elements
        if isinstance(els, list):
            blocks = [np.asarray(e, dtype=np.int64) for e in els if len(e)]
            if len(blocks) == 1:
                els = blocks[0]
            else:
                els = [r for b in blocks for r in b.tolist()]
        return Mesh.from_arrays(self.nodes, els, self.b_nodes, self.b_group_start, self.tags)

    def write_gmsh(self, path):
        """gmsh 2.2 ASCII: line elements first (grouped by tag), then triangles/quads."""
        tags = self.tags
        ng = len(tags)
        starts = list(self.b_group_start) + [len(self.b_nodes)]
        with open(path, "w") as f:
            f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$PhysicalNames\n%d\n" % (ng + 1))
            for i, t in enumerate(tags):
                f.write('1 %d "%s"\n' % (i + 1, t))
            f.write('2 %d "Flow"\n$EndPhysicalNames\n$Nodes\n%d\n' % (ng + 1, len(self.nodes)))
            idx = np.arange(1, len(self.nodes) + 1)
            np.savetxt(f, np.column_stack([idx, self.nodes[:, 0], self.nodes[:, 1], np.zeros(len(idx))]),
                       fmt=["%d", "%.17g", "%.17g", "%d"])
            blocks = self.elements if isinstance(self.elements, list) else [self.elements]
            nel = len(self.b_nodes) + sum(len(b) for b in blocks)
            f.write("$EndNodes\n$Elements\n%d\n" % nel)
            k = 1
            for g in range(ng):
                bn = self.b_nodes[starts[g]:starts[g + 1]] + 1
                n = len(bn)
                ids = np.arange(k, k + n)
                np.savetxt(f, np.column_stack([ids, np.ones(n, int), np.full(n, 2), np.full(n, g + 1),
                                               np.full(n, g + 1), bn]), fmt="%d")
                k += n
            for b in blocks:
                b = np.asarray(b, dtype=np.int64)
                if len(b) == 0:
                    continue
                n = len(b)
                typ = 2 if b.shape[1] == 3 else 3
                ids = np.arange(k, k + n)
                np.savetxt(f, np.column_stack([ids, np.full(n, typ), np.full(n, 2), np.full(n, ng + 1),
                                               np.full(n, ng + 1), b]), fmt="%d")
                k += n
            f.write("$EndElements\n")


def _boundary_groups(tri_nodes_xy, simplices, classify, tags):
    """Boundary edges of a triangulation (edges used once), grouped by classify(midx, midy) -> tag index."""
    e = np.concatenate([simplices[:, [0, 1]], simplices[:, [1, 2]], simplices[:, [2, 0]]])
    es = np.sort(e, axis=1)
    key = es[:, 0].astype(np.int64) * (len(tri_nodes_xy) + 1) + es[:, 1]
    uniq, inv, cnt = np.unique(key, return_inverse=True, return_counts=True)
    once = cnt[inv] == 1
    be = e[once]
    mid = 0.5 * (tri_nodes_xy[be[:, 0]] + tri_nodes_xy[be[:, 1]])
    g = classify(mid[:, 0], mid[:, 1])
    order = np.argsort(g, kind="stable")
    be, g = be[order], g[order]
    starts = [int(np.searchsorted(g, k)) for k in range(len(tags))]
    return be, starts


def _ccw(nodes, tris):
    x, y = nodes[:, 0], nodes[:, 1]
    a = (x[tris[:, 1]] - x[tris[:, 0]]) * (y[tris[:, 2]] - y[tris[:, 0]]) - \
        (x[tris[:, 2]] - x[tris[:, 0]]) * (y[tris[:, 1]] - y[tris[:, 0]])
    t = tris.copy()
    t[a < 0] = t[a < 0][:, [0, 2, 1]]
    return t, np.abs(a)


def _polyline(points, h_fn, closed=False):
    """Points along a polyline at local spacing h_fn(x, y)."""
    out = []
    pts = list(points) + ([points[0]] if closed else [])
    for a, b in zip(pts[:-1], pts[1:]):
        a, b = np.asarray(a, float), np.asarray(b, float)
        L = np.linalg.norm(b - a)
        s = 0.0
        seg = [a]
        while True:
            p = a + (b - a) * (s / L)
            s += h_fn(p[0], p[1])
            if s >= L - 0.3 * h_fn(b[0], b[1]):
                break
            seg.append(a + (b - a) * (s / L))
        out.extend(seg)
    if not closed:
        out.append(np.asarray(pts[-1], float))
    return np.array(out)


def _interior_points(rng, xlo, xhi, ylo, yhi, h_fn, inside, h0):
    """Jittered points with local spacing ~ h_fn: a fine jittered grid thinned by
    acceptance probability (h0/h)^2, keeping a minimum distance from the boundary."""
    nx = int(math.ceil((xhi - xlo) / h0))
    ny = int(math.ceil((yhi - ylo) / h0))
    gx, gy = np.meshgrid((np.arange(nx) + 0.5) * h0 + xlo, (np.arange(ny) + 0.5) * h0 + ylo)
    x = gx.ravel() + rng.uniform(-0.35, 0.35, gx.size) * h0
    y = gy.ravel() + rng.uniform(-0.35, 0.35, gy.size) * h0
    h = h_fn(x, y)
    keep = rng.uniform(0, 1, x.size) < (h0 / h) ** 2
    x, y = x[keep], y[keep]
    m = inside(x, y, 0.5 * h_fn(x, y))
    return np.column_stack([x[m], y[m]])


def _poisson_points(rng, xlo, xhi, ylo, yhi, h_fn, inside, h0, rho):
    """Poisson-disk points with local radius rho h(x, y): a jittered candidate grid
    (spacing 0.75 h0) reduced to a maximal independent set of the graph joining
    candidates closer than rho times their mean local spacing (Luby's random-priority
    rounds), then kept at least half a local spacing inside the boundary."""
    from scipy.spatial import cKDTree
    s = 0.75 * h0
    nx = int(math.ceil((xhi - xlo) / s))
    ny = int(math.ceil((yhi - ylo) / s))
    gx, gy = np.meshgrid((np.arange(nx) + 0.5) * s + xlo, (np.arange(ny) + 0.5) * s + ylo)
    x = gx.ravel() + rng.uniform(-0.4, 0.4, gx.size) * s
    y = gy.ravel() + rng.uniform(-0.4, 0.4, gy.size) * s
    m = inside(x, y, 0.5 * h_fn(x, y))
    x, y = x[m], y[m]
    h = h_fn(x, y)
    pts = np.column_stack([x, y])
    pairs = cKDTree(pts).query_pairs(rho * float(h.max()), output_type="ndarray")
    i, j = pairs[:, 0], pairs[:, 1]
    d = np.hypot(x[i] - x[j], y[i] - y[j])
    close = d < rho * 0.5 * (h[i] + h[j])
    i, j = i[close], j[close]
    n = len(x)
    prio = rng.permutation(n)
    alive = np.ones(n, bool)
    kept = np.zeros(n, bool)
    while True:
        a = alive[i] & alive[j]
        ii, jj = i[a], j[a]
        if len(ii) == 0:
            kept |= alive
            break
        lose = np.zeros(n, bool)
        lose[np.where(prio[ii] < prio[jj], ii, jj)] = True
        win = alive & ~lose
        kept |= win
        alive &= ~win
        alive[jj[win[ii]]] = False
        alive[ii[win[jj]]] = False
    return pts[kept]


def _graded_lattice(rng, x0, x1, ylo, yhi, h_of_y, jitter=0.08):
    """Points of a staggered triangular lattice graded in y: rows sqrt(3)/2 h(y) apart,
    points h(y) apart along each row (odd rows shifted by half a spacing), the row
    ends on x = x0 and x = x1, the first row at ylo excluded (it belongs to the caller)
    and the last row on yhi; interior points jittered by up to `jitter` h (seeded).
    Delaunay triangles of such points are close to equilateral wherever h varies slowly
    (no slivers), so the smallest 2 A / perimeter stays a fixed fraction of h."""
    rows = []
    y = ylo
    k = 0
    while True:
        y_next = y + 0.5 * math.sqrt(3.0) * float(h_of_y(y))
        if y_next >= yhi - 0.4 * 0.5 * math.sqrt(3.0) * float(h_of_y(yhi)):
            break
        y = y_next
        k += 1
        rows.append((y, k))
    rows.append((yhi, k + 1))
    out = []
    for y, k in rows:
        h = float(h_of_y(y))
        n = max(2, int(round((x1 - x0) / h)))
        s = (x1 - x0) / n
        if k % 2:
            xs = np.concatenate([[x0], x0 + (np.arange(n) + 0.5) * s, [x1]])
        else:
            xs = x0 + np.arange(n + 1) * s
        ys = np.full(xs.shape, y)
        if y < yhi:  # jitter interior points (row ends stay on the side boundaries)
            inner = slice(1, len(xs) - 1)
            xs[inner] += rng.uniform(-jitter, jitter, len(xs) - 2) * s
            ys[inner] += rng.uniform(-jitter, jitter, len(xs) - 2) * s
        out.append(np.column_stack([xs, ys]))
    return np.vstack(out)


def wedge(n_cells=1_000_000, seed=0, angle_deg=15.0, ramp_x=0.5):
    rng = np.random.default_rng(seed)
    ta = math.tan(math.radians(angle_deg))
    ymax_ramp = (3.0 - ramp_x) * ta

    def floor_y(x):
        return np.where(x > ramp_x, (x - ramp_x) * ta, 0.0)

    def dist_ramp(x, y):
        return np.hypot(np.maximum(x - 3.0, 0) + np.minimum(x - ramp_x, 0), 0) * 0 + np.abs(y - floor_y(x))

    # spacing graded 2x: h = hc near the floor/ramp (distance 0) to 2 hc at distance >= 0.5
    area = 3.0 - 0.5 * (3.0 - ramp_x) * ymax_ramp
    # triangles ~ 2 * points; mean (1/h^2) over the domain sets hc
    def inv_h2_mean(hc):
        xs = np.linspace(0, 3, 200)
        tot = 0.0
        for xv in xs:
            yl = float(floor_y(np.array([xv]))[0])
            ys = np.linspace(yl, 1, 100)
            d = ys - yl
            h = hc * (1 + np.clip(d / 0.5, 0, 1))
            tot += np.mean(1 / h ** 2) * (1 - yl)
        return tot / len(xs) * 3.0
    hc = math.sqrt(inv_h2_mean(1.0) / (n_cells / 2.0))

    def h_fn(x, y):
        d = np.abs(np.asarray(y) - floor_y(np.asarray(x)))
        return hc * (1 + np.clip(d / 0.5, 0, 1))

    corners = [(0.0, 0.0), (ramp_x, 0.0), (3.0, ymax_ramp), (3.0, 1.0), (0.0, 1.0)]
    bpts = _polyline(corners, lambda x, y: float(h_fn(np.array([x]), np.array([y]))[0]), closed=True)

    def inside(x, y, margin):
        return (x > margin) & (x < 3.0 - margin) & (y < 1.0 - margin) & (y - floor_y(x) > margin * 1.05)

    # Poisson-disk interior points; the point count goes as rho^-1.74 (measured), and
    # rho = 0.71 puts the triangle count near n_cells; a second pass corrects it when
    # it is off by more than 2%
    rho = 0.71
    for _ in range(2):
        ip = _poisson_points(np.random.default_rng(seed), 0.0, 3.0, 0.0, 1.0, h_fn, inside, hc, rho)
        ratio = (2 * len(ip) + len(bpts)) / n_cells
        if abs(ratio - 1) < 0.02:
            break
        rho *= ratio ** (1 / 1.74)
    nodes = np.vstack([bpts, ip])
    tri = Delaunay(nodes).simplices.astype(np.int64)
    tris, a = _ccw(nodes, tri)
    tris = tris[a > 1e-14]
    tags = ["Inflow", "Top", "Symmetry", "Ramp", "Outflow"]
    eps = 1e-9

    def classify(mx, my):
        g = np.full(mx.shape, 1)
        g[mx < eps] = 0
        g[mx > 3.0 - eps] = 4
        g[(my < eps) & (mx < ramp_x)] = 2
        g[(mx >= ramp_x) & (np.abs(my - floor_y(mx)) < 1e-7) & (mx < 3.0 - eps)] = 3
        return g

    be, starts = _boundary_groups(nodes, tris, classify, tags)
    return MeshArrays(nodes, tris + 1, be, starts, tags)


def bump_channel(n_cells=20000, h=0.05, seed=0):
    """Poisson-disk interior points (minimum triangle angle ~17 degrees and up; a
    jittered grid, the earlier choice, left angles down to ~10 degrees)."""

    def floor_y(x):
        x = np.asarray(x, float)
        return np.where((x >= 1) & (x <= 2), h * np.sin(np.pi * (x - 1)) ** 2, 0.0)

    area = 3.0 - 0.5 * h
    hc = math.sqrt(area / (n_cells / 2.0))
    hfun = lambda x, y: np.full(np.shape(x), hc)  # noqa: E731
    xs = np.arange(0, 3 + 1e-12, hc)
    xs[-1] = 3.0
    bottom = np.column_stack([xs, floor_y(xs)])
    top = np.column_stack([xs[::-1], np.ones_like(xs)])
    ys = np.arange(hc, 1 - 0.5 * hc, hc)
    right = np.column_stack([np.full_like(ys, 3.0), ys])
    left = np.column_stack([np.zeros_like(ys), ys[::-1]])
    bpts = np.vstack([bottom, right, top, left])

    def inside(x, y, margin):
        return (x > margin) & (x < 3 - margin) & (y < 1 - margin) & (y - floor_y(x) > margin)

    rho = 0.71  # the triangle count goes as rho^-1.74; a second pass corrects rho when off by > 2%
    for _ in range(2):
        ip = _poisson_points(np.random.default_rng(seed), 0, 3, 0, 1, hfun, inside, hc, rho)
        ratio = (2 * len(ip) + len(bpts)) / n_cells
        if abs(ratio - 1) < 0.02:
            break
        rho *= ratio ** (1 / 1.74)
    nodes = np.vstack([bpts, ip])
    tri = Delaunay(nodes).simplices.astype(np.int64)
    # the convex hull also covers the region under the bump: drop those triangles
    c = nodes[tri].mean(axis=1)
    tri = tri[c[:, 1] > floor_y(c[:, 0])]
    tris, a = _ccw(nodes, tri)
    tris = tris[a > 1e-14]
    used = np.unique(tris)
    remap = np.full(len(nodes), -1, np.int64)
    remap[used] = np.arange(len(used))
    nodes, tris = nodes[used], remap[tris]
    tags = ["Inflow", "Outflow", "Wall"]
    eps = 1e-9

    def classify(mx, my):
        g = np.full(mx.shape, 2)
        g[mx < eps] = 0
        g[mx > 3 - eps] = 1
        return g

    be, starts = _boundary_groups(nodes, tris, classify, tags)
    return MeshArrays(nodes, tris + 1, be, starts, tags)


def flat_plate(n_cells=4_000_000, h1=1e-4, growth=1.05, seed=0, layer_top=None):
    rng = np.random.default_rng(seed)
    x0, x1, y1 = -0.5, 2.0, 0.5
    # wall-layer column count sized so quads are ~12% of the cells
    nl = 0
    ys = [0.0]
    hh = h1
    while True:
        ys.append(ys[-1] + hh)
        hh *= growth
        nl += 1
        if (layer_top and ys[-1] >= layer_top) or (not layer_top and hh > 2.5e-3):
            break
    ys = np.array(ys)
    H = ys[-1]
    # tri region spacing graded from dx at the layer top to 4 dx at y1; a triangular
    # lattice of spacing h has 2 / (sqrt(3)/2 h^2) triangles per unit area
    def tri_count(dx):
        yy = np.linspace(H, y1, 400)
        h = dx * (1 + 3 * (yy - H) / (y1 - H))
        return 2 / (0.5 * math.sqrt(3.0)) * np.trapezoid((x1 - x0) / h ** 2, yy)
    lo, hi = 1e-5, 1e-1
    for _ in range(60):
        dx = math.sqrt(lo * hi)
        nc = tri_count(dx) + (x1 - x0) / dx * nl
        if nc > n_cells:
            lo = dx
        else:
            hi = dx
    dx = math.sqrt(lo * hi)
    # columns on x0 + i dx with the plate's leading edge x = 0 on a column
    nl_ = int(round(-x0 / dx))
    dx = -x0 / nl_
    nx = int(round((x1 - x0) / dx))
    xs = x0 + np.arange(nx + 1) * dx
    xs[-1] = x1
    X, Y = np.meshgrid(xs, ys)
    qnodes = np.column_stack([X.ravel(), Y.ravel()])
    ncol = len(xs)
    qid = np.arange(len(qnodes)).reshape(len(ys), ncol)
    quads = np.column_stack([qid[:-1, :-1].ravel(), qid[:-1, 1:].ravel(), qid[1:, 1:].ravel(), qid[1:, :-1].ravel()])

    def h_fn(x, y):
        return dx * (1 + 3 * np.clip((np.asarray(y) - H) / (y1 - H), 0, 1))

    # triangle region: the layer top row is shared with the quads; above it a seeded,
    # jittered triangular lattice graded with h_fn (its row ends form the side
    # boundaries, its last row the top)
    top_row = qid[-1]
    tnodes_extra = _graded_lattice(rng, x0, x1, H, y1, lambda y: h_fn(x0, y))
    nodes = np.vstack([qnodes, tnodes_extra])
    tri_set = np.concatenate([top_row, np.arange(len(qnodes), len(nodes))])
    local = nodes[tri_set]
    tri = Delaunay(local).simplices.astype(np.int64)
    tri = tri_set[tri]
    tris, a = _ccw(nodes, tri)
    tris = tris[a > 1e-16]
    # boundary: quads' left/right/bottom + triangles' outer edges
    tags = ["Inflow", "Top", "Outflow", "Symmetry", "Wall"]
    eps = 1e-12
    bl = []
    for j in range(ncol - 1):
        a_, b_ = qid[0, j], qid[0, j + 1]
        xm = 0.5 * (xs[j] + xs[j + 1])
        bl.append((4 if xm >= 0 else 3, b_, a_))
    for i in range(len(ys) - 1):
        bl.append((0, qid[i + 1, 0], qid[i, 0]))
        bl.append((2, qid[i, -1], qid[i + 1, -1]))

    def classify(mx, my):
        g = np.full(mx.shape, 1)
        g[mx < x0 + eps] = 0
        g[mx > x1 - eps] = 2
        return g

    tbe, tstarts = _boundary_groups(nodes, tris, classify, tags)
    # drop the layer-top edges (shared with quads, not boundary)
    mid_y = 0.5 * (nodes[tbe[:, 0], 1] + nodes[tbe[:, 1], 1])
    keep = mid_y > H + 1e-12
    tg = classify(0.5 * (nodes[tbe[:, 0], 0] + nodes[tbe[:, 1], 0]), mid_y)
    allb = [(int(g), int(a_), int(b_)) for g, (a_, b_) in zip(tg[keep], tbe[keep])] + bl
    allb.sort(key=lambda r: r[0])
    g = np.array([r[0] for r in allb])
    be = np.array([[r[1], r[2]] for r in allb], dtype=np.int64)
    starts = [int(np.searchsorted(g, k)) for k in range(len(tags))]
    return MeshArrays(nodes, [quads + 1, tris + 1], be, starts, tags)


def _cylinder_points(hw, growth, box, r0, rng):
    (x0, x1), (y0, y1) = box
    rmax = math.hypot(max(-x0, x1), max(-y0, y1))
    pts = []
    r = r0
    k = 0
    while r < rmax:
        h = hw * (1 + growth * (r - r0))
        n = max(8, int(math.ceil(2 * math.pi * r / h)))
        th = (np.arange(n) + 0.5 * (k % 2)) * (2 * math.pi / n) + rng.uniform(-0.05, 0.05) * (k > 0)
        x, y = r * np.cos(th), r * np.sin(th)
        m = (x > x0 + 0.5 * h) & (x < x1 - 0.5 * h) & (y > y0 + 0.5 * h) & (y < y1 - 0.5 * h)
        pts.append(np.column_stack([x[m], y[m]]))
        r += 0.866 * h
        k += 1
    return np.vstack(pts)


def cylinder(n_cells=20000, r=0.5, seed=0, growth=0.25):
    rng = np.random.default_rng(seed)
    box = ((-10.0, 30.0), (-10.0, 10.0))

    def count(hw):
        return 2 * len(_cylinder_points(hw, growth, box, r, np.random.default_rng(0)))

    lo, hi = 1e-4, 2.0  # wall spacing bracket
    for _ in range(40):
        mid = math.sqrt(lo * hi)
        if count(mid) > n_cells:
            lo = mid
        else:
            hi = mid
    hw = math.sqrt(lo * hi)
    ip = _cylinder_points(hw, growth, box, r, rng)
    h_fn = lambda x, y: hw * (1 + growth * (math.hypot(x, y) - r))
    (x0, x1), (y0, y1) = box
    bpts = _polyline([(x0, y0), (x1, y0), (x1, y1), (x0, y1)], h_fn, closed=True)
    nodes = np.vstack([bpts, ip])
    tri = Delaunay(nodes).simplices.astype(np.int64)
    c = nodes[tri].mean(axis=1)
    tri = tri[np.hypot(c[:, 0], c[:, 1]) > r]
    tris, a = _ccw(nodes, tri)
    tris = tris[a > 1e-14]
    used = np.unique(tris)
    remap = np.full(len(nodes), -1, np.int64)
    remap[used] = np.arange(len(used))
    nodes, tris = nodes[used], remap[tris]
    tags = ["Inflow", "Outflow", "Top", "Bottom", "Cylinder"]
    eps = 1e-9

    def classify(mx, my):
        g = np.full(mx.shape, 4)
        g[mx < x0 + eps] = 0
        g[mx > x1 - eps] = 1
        g[my > y1 - eps] = 2
        g[my < y0 + eps] = 3
        return g

    be, starts = _boundary_groups(nodes, tris, classify, tags)
    return MeshArrays(nodes, tris + 1, be, starts, tags)


def uniform_quads(n=32):
    xs = np.linspace(0, 1, n + 1)
    X, Y = np.meshgrid(xs, xs)
    nodes = np.column_stack([X.ravel(), Y.ravel()])
    qid = np.arange(len(nodes)).reshape(n + 1, n + 1)
    quads = np.column_stack([qid[:-1, :-1].ravel(), qid[:-1, 1:].ravel(), qid[1:, 1:].ravel(), qid[1:, :-1].ravel()])
    b = []
    for j in range(n):
        b.append((qid[0, j], qid[0, j + 1]))
    for i in range(n):
        b.append((qid[i, n], qid[i + 1, n]))
    for j in range(n, 0, -1):
        b.append((qid[n, j], qid[n, j - 1]))
    for i in range(n, 0, -1):
        b.append((qid[i, 0], qid[i - 1, 0]))
    return MeshArrays(nodes, quads + 1, np.array(b), [0], ["Freestream"])


def hanging_quads(n=16):
    """Non-conforming quads on [0,1]^2: an n x n grid (n even) whose cells with
    x index >= n/2 or y index >= n/2 are split 2 x 2.  The unsplit cells next to
    split ones carry the split side's middle node, so the mesh has pentagons along
    both interfaces and a hexagon at their corner (the reference's cells have up to
    six edges, source/mesh.d:26).  One tag (Freestream)."""
    assert n % 2 == 0 and n >= 4
    m = 2 * n + 1
    fid = lambda a, b: b * m + a  # noqa: E731  (fine-grid node id)
    split = lambda i, j: i >= n // 2 or j >= n // 2  # noqa: E731
    rows = []
    for j in range(n):
        for i in range(n):
            if split(i, j):
                for b in (2 * j, 2 * j + 1):
                    for a in (2 * i, 2 * i + 1):
                        rows.append([fid(a, b), fid(a + 1, b), fid(a + 1, b + 1), fid(a, b + 1)])
            else:
                v = [fid(2 * i, 2 * j), fid(2 * i + 2, 2 * j)]
                if i + 1 < n and split(i + 1, j):
                    v.append(fid(2 * i + 2, 2 * j + 1))
                v.append(fid(2 * i + 2, 2 * j + 2))
                if j + 1 < n and split(i, j + 1):
                    v.append(fid(2 * i + 1, 2 * j + 2))
                v.append(fid(2 * i, 2 * j + 2))
                rows.append(v)
    b = []
    for i in range(n):  # counter-clockwise walk: bottom, right, top, left
        b += [(fid(2 * i, 0), fid(2 * i + 1, 0)), (fid(2 * i + 1, 0), fid(2 * i + 2, 0))] if split(i, 0) \
            else [(fid(2 * i, 0), fid(2 * i + 2, 0))]
    b += [(fid(2 * n, k), fid(2 * n, k + 1)) for k in range(2 * n)]
    b += [(fid(k, 2 * n), fid(k - 1, 2 * n)) for k in range(2 * n, 0, -1)]
    for j in range(n - 1, -1, -1):
        b += [(fid(0, 2 * j + 2), fid(0, 2 * j + 1)), (fid(0, 2 * j + 1), fid(0, 2 * j))] if split(0, j) \
            else [(fid(0, 2 * j + 2), fid(0, 2 * j))]
    used = np.unique(np.concatenate([np.asarray(r) for r in rows]))
    new = np.full(m * m, -1, dtype=np.int64)
    new[used] = np.arange(len(used))
    xs = np.linspace(0.0, 1.0, m)
    nodes = np.column_stack([xs[used % m], xs[used // m]])
    blocks, run = [], []
    for r in rows:  # consecutive cells with the same edge count form one block
        if run and len(run[-1]) != len(r):
            blocks.append(np.asarray(run, dtype=np.int64) + 1)
            run = []
        run.append([int(new[v]) for v in r])
    blocks.append(np.asarray(run, dtype=np.int64) + 1)
    return MeshArrays(nodes, blocks, new[np.asarray(b)], [0], ["Freestream"])
