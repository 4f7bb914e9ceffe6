"""Particle surface meshes for the retarded BEM path.

``trisphere`` mirrors ``Particles/particleshapes/trisphere.m:18-61``: it loads
the stored minimum-energy point set closest in size to ``n`` (the table ships
as ``data/tables.npz``), triangulates it, and scales it to the requested
diameter.  The reference triangulates by a stereographic projection plus a
planar Delaunay triangulation (``misc/sphtriangulate.m``); for points on a
sphere that triangulation is the convex hull of the points, which is what is
computed here (same triangles, different face order).  Faces are oriented so
that ``(v1 - v2) x (v3 - v2)`` — the normal of ``norm_flat.m:36-38`` — points
outwards.

``fibsphere`` is this project's own deterministic mesher for sizes beyond the
stored sets (the largest has 1444 points): a Fibonacci spiral of points on the
sphere, triangulated the same way.  ``n_faces = 2 * n_points - 4``.

Faces are returned as ``int64 [n, 4]`` 0-based vertex indices with ``-1`` in
the 4th column for triangles (the reference uses NaN there).
"""
import os

import numpy as np

_TABLES = None


def tables():
    global _TABLES
    if _TABLES is None:
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "tables.npz")
        _TABLES = dict(np.load(path))
    return _TABLES


def _hull_faces(unit):
    from scipy.spatial import ConvexHull
    hull = ConvexHull(unit)
    faces = np.asarray(hull.simplices, dtype=np.int64)
    v1, v2, v3 = unit[faces[:, 0]], unit[faces[:, 1]], unit[faces[:, 2]]
    nvec = np.cross(v1 - v2, v3 - v2)
    cen = (v1 + v2 + v3) / 3
    flip = np.sum(nvec * cen, 1) < 0
    faces[flip] = faces[flip][:, ::-1]
    # deterministic order: sort faces by their smallest vertex index tuple
    rolled = np.array([np.roll(f, -int(np.argmin(f))) for f in faces])
    order = np.lexsort((rolled[:, 2], rolled[:, 1], rolled[:, 0]))
    faces = rolled[order]
    return np.hstack([faces, -np.ones((faces.shape[0], 1), np.int64)])


def trisphere(n, diameter=1.0):
    """Sphere from the stored point set closest to ``n`` points (trisphere.m)."""
    t = tables()
    sizes = t["sphere_sizes"]
    nsav = int(sizes[np.argmin(np.abs(sizes - n))])
    pts = t["sphere%d" % nsav].astype(np.float64)
    faces = _hull_faces(pts / np.linalg.norm(pts, axis=1)[:, None])
    v1 = 0.5 * pts * diameter
    verts = 0.5 * diameter * v1 / np.sqrt(np.sum(v1 * v1, 1))[:, None]
    return verts, faces


def midpoints_flat(verts, faces):
    """Nodes of curved elements from flat ones (Particles/@particle/midpoints.m,
    key 'flat'): every edge gets its midpoint and every quadrilateral its
    centroid.  Returns ``verts2`` (the corners, then the new nodes) and
    ``faces2 [n, 9]`` (corners 0-3 with -1 for triangles, midpoints of edges
    12, 23, 34 (31), 41 in 4-7, quadrilateral centre in 8; -1 where unused)."""
    verts = np.asarray(verts, dtype=np.float64)
    faces = np.asarray(faces, dtype=np.int64)
    if faces.shape[1] == 3:
        faces = np.hstack([faces, -np.ones((faces.shape[0], 1), np.int64)])
    n, nv = faces.shape[0], verts.shape[0]
    quad = faces[:, 3] >= 0
    # edges of every face in order, as (min, max) vertex pairs
    k = np.where(quad, 4, 3)
    a_list, b_list, slot = [], [], []
    for e in range(4):
        m = e < k
        a = faces[m, e]
        b = np.where(e + 1 < k[m], faces[m, (e + 1) % 4], faces[m, 0])
        a_list.append(a); b_list.append(b); slot.append((np.nonzero(m)[0], e))
    lo = np.concatenate([np.minimum(a, b) for a, b in zip(a_list, b_list)])
    hi = np.concatenate([np.maximum(a, b) for a, b in zip(a_list, b_list)])
    uniq, inv = np.unique(lo * (nv + 1) + hi, return_inverse=True)
    ulo, uhi = uniq // (nv + 1), uniq % (nv + 1)
    faces2 = -np.ones((n, 9), np.int64)
    faces2[:, :4] = faces
    off = 0
    for (rows, e) in slot:
        faces2[rows, 4 + e] = nv + inv[off:off + rows.size]
        off += rows.size
    mids = 0.5 * (verts[ulo] + verts[uhi])
    iq = np.nonzero(quad)[0]
    faces2[iq, 8] = nv + uniq.size + np.arange(iq.size)
    cents = 0.25 * verts[faces[iq, :4]].sum(1) if iq.size else np.zeros((0, 3))
    return np.vstack([verts, mids, cents]), faces2


def _split_triangles(faces):
    """Triangles of a face list (totriangles_flat.m): every face's corners
    1-2-3, then corners 3-4-1 of each quadrilateral; returns the triangles and
    the quadrilateral rows."""
    i4 = np.nonzero(faces[:, 3] >= 0)[0]
    return np.vstack([faces[:, :3], faces[i4][:, [2, 3, 0]]]), i4


def _neighbour_fans(tri, nv):
    """Ordered neighbour fan of every vertex, in the order of MNPBEM's
    vertex_neighbours.m (Particles/@particle/private/vertex_neighbours.m:1-76),
    which decides the opposite neighbours of the edge tangents.

    A face (a, b, c) gives a the pair (b, c), b the pair (c, a) and c the pair
    (a, b); a vertex's pairs are kept in face order.  The fan opens at the
    first pair whose first vertex closes no other pair (a boundary vertex),
    else at the first pair, and grows by sweeps over the pairs that append
    the second vertex of each pair continuing the fan; a sweep that appends
    nothing appends every missing vertex of every pair instead."""
    owner = tri.reshape(-1)
    other = tri[:, [1, 2, 2, 0, 0, 1]].reshape(-1, 2)
    order = np.argsort(owner, kind="stable")
    starts = np.searchsorted(owner[order], np.arange(nv + 1))
    fans = []
    for v in range(nv):
        pairs = other[order[starts[v]:starts[v + 1]]].tolist()
        if not pairs:
            fans.append([])
            continue
        seconds = {s for _, s in pairs}
        opening = next((k for k, (f, _) in enumerate(pairs) if f not in seconds), None)
        fan = list(pairs[opening if opening is not None else 0])
        seen = set(fan)
        for _ in range(len(pairs) - 1 - (opening is None)):
            grown = False
            for f, s in pairs:
                if f == fan[-1] and s not in seen:
                    fan.append(s)
                    seen.add(s)
                    grown = True
            if not grown:
                for f, s in pairs:
                    if f not in seen:
                        fan.append(f)
                        seen.add(f)
                        if s not in seen:
                            fan.append(s)
                            seen.add(s)
        for f, s in pairs:
            for x in (f, s):
                if x not in seen:
                    fan.append(x)
                    seen.add(x)
        fans.append(fan)
    return fans


def midpoints_curv(verts, faces):
    """Nodes of curved elements from the approximate curvature of a flat mesh
    (Particles/@particle/midpoints.m:47-49, key 'curv', through
    private/refine.m, edge_tangents.m and make_halfway_vertices.m).

    Every edge i-j gets the midpoint of the cubic Bezier curve whose end
    tangents are estimated at i and j: at a vertex P, the tangent towards the
    neighbour Pn bisects the angle of the planar triangle (P, Pn, Pnop), Pnop
    being the fan neighbour opposite Pn (the mean of the two nearest for an
    odd fan), and the handle length is (|P - Pn| + |Pn - Pnop| / 2) / 6.
    Returns ``verts2`` (the corners, then one node per edge in the order of
    the edge's first visit: lower vertex first, fan order) and ``faces2
    [n, 9]``: triangle midpoints of edges 12, 23, 31 in columns 4-6;
    quadrilateral midpoints of edges 12, 23, 34, 41 in 4-7 and of the
    diagonal 3-1 as its centre node in 8 (refine.m:35-48); -1 where unused."""
    verts = np.ascontiguousarray(verts, dtype=np.float64)
    faces = np.asarray(faces, dtype=np.int64)
    if faces.shape[1] == 3:
        faces = np.hstack([faces, -np.ones((faces.shape[0], 1), np.int64)])
    n, nv = faces.shape[0], verts.shape[0]
    tri, i4 = _split_triangles(faces)
    fans = _neighbour_fans(tri, nv)
    deg = np.array([len(f) for f in fans], np.int64)
    src = np.repeat(np.arange(nv), deg)
    dst = np.array([x for f in fans for x in f], np.int64)
    # position k of each directed edge in its fan, and the opposite neighbours
    base = np.repeat(np.cumsum(deg) - deg, deg)
    k = np.arange(src.size) - base
    L = deg[src]
    o1 = np.where(L % 2 == 0, (k + L // 2) % np.maximum(L, 1), (k + (L - 1) // 2) % np.maximum(L, 1))
    o2 = np.where(L % 2 == 0, o1, (k + (L + 1) // 2) % np.maximum(L, 1))
    P, pn = verts[src], verts[dst]
    pnop = (verts[dst[base + o1]] + verts[dst[base + o2]]) / 2

    def length(d):
        return np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
    ec = length(pn - P) + 1e-14
    eb = length(pnop - P) + 1e-14
    ea = length(pn - pnop) + 1e-14
    s = (ea + eb + ec) / 2
    # Heron's product is clamped at zero (collinear points under rounding)
    h = (2 / ea) * np.sqrt(np.maximum(s * (s - ea) * (s - eb) * (s - ec), 0.0)) + 1e-14
    x = (ea * ea - eb * eb + ec * ec) / (2 * ea)
    r1 = np.sqrt(h * h + x * x) + 1e-14
    r2 = np.sqrt(h * h + (ea - x) * (ea - x)) + 1e-14
    t0 = x / r1 + (ea - x) / r2          # 2-D tangent (t0, t1)
    t1 = -(-h / r1 + h / r2)
    pm = (pn * x[:, None] + pnop * (ea - x)[:, None]) / ea[:, None]
    tan = (pn - pnop) / ea[:, None] * t0[:, None] + (P - pm) / h[:, None] * t1[:, None]
    tan = tan / (length(tan) + 1e-14)[:, None]
    vel = 0.5 * (ec + 0.5 * ea)
    # one node per undirected edge, from its lower vertex's side
    key = src * nv + dst
    ordk = np.argsort(key)
    rev = ordk[np.searchsorted(key[ordk], dst * nv + src)]
    first = np.nonzero(dst > src)[0]
    p0, p3 = P[first], pn[first]
    p1 = p0 + tan[first] * vel[first][:, None] / 3
    p2 = p3 + tan[rev[first]] * vel[rev[first]][:, None] / 3
    c = 3 * (p1 - p0)
    b = 3 * (p2 - p1) - c
    a = p3 - p0 - c - b
    mids = a * 0.125 + b * 0.250 + c * 0.500 + p0
    ekey = key[first]
    eord = np.argsort(ekey)

    def node(u, w):
        q = np.minimum(u, w) * nv + np.maximum(u, w)
        return nv + eord[np.searchsorted(ekey[eord], q)]
    m = np.stack([node(tri[:, 0], tri[:, 1]), node(tri[:, 1], tri[:, 2]), node(tri[:, 2], tri[:, 0])], 1)
    faces2 = -np.ones((n, 9), np.int64)
    faces2[:, :4] = faces
    i3 = np.nonzero(faces[:, 3] < 0)[0]
    faces2[i3, 4:7] = m[i3]
    if i4.size:
        faces2[i4, 4:6] = m[i4, :2]
        faces2[i4, 6:9] = m[n:]
    return np.vstack([verts, mids]), faces2


def trisphere_curved(n, diameter=1.0):
    """``trisphere`` with the curved-element nodes of trisphere.m:54-61: edge
    midpoints projected onto the sphere.  Returns ``verts2, faces2``."""
    v, f = trisphere(n, diameter)
    v2, f2 = midpoints_flat(v, f)
    v2 = 0.5 * diameter * v2 / np.sqrt(np.sum(v2 * v2, 1))[:, None]
    return v2, f2


def fibsphere(n_faces, diameter=1.0, center=(0.0, 0.0, 0.0)):
    """Deterministic sphere with ``n_faces`` (even) flat triangles."""
    npts = n_faces // 2 + 2
    i = np.arange(npts, dtype=np.float64) + 0.5
    z = 1 - 2 * i / npts
    r = np.sqrt(np.maximum(0.0, 1 - z * z))
    golden = np.pi * (3 - np.sqrt(5.0))
    phi = golden * i
    unit = np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)
    faces = _hull_faces(unit)
    verts = 0.5 * diameter * unit + np.asarray(center, dtype=np.float64)[None, :]
    return verts, faces


def sphere(n_faces, diameter=1.0, center=(0.0, 0.0, 0.0)):
    """``trisphere`` when a stored set gives exactly ``n_faces``, else ``fibsphere``."""
    npts = n_faces // 2 + 2
    sizes = tables()["sphere_sizes"]
    if npts in set(int(s) for s in sizes):
        v, f = trisphere(npts, diameter)
        return v + np.asarray(center, dtype=np.float64)[None, :], f
    return fibsphere(n_faces, diameter, center)


def _orient_outward(verts, faces, center):
    """Flip faces whose normal (v1 - v2) x (v3 - v2) points towards ``center``."""
    out = faces.copy()
    for k, f in enumerate(out):
        idx = f[f >= 0]
        p = verts[idx]
        nv = np.cross(p[0] - p[1], p[2] - p[1])
        if np.dot(nv, p.mean(0) - center) < 0:
            out[k, :idx.size] = idx[::-1]
    return out


def _merge(verts, faces, tol=1e-9):
    """Merge coincident vertices; quads that collapse to three vertices become triangles."""
    key = np.round(verts / tol).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    inv = inv.reshape(-1)
    order = np.argsort(first)                 # keep first-occurrence order
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    new_verts = verts[first[order]]
    out = []
    for f in faces:
        idx = [int(rank[inv[i]]) for i in f if i >= 0]
        uniq = []
        for i in idx:
            if i not in uniq:
                uniq.append(i)
        if len(uniq) < 3:
            continue
        out.append(uniq + [-1] * (4 - len(uniq)))
    return new_verts, np.asarray(out, dtype=np.int64)


def trirod(diameter, height, n=(15, 20, 20), triangles=False):
    """Rod with hemispherical caps along z (``Particles/particleshapes/trirod.m``).

    ``n = (nphi, ntheta, nz)``: points around the axis (the first and last
    coincide), polar points per cap (pole to equator) and points along the
    cylinder.  The surface is a grid of quadrilaterals (triangles at the
    poles); ``(nphi - 1) * (2 * (ntheta - 1) + nz - 1)`` faces.  With
    ``triangles`` every quadrilateral is split in two.
    """
    nphi, nth, nz = n
    r = 0.5 * diameter
    half = 0.5 * (height - diameter)
    phi = np.linspace(0.0, 2 * np.pi, nphi)[:-1]
    theta = np.linspace(0.0, 0.5 * np.pi, nth)
    z = half * np.linspace(-1.0, 1.0, nz)
    m = phi.size
    verts, faces = [], []

    def ring(rho, zz):
        base = len(verts)
        for ph in phi:
            verts.append((rho * np.cos(ph), rho * np.sin(ph), zz))
        return base

    def band(b0, b1):
        for i in range(m):
            j = (i + 1) % m
            faces.append([b0 + i, b0 + j, b1 + j, b1 + i])

    # upper cap: pole ring (theta[1]) down to the equator, lower cap mirrored
    for sgn in (1.0, -1.0):
        pole = len(verts)
        verts.append((0.0, 0.0, sgn * (half + r)))
        rings = [ring(r * np.sin(t), sgn * (half + r * np.cos(t))) for t in theta[1:]]
        for i in range(m):
            faces.append([pole, rings[0] + i, rings[0] + (i + 1) % m, -1])
        for a, b in zip(rings[:-1], rings[1:]):
            band(a, b)
    cyl = [ring(r, zz) for zz in z]
    for a, b in zip(cyl[:-1], cyl[1:]):
        band(a, b)
    verts = np.asarray(verts, dtype=np.float64)
    faces = np.asarray(faces, dtype=np.int64)
    verts, faces = _merge(verts, faces, tol=1e-9 * max(1.0, height))
    if triangles:
        faces = _split_quads(faces)
    return verts, _orient_outward(verts, faces, np.zeros(3))


def _split_quads(faces):
    out = []
    for f in faces:
        if f[3] < 0:
            out.append(list(f))
        else:
            out.append([f[0], f[1], f[2], -1])
            out.append([f[2], f[3], f[0], -1])
    return np.asarray(out, dtype=np.int64)


def tricube(n, length=1.0, e=0.25, triangles=False):
    """Cube with rounded edges (``Particles/particleshapes/tricube.m``).

    Each side is an ``(n - 1) x (n - 1)`` grid whose coordinates
    ``sign(u) |u|^(1/e)`` (u uniform in ``[-0.5^e, 0.5^e]``) cluster towards
    the edges; the merged points are then moved onto the super-sphere
    ``x = 0.5 c(theta)^e c(phi)^e, y = 0.5 c(theta)^e s(phi)^e,
    z = 0.5 s(theta)^e`` (signed powers of sin / cos of the spherical angles),
    which rounds the edges, and scaled by ``length``.  6 (n - 1)^2 faces.
    """
    u = np.linspace(-0.5 ** e, 0.5 ** e, n)
    g = np.sign(u) * np.abs(u) ** (1.0 / e)
    X, Y = np.meshgrid(g, g, indexing="xy")
    x, y = X.ravel(), Y.ravel()
    zz = 0.5 * np.ones_like(x)
    quads = []
    for i in range(n - 1):
        for j in range(n - 1):
            a = i * n + j
            quads.append([a, a + 1, a + n + 1, a + n])
    quads = np.asarray(quads, dtype=np.int64)
    sides = [(x, y, zz), (y, x, -zz), (y, zz, x), (x, -zz, y), (zz, x, y), (-zz, y, x)]
    verts, faces = [], []
    for sx, sy, sz in sides:
        off = sum(v.shape[0] for v in verts)
        verts.append(np.stack([sx, sy, sz], 1))
        faces.append(quads + off)
    verts = np.vstack(verts)
    faces = np.vstack(faces)
    verts, faces = _merge(verts, faces, tol=1e-10)
    ph = np.arctan2(verts[:, 1], verts[:, 0])
    th = np.arctan2(verts[:, 2], np.hypot(verts[:, 0], verts[:, 1]))
    isin = lambda a: np.sign(np.sin(a)) * np.abs(np.sin(a)) ** e
    icos = lambda a: np.sign(np.cos(a)) * np.abs(np.cos(a)) ** e
    verts = np.stack([0.5 * icos(th) * icos(ph), 0.5 * icos(th) * isin(ph), 0.5 * isin(th)], 1) * length
    if triangles:
        faces = _split_quads(faces)
    return verts, _orient_outward(verts, faces, np.zeros(3))


def rounding_to_e(length, radius):
    """Super-sphere parameter ``e`` of ``tricube`` for an edge rounding ``radius``.

    Chosen so that the rounded edge passes through the point that a circular
    rounding of that radius gives on the diagonal of the cross section:
    ``h 2^(-e/2) = h - radius (1 - 1/sqrt(2))`` with ``h = length / 2``.
    """
    h = 0.5 * length
    return -2.0 * np.log2(1.0 - radius * (1.0 - 1.0 / np.sqrt(2.0)) / h)
