"""Particles, composite particles and their quadrature rules (host side).

Mirrors MNPBEM's ``particle`` (``Particles/@particle``), ``comparticle``
(``Particles/@comparticle``), ``quadface`` (``Misc/integration/@quadface``) and
``trisphere`` (``Particles/particleshapes/trisphere.m``).  The GPU library
recomputes every geometric quantity it uses (centroids, normals, areas,
quadrature points) from ``verts``/``faces``; the host-side ``pos``, ``nvec`` and
``area`` here serve user code and the sphere at infinity of the spectra.
"""
import numpy as np

from . import shapes


def lglnodes(n):
    """n+1 Legendre-Gauss-Lobatto nodes and weights on [-1, 1].

    Nodes are the roots of (1 - x^2) P_n'(x), found by Newton iterations on
    x P_n(x) - P_{n-1}(x) from the Chebyshev-Gauss-Lobatto points; weights are
    2 / (n (n+1) P_n(x)^2) (Misc/integration/lglnodes.m:13-32).
    """
    n1 = n + 1
    x = np.cos(np.pi * np.arange(n1) / n)
    prev = np.full(n1, 2.0)
    P = np.zeros((n1, n1))
    while np.max(np.abs(x - prev)) > np.finfo(float).eps:
        prev = x
        P[:, 0], P[:, 1] = 1.0, x
        for k in range(2, n1):
            P[:, k] = ((2 * k - 1) * x * P[:, k - 1] - (k - 1) * P[:, k - 2]) / k
        x = prev - (x * P[:, n] - P[:, n - 1]) / (n1 * P[:, n])
    return x, 2.0 / (n * n1 * P[:, n] ** 2)


class quadface:
    """Quadrature rules of boundary elements (@quadface/private/init.m:5-80).

    ``x, y, w``: 28-point triangle rule (rule 18, weights sum to 1);
    ``x3, y3, w3``: polar rule around the centroid of a triangle
    ((npol[0]+1) x (npol[1]+1) x 3 points, weights sum to 1);
    ``x4, y4, w4``: polar rule of a quadrilateral on [-1, 1]^2 (weights sum to 4).
    """

    def __init__(self, npol=(7, 5)):
        if np.isscalar(npol):
            npol = (int(npol), int(npol))
        self.npol = tuple(int(v) for v in npol)
        t = shapes.tables()
        self.x, self.y, self.w = t["rule18_x"].copy(), t["rule18_y"].copy(), t["rule18_w"].copy()
        self.x3, self.y3, self.w3 = self._polar(3)
        self.x4, self.y4, self.w4 = self._polar(4)

    def _polar(self, corners):
        x1, w1 = lglnodes(self.npol[0])
        x2, w2 = lglnodes(self.npol[1])
        rho = 0.5 * (x1 + 1 + 1e-6)
        if corners == 3:
            phi = (270 + 60 * x2) / 180 * np.pi
            step = 2 * np.pi / 3
        else:
            phi = (90 + 45 * x2) / 180 * np.pi
            step = np.pi / 2
        # radius (rho fastest) x angle grid, column-major like MATLAB's ndgrid(:)
        R = np.repeat(rho[:, None], phi.size, 1).ravel(order="F")
        PH = np.repeat(phi[None, :], rho.size, 0).ravel(order="F")
        rad = 1.0 / np.abs((2 if corners == 3 else 1) * np.sin(PH))
        ang = np.concatenate([PH + r * step for r in range(corners)])
        rr = np.tile(R * rad, corners)
        xx, yy = np.cos(ang) * rr, np.sin(ang) * rr
        if corners == 3:
            xx, yy = (1 - np.sqrt(3) * xx - yy) / 3, (1 + np.sqrt(3) * xx - yy) / 3
        w = np.tile((np.outer(w1, w2).ravel(order="F")) * R * rad ** 2, corners)
        w = (1.0 if corners == 3 else 4.0) * w / w.sum()
        return xx, yy, w


def _norm_flat(verts, faces):
    n = faces.shape[0]
    tri = faces[:, 3] < 0
    v = verts
    pos = np.where(tri[:, None], (v[faces[:, 0]] + v[faces[:, 1]] + v[faces[:, 2]]) / 3,
                   (v[faces[:, 0]] + v[faces[:, 1]] + v[faces[:, 2]] + v[np.maximum(faces[:, 3], 0)]) / 4)
    a1, b1 = v[faces[:, 0]] - v[faces[:, 1]], v[faces[:, 2]] - v[faces[:, 1]]
    n1 = np.cross(a1, b1)
    ar1 = 0.5 * np.linalg.norm(n1, axis=1)
    t1, nn, area = a1.copy(), n1.copy(), ar1.copy()
    q = np.nonzero(~tri)[0]
    if q.size:
        v4 = v[faces[q, 3]]
        a2, b2 = v[faces[q, 2]] - v4, v[faces[q, 0]] - v4
        n2 = np.cross(a2, b2)
        ar2 = 0.5 * np.linalg.norm(n2, axis=1)
        area[q] = ar1[q] + ar2
        big = ar2 > ar1[q]
        t1[q[big]], nn[q[big]] = a2[big], n2[big]
    t1 /= np.linalg.norm(t1, axis=1)[:, None]
    nn /= np.linalg.norm(nn, axis=1)[:, None]
    return pos, nn, np.cross(nn, t1), t1, area[:n]


def _tri6(x, y):
    z = 1 - x - y
    s = np.stack([x * (2 * x - 1), y * (2 * y - 1), z * (2 * z - 1), 4 * x * y, 4 * y * z, 4 * z * x], 1)
    sx = np.stack([4 * x - 1, 0 * y, 1 - 4 * z, 4 * y, -4 * y, 4 * (z - x)], 1)
    sy = np.stack([0 * x, 4 * y - 1, 1 - 4 * z, 4 * x, 4 * (z - y), -4 * x], 1)
    return s, sx, sy


def _norm_curv(verts2, faces2, quad):
    """Curved elements (norm_curv.m:8-62): area from the quad_curv.m weights,
    centroid and basis from the 6-node shape functions at the centre."""
    tri = faces2[:, 3] < 0
    n = faces2.shape[0]
    t1 = np.where(tri[:, None], faces2[:, [0, 1, 2, 4, 5, 6]], faces2[:, [0, 1, 2, 4, 5, 8]])
    s, sx, sy = _tri6(quad.x, quad.y)

    def tri_area(nodes):
        vv = verts2[nodes]
        nv = np.cross(np.einsum("pk,tkc->tpc", sx, vv), np.einsum("pk,tkc->tpc", sy, vv))
        return np.sum(0.5 * quad.w[None, :] * np.linalg.norm(nv, axis=2), 1)
    area = tri_area(t1)
    q = np.nonzero(~tri)[0]
    if q.size:
        area[q] += tri_area(faces2[q][:, [2, 3, 0, 6, 7, 8]])
    vv = verts2[t1]
    c = np.array([-1, -1, -1, 4, 4, 4]) / 9
    cx, cy = np.array([1, 0, -1, 4, -4, 0]) / 3, np.array([0, 1, -1, 4, 0, -4]) / 3
    qx, qy = np.array([1, 0, -1, 0, 0, 0], float), np.array([0, -1, -1, 2, 2, -2], float)
    pos = np.where(tri[:, None], np.einsum("k,tkc->tc", c, vv), verts2[t1[:, 5]])
    a = np.where(tri[:, None], np.einsum("k,tkc->tc", cy, vv), np.einsum("k,tkc->tc", qy, vv))
    b = np.where(tri[:, None], np.einsum("k,tkc->tc", cx, vv), np.einsum("k,tkc->tc", qx, vv))
    nn = np.cross(a, b)
    nn /= np.linalg.norm(nn, axis=1)[:, None]
    t1v = a / np.linalg.norm(a, axis=1)[:, None]
    return pos, nn, np.cross(nn, t1v), t1v, area


class particle:
    """Discretised surface: ``verts [nv, 3]``, ``faces [n, 4]`` (-1 in the 4th
    column for triangles; a ``[n, 3]`` array is accepted).  As in MNPBEM
    (Particles/@particle/init.m:17-38), ``faces [n, 9]`` gives the nodes of
    curved elements (``verts2`` / ``faces2``: corners, edge midpoints,
    quadrilateral centre; -1 or NaN where unused); ``op['interp']`` selects
    flat (default, the corners) or curved ('curv') elements."""

    def __init__(self, verts, faces, op=None):
        verts = np.ascontiguousarray(verts, dtype=np.float64)
        faces = np.asarray(faces)
        if faces.ndim != 2 or faces.shape[1] not in (3, 4, 9):
            raise ValueError("faces must be [n, 3], [n, 4] or [n, 9]")
        if np.issubdtype(faces.dtype, np.floating):
            faces = np.where(np.isnan(faces), -1, faces)
        faces = faces.astype(np.int64)
        if faces.shape[1] == 3:
            faces = np.hstack([faces, -np.ones((faces.shape[0], 1), dtype=np.int64)])
        self.verts2 = self.faces2 = None
        if faces.shape[1] == 9:
            self.verts2, self.faces2 = verts, np.ascontiguousarray(faces)
            faces = faces[:, :4]
        self.verts = verts
        self.faces = np.ascontiguousarray(faces, dtype=np.int64)
        op = op or {}
        self.op = dict(op)
        self.interp = op.get("interp", "flat")
        if self.interp not in ("flat", "curv"):
            raise ValueError("interp must be 'flat' or 'curv'")
        self.quad = quadface(op.get("npol", (7, 5)))
        if self.interp == "curv":
            if self.faces2 is None:
                # curved elements through flat midpoints (midpoints.m, key 'flat')
                self.verts2, self.faces2 = shapes.midpoints_flat(self.verts, self.faces)
            self.pos, self.nvec, self.tvec2, self.tvec1, self.area = _norm_curv(self.verts2, self.faces2, self.quad)
        else:
            self.pos, self.nvec, self.tvec2, self.tvec1, self.area = _norm_flat(self.verts, self.faces)

    @property
    def curved(self):
        return self.interp == "curv"

    @property
    def n(self):
        return self.faces.shape[0]

    nfaces = n

    def midpoints(self, key="flat"):
        """Particle with the nodes of curved elements
        (Particles/@particle/midpoints.m): key 'flat' puts them at the edge
        midpoints and quadrilateral centroids, 'curv' on cubic Bezier curves
        through the surface tangents estimated at the vertices (refine.m).
        As in midpoints.m:14 the element interpolation becomes ``key``."""
        if key not in ("flat", "curv"):
            raise ValueError("midpoints key must be 'flat' or 'curv'")
        make = shapes.midpoints_flat if key == "flat" else shapes.midpoints_curv
        v2, f2 = make(self.verts, self.faces)
        return particle(v2, f2, dict(self.op, interp=key))

    def _remake(self, verts, faces, verts2=None, faces2=None):
        if self.faces2 is not None:
            return particle(verts2, faces2, self.op)
        return particle(verts, faces, self.op)

    def rot(self, angle, dir=(0.0, 0.0, 1.0)):
        """Rotation by ``angle`` degrees about ``dir`` (Particles/@particle/
        rot.m): vertices times expm(-angle (d1 J1 + d2 J2 + d3 J3)) as row
        vectors, J the generators of rotations about x, y, z."""
        from scipy.linalg import expm
        d = np.asarray(dir, dtype=np.float64)
        d = d / np.linalg.norm(d)
        j1 = np.array([[0, 0, 0], [0, 0, -1], [0, 1, 0]], float)
        j2 = np.array([[0, 0, 1], [0, 0, 0], [-1, 0, 0]], float)
        j3 = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 0]], float)
        r = expm(-angle / 180 * np.pi * (d[0] * j1 + d[1] * j2 + d[2] * j3))
        return self._remake(self.verts @ r, self.faces,
                            None if self.verts2 is None else self.verts2 @ r, self.faces2)

    def scale(self, factor):
        """Vertices times a scalar or per-axis ``factor`` (scale.m)."""
        f = np.asarray(factor, dtype=np.float64)
        return self._remake(self.verts * f, self.faces,
                            None if self.verts2 is None else self.verts2 * f, self.faces2)

    def flipfaces(self):
        """Reversed face orientation (flipfaces.m): corner order reversed, the
        edge-midpoint columns of curved elements permuted to match."""
        faces = self.faces.copy()
        tri = faces[:, 3] < 0
        faces[tri, :3] = faces[tri][:, [2, 1, 0]]
        faces[~tri, :4] = faces[~tri][:, [3, 2, 1, 0]]
        faces2 = None
        if self.faces2 is not None:
            faces2 = self.faces2.copy()
            faces2[tri, :7] = self.faces2[tri][:, [2, 1, 0, 3, 5, 4, 6]]
            faces2[~tri, :8] = self.faces2[~tri][:, [3, 2, 1, 0, 6, 5, 4, 7]]
        return self._remake(self.verts, faces, self.verts2, faces2)

    def flip(self, dir=1):
        """Mirror image along axis ``dir`` (1-based: 1 = x, as flip.m), with
        the faces flipped so that the normals stay outward."""
        v = self.verts.copy()
        v[:, dir - 1] *= -1
        v2 = None
        if self.verts2 is not None:
            v2 = self.verts2.copy()
            v2[:, dir - 1] *= -1
        return self._remake(v, self.faces, v2, self.faces2).flipfaces()

    def shift(self, vec):
        d = np.asarray(vec, dtype=np.float64)[None, :]
        if self.faces2 is not None:
            return particle(self.verts2 + d, self.faces2, self.op)
        return particle(self.verts + d, self.faces, self.op)


def curved(p, key=None):
    """Particle with curved elements (Particles/@particle/curved.m:1-18): new
    nodes from ``p.midpoints(key)`` when ``p`` has none or a key is given
    (flat midpoints by default), else the nodes ``p`` carries."""
    if p.faces2 is None or key is not None:
        p = p.midpoints(key or "flat")
    return particle(p.verts2, p.faces2, dict(p.op, interp="curv"))


def trirod(diameter, height, n=(15, 20, 20), triangles=False, op=None):
    """Particle of ``shapes.trirod`` (Particles/particleshapes/trirod.m): rod
    along z with hemispherical caps; ``triangles`` splits the quadrilaterals."""
    v, f = shapes.trirod(diameter, height, n, triangles)
    return particle(v, f, op)


def tricube(n, length=1.0, e=0.25, triangles=False, op=None):
    """Particle of ``shapes.tricube`` (Particles/particleshapes/tricube.m):
    cube of edge ``length`` rounded by the super-sphere exponent ``e``."""
    v, f = shapes.tricube(n, length, e, triangles)
    return particle(v, f, op)


def trispheresegment(phi, theta, diameter=1.0, triangles=False, op=None):
    """Sphere segment on the grid of azimuths ``phi`` and polar angles
    ``theta`` (radians; Particles/particleshapes/trispheresegment.m): a
    quadrilateral (or, with ``triangles``, triangle) grid oriented with
    outward normals, cleaned as @particle/clean.m does (vertices rounded to 8
    decimals and merged in sorted order, quadrilaterals with a collapsed edge
    made triangles, faces below 1e-10 of the mean area dropped), then
    curved-element nodes at the flat midpoints projected onto the sphere."""
    ph, th = np.meshgrid(np.asarray(phi, float), np.asarray(theta, float))
    r = 0.5 * diameter
    xyz = np.stack([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)], -1)
    nt, nph = ph.shape
    verts = np.stack([xyz[..., k].ravel(order="F") for k in range(3)], 1)
    idx = np.arange(nt * nph).reshape(nph, nt).T          # column-major grid numbering
    a, b, c, d = idx[:-1, :-1], idx[1:, :-1], idx[1:, 1:], idx[:-1, 1:]
    quads = np.stack([q.ravel(order="F") for q in (a, d, c, b)], 1)      # outward for increasing phi, theta
    if triangles:
        faces = np.vstack([np.hstack([quads[:, [0, 1, 2]], -np.ones((quads.shape[0], 1), np.int64)]),
                           np.hstack([quads[:, [0, 2, 3]], -np.ones((quads.shape[0], 1), np.int64)])])
    else:
        faces = quads.astype(np.int64)
    # clean.m: merge vertices (rounded to 8 decimals, sorted rows), collapse faces
    uniq, inv = np.unique(np.round(verts, 8), axis=0, return_inverse=True)
    inv = inv.ravel()
    faces = np.where(faces >= 0, inv[np.maximum(faces, 0)], -1)
    out = []
    for row in faces:
        corners = row[row >= 0]
        _, first = np.unique(corners, return_index=True)
        keep = corners[np.sort(first)]
        if keep.size >= 3:
            out.append(np.concatenate([keep, -np.ones(4 - keep.size, np.int64)]))
    faces = np.asarray(out, np.int64)
    area = _norm_flat(uniq, faces)[4]
    faces = faces[area > 1e-10 * area.mean()]
    used = np.unique(faces[faces >= 0])
    remap = -np.ones(uniq.shape[0] + 1, np.int64)
    remap[used] = np.arange(used.size)
    faces = np.where(faces >= 0, remap[np.maximum(faces, 0)], -1)
    v2, f2 = shapes.midpoints_flat(uniq[used], faces)
    v2 = r * v2 / np.sqrt(np.sum(v2 * v2, 1))[:, None]
    return particle(v2, f2, op)


def trisphere(n, diameter=1.0, op=None):
    """Sphere triangulated from the stored point set closest to ``n`` points;
    with ``op['interp'] = 'curv'`` the curved elements of trisphere.m:54-61
    (edge midpoints on the sphere)."""
    if (op or {}).get("interp", "flat") == "curv":
        v2, f2 = shapes.trisphere_curved(n, diameter)
        return particle(v2, f2, op)
    v, f = shapes.trisphere(n, diameter)
    return particle(v, f, op)


class comparticle:
    """Compound of particles with dielectric environment.

    ``comparticle(eps, [p1, p2, ...], inout, closed..., op)``: ``eps`` is the
    list of dielectric functions, ``inout[i] = [inside, outside]`` (1-based
    indices into eps), ``closed`` are the (1-based) particles that are closed
    surfaces by themselves (comparticle.m; closedparticle.m).
    """

    def __init__(self, eps, p, inout, *closed, op=None):
        if isinstance(p, particle):
            p = [p]
        self.eps = list(eps)
        self.p = list(p)
        self.inout = np.asarray(inout, dtype=np.int32).reshape(-1, 2)
        if self.inout.shape[0] != len(self.p):
            raise ValueError("inout needs one row per particle")
        if self.inout.min() < 1 or self.inout.max() > len(self.eps):
            raise ValueError("inout refers to an undefined medium")
        flags = np.zeros(len(self.p), dtype=np.int32)
        for c in closed:
            for i in np.atleast_1d(c):
                flags[int(i) - 1] = 1
        self.closed = flags
        self.op = op or {}
        offs = np.cumsum([0] + [q.n for q in self.p])
        self.offsets = offs
        verts, faces = [], []
        voff = 0
        for q in self.p:
            verts.append(q.verts)
            f = q.faces.copy()
            f[f >= 0] += voff
            faces.append(f)
            voff += q.verts.shape[0]
        self.verts = np.ascontiguousarray(np.vstack(verts))
        self.faces = np.ascontiguousarray(np.vstack(faces))
        # a compound with a curved particle is curved as a whole; flat members
        # enter with flat midpoints, which reproduce their flat elements
        self.curved = any(q.curved for q in self.p)
        self.verts2 = self.faces2 = None
        if self.curved:
            v2s, f2s, voff = [], [], 0
            for q in self.p:
                if q.curved:
                    v2, f2 = q.verts2, q.faces2
                else:
                    v2, f2 = shapes.midpoints_flat(q.verts, q.faces)
                f2 = f2.copy()
                f2[f2 >= 0] += voff
                v2s.append(v2)
                f2s.append(f2)
                voff += v2.shape[0]
            self.verts2 = np.ascontiguousarray(np.vstack(v2s))
            self.faces2 = np.ascontiguousarray(np.vstack(f2s))
        self.pos = np.vstack([q.pos for q in self.p])
        self.nvec = np.vstack([q.nvec for q in self.p])
        self.area = np.concatenate([q.area for q in self.p])
        self.quad = self.p[0].quad

    @property
    def n(self):
        return int(self.offsets[-1])

    nfaces = n

    @property
    def np(self):
        return len(self.p)

    def index(self, i):
        """0-based face indices of particle i (0-based)."""
        return np.arange(self.offsets[i], self.offsets[i + 1])

    def eps_media(self, enei):
        """[len(enei), nmed] complex dielectric functions of all media."""
        enei = np.atleast_1d(np.asarray(enei, dtype=np.float64))
        return np.stack([np.broadcast_to(e(enei)[0], enei.shape) for e in self.eps], 1).astype(np.complex128)
