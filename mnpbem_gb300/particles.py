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


class particle:
    """Flat-faced discretised surface: ``verts [nv, 3]``, ``faces [n, 4]``
    (-1 in the 4th column for triangles; a ``[n, 3]`` array is accepted)."""

    def __init__(self, verts, faces, op=None):
        verts = np.ascontiguousarray(verts, dtype=np.float64)
        faces = np.asarray(faces)
        if faces.ndim != 2 or faces.shape[1] not in (3, 4):
            raise ValueError("faces must be [n, 3] or [n, 4]")
        if faces.shape[1] == 3:
            faces = np.hstack([faces, -np.ones((faces.shape[0], 1), dtype=np.int64)])
        if np.issubdtype(faces.dtype, np.floating):
            faces = np.where(np.isnan(faces), -1, faces)
        self.verts = verts
        self.faces = np.ascontiguousarray(faces, dtype=np.int64)
        op = op or {}
        self.interp = op.get("interp", "flat")
        if self.interp != "flat":
            raise NotImplementedError("only interp='flat' boundaries are implemented")
        self.quad = quadface(op.get("npol", (7, 5)))
        self.pos, self.nvec, self.tvec2, self.tvec1, self.area = _norm_flat(self.verts, self.faces)

    @property
    def n(self):
        return self.faces.shape[0]

    nfaces = n

    def shift(self, vec):
        return particle(self.verts + np.asarray(vec, dtype=np.float64)[None, :], self.faces,
                        {"npol": self.quad.npol})


def trisphere(n, diameter=1.0, op=None):
    """Sphere triangulated from the stored point set closest to ``n`` points."""
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
