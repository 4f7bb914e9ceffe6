"""FP64 NumPy restatement of the MNPBEM retarded BEM path (oracle; test-only).

Conventions follow the reference: faces are ``[n, 4]`` 0-based vertex indices
with ``-1`` in the 4th column for triangles (the reference uses NaN), arrays of
surface vectors are ``[n, 3, npol]``, matrices are ``[n1, n2]`` with rows the
observation faces and columns the source faces.  Linear indices into matrices
are column-major like MATLAB's (``i + j * n1``), so the ordering of near-field
pairs is the reference's ordering.
"""
import math

import numpy as np
import scipy.special

EPS = np.finfo(float).eps
EV2NM = 1.0 / 8.0655477e-4          # Misc/units.m:2


# --------------------------------------------------------------------------
# materials  (Material/@epsconst/subsref.m:15-17, Material/epsfun.m:41-58)
# --------------------------------------------------------------------------
class EpsConst:
    def __init__(self, eps):
        self.eps = complex(eps)

    def __call__(self, enei):
        enei = np.asarray(enei, dtype=float)
        eps = np.full(enei.shape, self.eps, dtype=complex)
        return eps, 2 * np.pi / enei * np.sqrt(eps)


class EpsFun:
    """``epsfun(fun, key)``: user function of wavelength (nm) or energy (eV)."""

    def __init__(self, fun, key="nm"):
        self.fun, self.key = fun, key

    def __call__(self, enei):
        enei = np.asarray(enei, dtype=float)
        arg = enei if self.key == "nm" else EV2NM / enei
        eps = np.asarray(self.fun(arg), dtype=complex)
        return eps, 2 * np.pi / enei * np.sqrt(eps)


def spline_not_a_knot(x, y):
    """Cubic interpolating spline with not-a-knot ends, as MATLAB's
    ``spline(x, y)`` for four or more distinct sites (used by
    Material/@epstable/epstable.m:38-39; evaluated like ``ppval``).
    Restated from the textbook second-derivative form: continuity of the
    first derivative at the interior sites, and continuity of the third
    derivative at the second and the last-but-one site.  Returns a function
    of the evaluation points."""
    order = np.argsort(x)
    x, y = np.asarray(x, float)[order], np.asarray(y, float)[order]
    n = x.size
    h = np.diff(x)
    A = np.zeros((n, n))
    r = np.zeros(n)
    A[0, 0], A[0, 1], A[0, 2] = h[1], -(h[0] + h[1]), h[0]
    A[n - 1, n - 3], A[n - 1, n - 2], A[n - 1, n - 1] = h[n - 2], -(h[n - 3] + h[n - 2]), h[n - 3]
    for i in range(1, n - 1):
        A[i, i - 1], A[i, i], A[i, i + 1] = h[i - 1], 2 * (h[i - 1] + h[i]), h[i]
        r[i] = 6 * ((y[i + 1] - y[i]) / h[i] - (y[i] - y[i - 1]) / h[i - 1])
    M = np.linalg.solve(A, r)

    def ev(t):
        t = np.asarray(t, float)
        i = np.clip(np.searchsorted(x, t, side="right") - 1, 0, n - 2)
        hi, a, b = h[i], x[i + 1] - t, t - x[i]
        return (M[i] * a ** 3 + M[i + 1] * b ** 3) / (6 * hi) + (y[i] / hi - M[i] * hi / 6) * a \
            + (y[i + 1] / hi - M[i + 1] * hi / 6) * b
    return ev


class EpsTable:
    """``epstable(finp)`` (Material/@epstable/epstable.m:34-40, subsref.m:17-26)
    from rows ``ene n k`` (eV): splines of n and k over ``EV2NM / ene``,
    eps = (n + ik)^2; wavelengths outside the table are an error."""

    def __init__(self, table):
        table = np.asarray(table, float)
        self.enei = EV2NM / table[:, 0]
        self.n = spline_not_a_knot(self.enei, table[:, 1])
        self.k = spline_not_a_knot(self.enei, table[:, 2])

    def __call__(self, enei):
        enei = np.asarray(enei, dtype=float)
        if enei.min() < self.enei.min() or enei.max() > self.enei.max():
            raise ValueError("wavelength outside the table")
        eps = (self.n(enei) + 1j * self.k(enei)) ** 2
        return eps, 2 * np.pi / enei * np.sqrt(eps)


def drude_eps(eps_inf=10.0, wp=9.065, gamma=0.0708):
    """Drude metal as ``epsfun(@(w) eps_inf - wp^2./(w.*(w+1i*gamma)), 'eV')``."""
    return EpsFun(lambda w: eps_inf - wp ** 2 / (w * (w + 1j * gamma)), "eV")


# --------------------------------------------------------------------------
# quadrature rules  (Misc/integration/lglnodes.m:13-32,
#                    Misc/integration/@quadface/private/init.m:5-80)
# --------------------------------------------------------------------------
def lglnodes(n):
    """Legendre-Gauss-Lobatto nodes/weights, n+1 points (lglnodes.m:13-32)."""
    n1 = n + 1
    x = np.cos(np.pi * np.arange(n1) / n)
    P = np.zeros((n1, n1))
    xold = 2.0 * np.ones_like(x)
    while np.max(np.abs(x - xold)) > EPS:
        xold = x
        P[:, 0] = 1.0
        P[:, 1] = x
        for k in range(2, n1):
            P[:, k] = ((2 * k - 1) * x * P[:, k - 1] - (k - 1) * P[:, k - 2]) / k
        x = xold - (x * P[:, n] - P[:, n - 1]) / (n1 * P[:, n])
    w = 2.0 / (n * n1 * P[:, n] ** 2)
    return x, w


class QuadFace:
    """``quadface`` with ``rule = 18`` (28 points) and ``npol = [7, 5]``.

    ``rule18`` is the (x, y, w) table of the 28-point Lyness-Jespersen rule
    (triangle_unit_set.m:471-505), passed in by the caller.
    """

    def __init__(self, rule18, npol=(7, 5)):
        self.x, self.y, self.w = [np.asarray(a, dtype=float) for a in rule18]
        # polar triangle integration (init.m:27-53)
        x1, w1 = lglnodes(npol[0])
        rho = 0.5 * (x1 + 1 + 1e-6)
        x2, w2 = lglnodes(npol[1])
        phi = (270 + 60 * x2) / 180 * np.pi
        phi0 = 120 / 180 * np.pi
        rho_g, phi_g = np.meshgrid(rho, phi, indexing="ij")
        rho_f, phi_f = rho_g.ravel(order="F"), phi_g.ravel(order="F")
        rad = 1.0 / np.abs(2 * np.sin(phi_f))
        phis = np.stack([phi_f, phi_f + phi0, phi_f + 2 * phi0], axis=1)
        xx = (np.cos(phis) * (rho_f * rad)[:, None]).ravel(order="F")
        yy = (np.sin(phis) * (rho_f * rad)[:, None]).ravel(order="F")
        self.x3 = (1 - np.sqrt(3) * xx - yy) / 3
        self.y3 = (1 + np.sqrt(3) * xx - yy) / 3
        w = np.outer(w1, w2).ravel(order="F")
        w = np.tile(w * rho_f * rad ** 2, 3)
        self.w3 = w / w.sum()
        # polar quadrilateral integration (init.m:57-80)
        x1, w1 = lglnodes(npol[0])
        rho = 0.5 * (x1 + 1 + 1e-6)
        x2, w2 = lglnodes(npol[1])
        phi = (90 + 45 * x2) / 180 * np.pi
        phi0 = np.pi / 2
        rho_g, phi_g = np.meshgrid(rho, phi, indexing="ij")
        rho_f, phi_f = rho_g.ravel(order="F"), phi_g.ravel(order="F")
        rad = 1.0 / np.abs(np.sin(phi_f))
        phis = np.stack([phi_f + i * phi0 for i in range(4)], axis=1)
        self.x4 = (np.cos(phis) * (rho_f * rad)[:, None]).ravel(order="F")
        self.y4 = (np.sin(phis) * (rho_f * rad)[:, None]).ravel(order="F")
        w = np.outer(w1, w2).ravel(order="F")
        w = np.tile(w * rho_f * rad ** 2, 4)
        self.w4 = 4 * w / w.sum()


# --------------------------------------------------------------------------
# particle geometry  (Particles/@particle/private/norm_flat.m:8-62,
#   quad_flat.m:13-56, quadpol_flat.m:15-78, Misc/+misc/bradius.m:11-32)
# --------------------------------------------------------------------------
def _quad_shape(x, y):
    """Bilinear 4-node shape functions and derivatives (Misc/+shape/@quad)."""
    s = 0.25 * np.stack([(1 - x) * (1 - y), (1 + x) * (1 - y), (1 + x) * (1 + y), (1 - x) * (1 + y)], 1)
    sx = 0.25 * np.stack([-(1 - y), (1 - y), (1 + y), -(1 + y)], 1)
    sy = 0.25 * np.stack([-(1 - x), -(1 + x), (1 + x), (1 - x)], 1)
    return s, sx, sy


def _tri6_shape(x, y):
    """6-node triangle shape functions and first derivatives
    (Misc/+shape/@tri/eval.m:16-22, deriv.m:45-56): nodes 1-3 corners,
    4-6 the midpoints of edges 12, 23, 31."""
    x, y = np.asarray(x, float), np.asarray(y, float)
    z = 1 - x - y
    s = np.stack([x * (2 * x - 1), y * (2 * y - 1), z * (2 * z - 1), 4 * x * y, 4 * y * z, 4 * z * x], 1)
    sx = np.stack([4 * x - 1, 0 * y, 1 - 4 * z, 4 * y, -4 * y, 4 * (z - x)], 1)
    sy = np.stack([0 * x, 4 * y - 1, 1 - 4 * z, 4 * x, 4 * (z - y), -4 * x], 1)
    return s, sx, sy


def _quad9_shape(x, y):
    """9-node quadrilateral shape functions and first derivatives
    (Misc/+shape/@quad/eval.m:19-27, deriv.m:47-66): corners 1-4, edge
    midpoints 5-8 (edges 12, 23, 34, 41), centre 9."""
    x, y = np.asarray(x, float), np.asarray(y, float)

    def asm(a, b):
        return np.stack([a[0] * b[0], a[2] * b[0], a[2] * b[2], a[0] * b[2], a[1] * b[0], a[2] * b[1],
                         a[1] * b[2], a[0] * b[1], a[1] * b[1]], 1)
    sx0 = [0.5 * x * (x - 1), 1 - x ** 2, 0.5 * x * (1 + x)]
    sy0 = [0.5 * y * (y - 1), 1 - y ** 2, 0.5 * y * (1 + y)]
    sx1 = [x - 0.5, -2 * x, x + 0.5]
    sy1 = [y - 0.5, -2 * y, y + 0.5]
    return asm(sx0, sy0), asm(sx1, sy0), asm(sx0, sy1)


def midpoints_flat(verts, faces):
    """Edge midpoints and quadrilateral centroids for curved interpolation
    (Particles/@particle/midpoints.m:16-45, key 'flat'): returns ``verts2``
    (the corner vertices followed by the new points) and ``faces2 [n, 9]``
    (corners 0-3, -1 for triangles; edge midpoints 4-7; quadrilateral centre 8).
    The numbering of the new points follows this function's own edge order."""
    verts = np.asarray(verts, float)
    faces = np.asarray(faces, np.int64)
    if faces.shape[1] == 3:
        faces = np.hstack([faces, -np.ones((faces.shape[0], 1), np.int64)])
    n, nv = faces.shape[0], verts.shape[0]
    edge_id, new = {}, []
    faces2 = -np.ones((n, 9), np.int64)
    faces2[:, :4] = faces
    for i in range(n):
        k = 3 if faces[i, 3] < 0 else 4
        for e in range(k):
            a, b = int(faces[i, e]), int(faces[i, (e + 1) % k])
            key = (min(a, b), max(a, b))
            if key not in edge_id:
                edge_id[key] = nv + len(new)
                new.append(0.5 * (verts[a] + verts[b]))
            faces2[i, 4 + e] = edge_id[key]
    ind4 = np.nonzero(faces[:, 3] >= 0)[0]
    for i in ind4:
        faces2[i, 8] = nv + len(new)
        new.append(0.25 * verts[faces[i, :4]].sum(0))
    verts2 = np.vstack([verts] + ([np.asarray(new)] if new else []))
    return verts2, faces2


def _norm3(d):
    """sqrt(sum(d.^2)) of a 3-vector, summed in MATLAB's order."""
    return np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])


def vertex_neighbours(tri, nv):
    """Ordered neighbour fan of every vertex
    (Particles/@particle/private/vertex_neighbours.m:1-76), 0-based.

    Each face (a, b, c) appends the pairs (b, c), (c, a), (a, b) to the lists
    of a, b, c (:10-17).  The fan starts at the first pair whose first vertex
    is no pair's second vertex (an open fan), else at the first pair
    (:25-37); it is then continued by appending the second vertex of every
    pair whose first vertex is the current last one (:42-50), with the
    fallbacks of :51-60 and :63-69 for irregular vertices."""
    pairs = [[] for _ in range(nv)]
    for a, b, c in tri:
        a, b, c = int(a), int(b), int(c)
        pairs[a] += [b, c]
        pairs[b] += [c, a]
        pairs[c] += [a, b]
    out = []
    for i in range(nv):
        pf = pairs[i]
        m = len(pf)
        if m == 0:
            out.append([])
            continue
        start, found = 0, False
        for i1 in range(0, m, 2):
            found = False
            for i2 in range(1, m, 2):
                if pf[i1] == pf[i2]:
                    found = True
                    break
            if not found:
                start = i1
                break
        pn = [pf[start], pf[start + 1]]
        for _ in range(2 + int(found), m // 2 + 1):
            hit = False
            for idx in range(0, m, 2):
                if pf[idx] == pn[-1] and pf[idx + 1] not in pn:
                    hit = True
                    pn.append(pf[idx + 1])
            if not hit:
                for idx in range(0, m, 2):
                    if pf[idx] not in pn:
                        pn.append(pf[idx])
                        if pf[idx + 1] not in pn:
                            pn.append(pf[idx + 1])
        if len(pn) < m:
            for x in pf:
                if x not in pn:
                    pn.append(x)
        out.append(pn)
    return out


def edge_tangents(verts, ne):
    """Tangent and velocity of every directed edge i -> ne[i][k]
    (Particles/@particle/private/edge_tangents.m:1-72): the opposite neighbour
    is ne[i][k + L/2] (the mean of the two nearest for odd L, :14-28); the
    tangent bisects the 2-D triangle (P, neighbour, opposite) and is mapped
    back to 3-D (:30-65); the velocity is (|P - Pn| + |Pn - Pnop| / 2) / 2.

    The Heron product s(s-a)(s-b)(s-c) is clamped at zero: MATLAB's sqrt
    would return a complex number for a negative product (possible only for
    collinear points whose rounding beats the 1e-14 guards added to every
    length)."""
    rows, tang, vel = [], [], []
    for i in range(len(ne)):
        nb = ne[i]
        L = len(nb)
        P = verts[i]
        for k in range(L):
            if L % 2 == 0:
                pnop = verts[nb[(k + L // 2) % L]]
            else:
                o1, o2 = (k + (L - 1) // 2) % L, (k + (L + 1) // 2) % L
                pnop = (verts[nb[o1]] + verts[nb[o2]]) / 2
            pn = verts[nb[k]]
            ec = _norm3(pn - P) + 1e-14
            eb = _norm3(pnop - P) + 1e-14
            ea = _norm3(pn - pnop) + 1e-14
            s = (ea + eb + ec) / 2
            h = (2 / ea) * np.sqrt(max(s * (s - ea) * (s - eb) * (s - ec), 0.0)) + 1e-14
            x = (ea * ea - eb * eb + ec * ec) / (2 * ea)
            npv = np.array([-h, x])
            npv = npv / (np.sqrt(npv[0] * npv[0] + npv[1] * npv[1]) + 1e-14)
            nsv = np.array([h, ea - x])
            nsv = nsv / (np.sqrt(nsv[0] * nsv[0] + nsv[1] * nsv[1]) + 1e-14)
            nbv = npv + nsv
            tb = (nbv[1], -nbv[0])
            pm = (pn * x + pnop * (ea - x)) / ea
            x3 = (pn - pnop) / ea
            y3 = (P - pm) / h
            t3 = x3 * tb[0] + y3 * tb[1]
            t3 = t3 / (_norm3(t3) + 1e-14)
            rows.append((i, nb[k]))
            tang.append(t3)
            vel.append(0.5 * (ec + 0.5 * ea))
    return rows, np.asarray(tang).reshape(-1, 3), np.asarray(vel)


def make_halfway_vertices(vel, tang, rows, verts, ne):
    """Cubic Bezier midpoint of every edge from the end tangents and
    velocities (Particles/@particle/private/make_halfway_vertices.m:1-69):
    P1 = P0 + T01 v01 / 3, P2 = P3 + T10 v10 / 3, point at t = 1/2.  New
    points are numbered in the order (i ascending, fan order of i) of the
    edge's first visit.  Returns ``verts2`` and the map {(i, j): index}."""
    pos = {r: k for k, r in enumerate(rows)}
    new, idx = [], {}
    nv = verts.shape[0]
    for i in range(len(ne)):
        for j in ne[i]:
            if (i, j) in idx:
                continue
            a = pos[(i, j)]
            b = pos[(j, i)]
            p0, p3 = verts[i], verts[j]
            p1 = p0 + tang[a] * vel[a] / 3
            p2 = p3 + tang[b] * vel[b] / 3
            c = 3 * (p1 - p0)
            bb = 3 * (p2 - p1) - c
            aa = p3 - p0 - c - bb
            new.append(aa * 0.125 + bb * 0.250 + c * 0.500 + p0)
            idx[(i, j)] = idx[(j, i)] = nv + len(new) - 1
    verts2 = np.vstack([verts] + ([np.asarray(new)] if new else []))
    return verts2, idx


def midpoints_curv(verts, faces):
    """Curved-element nodes from the approximate curvature
    (Particles/@particle/midpoints.m:47-49 -> private/refine.m:1-52): the
    faces are split into triangles (totriangles_flat.m), every edge gets the
    Bezier midpoint of make_halfway_vertices.m, and faces2 takes for a
    triangle the midpoints of edges 12, 23, 31 (columns 4-6) and for a
    quadrilateral those of 12, 23 (triangle 123) and 34, 41, 13 (triangle
    341) in columns 4-8, so that the quadrilateral's centre node is the
    midpoint of its diagonal 3-1 (refine.m:35-48).  0-based, -1 where
    unused."""
    verts = np.asarray(verts, float)
    faces = np.asarray(faces, np.int64)
    if faces.shape[1] == 3:
        faces = np.hstack([faces, -np.ones((faces.shape[0], 1), np.int64)])
    n = faces.shape[0]
    i4 = np.nonzero(faces[:, 3] >= 0)[0]
    tri = np.vstack([faces[:, :3], faces[i4][:, [2, 3, 0]]])
    ne = vertex_neighbours(tri, verts.shape[0])
    rows, tang, vel = edge_tangents(verts, ne)
    verts2, idx = make_halfway_vertices(vel, tang, rows, verts, ne)
    mids = np.array([[idx[(a, b)], idx[(b, c)], idx[(c, a)]] for a, b, c in tri.tolist()],
                    np.int64).reshape(-1, 3)
    faces2 = -np.ones((n, 9), np.int64)
    faces2[:, :4] = faces
    i3 = np.nonzero(faces[:, 3] < 0)[0]
    faces2[i3, 4:7] = mids[i3]
    if i4.size:
        ib = n + np.arange(i4.size)
        faces2[i4, 4:6] = mids[i4][:, :2]
        faces2[i4, 6:9] = mids[ib]
    return verts2, faces2


class Particle:
    """Particle boundary: ``pos``, ``area``, ``tvec1``, ``tvec2``, ``nvec``.

    Flat faces (``interp = 'flat'``, norm_flat.m) by default; with
    ``verts2, faces2`` (9-node connectivity, midpoints.m) and
    ``interp = 'curv'`` the elements are the quadratic (6-node triangle,
    9-node quadrilateral) interpolations of norm_curv.m, quad_curv.m and
    quadpol_curv.m.  ``verts`` / ``faces`` hold the corner vertices (the
    flat particle and bradius.m use them).
    """

    def __init__(self, verts, faces, quad, verts2=None, faces2=None, interp="flat"):
        self.verts = np.asarray(verts, dtype=float)
        faces = np.asarray(faces, dtype=np.int64)
        if faces.shape[1] == 3:
            faces = np.hstack([faces, -np.ones((faces.shape[0], 1), np.int64)])
        self.faces = faces
        self.quad = quad
        self.n = faces.shape[0]
        self.interp = interp
        self.verts2 = None if verts2 is None else np.asarray(verts2, float)
        self.faces2 = None if faces2 is None else np.asarray(faces2, np.int64)
        if interp == "curv":
            if self.verts2 is None:
                raise ValueError("interp='curv' needs verts2 / faces2")
            self._norm_curv()
        else:
            self._norm_flat()

    @classmethod
    def curved(cls, verts2, faces2, quad):
        """Curved particle from 9-node connectivity into ``verts2``."""
        faces2 = np.asarray(faces2, np.int64)
        return cls(verts2, faces2[:, :4], quad, verts2, faces2, "curv")

    # index34.m
    def index34(self, ind=None):
        f = self.faces if ind is None else self.faces[ind]
        return np.nonzero(f[:, 3] < 0)[0], np.nonzero(f[:, 3] >= 0)[0]

    # totriangles_flat.m
    def totriangles(self, ind=None):
        ind = np.arange(self.n) if ind is None else np.asarray(ind)
        _, i4 = self.index34(ind)
        faces = self.faces[ind][:, [0, 1, 2]]
        if i4.size:
            faces = np.vstack([faces, self.faces[ind[i4]][:, [2, 3, 0]]])
            i4 = np.stack([i4, ind.size + np.arange(i4.size)], 1)
        else:
            i4 = np.zeros((0, 2), np.int64)
        return faces, i4

    def _norm_flat(self):
        v, f, n = self.verts, self.faces, self.n
        i3, i4 = self.index34()
        pos = np.zeros((n, 3))
        pos[i3] = (v[f[i3, 0]] + v[f[i3, 1]] + v[f[i3, 2]]) / 3
        if i4.size:
            pos[i4] = (v[f[i4, 0]] + v[f[i4, 1]] + v[f[i4, 2]] + v[f[i4, 3]]) / 4
        faces, ind4 = self.totriangles()
        v1, v2, v3 = v[faces[:, 0]], v[faces[:, 1]], v[faces[:, 2]]
        vec1, vec2 = v1 - v2, v3 - v2
        nvec = np.cross(vec1, vec2)
        area = 0.5 * np.sqrt(np.sum(nvec * nvec, 1))
        vec1 = vec1 / np.sqrt(np.sum(vec1 * vec1, 1))[:, None]
        nvec = nvec / np.sqrt(np.sum(nvec * nvec, 1))[:, None]
        vec2 = np.cross(nvec, vec1)
        if ind4.shape[0] == 0:
            self.area = area
        else:
            self.area = area[:n].copy()
            np.add.at(self.area, ind4[:, 0], area[ind4[:, 1]])
            big2 = area[ind4[:, 1]] > area[ind4[:, 0]]
            src, dst = ind4[big2, 1], ind4[big2, 0]
            vec1[dst], vec2[dst], nvec[dst] = vec1[src], vec2[src], nvec[src]
        self.pos = pos
        self.tvec1, self.tvec2, self.nvec = vec1[:n], vec2[:n], nvec[:n]

    # totriangles_curv.m:14-31 (6-node triangles; quads split into (1,2,3,5,6,9), (3,4,1,7,8,9))
    def totriangles_curv(self, ind=None):
        ind = np.arange(self.n) if ind is None else np.asarray(ind)
        _, i4 = self.index34(ind)
        f2 = self.faces2[ind]
        faces = f2[:, [0, 1, 2, 4, 5, 6]].copy()
        if i4.size:
            faces[i4] = f2[i4][:, [0, 1, 2, 4, 5, 8]]
            faces = np.vstack([faces, f2[i4][:, [2, 3, 0, 6, 7, 8]]])
            i4 = np.stack([i4, ind.size + np.arange(i4.size)], 1)
        else:
            i4 = np.zeros((0, 2), np.int64)
        return faces, i4

    def _norm_curv(self):
        """Centroids, areas and bases of curved elements (norm_curv.m:8-62)."""
        n, v2 = self.n, self.verts2
        _, w, row = self.quad_points(np.arange(n))
        self.area = np.bincount(row, weights=w, minlength=n)
        i3, i4 = self.index34()
        faces, _ = self.totriangles_curv()
        pos, vec1, vec2 = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        if i3.size:
            tri = np.array([-1, -1, -1, 4, 4, 4]) / 9
            trix = np.array([1, 0, -1, 4, -4, 0]) / 3
            triy = np.array([0, 1, -1, 4, 0, -4]) / 3
            vv = v2[faces[i3]]
            pos[i3] = np.einsum("k,fkc->fc", tri, vv)
            vec1[i3] = np.einsum("k,fkc->fc", triy, vv)
            vec2[i3] = np.einsum("k,fkc->fc", trix, vv)
        if i4.size:
            pos[i4] = v2[faces[i4, 5]]
            trix = np.array([1, 0, -1, 0, 0, 0], float)
            triy = np.array([0, -1, -1, 2, 2, -2], float)
            vv = v2[faces[i4]]
            vec1[i4] = np.einsum("k,fkc->fc", triy, vv)
            vec2[i4] = np.einsum("k,fkc->fc", trix, vv)
        nrm = lambda x: x / np.sqrt(np.sum(x * x, 1))[:, None]
        nvec = nrm(np.cross(vec1, vec2))
        vec1 = nrm(vec1)
        self.pos, self.tvec1, self.tvec2, self.nvec = pos, vec1, np.cross(nvec, vec1), nvec

    def quad_points(self, ind):
        """Boundary-element points/weights for faces ``ind`` (quad_flat.m:13-56,
        quad_curv.m:13-59 for curved elements).

        Returns ``pos [m, 3]``, ``w [m]`` and ``row [m]`` (index into ``ind``).
        """
        ind = np.asarray(ind)
        if self.interp == "curv":
            faces, ind4 = self.totriangles_curv(ind)
            ind3 = np.arange(ind.size)
            if ind4.shape[0]:
                ind3 = np.concatenate([ind3, ind4[:, 0]])
            q = self.quad
            s, sx, sy = _tri6_shape(q.x, q.y)
            vv = self.verts2[faces]                     # [t, 6, 3]
            pos = np.einsum("pk,tkc->tpc", s, vv).reshape(-1, 3)
            px = np.einsum("pk,tkc->tpc", sx, vv)
            py = np.einsum("pk,tkc->tpc", sy, vv)
            nv = np.cross(px, py)
            w = (0.5 * q.w[None, :] * np.sqrt(np.sum(nv * nv, 2))).ravel()
            row = np.repeat(ind3, q.w.size)
            return pos, w, row
        faces, ind4 = self.totriangles(ind)
        ind3 = np.arange(ind.size)
        if ind4.shape[0]:
            ind3 = np.concatenate([ind3, ind4[:, 0]])
        v = self.verts
        nv = np.cross(v[faces[:, 1]] - v[faces[:, 0]], v[faces[:, 2]] - v[faces[:, 0]])
        area = 0.5 * np.sqrt(np.sum(nv * nv, 1))
        q = self.quad
        tri = np.stack([q.x, q.y, 1 - q.x - q.y], 1)
        pos = np.einsum("pk,tkc->tpc", tri, v[faces[:, :3]]).reshape(-1, 3)
        w = (q.w[None, :] * area[:, None]).ravel()
        row = np.repeat(ind3, q.w.size)
        return pos, w, row

    def quadpol_points(self, ind):
        """Polar points/weights around centroids (quadpol_flat.m:15-78,
        quadpol_curv.m:15-88 for curved elements)."""
        ind = np.asarray(ind)
        i3, i4 = self.index34(ind)
        q, v = self.quad, self.verts
        pos, w, row = [], [], []
        if self.interp == "curv":
            f2, v2 = self.faces2, self.verts2
            if i3.size:
                s, sx, sy = _tri6_shape(q.x3, q.y3)
                for i in i3:
                    vv = v2[f2[ind[i], [0, 1, 2, 4, 5, 6]]]
                    nv = np.cross(sx @ vv, sy @ vv)
                    pos.append(s @ vv)
                    w.append(0.5 * q.w3 * np.sqrt(np.sum(nv * nv, 1)))
                    row.append(np.full(q.w3.size, i))
            if i4.size:
                s, sx, sy = _quad9_shape(q.x4, q.y4)
                for i in i4:
                    vv = v2[f2[ind[i], :9]]
                    nv = np.cross(sx @ vv, sy @ vv)
                    pos.append(s @ vv)
                    w.append(q.w4 * np.sqrt(np.sum(nv * nv, 1)))
                    row.append(np.full(q.w4.size, i))
            return np.vstack(pos), np.concatenate(w), np.concatenate(row)
        if i3.size:
            tri = np.stack([q.x3, q.y3, 1 - q.x3 - q.y3], 1)
            for i in i3:
                pos.append(tri @ v[self.faces[ind[i], :3]])
                w.append(q.w3 * self.area[ind[i]])
                row.append(np.full(q.w3.size, i))
        if i4.size:
            s, sx, sy = _quad_shape(q.x4, q.y4)
            for i in i4:
                vv = v[self.faces[ind[i], :4]]
                px, py = sx @ vv, sy @ vv
                nv = np.cross(px, py)
                pos.append(s @ vv)
                w.append(q.w4 * np.sqrt(np.sum(nv * nv, 1)))
                row.append(np.full(q.w4.size, i))
        return np.vstack(pos), np.concatenate(w), np.concatenate(row)

    def bradius(self):
        """Max centroid-to-vertex distance per face (bradius.m:11-32)."""
        r = np.zeros(self.n)
        i3, i4 = self.index34()
        for idx, nvert in ((i3, 3), (i4, 4)):
            for k in range(nvert):
                d = np.sqrt(np.sum((self.pos[idx] - self.verts[self.faces[idx, k]]) ** 2, 1))
                r[idx] = np.maximum(r[idx], d)
        return r


# --------------------------------------------------------------------------
# composite particle  (Particles/@comparticle, Particles/@compound/connect.m)
# --------------------------------------------------------------------------
class ComParticle:
    """Concatenation of particles with their media (``inout``) and closed flags.

    ``inout[i] = (medium inside, medium outside)`` (1-based medium indices into
    ``eps``), ``closed[i]`` is True when particle i is a closed surface by
    itself (the ``comparticle(..., 1, 2, ...)`` case of the demos).
    """

    def __init__(self, eps, parts, inout, closed):
        self.eps = eps
        self.parts = parts
        self.inout = np.asarray(inout, dtype=np.int64).reshape(-1, 2)
        self.closed = list(closed)
        offs = np.cumsum([0] + [p.n for p in parts])
        self.offsets = offs
        self.n = int(offs[-1])
        curved = any(p.interp == "curv" for p in parts)
        verts, faces = [], []
        voff = 0
        for p in parts:
            if curved:
                # a compound is curved as a whole; flat members get flat midpoints
                # (which reproduce their flat elements exactly)
                if p.interp == "curv":
                    v2, f2 = p.verts2, p.faces2
                else:
                    v2, f2 = midpoints_flat(p.verts, p.faces)
                verts.append(v2)
                f = f2.copy()
                f[f >= 0] += voff
                faces.append(f)
                voff += v2.shape[0]
            else:
                verts.append(p.verts)
                f = p.faces.copy()
                f[f >= 0] += voff
                faces.append(f)
                voff += p.verts.shape[0]
        if curved:
            self.pc = Particle.curved(np.vstack(verts), np.vstack(faces), parts[0].quad)
        else:
            self.pc = Particle(np.vstack(verts), np.vstack(faces), parts[0].quad)
        self.pos, self.area, self.nvec = self.pc.pos, self.pc.area, self.pc.nvec
        self.tvec1, self.tvec2 = self.pc.tvec1, self.pc.tvec2

    def index(self, i):
        return np.arange(self.offsets[i], self.offsets[i + 1])

    def bradius(self):
        return self.pc.bradius()

    def quad_points(self, ind):
        return self.pc.quad_points(ind)

    def quadpol_points(self, ind):
        return self.pc.quadpol_points(ind)

    def face_media(self):
        """Per-face inside/outside medium (``expand`` of inout)."""
        return np.repeat(self.inout, [p.n for p in self.parts], axis=0)

    def eps_faces(self, enei, side):
        med = self.face_media()[:, side]
        vals = {m: self.eps[m - 1](enei)[0] for m in np.unique(med)}
        return np.array([vals[m] for m in med], dtype=complex)


def connect(inout):
    """Connectivity ``con[a][b][i1, i2]`` (Particles/@compound/connect.m:40-57)."""
    con = [[None, None], [None, None]]
    for a in range(2):
        for b in range(2):
            c1 = inout[:, a][:, None]
            c2 = inout[:, b][None, :]
            con[a][b] = np.where(c1 == c2, c1 + 0 * c2, 0)
    return con


# --------------------------------------------------------------------------
# refinement pattern  (Greenfun/+green/refinematrix.m:28-68,
#                      Misc/+misc/pdist2.m:13-17)
# --------------------------------------------------------------------------
def refinematrix(p, rel_cutoff=3.0, abs_cutoff=0.0):
    """Dense int8 pattern: 2 = self element, 1 = near pair, 0 = far."""
    pos = p.pos
    rad = p.bradius()
    sq = np.sum(pos * pos, 1)
    d2 = sq[:, None] + sq[None, :] - 2 * pos @ pos.T
    d2[d2 < 1e-10] = 0
    d = np.sqrt(d2)
    dd = d - rad[None, :]
    idist = dd / rad[:, None]
    ir = np.zeros(d.shape, np.int8)
    ir[d == 0] = 2
    ir[((dd < abs_cutoff) | (idist < rel_cutoff)) & (d != 0)] = 1
    return ir


# --------------------------------------------------------------------------
# greenret: refined Taylor coefficients  (Greenfun/@greenret/private/init.m)
# --------------------------------------------------------------------------
class GreenRet:
    """Retarded Green function with 'cart' derivative and near-field refinement.

    ``ind`` are the column-major linear indices of refined elements
    (init.m:24), ``g [nref, order+1]`` and ``f [nref, 3, order+1]`` their Taylor
    coefficients in powers of (i k).
    """

    def __init__(self, p, order=5, rel_cutoff=3.0, abs_cutoff=0.0, pattern=None):
        self.p = p
        self.order = order
        # pattern: a fixed refinement pattern (finite-difference checks keep
        # it constant while the vertices move)
        ir = refinematrix(p, rel_cutoff, abs_cutoff) if pattern is None else pattern
        self.pattern = ir
        n = p.n
        rows, cols = np.nonzero(ir.T)          # column-major order of find()
        rows, cols = cols, rows
        self.ind = rows + cols * n
        self.rows, self.cols = rows, cols
        lookup = {(int(r), int(c)): k for k, (r, c) in enumerate(zip(rows, cols))}
        g = np.zeros((rows.size, order + 1))
        f = np.zeros((rows.size, 3, order + 1))
        pos1 = p.pos
        # ---- diagonal elements (init.m:42-95)
        dface = np.nonzero(np.diag(ir) == 2)[0]
        if dface.size:
            iface = np.array([lookup[(int(i), int(i))] for i in dface])
            pos, w, row = p.quadpol_points(dface)
            vec = pos1[dface[row]] - pos
            r = np.sqrt(np.sum(vec * vec, 1))

            def acc(x, o):
                return np.bincount(row, weights=w * x, minlength=dface.size) / math.factorial(o)

            for o in range(order + 1):
                g[iface, o] = acc(r ** (o - 1), o)
            nv, t1, t2 = p.nvec[dface[row]], p.tvec1[dface[row]], p.tvec2[dface[row]]
            inn = np.sum(vec * nv, 1)
            rr = np.maximum(r, 1e-4 * np.max(r))
            in1 = np.sum(vec * t1, 1)
            in2 = np.sum(vec * t2, 1)
            for o in range(order + 1):
                fn = acc((o - 1) * inn * r ** (o - 3), o)
                f1 = acc((o - 1) * in1 * r ** o / rr ** 3, o)
                f2 = acc((o - 1) * in2 * r ** o / rr ** 3, o)
                f[iface, :, o] = (p.nvec[dface] * fn[:, None] + p.tvec1[dface] * f1[:, None]
                                  + p.tvec2[dface] * f2[:, None])
        # ---- off-diagonal elements (init.m:98-177)
        reface = np.nonzero(np.any(ir == 1, axis=0))[0]
        if reface.size:
            postab, wtab, rowtab = p.quad_points(reface)
            for k2, face in enumerate(reface):
                nb = np.nonzero(ir[:, face] == 1)[0]
                iface = np.array([lookup[(int(i), int(face))] for i in nb])
                sel = rowtab == k2
                pts, w = postab[sel], wtab[sel]
                x = pos1[nb, 0][:, None] - pts[None, :, 0]
                y = pos1[nb, 1][:, None] - pts[None, :, 1]
                z = pos1[nb, 2][:, None] - pts[None, :, 2]
                r = np.sqrt(x ** 2 + y ** 2 + z ** 2)
                vec0 = -(pos1[nb] - p.pos[face])
                r0 = np.sqrt(np.sum(vec0 * vec0, 1))
                dr = r - r0[:, None]
                for o in range(order + 1):
                    g[iface, o] = (dr ** o / r / math.factorial(o)) @ w

                def fun(ff):
                    return np.stack([(x * ff) @ w, (y * ff) @ w, (z * ff) @ w], 1)

                f[iface, :, 0] = -fun(1.0 / r ** 3)
                for o in range(1, order + 1):
                    f[iface, :, o] = fun(-dr ** o / (r ** 3 * math.factorial(o))
                                         + dr ** (o - 1) / (r ** 2 * math.factorial(o - 1)))
        self.g, self.f = g, f

    # greenret/private/eval2.m:19-117, 'cart' branch with only F requested
    def eval_F_indexed(self, rows, cols, k):
        p = self.p
        d = np.maximum(np.sqrt(np.sum((p.pos[rows] - p.pos[cols]) ** 2, 1)), EPS)
        fr = (1j * k) ** np.arange(self.order + 1)
        inn = np.sum(p.nvec[rows] * (p.pos[rows] - p.pos[cols]), 1)
        F = inn * (1j * k - 1 / d) / d ** 2 * p.area[cols]
        lin = rows + cols * p.n
        _, i1, i2 = np.intersect1d(self.ind, lin, return_indices=True)
        if i1.size:
            F[i2] = np.einsum("kc,kco->ko", p.nvec[rows[i2]], self.f[i1]) @ fr
        return F * np.exp(1j * k * d)

    # greenret/diag.m:10-30 ('cart' f: add a 3-vector to the order-0 term)
    def add_diag(self, faces, fvec):
        lin = faces + faces * self.p.n
        pos = np.searchsorted(self.ind, lin)
        assert np.all(self.ind[pos] == lin)
        self.f[pos, :, 0] += fvec

    def eval_full(self, k, rows, cols):
        """G and F for the sub-block rows x cols (eval1.m:18-40, 110-124).

        Returns the block of G and F (before adding +-2*pi on the diagonal)
        and a mask of the d == 0 entries.
        """
        p = self.p
        x = p.pos[rows, 0][:, None] - p.pos[cols, 0][None, :]
        y = p.pos[rows, 1][:, None] - p.pos[cols, 1][None, :]
        z = p.pos[rows, 2][:, None] - p.pos[cols, 2][None, :]
        d = np.maximum(np.sqrt(x ** 2 + y ** 2 + z ** 2), EPS)
        area = p.area[cols][None, :]
        G = (1.0 / d * area).astype(complex)
        ff = (1j * k - 1.0 / d) / d ** 2
        nv = p.nvec[rows]
        F = (ff * x * nv[:, 0:1] + ff * y * nv[:, 1:2] + ff * z * nv[:, 2:3]) * area
        # refined entries that fall inside the block
        n = p.n
        rpos = np.full(n, -1)
        rpos[rows] = np.arange(rows.size)
        cpos = np.full(n, -1)
        cpos[cols] = np.arange(cols.size)
        sel = (rpos[self.rows] >= 0) & (cpos[self.cols] >= 0)
        if np.any(sel):
            fr = (1j * k) ** np.arange(self.order + 1)
            ri, ci = rpos[self.rows[sel]], cpos[self.cols[sel]]
            G[ri, ci] = self.g[sel] @ fr
            F[ri, ci] = np.einsum("kc,kco->ko", p.nvec[self.rows[sel]], self.f[sel]) @ fr
        ph = np.exp(1j * k * d)
        return G * ph, F * ph, d == EPS


def _eval_gp(gr, k, rows, cols):
    """Cartesian derivative Gp [rows, 3, cols] of greenret (eval1.m:86-102,
    'cart'): (ik - 1/d)/d^2 * A_j * (r_i - r_j), refined entries
    f @ (ik)^o, all times exp(ik d); and the d == 0 mask."""
    p = gr.p
    x = p.pos[rows, 0][:, None] - p.pos[cols, 0][None, :]
    y = p.pos[rows, 1][:, None] - p.pos[cols, 1][None, :]
    z = p.pos[rows, 2][:, None] - p.pos[cols, 2][None, :]
    d = np.maximum(np.sqrt(x ** 2 + y ** 2 + z ** 2), EPS)
    ff = (1j * k - 1.0 / d) / d ** 2 * p.area[cols][None, :]
    Gp = np.stack([ff * x, ff * y, ff * z], 1)
    n = p.n
    rpos = np.full(n, -1)
    rpos[rows] = np.arange(rows.size)
    cpos = np.full(n, -1)
    cpos[cols] = np.arange(cols.size)
    sel = (rpos[gr.rows] >= 0) & (cpos[gr.cols] >= 0)
    if np.any(sel):
        fr = (1j * k) ** np.arange(gr.order + 1)
        Gp[rpos[gr.rows[sel]], :, cpos[gr.cols[sel]]] = gr.f[sel] @ fr
    return Gp * np.exp(1j * k * d)[:, None, :], d == EPS


def initclosed(gr, cp):
    """Fuchs-Liu sum rule on the order-0 diagonal (initclosed.m:19-89)."""
    for i in range(len(cp.parts)):
        if not cp.closed[i]:
            continue
        ind = cp.index(i)
        rows = np.repeat(ind, ind.size)           # closed surface = particle i
        cols = np.tile(ind, ind.size)
        F = gr.eval_F_indexed(rows, cols, 0.0).real.reshape(ind.size, ind.size)
        f = np.sum(cp.area[ind][:, None] * F / cp.area[ind][None, :], 0)
        gr.add_diag(ind, cp.nvec[ind] * (-2 * np.pi * 1 - f)[:, None])


class CompGreenRet:
    """compgreenret(p, p, op): greenret + closed-surface diagonal + con."""

    def __init__(self, cp, order=5, rel_cutoff=3.0, abs_cutoff=0.0, pattern=None):
        self.p = cp
        self.g = GreenRet(cp, order, rel_cutoff, abs_cutoff, pattern)
        initclosed(self.g, cp)
        self.con = connect(cp.inout)

    # compgreenret/private/eval1.m:16-51
    def eval(self, a, b, key, enei):
        cp = self.p
        k = np.array([e(enei)[1] for e in cp.eps], dtype=complex)
        con = self.con[a][b]
        out = np.zeros((cp.n, cp.n), dtype=complex)
        any_block = False
        for i1 in range(con.shape[0]):
            for i2 in range(con.shape[1]):
                if con[i1, i2]:
                    any_block = True
                    r, c = cp.index(i1), cp.index(i2)
                    G, F, dz = self.g.eval_full(k[con[i1, i2] - 1], r, c)
                    if key == "G":
                        blk = G
                    elif key == "F":
                        blk = F
                    elif key == "H1":
                        blk = F + 2 * np.pi * dz
                    elif key == "H2":
                        blk = F - 2 * np.pi * dz
                    out[np.ix_(r, c)] = blk
        if not any_block or not np.any(out):
            return 0
        return out


    # compgreenret eval of 'Gp', 'H1p', 'H2p' (eval1.m:144-149; H1p = Gp + 2 pi
    # outer(nvec, d == 0), H2p with -2 pi); 0 where no block connects
    def eval_p(self, a, b, key, enei):
        cp = self.p
        k = np.array([e(enei)[1] for e in cp.eps], dtype=complex)
        con = self.con[a][b]
        out = np.zeros((cp.n, 3, cp.n), dtype=complex)
        any_block = False
        for i1 in range(con.shape[0]):
            for i2 in range(con.shape[1]):
                if con[i1, i2]:
                    any_block = True
                    r, c = cp.index(i1), cp.index(i2)
                    Gp, dz = _eval_gp(self.g, k[con[i1, i2] - 1], r, c)
                    if key != "Gp":
                        sgn = 2 * np.pi if key == "H1p" else -2 * np.pi
                        Gp = Gp + sgn * cp.nvec[r][:, :, None] * dz[:, None, :]
                    out[np.ix_(r, np.arange(3), c)] = Gp
        if not any_block or not np.any(out):
            return 0
        return out


def _cross_p(Gp, h):
    """field.m:41-57: Gp x h for Gp [n, 3, n'] and h [n', 3, npol]."""
    if np.isscalar(Gp):
        return 0
    return np.stack([Gp[:, 1] @ h[:, 2] - Gp[:, 2] @ h[:, 1],
                     Gp[:, 2] @ h[:, 0] - Gp[:, 0] @ h[:, 2],
                     Gp[:, 0] @ h[:, 1] - Gp[:, 1] @ h[:, 0]], 1)


def _mm(a, x):
    """matmul.m for a Green block: 0, [n, n'] @ [n', ...] or Gp [n, 3, n'] @ [n', npol]."""
    if np.isscalar(a):
        return 0
    if a.ndim == 3:
        return np.einsum("icj,jp->icp", a, x)
    return (a @ x.reshape(x.shape[0], -1)).reshape((a.shape[0],) + x.shape[1:])


def surface_field(g, enei, sig1, sig2, h1, h2, inout=2):
    """E and H at the faces, on side ``inout`` (1 inside, 2 outside), from the
    surface charges and currents (Greenfun/@compgreenret/field.m:14-38):
    E = i k0 (G{inout,1} h1 + G{inout,2} h2) - H{inout}p{inout,1} sig1 - ...,
    H = Hp1 x h1 + Hp2 x h2, with H1p for inout = 1 and H2p for inout = 2.
    Returns ``e, h [n, 3, npol]``."""
    k0 = 2 * np.pi / enei
    a, key = inout - 1, ("H1p" if inout == 1 else "H2p")
    G1, G2 = g.eval(a, 0, "G", enei), g.eval(a, 1, "G", enei)
    P1, P2 = g.eval_p(a, 0, key, enei), g.eval_p(a, 1, key, enei)
    e = 1j * k0 * (_mm(G1, h1) + _mm(G2, h2)) - _mm(P1, sig1) - _mm(P2, sig2)
    h = _cross_p(P1, h1) + _cross_p(P2, h2)
    n, P = sig1.shape
    return np.broadcast_to(e, (n, 3, P)).copy(), np.broadcast_to(h, (n, 3, P)).copy()


def surface_potential(g, enei, sig1, sig2, h1, h2, inout=2):
    """Potentials and their surface derivatives at the faces, on side
    ``inout`` (Greenfun/@compgreenret/potential.m:16-48): phi = G1 sig1 +
    G2 sig2, phip = H1 sig1 + H2 sig2, a = G1 h1 + G2 h2, ap = H1 h1 + H2 h2
    with the blocks {inout, 1}, {inout, 2} and H = 'H1' (inout = 1) or 'H2'.
    Returns ``phi, phip [n, npol]`` and ``a, ap [n, 3, npol]``."""
    a, key = inout - 1, ("H1" if inout == 1 else "H2")
    G1, G2 = g.eval(a, 0, "G", enei), g.eval(a, 1, "G", enei)
    H1, H2 = g.eval(a, 0, key, enei), g.eval(a, 1, key, enei)
    n, P = sig1.shape
    phi = _matmul(G1, sig1) + _matmul(G2, sig2)
    phip = _matmul(H1, sig1) + _matmul(H2, sig2)
    av = _matmul(G1, h1) + _matmul(G2, h2)
    ap = _matmul(H1, h1) + _matmul(H2, h2)

    def full(x, shape):
        return np.broadcast_to(x, shape).astype(complex)
    return (full(phi, (n, P)), full(phip, (n, P)), full(av, (n, 3, P)), full(ap, (n, 3, P)))


# --------------------------------------------------------------------------
# bemret  (BEM/@bemret/private/initmat.m:5-74, excitation.m:4-29,
#          mldivide.m:12-49)
# --------------------------------------------------------------------------
def _matmul(a, x):
    """Misc/matmul.m: scalar / matrix times [n, ...] array."""
    if np.isscalar(a) or np.ndim(a) == 0:
        return 0 if a == 0 else a * x
    if np.isscalar(x) and x == 0:
        return 0
    sh = x.shape
    return (a @ x.reshape(sh[0], -1)).reshape(sh)


def _inner(nvec, a):
    """Misc/inner.m: sum_k nvec[i,k] * a[i,k,...] (nvec real)."""
    if np.isscalar(a):
        return 0
    return np.einsum("ik,ik...->i...", nvec, a)


def _outer(nvec, val):
    """Misc/outer.m: a[i,k,...] = nvec[i,k] * val[i,...]."""
    if np.isscalar(val):
        return 0
    return nvec[:, :, None] * val[:, None, ...] if val.ndim == 2 else np.einsum("ik,i->ik", nvec, val)


class BemRet:
    def __init__(self, cp, order=5, rel_cutoff=3.0, abs_cutoff=0.0, pattern=None):
        self.p = cp
        self.g = CompGreenRet(cp, order, rel_cutoff, abs_cutoff, pattern)
        self.enei = None

    def matrices(self, enei):
        """G1, H1, G2, H2 as in initmat.m:27-31."""
        g = self.g

        def sub(a, b):
            if np.isscalar(b) and b == 0:
                return a
            return a - b
        G1 = sub(g.eval(0, 0, "G", enei), g.eval(1, 0, "G", enei))
        G2 = sub(g.eval(1, 1, "G", enei), g.eval(0, 1, "G", enei))
        H1 = sub(g.eval(0, 0, "H1", enei), g.eval(1, 0, "H1", enei))
        H2 = sub(g.eval(1, 1, "H2", enei), g.eval(0, 1, "H2", enei))
        return G1, H1, G2, H2

    def _eps12(self, enei):
        cp = self.p
        e1, e2 = cp.eps_faces(enei, 0), cp.eps_faces(enei, 1)
        if np.unique(e1).size == 1 and np.unique(e2).size == 1:
            return e1[0], e2[0]
        return np.diag(e1), np.diag(e2)

    def initmat(self, enei):
        if self.enei == enei:
            return
        self.enei = enei
        nvec = self.p.nvec
        k = 2 * np.pi / enei
        eps1, eps2 = self._eps12(enei)
        G1, H1, G2, H2 = self.matrices(enei)
        G1i = np.linalg.inv(G1)
        G2i = np.linalg.inv(G2)
        if not np.any(self.g.con[0][1]):
            L1, L2 = eps1, eps2
        else:
            L1 = G1 @ (eps1 * np.eye(G1.shape[0]) if np.ndim(eps1) == 0 else eps1) @ G1i
            L2 = G2 @ (eps2 * np.eye(G2.shape[0]) if np.ndim(eps2) == 0 else eps2) @ G2i
        Sigma1 = H1 @ G1i
        Sigma2 = H2 @ G2i
        Deltai = np.linalg.inv(Sigma1 - Sigma2)
        L = L1 - L2
        nn = nvec @ nvec.T
        if np.ndim(L) == 0:
            Sigma = Sigma1 * L1 - Sigma2 * L2 + k ** 2 * ((L * Deltai) * nn) * L
        else:
            Sigma = Sigma1 @ L1 - Sigma2 @ L2 + k ** 2 * ((L @ Deltai) * nn) @ L
        self.k, self.nvec = k, nvec
        self.eps1, self.eps2 = eps1, eps2
        self.G1i, self.G2i, self.L1, self.L2 = G1i, G2i, L1, L2
        self.Sigma1, self.Deltai = Sigma1, Deltai
        self.Sigmai = np.linalg.inv(Sigma)
        self.G1, self.H1, self.G2, self.H2 = G1, H1, G2, H2

    def excitation(self, exc):
        """excitation.m:4-29 (Garcia de Abajo and Howie Eqs. 10, 11, 15, 18);
        missing potentials are zero."""
        k = 2 * np.pi / exc["enei"]
        eps1 = self.p.eps_faces(exc["enei"], 0)
        eps2 = self.p.eps_faces(exc["enei"], 1)
        nvec = self.nvec
        n = nvec.shape[0]
        P = next(v.shape[-1] for key, v in exc.items() if key != "enei")
        z1, z3 = np.zeros((n, P), complex), np.zeros((n, 3, P), complex)
        get = lambda key, z: exc.get(key, z)
        phi1, phi1p, phi2, phi2p = get("phi1", z1), get("phi1p", z1), get("phi2", z1), get("phi2p", z1)
        a1, a1p, a2, a2p = get("a1", z3), get("a1p", z3), get("a2", z3), get("a2p", z3)
        phi = phi2 - phi1
        a = a2 - a1
        alpha = a2p - a1p - 1j * k * (nvec[:, :, None] * (eps2[:, None] * phi2)[:, None, :]
                                      - nvec[:, :, None] * (eps1[:, None] * phi1)[:, None, :])
        De = (eps2[:, None] * phi2p - eps1[:, None] * phi1p
              - 1j * k * (eps2[:, None] * _inner(nvec, a2) - eps1[:, None] * _inner(nvec, a1)))
        return phi, a, alpha, De

    def solve(self, exc):
        """mldivide.m:12-49 -> dict with sig1, sig2 [n, npol], h1, h2 [n, 3, npol]."""
        self.initmat(exc["enei"])
        phi, a, alpha, De = self.excitation(exc)
        out = self.chain(phi, a, alpha, De)
        out["enei"] = exc["enei"]
        return out

    def chain(self, phi, a, alpha, De):
        """mldivide.m:20-49 on excitation variables (after initmat)."""
        k, nvec = self.k, self.nvec
        G1i, G2i, L1, L2 = self.G1i, self.G2i, self.L1, self.L2
        Sigma1, Deltai, Sigmai = self.Sigma1, self.Deltai, self.Sigmai
        alpha = alpha - _matmul(Sigma1, a) + 1j * k * _outer(nvec, _matmul(L1, phi))
        De = De - _matmul(Sigma1, _matmul(L1, phi)) + 1j * k * _inner(nvec, _matmul(L1, a))
        sig2 = _matmul(Sigmai, De + 1j * k * _inner(nvec, _matmul(L1 - L2, _matmul(Deltai, alpha))))
        h2 = _matmul(Deltai, 1j * k * _outer(nvec, _matmul(L1 - L2, sig2)) + alpha)
        sig1 = _matmul(G1i, sig2 + phi)
        h1 = _matmul(G1i, h2 + a)
        sig2 = _matmul(G2i, sig2)
        h2 = _matmul(G2i, h2)
        return {"sig1": sig1, "sig2": sig2, "h1": h1, "h2": h2}

    def afun(self, sig1, h1, sig2, h2):
        """Full BEM operator (BEM/@bemretiter/private/afun.m:6-35).

        Maps (sig1, h1, sig2, h2) to (phi, a, De, alpha) using the stored
        G1, G2, H1, H2 and per-face eps1, eps2.
        """
        k, nvec = self.k, self.nvec
        e1 = self.p.eps_faces(self.enei, 0)
        e2 = self.p.eps_faces(self.enei, 1)
        G1, G2, H1, H2 = self.G1, self.G2, self.H1, self.H2
        Gs1, Gh1 = _matmul(G1, sig1), _matmul(G1, h1)
        Gs2, Gh2 = _matmul(G2, sig2), _matmul(G2, h2)
        Hs1, Hh1 = _matmul(H1, sig1), _matmul(H1, h1)
        Hs2, Hh2 = _matmul(H2, sig2), _matmul(H2, h2)
        phi = Gs1 - Gs2
        a = Gh1 - Gh2
        alpha = Hh1 - Hh2 - 1j * k * _outer(nvec, e1[:, None] * Gs1 - e2[:, None] * Gs2)
        De = (e1[:, None] * Hs1 - e2[:, None] * Hs2
              - 1j * k * _inner(nvec, e1[:, None, None] * Gh1 - e2[:, None, None] * Gh2))
        return phi, a, De, alpha


# --------------------------------------------------------------------------
# plane wave + spectra  (Simulation/retarded/@planewaveret/potential.m:13-57,
#   extinction.m:12-16, scattering.m:13-19, @spectrumret/farfield.m:15-74,
#   Simulation/retarded/scattering.m:14-31)
# --------------------------------------------------------------------------
class PlaneWaveRet:
    def __init__(self, pol, dir, pinfty, medium=1):
        self.pol = np.atleast_2d(np.asarray(pol, dtype=float))
        self.dir = np.atleast_2d(np.asarray(dir, dtype=float))
        assert not np.any(np.sum(self.pol * self.dir, 1))
        self.medium = medium
        self.pinfty = pinfty        # Particle: unit sphere at infinity

    def potential(self, cp, enei):
        nb = np.sqrt(cp.eps[self.medium - 1](enei)[0])
        k0 = 2 * np.pi / enei
        k = k0 * nb
        npol = self.pol.shape[0]
        media = cp.face_media()
        exc = {"enei": enei}
        for side, (ka, kp) in enumerate((("a1", "a1p"), ("a2", "a2p"))):
            a = np.zeros((cp.n, 3, npol), dtype=complex)
            ap = np.zeros((cp.n, 3, npol), dtype=complex)
            ind = np.nonzero(media[:, side] == self.medium)[0]
            for i in range(npol):
                phase = np.exp(1j * k * cp.pos[ind] @ self.dir[i]) / (1j * k0)
                a[ind, :, i] = phase[:, None] * self.pol[i][None, :]
                ap[ind, :, i] = ((1j * k * cp.nvec[ind] @ self.dir[i]) * phase)[:, None] * self.pol[i][None, :]
            exc[ka], exc[kp] = a, ap
        return exc

    def farfield(self, cp, sig, dirs):
        enei = sig["enei"]
        k = cp.eps[self.medium - 1](enei)[1]
        k0 = 2 * np.pi / enei
        phase = np.exp(-1j * k * dirs @ cp.pos.T) * cp.area[None, :]
        media = cp.face_media()
        npol = sig["sig2"].shape[1]
        e = np.zeros((dirs.shape[0], 3, npol), dtype=complex)
        h = np.zeros_like(e)
        for side, (ks, kh) in enumerate((("sig1", "h1"), ("sig2", "h2"))):
            ind = np.nonzero(media[:, side] == self.medium)[0]
            if ind.size == 0:
                continue
            ph = phase[:, ind]
            Ph = np.einsum("dn,nkp->dkp", ph, sig[kh][ind])
            Ps = ph @ sig[ks][ind]
            e += 1j * k0 * Ph - 1j * k * dirs[:, :, None] * Ps[:, None, :]
            h += 1j * k * np.cross(np.broadcast_to(dirs[:, :, None], Ph.shape), Ph, axis=1)
        return e, h, k

    def field(self, cp, enei, inout=1):
        """Incoming fields at the faces (@planewaveret/field.m): faces whose
        medium column ``inout`` is the excitation medium get
        e = i k0 exp(i k r.dir)/(i k0) pol; h = nb dir x e everywhere."""
        nb = np.sqrt(complex(cp.eps[self.medium - 1](enei)[0]))
        k0 = 2 * np.pi / enei
        k = k0 * nb
        ind = np.nonzero(cp.face_media()[:, inout - 1] == self.medium)[0]
        n, P = cp.n, self.pol.shape[0]
        e = np.zeros((n, 3, P), complex)
        h = np.zeros((n, 3, P), complex)
        for i in range(P):
            phase = np.exp(1j * k * cp.pos[ind] @ self.dir[i]) / (1j * k0)
            e[ind, :, i] = 1j * k0 * phase[:, None] * self.pol[i][None, :]
            h[:, :, i] = nb * np.cross(np.tile(self.dir[i], (n, 1)), e[:, :, i])
        return e, h

    def extinction(self, cp, sig):
        e, h, k = self.farfield(cp, sig, self.dir)
        npol = self.pol.shape[0]
        val = np.array([np.sum(np.conj(self.pol[i]) * e[i, :, i]) for i in range(npol)])
        return np.real(4 * np.pi / k * np.imag(val))

    def scattering(self, cp, sig):
        pinf = self.pinfty
        e, h, k = self.farfield(cp, sig, pinf.nvec)
        dsca = 0.5 * np.real(np.einsum("dk,dkp->dp", pinf.nvec, np.cross(e, np.conj(h), axis=1)))
        sca = pinf.area @ dsca
        nb = np.sqrt(cp.eps[0](sig["enei"])[0])
        return np.real(sca / (0.5 * nb))


# --------------------------------------------------------------------------
# Mie theory  (Mie/@mieret/extinction.m:9-28, scattering.m:9-28,
#   private/miecoefficients.m:14-31, private/riccatibessel.m:17-34)
# --------------------------------------------------------------------------
def _riccatibessel(z, lmax):
    l = np.arange(1, lmax + 1)
    j0 = np.sin(z) / z
    j = np.sqrt(np.pi / (2 * z)) * scipy.special.jv(l + 0.5, z)
    y0 = -np.cos(z) / z
    y = np.sqrt(np.pi / (2 * z)) * scipy.special.yv(l + 0.5, z)
    h0 = j0 + 1j * y0
    h = j + 1j * y
    zjp = z * np.concatenate([[j0], j[:-1]]) - l * j
    zhp = z * np.concatenate([[h0], h[:-1]]) - l * h
    return j, h, zjp, zhp


def mie_coefficients(k, diameter, epsr, lmax=20, mur=1.0):
    nr = np.sqrt(epsr * mur)
    j1, _, zjp1, _ = _riccatibessel(nr * k * diameter / 2, lmax)
    j2, h2, zjp2, zhp2 = _riccatibessel(k * diameter / 2 + 0j, lmax)
    a = (nr ** 2 * j1 * zjp2 - mur * j2 * zjp1) / (nr ** 2 * j1 * zhp2 - mur * h2 * zjp1)
    b = (mur * j1 * zjp2 - j2 * zjp1) / (mur * j1 * zhp2 - h2 * zjp1)
    return a, b


def mie_ext_sca(epsin, epsout, diameter, enei, lmax=20):
    enei = np.atleast_1d(np.asarray(enei, dtype=float))
    epsb = epsout(enei)[0]
    nb = np.sqrt(epsb)
    k = 2 * np.pi / enei * nb
    epsz = epsin(enei)[0] / epsb
    l = np.arange(1, lmax + 1)
    ext, sca = np.zeros(enei.size), np.zeros(enei.size)
    for i in range(enei.size):
        a, b = mie_coefficients(k[i], diameter, epsz[i], lmax)
        ext[i] = np.real(2 * np.pi / k[i] ** 2 * np.sum((2 * l + 1) * np.real(a + b)))
        sca[i] = np.real(2 * np.pi / k[i] ** 2 * np.sum((2 * l + 1) * (np.abs(a) ** 2 + np.abs(b) ** 2)))
    return ext, sca


# --------------------------------------------------------------------------
# one-call driver used by tests and the CPU baseline
# --------------------------------------------------------------------------
def solve_spectrum(cp, pw, eneis, order=5, rel_cutoff=3.0):
    """bemsolver + loop over wavelengths: returns ext, sca [nenei, npol] and
    the list of solutions (demospecret1.m:20-41)."""
    bem = BemRet(cp, order, rel_cutoff)
    ext, sca, sols = [], [], []
    for enei in eneis:
        sig = bem.solve(pw.potential(cp, enei))
        ext.append(pw.extinction(cp, sig))
        sca.append(pw.scattering(cp, sig))
        sols.append(sig)
    return np.array(ext), np.array(sca), sols, bem


# --------------------------------------------------------------------------
# fields at points off the boundary (Greenfun/@compgreenret/field.m:17-38
# with the Green function between a compoint and the particle:
# refinematrix.m:27-67 for points (radius of the boundary element, no self
# elements), greenret/private/init.m:98-177 near coefficients with the points
# as first argument, eval1.m:18-40,110-124 for G and its Cartesian derivative)
# --------------------------------------------------------------------------
def point_refinement(cp, pts, rel_cutoff=3.0, abs_cutoff=0.0, order=5):
    """Refined (point, face) pairs and their Taylor coefficients.

    Returns ``rows, cols`` (point, face) in row-major order and ``g [m,
    order+1]``, ``f [m, 3, order+1]``.
    """
    pts = np.asarray(pts, float)
    rad2 = cp.bradius()
    d = np.sqrt(np.sum((pts[:, None, :] - cp.pos[None, :, :]) ** 2, 2))
    d2 = d - rad2[None, :]
    ir = (d2 < abs_cutoff) | (d2 / rad2[None, :] < rel_cutoff)
    rows, cols = np.nonzero(ir)
    g = np.zeros((rows.size, order + 1))
    f = np.zeros((rows.size, 3, order + 1))
    faces = np.unique(cols)
    if faces.size:
        postab, wtab, rowtab = cp.quad_points(faces)
        for k2, face in enumerate(faces):
            sel_pairs = np.nonzero(cols == face)[0]
            nb = rows[sel_pairs]
            sel = rowtab == k2
            q, w = postab[sel], wtab[sel]
            x = pts[nb, 0][:, None] - q[None, :, 0]
            y = pts[nb, 1][:, None] - q[None, :, 1]
            z = pts[nb, 2][:, None] - q[None, :, 2]
            r = np.sqrt(x ** 2 + y ** 2 + z ** 2)
            r0 = np.sqrt(np.sum((pts[nb] - cp.pos[face]) ** 2, 1))
            dr = r - r0[:, None]
            for o in range(order + 1):
                g[sel_pairs, o] = (dr ** o / r / math.factorial(o)) @ w

            def fun(ff):
                return np.stack([(x * ff) @ w, (y * ff) @ w, (z * ff) @ w], 1)
            f[sel_pairs, :, 0] = -fun(1.0 / r ** 3)
            for o in range(1, order + 1):
                f[sel_pairs, :, o] = fun(-dr ** o / (r ** 3 * math.factorial(o))
                                         + dr ** (o - 1) / (r ** 2 * math.factorial(o - 1)))
    return rows, cols, g, f


def point_fields(cp, pts, pt_medium, enei, sig1, sig2, h1, h2, rel_cutoff=3.0, abs_cutoff=0.0, order=5):
    """E and H at points ``pts`` lying in media ``pt_medium`` (1-based) from the
    surface charges ``sig1, sig2 [n, npol]`` and currents ``h1, h2 [n, 3, npol]``
    (field.m:17-38): faces whose inside (outside) medium is the point's medium
    contribute with sig1 / h1 (sig2 / h2); the Green function takes
    k = k0 sqrt(eps(medium)), the vector-potential term E = i k0 A the vacuum k0.
    Returns ``e, h [m, 3, npol]``."""
    pts = np.asarray(pts, float)
    pt_medium = np.asarray(pt_medium, int)
    m, n = pts.shape[0], cp.n
    k0 = 2 * np.pi / enei
    rows, cols, gc, fc = point_refinement(cp, pts, rel_cutoff, abs_cutoff, order)
    med = cp.face_media()                       # [n, 2] inside, outside
    x = pts[:, None, 0] - cp.pos[None, :, 0]
    y = pts[:, None, 1] - cp.pos[None, :, 1]
    z = pts[:, None, 2] - cp.pos[None, :, 2]
    d = np.maximum(np.sqrt(x ** 2 + y ** 2 + z ** 2), EPS)
    P = sig1.shape[1]
    e = np.zeros((m, 3, P), complex)
    h = np.zeros((m, 3, P), complex)
    for mm in np.unique(pt_medium):
        ip = np.nonzero(pt_medium == mm)[0]
        k = k0 * np.sqrt(complex(cp.eps[mm - 1](enei)[0]))
        area = cp.area[None, :]
        G = (1.0 / d[ip] * area).astype(complex)
        ff = (1j * k - 1.0 / d[ip]) / d[ip] ** 2 * area
        Gp = np.stack([ff * x[ip], ff * y[ip], ff * z[ip]], 1)     # [mi, 3, n]
        # refined pairs of these points
        fr = (1j * k) ** np.arange(order + 1)
        pos_in = np.full(m, -1)
        pos_in[ip] = np.arange(ip.size)
        sel = pos_in[rows] >= 0
        ri, ci = pos_in[rows[sel]], cols[sel]
        G[ri, ci] = gc[sel] @ fr
        Gp[ri, :, ci] = fc[sel] @ fr
        ph = np.exp(1j * k * d[ip])
        G, Gp = G * ph, Gp * ph[:, None, :]
        for side, (s, hh) in enumerate(((sig1, h1), (sig2, h2))):
            mask = (med[:, side] == mm).astype(float)         # faces of this side facing medium mm
            Gs, Gps = G * mask[None, :], Gp * mask[None, None, :]
            # E = i k0 A - grad(phi) with the vacuum wavenumber (field.m:17-21)
            e[ip] += 1j * k0 * np.einsum("ij,jcp->icp", Gs, hh) - np.einsum("icj,jp->icp", Gps, s)
            hx = np.einsum("ij,jp->ip", Gps[:, 1], hh[:, 2]) - np.einsum("ij,jp->ip", Gps[:, 2], hh[:, 1])
            hy = np.einsum("ij,jp->ip", Gps[:, 2], hh[:, 0]) - np.einsum("ij,jp->ip", Gps[:, 0], hh[:, 2])
            hz = np.einsum("ij,jp->ip", Gps[:, 0], hh[:, 1]) - np.einsum("ij,jp->ip", Gps[:, 1], hh[:, 0])
            h[ip] += np.stack([hx, hy, hz], 1)
    return e, h



# --------------------------------------------------------------------------
# dipole excitation (Simulation/retarded/@dipoleret: potential.m:14-117,
# farfield.m:11-55, scattering.m, decayrate.m:13-62)
# --------------------------------------------------------------------------
class DipoleRet:
    """Oscillating dipoles at ``pos [npt, 3]`` in media ``medium [npt]``
    (1-based) with moments ``dip [npt, 3, ndip]``; ``pinfty`` the unit sphere
    at infinity of the radiative rate.  Columns of the potentials are the
    (position, orientation) pairs, position-major."""

    def __init__(self, pos, dip, medium, pinfty, spec_medium=1):
        self.pos = np.asarray(pos, float).reshape(-1, 3)
        self.dip = np.asarray(dip, float)
        self.medium = np.asarray(medium, int)
        self.pinfty = pinfty
        self.spec_medium = spec_medium

    def potential(self, cp, enei):
        npt, ndip = self.pos.shape[0], self.dip.shape[2]
        P = npt * ndip
        n = cp.n
        out = {"enei": enei}
        for key in ("phi1", "phi1p", "phi2", "phi2p"):
            out[key] = np.zeros((n, P), complex)
        for key in ("a1", "a1p", "a2", "a2p"):
            out[key] = np.zeros((n, 3, P), complex)
        media = cp.face_media()
        k0 = 2 * np.pi / enei
        for ipt in range(npt):
            mm = self.medium[ipt]
            eps = complex(cp.eps[mm - 1](enei)[0])
            k = k0 * np.sqrt(eps)
            for side, sfx in ((0, "1"), (1, "2")):
                ind = np.nonzero(media[:, side] == mm)[0]
                if ind.size == 0:
                    continue
                v = cp.pos[ind] - self.pos[ipt][None, :]
                r = np.sqrt(np.sum(v * v, 1))
                u = v / r[:, None]
                G = np.exp(1j * k * r) / r
                F = (1j * k - 1 / r) * G
                nv = cp.nvec[ind]
                en = np.sum(nv * u, 1)
                for idip in range(ndip):
                    d = self.dip[ipt, :, idip]
                    col = ipt * ndip + idip
                    ep, npd = u @ d, nv @ d
                    out["phi" + sfx][ind, col] = -ep * F / eps
                    out["phi" + sfx + "p"][ind, col] = ((npd - 3 * en * ep) / r ** 2 * (1 - 1j * k * r) * G / eps
                                                         + k ** 2 * ep * en * G / eps)
                    out["a" + sfx][ind, :, col] = -1j * k0 * d[None, :] * G[:, None]
                    out["a" + sfx + "p"][ind, :, col] = -1j * k0 * d[None, :] * (en * F)[:, None]
        return out

    def farfield(self, cp, enei):
        """Far fields of the dipoles themselves (farfield.m:11-55)."""
        dirs = self.pinfty.nvec
        eps = complex(cp.eps[self.spec_medium - 1](enei)[0])
        k = 2 * np.pi / enei * np.sqrt(eps)
        npt, ndip = self.pos.shape[0], self.dip.shape[2]
        e = np.zeros((dirs.shape[0], 3, npt * ndip), complex)
        h = np.zeros_like(e)
        for ipt in range(npt):
            if self.medium[ipt] != self.spec_medium:
                continue
            g = np.exp(-1j * k * dirs @ self.pos[ipt])
            for idip in range(ndip):
                hh = np.cross(dirs, self.dip[ipt, :, idip][None, :]) * g[:, None]
                ee = np.cross(hh, dirs)
                e[:, :, ipt * ndip + idip] = k ** 2 * ee / eps
                h[:, :, ipt * ndip + idip] = k ** 2 * hh / np.sqrt(eps)
        return e, h

    def decayrate(self, cp, sig):
        """Total and radiative decay rates in units of the free-space rate
        (decayrate.m:13-62): tot = 1 + Im(e_ind . dip*) / (nb gamma / 2) with
        gamma = 4/3 k0^3 and e_ind the induced field at the dipole; rad = the
        power scattered by dipole + induced far fields / (2 pi k0), in the same
        units."""
        enei = sig["enei"]
        k0 = 2 * np.pi / enei
        gamma = 4.0 / 3.0 * k0 ** 3
        npt, ndip = self.pos.shape[0], self.dip.shape[2]
        e, _ = point_fields(cp, self.pos, self.medium, enei, sig["sig1"], sig["sig2"], sig["h1"], sig["h2"])
        # far fields: induced charges (spectrumret/farfield.m, as PlaneWaveRet.farfield) + dipoles
        pw = PlaneWaveRet([1, 0, 0], [0, 0, 1], self.pinfty, self.spec_medium)
        ef, hf, _ = pw.farfield(cp, sig, self.pinfty.nvec)
        ed, hd = self.farfield(cp, enei)
        et, ht = ef + ed, hf + hd
        flux = 0.5 * np.real(np.einsum("dc,dcp->dp", self.pinfty.nvec, np.cross(et, np.conj(ht), axis=1)))
        sca = self.pinfty.area @ flux
        tot = np.zeros((npt, ndip))
        rad = np.zeros((npt, ndip))
        for ipt in range(npt):
            nb = np.sqrt(complex(cp.eps[self.medium[ipt] - 1](enei)[0])).real
            for idip in range(ndip):
                col = ipt * ndip + idip
                tot[ipt, idip] = 1 + np.imag(e[ipt, :, col] @ np.conj(self.dip[ipt, :, idip])) / (0.5 * nb * gamma)
                rad[ipt, idip] = sca[col] / (2 * np.pi * k0) / (0.5 * nb * gamma)
        return tot, rad
