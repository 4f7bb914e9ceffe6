"""Cluster tree and block partition of the H-matrices (host side).

``clustertree(p, cleaf)`` follows Greenfun/hmatrices/@clustertree/private/
init.m and bisection.m: the face centroids are split by particle first, then
at the middle of the longest edge of their bounding box, until a cluster has
at most ``cleaf`` faces.  ``hmatrix_blocks(tree, eta)`` follows
@clustertree/admissibility.m: a pair of leaves is a full block, a pair of
clusters inside one particle each with ``eta min(rad1, rad2) < dist`` a
low-rank block; other pairs recurse into their sons.  ``hpartition(p).c``
hands both to the library (``mnpbem_cluster_tree``), as treemex.m hands them
to the H-matrix MEX functions.  ``hmatrix_gpu`` is an H-matrix on such a tree
with the arithmetic of those MEX functions (LU, right solve, inverse, sum,
diagonal scaling, solve, product) run by the library.
"""
import ctypes

import numpy as np

from . import _lib


class clustertree:
    """Binary cluster tree of a comparticle's face centroids.

    Attributes (0-based): ``son [ncl, 2]`` (-1 for leaves), ``cind [ncl, 2]``
    first / last cluster-order position, ``mid [ncl, 3]``, ``rad [ncl]``
    bounding-box centre and half diagonal, ``ipart [ncl]`` particle of the
    cluster (-1 if several), ``perm [n]`` face at each cluster position
    (``ind(:, 1)``), ``iperm [n]`` cluster position of each face."""

    def __init__(self, p, cleaf=200):
        pos = np.asarray(p.pos, dtype=np.float64)
        n = pos.shape[0]
        offs = np.asarray(p.offsets)
        part = np.searchsorted(offs, np.arange(n), side="right") - 1
        self.cleaf = int(cleaf)
        son, cind, mid, rad = [[-1, -1]], [[0, n - 1]], [], []

        def box(ind):
            lo, hi = pos[ind].min(axis=0), pos[ind].max(axis=0)
            return 0.5 * (lo + hi), 0.5 * float(np.linalg.norm(hi - lo))

        m0, r0 = box(np.arange(n))
        mid.append(m0)
        rad.append(r0)
        perm = np.empty(n, dtype=np.int64)
        # explicit stack in the order of the recursive bisection (first son's
        # subtree before the second son's)
        stack = [(0, np.arange(n), 0)]
        while stack:
            ic, ind, c0 = stack.pop()
            ip = part[ind]
            psplit = np.any(ip != ip[0])
            if psplit:
                sel = ip == ip[0]
            else:
                lo, hi = pos[ind].min(axis=0), pos[ind].max(axis=0)
                k = int(np.argmax(hi - lo))
                sel = pos[ind, k] < lo[k] + 0.5 * (hi[k] - lo[k])
            ind1, ind2 = ind[sel], ind[~sel]
            if ind1.size == 0 or ind2.size == 0:
                raise ValueError("clustertree: a cluster of coincident centroids cannot be split")
            s1 = len(son)
            son[ic] = [s1, s1 + 1]
            todo = []
            for s, sub, cs in ((s1, ind1, c0), (s1 + 1, ind2, c0 + ind1.size)):
                son.append([-1, -1])
                cind.append([cs, cs + sub.size - 1])
                m, r = box(sub)
                mid.append(m)
                rad.append(r)
                if sub.size > self.cleaf or psplit:
                    todo.append((s, sub, cs))
                else:
                    perm[cs:cs + sub.size] = sub
            stack.extend(reversed(todo))
        self.n = n
        self.son = np.asarray(son, dtype=np.int32)
        self.cind = np.asarray(cind, dtype=np.int32)
        self.mid = np.asarray(mid)
        self.rad = np.asarray(rad)
        self.perm = perm.astype(np.int32)
        self.iperm = np.empty(n, dtype=np.int32)
        self.iperm[self.perm] = np.arange(n, dtype=np.int32)
        p0 = part[self.perm[self.cind[:, 0]]]
        p1 = part[self.perm[self.cind[:, 1]]]
        self.ipart = np.where(p0 == p1, p0, -1).astype(np.int32)

    @property
    def leaves(self):
        return np.flatnonzero(self.son[:, 0] < 0)


def hmatrix_blocks(tree, eta=2.5):
    """Full and low-rank blocks ``[nb, 2]`` (row cluster, column cluster),
    each ordered as MATLAB's ``find`` on the admissibility matrix."""
    full, low = [], []
    stack = [(0, 0)]
    leaf = tree.son[:, 0] < 0
    while stack:
        i1, i2 = stack.pop()
        if leaf[i1] and leaf[i2]:
            full.append((i1, i2))
            continue
        if tree.ipart[i1] >= 0 and tree.ipart[i2] >= 0:
            d = float(np.linalg.norm(tree.mid[i1] - tree.mid[i2]))
            if eta * min(tree.rad[i1], tree.rad[i2]) < d:
                low.append((i1, i2))
                continue
        s1 = [i1] if leaf[i1] else list(tree.son[i1])
        s2 = [i2] if leaf[i2] else list(tree.son[i2])
        stack.extend((a, b) for a in s1 for b in s2)

    def order(lst):
        a = np.asarray(lst, dtype=np.int32).reshape(-1, 2)
        return np.ascontiguousarray(a[np.lexsort((a[:, 0], a[:, 1]))])
    return order(full), order(low)


class hpartition:
    """Cluster tree plus block partition, packed for the library."""

    def __init__(self, p, cleaf=200, eta=2.5):
        self.tree = clustertree(p, cleaf)
        self.full, self.low = hmatrix_blocks(self.tree, eta)
        t = self.tree
        self._keep = [np.ascontiguousarray(a, dtype=np.int32) for a in
                      (t.son, t.cind, t.ipart, t.perm, self.full, self.low)]
        s = _lib.ClusterTree()
        s.ncluster = t.son.shape[0]
        s.son, s.cind, s.ipart, s.perm = (a.ctypes.data for a in self._keep[:4])
        s.nfull, s.full = self.full.shape[0], self._keep[4].ctypes.data
        s.nlow, s.low = self.low.shape[0], self._keep[5].ctypes.data
        self.c = s

    def dense_fraction(self):
        c = self.tree.cind
        sz = c[:, 1] - c[:, 0] + 1
        return float(np.sum(sz[self.full[:, 0]].astype(float) * sz[self.full[:, 1]])) / self.tree.n ** 2


class treearrays:
    """Cluster tree given as arrays (0-based, as ``clustertree``): son [nc, 2]
    (-1 for leaves), cind [nc, 2] (inclusive), perm [n], full / low [nb, 2];
    ``.c`` is the library's view."""

    def __init__(self, son, cind, perm, full, low, ipart=None):
        son = np.ascontiguousarray(son, dtype=np.int32)
        nc = son.shape[0]
        self._keep = [son, np.ascontiguousarray(cind, dtype=np.int32),
                      np.ascontiguousarray(ipart if ipart is not None else np.full(nc, -1), dtype=np.int32),
                      np.ascontiguousarray(perm, dtype=np.int32),
                      np.ascontiguousarray(full, dtype=np.int32).reshape(-1, 2),
                      np.ascontiguousarray(low, dtype=np.int32).reshape(-1, 2)]
        self.son, self.cind, _, self.perm, self.full, self.low = self._keep
        self.n = int(self.cind[0, 1]) + 1
        s = _lib.ClusterTree()
        s.ncluster = nc
        s.son, s.cind, s.ipart, s.perm = (a.ctypes.data for a in self._keep[:4])
        s.nfull, s.full = self.full.shape[0], self._keep[4].ctypes.data
        s.nlow, s.low = self.low.shape[0], self._keep[5].ctypes.data
        self.c = s

    @classmethod
    def of(cls, part):
        t = part.tree
        return cls(t.son, t.cind, t.perm, part.full, part.low, t.ipart)

    def rows(self, c):
        return int(self.cind[c, 1] - self.cind[c, 0] + 1)


class hmatrix_gpu:
    """H-matrix on the GPU (Greenfun/hmatrices/@hmatrix): full blocks and
    low-rank factors on a cluster tree, with the arithmetic of the reference's
    MEX functions (hmatlu, hmatrsolve, hmatinv, hmatadd, hmatsolve) run by the
    library in FP64.  ``vals``: full blocks (tree.full order), ``lhs`` /
    ``rhs``: factors of the low-rank blocks (block = lhs @ rhs.T), all in
    cluster order.  ``htol`` / ``kmax`` are the truncation options of later
    operations (@hmatrix htol / kmax)."""

    def __init__(self, tree, vals=None, lhs=None, rhs=None, htol=1e-6, kmax=100, device=0, _handle=None):
        self.tree = tree if isinstance(tree, treearrays) else treearrays.of(tree)
        self.lib = _lib.load()
        if _handle is not None:
            self.h = _handle
            return
        v = np.concatenate([np.asarray(x, dtype=np.complex128).ravel(order="F") for x in vals])
        ranks = np.array([np.asarray(x).shape[1] for x in lhs], dtype=np.int32)
        cat = lambda xs: (np.concatenate([np.asarray(x, dtype=np.complex128).ravel(order="F") for x in xs])
                          if len(xs) else np.zeros(1, dtype=np.complex128))
        L, R = cat(lhs), cat(rhs)
        if ranks.size == 0:
            ranks = np.zeros(1, dtype=np.int32)
        h = ctypes.c_void_p()
        _lib.check(self.lib.mnpbem_hm_create(int(device), ctypes.byref(self.tree.c), float(htol), int(kmax),
                                             v.ctypes.data, ranks.ctypes.data, L.ctypes.data, R.ctypes.data,
                                             ctypes.byref(h)))
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            self.lib.mnpbem_hm_free(h)
            self.h = None

    def _new(self, fn, *args):
        out = ctypes.c_void_p()
        _lib.check(fn(self.h, *args, ctypes.byref(out)))
        return hmatrix_gpu(self.tree, _handle=out)

    def set_options(self, htol, kmax):
        _lib.check(self.lib.mnpbem_hm_set_options(self.h, float(htol), int(kmax)))
        return self

    def lu(self):
        """@hmatrix/lu.m"""
        return self._new(self.lib.mnpbem_hm_lu)

    def rsolve(self, lu, key="N"):
        """@hmatrix/rsolve.m: X with X (L U) = self"""
        return self._new(lambda h, *a: self.lib.mnpbem_hm_rsolve(h, lu.h, key.encode(), *a))

    def lsolve(self, lu, key="N"):
        """@hmatrix/lsolve.m: X with (L U) X = self"""
        return self._new(lambda h, *a: self.lib.mnpbem_hm_lsolve(h, lu.h, key.encode(), *a))

    def __matmul__(self, other):
        """self * other of two H-matrices (@hmatrix/mtimes.m, hmatmul2)"""
        return self._new(lambda h, *a: self.lib.mnpbem_hm_matmul(h, other.h, *a))

    def inv(self):
        return self._new(self.lib.mnpbem_hm_inv)

    def __add__(self, other):
        return self._new(lambda h, *a: self.lib.mnpbem_hm_add(h, other.h, 1.0, *a))

    def __sub__(self, other):
        return self._new(lambda h, *a: self.lib.mnpbem_hm_add(h, other.h, -1.0, *a))

    def scale(self, d, side):
        """diag(d) self (side 'L') or self diag(d) ('R'); d in cluster order"""
        d = np.ascontiguousarray(d, dtype=np.complex128)
        return self._new(lambda h, *a: self.lib.mnpbem_hm_scale(h, d.ctypes.data, side.encode(), *a))

    def solve(self, b, key="N"):
        """@hmatrix/solve.m on cluster-order b [n] or [n, N] (self from lu())"""
        b = np.asarray(b, dtype=np.complex128)
        x = np.asfortranarray(b.reshape(self.tree.n, -1)).copy(order="F")
        _lib.check(self.lib.mnpbem_hm_solve(self.h, key.encode(), x.ctypes.data, x.shape[1]))
        return x.reshape(b.shape)

    def mul(self, x):
        x = np.asfortranarray(np.asarray(x, dtype=np.complex128).reshape(self.tree.n, -1))
        y = np.zeros_like(x, order="F")
        _lib.check(self.lib.mnpbem_hm_mul(self.h, x.ctypes.data, y.ctypes.data, x.shape[1]))
        return y

    def full(self):
        """expanded matrix in cluster order"""
        n = self.tree.n
        out = np.zeros((n, n), dtype=np.complex128, order="F")
        _lib.check(self.lib.mnpbem_hm_full(self.h, out.ctypes.data))
        return out

    def export(self):
        """(vals, lhs, rhs) lists in tree order"""
        nv, nl, nr = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(self.lib.mnpbem_hm_sizes(self.h, ctypes.byref(nv), ctypes.byref(nl), ctypes.byref(nr)))
        V = np.zeros(max(1, nv.value), dtype=np.complex128)
        L = np.zeros(max(1, nl.value), dtype=np.complex128)
        R = np.zeros(max(1, nr.value), dtype=np.complex128)
        ranks = np.zeros(max(1, self.tree.low.shape[0]), dtype=np.int32)
        _lib.check(self.lib.mnpbem_hm_export(self.h, V.ctypes.data, ranks.ctypes.data, L.ctypes.data, R.ctypes.data))
        t = self.tree
        vals, lhs, rhs = [], [], []
        o = 0
        for r, c in t.full:
            m, n = t.rows(r), t.rows(c)
            vals.append(V[o:o + m * n].reshape((m, n), order="F"))
            o += m * n
        ol = orr = 0
        for b, (r, c) in enumerate(t.low):
            m, n, k = t.rows(r), t.rows(c), int(ranks[b])
            lhs.append(L[ol:ol + m * k].reshape((m, k), order="F"))
            rhs.append(R[orr:orr + n * k].reshape((n, k), order="F"))
            ol += m * k
            orr += n * k
        return vals, lhs, rhs


__all__ = ["clustertree", "hmatrix_blocks", "hpartition", "treearrays", "hmatrix_gpu"]
