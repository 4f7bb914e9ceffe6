"""Cluster tree and block partition of the H-matrices (host side).

``clustertree(p, cleaf)`` follows Greenfun/hmatrices/@clustertree/private/
init.m and bisection.m: the face centroids are split by particle first, then
at the middle of the longest edge of their bounding box, until a cluster has
at most ``cleaf`` faces.  ``hmatrix_blocks(tree, eta)`` follows
@clustertree/admissibility.m: a pair of leaves is a full block, a pair of
clusters inside one particle each with ``eta min(rad1, rad2) < dist`` a
low-rank block; other pairs recurse into their sons.  ``hpartition(p).c``
hands both to the library (``mnpbem_cluster_tree``), as treemex.m hands them
to the H-matrix MEX functions.
"""
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


__all__ = ["clustertree", "hmatrix_blocks", "hpartition"]
