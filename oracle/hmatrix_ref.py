"""FP64 NumPy restatement of MNPBEM's iterative retarded solver (oracle; test-only).

Test infrastructure: cluster tree, admissibility, adaptive cross approximation
(ACA) of the far blocks of G1, H1, G2, H2, the H-matrix product and the
preconditioned GMRES of ``bemretiter``.  Followed files:

* ``Greenfun/hmatrices/@clustertree/private/init.m:1-60`` and
  ``bisection.m:1-110`` -- bisection of the face centroids (split by particle
  first, then at the middle of the longest bounding-box edge) down to
  ``cleaf`` faces; cluster boxes as (centre, half diagonal);
* ``@clustertree/admissibility.m:1-75`` -- block tree: two leaves give a full
  block, a pair inside one particle each with ``fadmiss(rad1, rad2, dist) =
  2.5 min(rad1, rad2) < dist`` a low-rank block, else recurse into the sons;
* ``mex/hlib/aca.cpp:150-218`` -- partial-pivot ACA (pivot search by
  |re| + |im|, first maximum; stop when the raw row norm is below 1e-10, when
  ||a_k|| ||b_k|| < tol * (accumulated norm), or when no rows are left);
* ``mex/acagreen/acagreen.cpp:76-131`` -- the retarded kernel of the far
  blocks: G = exp(ikd)/d area_j, F = (r . n_i)(ik - 1/d) exp(ikd)/d^2 area_j;
* ``Greenfun/+aca/@compgreenret/eval.m:18-68``, ``@hmatrix/fillval.m`` --
  full blocks hold the entries of the complete Green function (refinement
  included);
* ``BEM/@bemretiter/private/afun.m:6-35``, ``mfun.m:1-52``,
  ``initprecond.m:1-76`` ('full'; 'hmat' through oracle/hlu_ref.py), ``@bemiter/solve.m:1-45`` (gmres, cgs,
  bicgstab; cgs and bicgstab restated from their published algorithms with
  the preconditioner applied to the search directions).

Deviations (also made by the GPU path, so both agree): the low-rank blocks of
G1 = g{1,1} - g{2,1} (and H1, G2, H2) are compressed as one kernel (the
difference evaluated entry by entry) instead of compressing each term and
adding with truncation (hmatadd); the 'full' preconditioner uses the exact
dense matrices instead of the expanded H-matrices (it changes the number of
iterations, not the solution); GMRES is restated as restarted, left-
preconditioned GMRES with classical Gram-Schmidt applied twice and complex
Givens rotations (MATLAB's gmres uses Householder reflections; both stop on
the preconditioned residual ||M (b - A x)|| <= tol ||M b||).
"""
import numpy as np

from . import mnpbem_ref as R

ACATOL = 1e-10


# --------------------------------------------------------------------------
# cluster tree
# --------------------------------------------------------------------------
class ClusterTree:
    """Binary cluster tree of the face centroids.

    ``son [ncl, 2]`` (-1: leaf), ``cind [ncl, 2]`` first / last cluster-order
    position (0-based, inclusive), ``mid``, ``rad`` box centre and half
    diagonal, ``perm [n]`` face index of each cluster-order position
    (``ind(:, 1)``), ``iperm`` its inverse (``ind(:, 2)``), ``ipart [ncl]``
    particle (0-based) of a cluster, -1 when it spans several.
    """

    def __init__(self, pos, face_part, cleaf=200):
        pos = np.asarray(pos, dtype=float)
        face_part = np.asarray(face_part)
        n = pos.shape[0]
        nodes = []

        def sphbox(ind):
            lo, hi = pos[ind].min(axis=0), pos[ind].max(axis=0)
            return 0.5 * (lo + hi), 0.5 * np.linalg.norm(hi - lo)

        def split(ind):
            ip = face_part[ind]
            if np.unique(ip).size > 1:
                ind1 = ind[ip == ip[0]]
                return ind1, np.setdiff1d(ind, ind1), True
            lo, hi = pos[ind].min(axis=0), pos[ind].max(axis=0)
            k = int(np.argmax(hi - lo))
            mid = lo[k] + 0.5 * (hi[k] - lo[k])
            ind1 = ind[pos[ind, k] < mid]
            return ind1, np.setdiff1d(ind, ind1), False

        leaves = {}

        def bisection(ic, ind, c0):
            siz = len(nodes)
            nodes[ic]["son"] = (siz, siz + 1)
            ind1, ind2, psplit = split(ind)
            for s, sub, cs in ((siz, ind1, c0), (siz + 1, ind2, c0 + ind1.size)):
                m, r = sphbox(sub)
                nodes.append({"cind": (cs, cs + sub.size - 1), "mid": m, "rad": r, "son": (-1, -1)})
            for s, sub, cs in ((siz, ind1, c0), (siz + 1, ind2, c0 + ind1.size)):
                if sub.size > cleaf or psplit:
                    bisection(s, sub, cs)
                else:
                    leaves[s] = sub

        m, r = sphbox(np.arange(n))
        nodes.append({"cind": (0, n - 1), "mid": m, "rad": r, "son": (-1, -1)})
        bisection(0, np.arange(n), 0)
        self.n = n
        self.son = np.array([nd["son"] for nd in nodes], dtype=np.int64)
        self.cind = np.array([nd["cind"] for nd in nodes], dtype=np.int64)
        self.mid = np.array([nd["mid"] for nd in nodes])
        self.rad = np.array([nd["rad"] for nd in nodes])
        self.perm = np.empty(n, dtype=np.int64)
        for s, sub in leaves.items():
            c0, c1 = self.cind[s]
            self.perm[c0:c1 + 1] = sub
        self.iperm = np.empty(n, dtype=np.int64)
        self.iperm[self.perm] = np.arange(n)
        p0 = face_part[self.perm[self.cind[:, 0]]]
        p1 = face_part[self.perm[self.cind[:, 1]]]
        self.ipart = np.where(p0 == p1, p0, -1).astype(np.int64)

    def is_leaf(self, i):
        return self.son[i, 0] < 0

    def admissibility(self, eta=2.5):
        """Lists of full (both leaves) and low-rank blocks (row cluster, col
        cluster), each sorted like MATLAB's ``find`` (by column, then row)."""
        full, low = [], []

        def blocktree(i1, i2):
            if self.is_leaf(i1) and self.is_leaf(i2):
                full.append((i1, i2))
                return
            if self.ipart[i1] >= 0 and self.ipart[i2] >= 0:
                d = np.linalg.norm(self.mid[i1] - self.mid[i2])
                if eta * min(self.rad[i1], self.rad[i2]) < d:
                    low.append((i1, i2))
                    return
            s1 = [i1] if self.is_leaf(i1) else list(self.son[i1])
            s2 = [i2] if self.is_leaf(i2) else list(self.son[i2])
            for a in s1:
                for b in s2:
                    blocktree(a, b)

        blocktree(0, 0)
        key = lambda t: (t[1], t[0])
        return sorted(full, key=key), sorted(low, key=key)


# --------------------------------------------------------------------------
# ACA  (mex/hlib/aca.cpp:150-218)
# --------------------------------------------------------------------------
def cabs1(z):
    return np.abs(z.real) + np.abs(z.imag)


def aca(getrow, getcol, m, n, tol, kmax):
    """Partial-pivot ACA of an m x n block: returns L [m, r], R [n, r] with
    block ~ L R^T.  A zero pivot ends the loop (guard; the reference would
    divide by zero)."""
    kmax = min(m, n, kmax)
    A = np.zeros((m, kmax), dtype=complex)
    B = np.zeros((n, kmax), dtype=complex)
    used = np.zeros(m, dtype=bool)
    r, nsum, k = 0, 0.0, 0
    while k < kmax:
        B[:, k] = getrow(r)
        if np.linalg.norm(B[:, k]) < ACATOL:
            break
        if k:
            B[:, k] -= B[:, :k] @ A[r, :k]
        c = int(np.argmax(cabs1(B[:, k])))
        if B[c, k] == 0:
            B[:, k] = 0
            return A[:, :k], B[:, :k]
        B[:, k] *= 1.0 / B[c, k]
        A[:, k] = getcol(c)
        if k:
            A[:, k] -= A[:, :k] @ B[c, :k]
        used[r] = True
        work = np.where(used, 0, A[:, k])
        r = int(np.argmax(cabs1(work)))
        nk = np.linalg.norm(A[:, k]) * np.linalg.norm(B[:, k])
        if nk < tol * nsum or used.all():
            break
        nsum = np.sqrt(nsum ** 2 + nk ** 2)
        k += 1
    rank = min(k + 1, kmax)
    return A[:, :rank], B[:, :rank]


# --------------------------------------------------------------------------
# H-matrices of G1, H1, G2, H2
# --------------------------------------------------------------------------
class HMatrix:
    """Full blocks ``val[b]`` and low-rank blocks ``lhs[b] @ rhs[b].T`` on the
    cluster ordering of ``tree``."""

    def __init__(self, tree, full, low):
        self.tree, self.full, self.low = tree, full, low
        self.val, self.lhs, self.rhs = [], [], []

    def rng(self, c):
        c0, c1 = self.tree.cind[c]
        return slice(c0, c1 + 1)

    def matvec(self, x):
        """H x for x [n, ...] in face order (hmatmul1 on part2cluster'ed x)."""
        t = self.tree
        sh = x.shape
        xc = x.reshape(sh[0], -1)[t.perm]
        yc = np.zeros_like(xc, dtype=complex)
        for (rc, cc), v in zip(self.full, self.val):
            yc[self.rng(rc)] += v @ xc[self.rng(cc)]
        for (rc, cc), L, Rr in zip(self.low, self.lhs, self.rhs):
            yc[self.rng(rc)] += L @ (Rr.T @ xc[self.rng(cc)])
        y = np.empty_like(yc)
        y[t.perm] = yc
        return y.reshape(sh)

    def full_matrix(self):
        """Expanded matrix in face order (@hmatrix/full.m)."""
        t = self.tree
        M = np.zeros((t.n, t.n), dtype=complex)
        for (rc, cc), v in zip(self.full, self.val):
            M[self.rng(rc), self.rng(cc)] = v
        for (rc, cc), L, Rr in zip(self.low, self.lhs, self.rhs):
            M[self.rng(rc), self.rng(cc)] = L @ Rr.T
        out = np.empty_like(M)
        out[np.ix_(t.perm, t.perm)] = M
        return out

    def ranks(self):
        return [L.shape[1] for L in self.lhs]


def kernel_block(cp, tree, key, k_terms, rows, cols):
    """Far-field kernel entries (cluster-order rows / cols) of a combined key:
    sum over (sign, k) of G or F (acagreen.cpp greenret::getrow / getcol)."""
    fi, fj = tree.perm[rows], tree.perm[cols]
    r = cp.pos[fi][:, None, :] - cp.pos[fj][None, :, :]
    d = np.linalg.norm(r, axis=2)
    area = cp.area[fj][None, :]
    out = np.zeros(d.shape, dtype=complex)
    for sign, k in k_terms:
        fac = np.exp(1j * k * d)
        if key == "G":
            out += sign * fac / d * area
        else:
            inn = np.einsum("ijk,ik->ij", r, cp.nvec[fi])
            out += sign * inn * (1j * k - 1.0 / d) * fac / d ** 2 * area
    return out


def build_hmatrices(cp, tree, dense, enei, htol=1e-6, kmax=100, eta=2.5):
    """H-matrices of G1, H1, G2, H2 at one wavelength: full blocks from the
    dense matrices ``dense = (G1, H1, G2, H2)`` (complete Green function),
    low-rank blocks by ACA of the far-field kernel."""
    full, low = tree.admissibility(eta)
    k = np.array([e(enei)[1] for e in cp.eps], dtype=complex)
    con = R.connect(cp.inout)
    # (key, [(+1, con block), (-1, con block)]) of G1, H1, G2, H2 (initmat.m:27-31)
    spec = [("G", (con[0][0], con[1][0])), ("F", (con[0][0], con[1][0])),
            ("G", (con[1][1], con[0][1])), ("F", (con[1][1], con[0][1]))]
    out = []
    for q, (key, (cplus, cminus)) in enumerate(spec):
        H = HMatrix(tree, full, low)
        P = tree.perm
        for rc, cc in full:
            rs, cs = H.rng(rc), H.rng(cc)
            H.val.append(dense[q][np.ix_(P[rs], P[cs])])
        for rc, cc in low:
            rs, cs = H.rng(rc), H.rng(cc)
            pi, pj = tree.ipart[rc], tree.ipart[cc]
            terms = []
            if cplus[pi, pj]:
                terms.append((1.0, k[cplus[pi, pj] - 1]))
            if cminus[pi, pj]:
                terms.append((-1.0, k[cminus[pi, pj] - 1]))
            rows = np.arange(rs.start, rs.stop)
            cols = np.arange(cs.start, cs.stop)
            L, Rr = aca(lambda i: kernel_block(cp, tree, key, terms, rows[i:i + 1], cols)[0],
                        lambda j: kernel_block(cp, tree, key, terms, rows, cols[j:j + 1])[:, 0],
                        rows.size, cols.size, htol, kmax)
            H.lhs.append(L)
            H.rhs.append(Rr)
        out.append(H)
    return out


# --------------------------------------------------------------------------
# GMRES
# --------------------------------------------------------------------------
def gmres(afun, b, tol=1e-6, maxit=100, restart=None, mfun=None):
    """Restarted, left-preconditioned GMRES (x0 = 0).

    restart None: cycles of up to ``maxit`` steps, at most ``maxit`` steps in
    all; else cycles of ``restart`` steps, at most ``maxit`` cycles (MATLAB's
    gmres counting).  A cycle ends when the estimated residual reaches the
    tolerance; when the true preconditioned residual has not (an inexact
    preconditioner), the next cycle continues from x within the same step
    budget.  Returns x, flag (0 converged), relres = ||M (b - A x)|| / ||M b||,
    total inner steps."""
    M = (lambda v: v) if mfun is None else mfun
    inner = restart if restart else maxit
    budget = maxit * restart if restart else maxit
    Mb = M(b)
    nmb = np.linalg.norm(Mb)
    x = np.zeros_like(b)
    if nmb == 0:
        return x, 0, 0.0, 0
    tolb = tol * nmb
    steps = 0
    r = Mb
    while steps < budget:
        beta = np.linalg.norm(r)
        if beta <= tolb:
            return x, 0, beta / nmb, steps
        inner_c = min(inner, budget - steps)
        V = [r / beta]
        H = np.zeros((inner + 1, inner), dtype=complex)
        cs = np.zeros(inner)
        sn = np.zeros(inner, dtype=complex)
        g = np.zeros(inner + 1, dtype=complex)
        g[0] = beta
        j_last = -1
        for j in range(inner_c):
            w = M(afun(V[j]))
            steps += 1
            Vm = np.array(V)
            h = Vm.conj() @ w
            w = w - Vm.T @ h
            h2 = Vm.conj() @ w
            w = w - Vm.T @ h2
            h = h + h2
            hn = np.linalg.norm(w)
            col = np.zeros(inner + 1, dtype=complex)
            col[:j + 1] = h
            col[j + 1] = hn
            for i in range(j):
                a0, a1 = col[i], col[i + 1]
                col[i] = cs[i] * a0 + sn[i] * a1
                col[i + 1] = -np.conj(sn[i]) * a0 + cs[i] * a1
            a, bb = col[j], col[j + 1]
            t = np.hypot(abs(a), abs(bb))
            if abs(a) == 0:
                cs[j], sn[j] = 0.0, 1.0
            else:
                cs[j] = abs(a) / t
                sn[j] = (a / abs(a)) * np.conj(bb) / t
            col[j] = cs[j] * a + sn[j] * bb
            col[j + 1] = 0
            H[:, j] = col
            g[j + 1] = -np.conj(sn[j]) * g[j]
            g[j] = cs[j] * g[j]
            j_last = j
            if hn == 0 or abs(g[j + 1]) <= tolb:
                break
            V.append(w / hn)
        m = j_last + 1
        y = np.zeros(m, dtype=complex)
        for i in range(m - 1, -1, -1):
            y[i] = (g[i] - H[i, i + 1:m] @ y[i + 1:m]) / H[i, i]
        x = x + np.array(V[:m]).T @ y
        r = M(b - afun(x))
        if np.linalg.norm(r) <= tolb:
            return x, 0, np.linalg.norm(r) / nmb, steps
    return x, 1, np.linalg.norm(r) / nmb, steps


def cgs(afun, b, tol=1e-6, maxit=100, mfun=None):
    """Preconditioned conjugate gradients squared (x0 = 0; the preconditioner
    M applied to the search directions, residuals unpreconditioned; stop when
    the recurrence residual ||r|| <= tol ||b||).  Returns x, flag, relres =
    ||b - A x|| / ||b|| (true residual), iterations."""
    M = (lambda v: v) if mfun is None else mfun
    nb = np.linalg.norm(b)
    x = M(np.zeros_like(b)) * 0
    if nb == 0:
        return x, 0, 0.0, 0
    tolb = tol * nb
    r = b.copy()
    rt = r.copy()
    rho = 1.0
    u = q = p = None
    flag, it = 1, 0
    for ii in range(1, maxit + 1):
        rho1, rho = rho, np.vdot(rt, r)
        if rho == 0:
            break
        if ii == 1:
            u = r.copy()
            p = u.copy()
        else:
            beta = rho / rho1
            u = r + beta * q
            p = u + beta * (q + beta * p)
        ph = M(p)
        vh = afun(ph)
        rtv = np.vdot(rt, vh)
        if rtv == 0:
            break
        alpha = rho / rtv
        q = u - alpha * vh
        uh = M(u + q)
        x = x + alpha * uh
        r = r - alpha * afun(uh)
        it = ii
        if np.linalg.norm(r) <= tolb:
            flag = 0
            break
    return x, flag, np.linalg.norm(b - afun(x)) / nb, it


def bicgstab(afun, b, tol=1e-6, maxit=100, mfun=None):
    """Preconditioned BiCGStab (x0 = 0; residuals unpreconditioned; stop when
    ||s|| or ||r|| <= tol ||b||, the half step counting as its iteration).
    Returns x, flag, relres = ||b - A x|| / ||b||, iterations."""
    M = (lambda v: v) if mfun is None else mfun
    nb = np.linalg.norm(b)
    x = M(np.zeros_like(b)) * 0
    if nb == 0:
        return x, 0, 0.0, 0
    tolb = tol * nb
    r = b.copy()
    rt = r.copy()
    rho = alpha = omega = 1.0
    p = v = None
    flag, it = 1, 0
    for ii in range(1, maxit + 1):
        rho1, rho = rho, np.vdot(rt, r)
        if rho == 0:
            break
        if ii == 1:
            p = r.copy()
        else:
            beta = (rho / rho1) * (alpha / omega)
            p = r + beta * (p - omega * v)
        ph = M(p)
        v = afun(ph)
        rtv = np.vdot(rt, v)
        if rtv == 0:
            break
        alpha = rho / rtv
        s = r - alpha * v
        it = ii
        if np.linalg.norm(s) <= tolb:
            x = x + alpha * ph
            flag = 0
            break
        sh = M(s)
        t = afun(sh)
        tt = np.vdot(t, t)
        if tt == 0:
            break
        omega = np.vdot(t, s) / tt
        x = x + alpha * ph + omega * sh
        r = s - omega * t
        if np.linalg.norm(r) <= tolb:
            flag = 0
            break
    return x, flag, np.linalg.norm(b - afun(x)) / nb, it


# --------------------------------------------------------------------------
# bemretiter
# --------------------------------------------------------------------------
class BemRetIter:
    """Iterative retarded solver: A from the H-matrices, preconditioner
    'full' (dense chain of mldivide.m) or None."""

    def __init__(self, cp, cleaf=200, htol=1e-6, kmax=100, tol=1e-6, maxit=100, restart=None,
                 precond="full", eta=2.5, solver="gmres", kmax_precond=4):
        self.p = cp
        self.bem = R.BemRet(cp)
        face_part = np.repeat(np.arange(len(cp.parts)), [q.n for q in cp.parts])
        self.tree = ClusterTree(cp.pos, face_part, cleaf)
        self.htol, self.kmax, self.eta = htol, kmax, eta
        self.tol, self.maxit, self.restart, self.precond = tol, maxit, restart, precond
        self.solver = solver
        self.kmax_precond = kmax_precond
        self.enei = None

    def initmat(self, enei):
        if self.enei == enei:
            return
        self.enei = enei
        self.bem.initmat(enei)
        b = self.bem
        self.H = build_hmatrices(self.p, self.tree, (b.G1, b.H1, b.G2, b.H2), enei, self.htol,
                                 self.kmax, self.eta)
        if self.precond == "hmat":
            # initprecond.m 'hmat' on the compressed H-matrices (compress.m:
            # htol, min(op.kmax))
            from . import hlu_ref as HL
            t = self.tree
            full, low = self.H[0].full, self.H[0].low
            T = HL.Tree(t.son, t.cind, full, low)
            mats = [HL.from_blocks(T, full, low, H.val, H.lhs, H.rhs) for H in self.H]
            e1 = self.p.eps_faces(enei, 0)
            e2 = self.p.eps_faces(enei, 1)
            self.hpc = HL.HmatPrecond(T, t.perm, *mats, b.k, e1, e2, b.nvec, self.htol, self.kmax_precond)

    def _split(self, x):
        n = self.p.n
        P = x.size // (8 * n)
        o = np.cumsum([0, n * P, 3 * n * P, n * P, 3 * n * P])
        return (x[o[0]:o[1]].reshape(n, P), x[o[1]:o[2]].reshape(n, 3, P),
                x[o[2]:o[3]].reshape(n, P), x[o[3]:o[4]].reshape(n, 3, P))

    @staticmethod
    def _pack(*parts):
        return np.concatenate([q.ravel() for q in parts])

    def afun(self, x):
        """(sig1, h1, sig2, h2) -> (phi, a, De, alpha) with the H-matrices."""
        sig1, h1, sig2, h2 = self._split(x)
        b = self.bem
        G1, H1, G2, H2 = self.H
        k, nvec = b.k, b.nvec
        e1 = self.p.eps_faces(self.enei, 0)
        e2 = self.p.eps_faces(self.enei, 1)
        Gs1, Gh1 = G1.matvec(sig1), G1.matvec(h1)
        Gs2, Gh2 = G2.matvec(sig2), G2.matvec(h2)
        Hs1, Hh1 = H1.matvec(sig1), H1.matvec(h1)
        Hs2, Hh2 = H2.matvec(sig2), H2.matvec(h2)
        phi = Gs1 - Gs2
        a = Gh1 - Gh2
        alpha = Hh1 - Hh2 - 1j * k * R._outer(nvec, e1[:, None] * Gs1 - e2[:, None] * Gs2)
        De = (e1[:, None] * Hs1 - e2[:, None] * Hs2
              - 1j * k * R._inner(nvec, e1[:, None, None] * Gh1 - e2[:, None, None] * Gh2))
        return self._pack(phi, a, De, alpha)

    def mfun(self, v):
        phi, a, De, alpha = self._split(v)
        if self.precond == "hmat":
            return self._pack(*self.hpc.apply(phi, a, De, alpha))
        s = self.bem.chain(phi, a, alpha, De)
        return self._pack(s["sig1"], s["h1"], s["sig2"], s["h2"])

    def solve(self, exc):
        self.initmat(exc["enei"])
        phi, a, alpha, De = self.bem.excitation(exc)
        b = self._pack(phi, a, De, alpha)
        mf = self.mfun if self.precond in ("full", "hmat") else None
        if self.solver == "gmres":
            x, flag, relres, it = gmres(self.afun, b, self.tol, self.maxit, self.restart, mf)
        else:
            # the unpreconditioned operator maps unknowns to equations of the same
            # layout (pack.m / unpack.m), so both solvers run on one vector space
            fn = cgs if self.solver == "cgs" else bicgstab
            x, flag, relres, it = fn(self.afun, b, self.tol, self.maxit, mf)
        sig1, h1, sig2, h2 = self._split(x)
        self.flag, self.relres, self.iter = flag, relres, it
        self.true_relres = np.linalg.norm(b - self.afun(x)) / np.linalg.norm(b)
        return {"enei": exc["enei"], "sig1": sig1, "sig2": sig2, "h1": h1, "h2": h2}
