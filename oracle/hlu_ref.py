"""FP64 NumPy restatement of MNPBEM's H-matrix arithmetic (oracle; test-only).

Test infrastructure: the checker of the GPU H-matrix LU, triangular solves,
inversion and addition that make the 'hmat' preconditioner of the iterative
retarded solver.  Followed files:

* ``mex/hlib/clustertree.h:100-203`` -- sons, cluster ranges, admissibility
  flags (flagRk 1, flagFull 2), son iteration (a leaf iterates over itself),
  the pair iterator over the leaf blocks below a cluster pair;
* ``mex/hlib/submatrix.h:50-263`` -- full / low-rank sub-matrices: storage
  conversion (low-rank -> full by L R^T, full -> low-rank by ACA), ACA
  truncation of low-rank sums, masks to sub-clusters, products of two
  sub-matrices, concatenation of 1x1 / 2x1 / 1x2 / 2x2 sub-matrices;
* ``mex/hlib/hmatrix.h:150-446`` -- addition, subtraction, negation over the
  leaf pairs below a cluster pair, the recursive products ``add_mul`` /
  ``add_mul2`` and the recursive inversion by Schur complements;
* ``mex/hlib/lu.h:30-223`` -- H-LU (``lu``), the triangular solves of
  sub-matrices and H-matrices from the left (``lsolve``) and the right
  (``rsolve``), and the forward / backward solve of a vector (``solve``);
* ``mex/hlib/lu.cpp:14-137`` -- LU of a full leaf without row interchanges
  (L lower with its diagonal, U unit upper) and the dense triangular solves
  (``?trsm`` with a non-unit L and a unit U);
* ``mex/hlib/aca.cpp:150-218`` -- partial-pivot ACA of a full matrix and of
  a low-rank product (``acafull`` / ``acaRk``, rank cap min(max_rank, kmax));
* ``mex/hlib/basemat.cpp:225-240`` -- inverse of a full leaf (LAPACK
  getrf / getri, i.e. with partial pivoting);
* ``mex/hmatlu.cpp``, ``hmatrsolve.cpp`` (X (L U) = B: the 'U' then the 'L'
  right solve), ``hmatlsolve.cpp`` ((L U) X = B: 'L' then 'U'),
  ``hmatsolve.cpp`` (L then U), ``hmatinv.cpp``, ``hmatadd.cpp``,
  ``hmatmul2.cpp`` (A B, hmatrix.h operator*); ``Greenfun/hmatrices/@hmatrix/private/mtimes1.m``
  (diagonal times H-matrix) and ``plus2.m``;
* ``BEM/@bemretiter/private/initprecond.m:1-76`` ('hmat'), ``compress.m``
  (the preconditioner works with htol = max(op.htol), kmax = min(op.kmax))
  and ``mfun.m:1-52``.

Clusters are numbered as in the library's cluster tree (0 the root, son -1
for none); ranges are [first, one past last) in cluster order.  A guard not
in the reference: an ACA pivot that is exactly zero ends the loop (the
reference would divide by zero).
"""
import numpy as np

ACATOL = 1e-10
FLAG_RK, FLAG_FULL = 1, 2


# --------------------------------------------------------------------------
# cluster tree with admissibility (clustertree.h)
# --------------------------------------------------------------------------
class Tree:
    """``son [nc, 2]`` (-1 none), ``cind [nc, 2]`` first / last position
    (inclusive, as the library's tree), ``full`` / ``low`` leaf blocks."""

    def __init__(self, son, cind, full, low):
        self.son = np.asarray(son, dtype=np.int64)
        c = np.asarray(cind, dtype=np.int64)
        self.lo, self.hi = c[:, 0], c[:, 1] + 1
        self.ad = {}
        for r, cc in np.asarray(full, dtype=np.int64).reshape(-1, 2):
            self.ad[(int(r), int(cc))] = FLAG_FULL
        for r, cc in np.asarray(low, dtype=np.int64).reshape(-1, 2):
            self.ad[(int(r), int(cc))] = FLAG_RK
        self.n = int(self.hi[0])

    def leaf(self, i):
        return self.son[i, 0] < 0

    def sons(self, i, s):
        return int(self.son[i, s])

    def begin(self, i):
        """sons of i in order, or i itself for a leaf (treeiterator)"""
        return [i] if self.leaf(i) else [int(self.son[i, 0]), int(self.son[i, 1])]

    def nrows(self, i):
        return int(self.hi[i] - self.lo[i])

    def rel(self, i, j):
        """positions of cluster i inside its ancestor j (size(i, j))"""
        return slice(int(self.lo[i] - self.lo[j]), int(self.hi[i] - self.lo[j]))

    def rng(self, i):
        return slice(int(self.lo[i]), int(self.hi[i]))

    def admiss(self, r, c):
        return self.ad.get((r, c), 0)

    def pairs(self, r, c):
        """leaf blocks below (r, c) in the pair iterator's order"""
        out = []

        def walk(a, b):
            if self.admiss(a, b):
                out.append((a, b))
                return
            for x in self.begin(a):
                for y in self.begin(b):
                    walk(x, y)
        walk(r, c)
        return out


# --------------------------------------------------------------------------
# dense kernels (lu.cpp, aca.cpp, basemat.cpp)
# --------------------------------------------------------------------------
def cabs1(z):
    return np.abs(z.real) + np.abs(z.imag)


def aca(getrow, getcol, m, n, tol, kcap):
    """aca.cpp:150-218: L [m, r], R [n, r] with block ~ L R^T, at most kcap terms."""
    A = np.zeros((m, kcap), dtype=complex)
    B = np.zeros((n, kcap), dtype=complex)
    used = np.zeros(m, dtype=bool)
    r, nsum, k = 0, 0.0, 0
    while k < kcap:
        B[:, k] = getrow(r)
        if np.linalg.norm(B[:, k]) < ACATOL:
            break
        if k:
            B[:, k] -= B[:, :k] @ A[r, :k]
        c = int(np.argmax(cabs1(B[:, k])))
        if B[c, k] == 0:
            return A[:, :k], B[:, :k]
        B[:, k] *= 1.0 / B[c, k]
        A[:, k] = getcol(c)
        if k:
            A[:, k] -= A[:, :k] @ B[c, :k]
        used[r] = True
        r = int(np.argmax(cabs1(np.where(used, 0, A[:, k]))))
        nk = np.linalg.norm(A[:, k]) * np.linalg.norm(B[:, k])
        if nk < tol * nsum or used.all():
            break
        nsum = np.sqrt(nsum ** 2 + nk ** 2)
        k += 1
    rank = min(k + 1, kcap)
    return A[:, :rank], B[:, :rank]


def aca_full(M, tol, kmax):
    m, n = M.shape
    return aca(lambda i: M[i, :].copy(), lambda j: M[:, j].copy(), m, n, tol, min(m, n, kmax))


def aca_rk(L, R, tol, kmax):
    return aca(lambda i: R @ L[i, :], lambda j: L @ R[j, :], L.shape[0], R.shape[0], tol,
               min(L.shape[1], kmax))


def lu_dense(A):
    """lu.cpp:82-106: A = L U, L lower with its diagonal, U unit upper (no
    row interchanges), both returned in one array."""
    B = np.array(A, dtype=complex)
    n = B.shape[0]
    for j in range(n):
        B[j:, j] -= B[j:, :j] @ B[:j, j]
        B[j, j + 1:] = (B[j, j + 1:] - B[j, :j] @ B[:j, j + 1:]) / B[j, j]
    return B


def tri(A, uplo):
    """the triangle ?trsm reads: L with its diagonal, or U with a unit one"""
    if uplo == "L":
        return np.tril(A)
    return np.triu(A, 1) + np.eye(A.shape[0])


def trsm(side, B, trans, A, uplo):
    """lu.cpp:110-124: side 'L' op(A) X = B, side 'R' X op(A) = B."""
    T = tri(A, uplo)
    if trans == "T":
        T = T.T
    if side == "L":
        return np.linalg.solve(T, B)
    return np.linalg.solve(T.T, B.T).T


# --------------------------------------------------------------------------
# sub-matrices (submatrix.h)
# --------------------------------------------------------------------------
class Sub:
    """Block of cluster pair (row, col): full ``mat`` or low-rank ``lhs rhs^T``."""
    __slots__ = ("row", "col", "mat", "lhs", "rhs")

    def __init__(self, row, col, mat=None, lhs=None, rhs=None):
        self.row, self.col, self.mat, self.lhs, self.rhs = row, col, mat, lhs, rhs

    @property
    def flag(self):
        if self.lhs is not None:
            return FLAG_RK
        return FLAG_FULL if self.mat is not None else 0

    def copy(self):
        return Sub(self.row, self.col, *(None if a is None else a.copy() for a in (self.mat, self.lhs, self.rhs)))


class HOpts:
    def __init__(self, tol=1e-6, kmax=100):
        self.tol, self.kmax = tol, kmax


class HArith:
    """The H-matrix arithmetic of one cluster tree and option set."""

    def __init__(self, tree, tol=1e-6, kmax=100):
        self.t = tree
        self.o = HOpts(tol, kmax)

    # ---- sub-matrix helpers
    def convert(self, A, flag):
        """submatrix.h:104-118"""
        if A.flag == flag:
            return A
        if A.flag == FLAG_RK:
            return Sub(A.row, A.col, mat=A.lhs @ A.rhs.T)
        L, R = aca_full(A.mat, self.o.tol, self.o.kmax)
        return Sub(A.row, A.col, lhs=L, rhs=R)

    def truncate(self, A):
        """submatrix.h:127-133"""
        if A.flag == FLAG_RK:
            A.lhs, A.rhs = aca_rk(A.lhs, A.rhs, self.o.tol, self.o.kmax)
        return A

    def mask(self, A, r, c):
        """submatrix.h:136-143: A restricted to sub-clusters (r, c)"""
        t = self.t
        rr, cc = t.rel(r, A.row), t.rel(c, A.col)
        if A.flag == FLAG_FULL:
            return Sub(r, c, mat=A.mat[rr, cc].copy())
        return Sub(r, c, lhs=A.lhs[rr].copy(), rhs=A.rhs[cc].copy())

    def iadd(self, A, B):
        """A += B (submatrix.h:165-182); returns the result"""
        if A is None or A.flag == 0:
            return B.copy()
        if A.flag == FLAG_FULL:
            return Sub(A.row, A.col, mat=A.mat + B.mat)
        S = Sub(A.row, A.col, lhs=np.hstack([A.lhs, B.lhs]), rhs=np.hstack([A.rhs, B.rhs]))
        return self.truncate(S)

    @staticmethod
    def neg(A):
        if A.flag == FLAG_FULL:
            return Sub(A.row, A.col, mat=-A.mat)
        return Sub(A.row, A.col, lhs=-A.lhs, rhs=A.rhs.copy())

    def mul_sub(self, A, B, i, j, k):
        """C(i, j) = A(i, k) B(k, j) of two sub-matrices (submatrix.h:196-219)"""
        t = self.t
        fa, fb = A.flag, B.flag
        if fa == FLAG_FULL and fb == FLAG_FULL:
            return Sub(i, j, mat=A.mat[t.rel(i, A.row), t.rel(k, A.col)] @ B.mat[t.rel(k, B.row), t.rel(j, B.col)])
        if fa == FLAG_FULL and fb == FLAG_RK:
            return Sub(i, j, lhs=A.mat[t.rel(i, A.row), t.rel(k, A.col)] @ B.lhs[t.rel(k, B.row)],
                       rhs=B.rhs[t.rel(j, B.col)].copy())
        if fa == FLAG_RK and fb == FLAG_FULL:
            return Sub(i, j, lhs=A.lhs[t.rel(i, A.row)].copy(),
                       rhs=B.mat[t.rel(k, B.row), t.rel(j, B.col)].T @ A.rhs[t.rel(k, A.col)])
        S = A.rhs[t.rel(k, A.col)].T @ B.lhs[t.rel(k, B.row)]
        if S.shape[0] > S.shape[1]:
            return Sub(i, j, lhs=A.lhs[t.rel(i, A.row)] @ S, rhs=B.rhs[t.rel(j, B.col)].copy())
        return Sub(i, j, lhs=A.lhs[t.rel(i, A.row)].copy(), rhs=B.rhs[t.rel(j, B.col)] @ S.T)

    def cat(self, C, row, col):
        """submatrix.h:222-261; C is a list of rows of sub-matrices (1 or 2 x 1 or 2)"""
        m, n = len(C), len(C[0])
        if C[0][0].flag == FLAG_FULL:
            return Sub(row, col, mat=np.block([[C[a][b].mat for b in range(n)] for a in range(m)]))
        if m == 1 and n == 1:
            return Sub(row, col, lhs=C[0][0].lhs, rhs=C[0][0].rhs)

        def z(r, c):
            return np.zeros((r, c), dtype=complex)
        if m == 2 and n == 1:
            L0, L1 = C[0][0].lhs, C[1][0].lhs
            return Sub(row, col, lhs=np.block([[L0, z(L0.shape[0], L1.shape[1])], [z(L1.shape[0], L0.shape[1]), L1]]),
                       rhs=np.hstack([C[0][0].rhs, C[1][0].rhs]))
        if m == 1 and n == 2:
            R0, R1 = C[0][0].rhs, C[0][1].rhs
            return Sub(row, col, lhs=np.hstack([C[0][0].lhs, C[0][1].lhs]),
                       rhs=np.block([[R0, z(R0.shape[0], R1.shape[1])], [z(R1.shape[0], R0.shape[1]), R1]]))
        L00, L10, L01, L11 = C[0][0].lhs, C[1][0].lhs, C[0][1].lhs, C[1][1].lhs
        R00, R10, R01, R11 = C[0][0].rhs, C[1][0].rhs, C[0][1].rhs, C[1][1].rhs
        # columns: (0,0), (1,1), (1,0), (0,1)
        lhs = np.block([[L00, z(L00.shape[0], L11.shape[1]), z(L00.shape[0], L10.shape[1]), L01],
                        [z(L10.shape[0], L00.shape[1]), L11, L10, z(L11.shape[0], L01.shape[1])]])
        rhs = np.block([[R00, z(R00.shape[0], R11.shape[1]), R10, z(R00.shape[0], R01.shape[1])],
                        [z(R01.shape[0], R00.shape[1]), R11, z(R11.shape[0], R10.shape[1]), R01]])
        return Sub(row, col, lhs=lhs, rhs=rhs)

    # ---- H-matrices: dict (row, col) -> Sub over leaf pairs
    @staticmethod
    def find(A, i, j):
        if isinstance(A, Sub):
            return A
        return A.get((i, j))

    def add(self, A, B, i=0, j=0, C=None):
        """C(H) (+)= A(H) + B(H) over the pairs below (i, j) (hmatrix.h:166-185)"""
        out = {} if C is None else C
        for p in self.t.pairs(i, j):
            s = self.iadd(A[p].copy(), B[p])
            out[p] = self.iadd(out.get(p), s) if C is not None else s
        return out

    def subtract(self, A, B, i, j):
        """hmatrix.h:199-208"""
        return {p: self.iadd(A[p].copy(), self.neg(B[p])) for p in self.t.pairs(i, j)}

    def uminus(self, A, i, j):
        return {p: self.neg(A[p]) for p in self.t.pairs(i, j)}

    def add_mul2(self, A, B, i, j, k, flag):
        """C(sub) = A(i, k) B(k, j) with A or B subdivided (hmatrix.h:221-251)"""
        pA, pB = self.find(A, i, k), self.find(B, k, j)
        if pA is not None and pB is not None:
            return self.convert(self.mul_sub(pA, pB, i, j, k), flag)
        t = self.t
        bi, bj, bk = t.begin(i), t.begin(j), t.begin(k)
        C = [[None] * len(bj) for _ in bi]
        for a, ii in enumerate(bi):
            for b, jj in enumerate(bj):
                for kk in bk:
                    if pA is not None:
                        s = self.add_mul2(pA, B, ii, jj, kk, flag)
                    elif pB is not None:
                        s = self.add_mul2(A, pB, ii, jj, kk, flag)
                    else:
                        s = self.add_mul2(A, B, ii, jj, kk, flag)
                    C[a][b] = self.iadd(C[a][b], s)
        return self.cat(C, i, j)

    def add_mul(self, A, B, C, i, j, k):
        """C(H) += A(i, k) B(k, j) (hmatrix.h:254-287)"""
        pA, pB = self.find(A, i, k), self.find(B, k, j)
        adC = self.t.admiss(i, j)
        if adC == 0:
            t = self.t
            for ii in t.begin(i):
                for jj in t.begin(j):
                    for kk in t.begin(k):
                        self.add_mul(A if pA is None else pA, B if pB is None else pB, C, ii, jj, kk)
        elif pA is not None and pB is not None:
            C[(i, j)] = self.iadd(C.get((i, j)), self.convert(self.mul_sub(pA, pB, i, j, k), adC))
        else:
            C[(i, j)] = self.iadd(C.get((i, j)), self.add_mul2(A, B, i, j, k, adC))

    def mul(self, A, B, i=0, j=0, k=0):
        C = {}
        self.add_mul(A, B, C, i, j, k)
        return C

    # ---- inversion (hmatrix.h:310-345)
    def inv(self, A, i=0):
        t = self.t
        if t.leaf(i):
            return {(i, i): Sub(i, i, mat=np.linalg.inv(A[(i, i)].mat))}
        i0, i1 = t.sons(i, 0), t.sons(i, 1)
        Y = self.inv(A, i0)
        S = self.subtract(A, self.mul(A, self.mul(Y, A, i0, i1, i0), i1, i1, i0), i1, i1)
        C = self.inv(S, i1)
        tt = self.mul(Y, self.mul(A, self.mul(C, self.mul(A, Y, i1, i0, i0), i1, i0, i1), i0, i0, i1), i0, i0, i0)
        self.add(Y, tt, i0, i0, C)
        self.add_mul(self.uminus(Y, i0, i0), self.mul(A, C, i0, i1, i1), C, i0, i1, i0)
        self.add_mul(C, self.mul(A, self.uminus(Y, i0, i0), i1, i0, i0), C, i1, i0, i1)
        return C

    # ---- triangular solves of sub-matrices with a full leaf (lu.h:30-60)
    def rsolve_ss(self, B, A, i, j, uplo):
        t = self.t
        if B.flag == FLAG_FULL:
            return Sub(i, j, mat=trsm("R", B.mat[t.rel(i, B.row), t.rel(j, B.col)], "N", A.mat, uplo))
        return Sub(i, j, lhs=B.lhs[t.rel(i, B.row)].copy(),
                   rhs=trsm("L", B.rhs[t.rel(j, B.col)], "T", A.mat, uplo))

    def lsolve_ss(self, B, A, i, j, uplo):
        t = self.t
        if B.flag == FLAG_FULL:
            return Sub(i, j, mat=trsm("L", B.mat[t.rel(i, B.row), t.rel(j, B.col)], "N", A.mat, uplo))
        return Sub(i, j, lhs=trsm("L", B.lhs[t.rel(i, B.row)], "N", A.mat, uplo),
                   rhs=B.rhs[t.rel(j, B.col)].copy())

    # ---- sub-matrix with an H-matrix factor (lu.h:66-113)
    def rsolve_sh(self, B, A, i, j, uplo):
        t = self.t
        if t.admiss(j, j):
            return self.rsolve_ss(B, A[(j, j)], i, j, uplo)
        first, second = (0, 1) if uplo == "U" else (1, 0)
        j0, j1 = t.sons(j, first), t.sons(j, second)
        X = [None, None]
        X[first] = self.rsolve_sh(B, A, i, j0, uplo)
        rhs = self.iadd(self.mask(B, i, j1), self.neg(self.add_mul2(X[first], A, i, j1, j0, B.flag)))
        X[second] = self.rsolve_sh(rhs, A, i, j1, uplo)
        return self.truncate(self.cat([X], i, j))

    def lsolve_sh(self, B, A, i, j, uplo):
        t = self.t
        if t.admiss(i, i):
            return self.lsolve_ss(B, A[(i, i)], i, j, uplo)
        first, second = (0, 1) if uplo == "L" else (1, 0)
        i0, i1 = t.sons(i, first), t.sons(i, second)
        X = [None, None]
        X[first] = self.lsolve_sh(B, A, i0, j, uplo)
        rhs = self.iadd(self.mask(B, i1, j), self.neg(self.add_mul2(A, X[first], i1, j, i0, B.flag)))
        X[second] = self.lsolve_sh(rhs, A, i1, j, uplo)
        return self.truncate(self.cat([[X[0]], [X[1]]], i, j))

    # ---- H-matrix solves (lu.h:118-176)
    def rsolve(self, B, A, X, i, j, uplo):
        """X(i, j) op(A)(j, j) = B(i, j)"""
        t = self.t
        pA, pB = A.get((j, j)), B.get((i, j))
        if pA is not None and pB is not None:
            X[(i, j)] = self.rsolve_ss(pB, pA, i, j, uplo)
        elif pA is not None:
            for ii in t.begin(i):
                self.rsolve(B, A, X, ii, j, uplo)
        elif pB is None:
            js = t.begin(j)
            if uplo != "U":
                js = js[::-1]
            kf = t.sons(j, 0 if uplo == "U" else 1)
            for num, jj in enumerate(js):
                for ii in t.begin(i):
                    Bn = self.subtract(B, self.mul(X, A, ii, jj, kf), ii, jj) if num else B
                    self.rsolve(Bn, A, X, ii, jj, uplo)
        else:
            X[(i, j)] = self.rsolve_sh(pB, A, i, j, uplo)

    def lsolve(self, B, A, X, i, j, uplo):
        """op(A)(i, i) X(i, j) = B(i, j)"""
        t = self.t
        pA, pB = A.get((i, i)), B.get((i, j))
        if pA is not None and pB is not None:
            X[(i, j)] = self.lsolve_ss(pB, pA, i, j, uplo)
        elif pA is not None:
            for jj in t.begin(j):
                self.lsolve(B, A, X, i, jj, uplo)
        elif pB is None:
            is_ = t.begin(i)
            if uplo != "L":
                is_ = is_[::-1]
            kf = t.sons(i, 0 if uplo == "L" else 1)
            for num, ii in enumerate(is_):
                for jj in t.begin(j):
                    Bn = self.subtract(B, self.mul(A, X, ii, jj, kf), ii, jj) if num else B
                    self.lsolve(Bn, A, X, ii, jj, uplo)
        else:
            X[(i, j)] = self.lsolve_sh(pB, A, i, j, uplo)

    def lu(self, B, A=None, i=0):
        """lu.h:180-198: A = L U of B (leaf diagonals by lu_dense)"""
        A = {} if A is None else A
        t = self.t
        if t.leaf(i):
            A[(i, i)] = Sub(i, i, mat=lu_dense(B[(i, i)].mat))
            return A
        i0, i1 = t.sons(i, 0), t.sons(i, 1)
        self.lu(B, A, i0)
        self.lsolve(B, A, A, i0, i1, "L")
        self.rsolve(B, A, A, i1, i0, "U")
        self.lu(self.subtract(B, self.mul(A, A, i1, i1, i0), i1, i1), A, i1)
        return A

    def rsolve_lu(self, B, A, key="N"):
        """hmatrsolve.cpp: X (L U) = B"""
        X = {}
        if key in ("U", "N"):
            self.rsolve(B, A, X, 0, 0, "U")
        if key in ("L", "N"):
            self.rsolve(dict(X), A, X, 0, 0, "L")
        return X

    def lsolve_lu(self, B, A, key="N"):
        """hmatlsolve.cpp: X with (L U) X = B"""
        X = {}
        if key in ("L", "N"):
            self.lsolve(B, A, X, 0, 0, "L")
        if key in ("U", "N"):
            self.lsolve(dict(X) if key == "N" else B, A, X, 0, 0, "U")
        return X

    def solve_vec(self, A, b, i=0, uplo="L"):
        """lu.h:204-221: op(A) x = b in place on b [n, N] (cluster order)"""
        t = self.t
        if t.admiss(i, i):
            rs = t.rng(i)
            b[rs] = trsm("L", b[rs], "N", A[(i, i)].mat, uplo)
            return
        i0 = t.sons(i, 0) if uplo == "L" else t.sons(i, 1)
        i1 = t.sons(i, 1) if uplo == "L" else t.sons(i, 0)
        self.solve_vec(A, b, i0, uplo)
        for p in t.pairs(i1, i0):
            b[t.rng(p[0])] -= self.sub_full(A[p]) @ b[t.rng(p[1])]
        self.solve_vec(A, b, i1, uplo)

    def solve(self, A, b, key="N"):
        """hmatsolve.cpp: L then U"""
        x = np.array(b, dtype=complex)
        if key in ("L", "N"):
            self.solve_vec(A, x, 0, "L")
        if key in ("U", "N"):
            self.solve_vec(A, x, 0, "U")
        return x

    # ---- helpers outside the C++ library
    @staticmethod
    def sub_full(S):
        return S.mat if S.flag == FLAG_FULL else S.lhs @ S.rhs.T

    def full(self, A):
        """expanded matrix in cluster order (hmatrix.h full)"""
        M = np.zeros((self.t.n, self.t.n), dtype=complex)
        for (r, c), S in A.items():
            M[self.t.rng(r), self.t.rng(c)] = self.sub_full(S)
        return M

    def matvec(self, A, x):
        y = np.zeros_like(x, dtype=complex)
        for (r, c), S in A.items():
            if S.flag == FLAG_FULL:
                y[self.t.rng(r)] += S.mat @ x[self.t.rng(c)]
            else:
                y[self.t.rng(r)] += S.lhs @ (S.rhs.T @ x[self.t.rng(c)])
        return y

    def scale(self, A, d, side):
        """mtimes1.m: diag(d) A (side 'L', rows) or A diag(d) (side 'R');
        d in cluster order"""
        out = {}
        for (r, c), S in A.items():
            if side == "L":
                dr = d[self.t.rng(r)][:, None]
                out[(r, c)] = Sub(r, c, mat=S.mat * dr) if S.flag == FLAG_FULL else \
                    Sub(r, c, lhs=S.lhs * dr, rhs=S.rhs.copy())
            else:
                dc = d[self.t.rng(c)]
                out[(r, c)] = Sub(r, c, mat=S.mat * dc[None, :]) if S.flag == FLAG_FULL else \
                    Sub(r, c, lhs=S.lhs.copy(), rhs=S.rhs * dc[:, None])
        return out


def from_blocks(tree, full, low, vals, lhs, rhs):
    """H-matrix dict from block lists (the oracle's HMatrix layout)."""
    A = {}
    for (r, c), v in zip(full, vals):
        A[(int(r), int(c))] = Sub(int(r), int(c), mat=np.array(v, dtype=complex))
    for (r, c), L, R in zip(low, lhs, rhs):
        A[(int(r), int(c))] = Sub(int(r), int(c), lhs=np.array(L, dtype=complex), rhs=np.array(R, dtype=complex))
    return A


# --------------------------------------------------------------------------
# the 'hmat' preconditioner (initprecond.m, mfun.m)
# --------------------------------------------------------------------------
class HmatPrecond:
    """G1i, G2i, Sigma1, Deltai, Sigmai of initprecond.m ('hmat') from the
    H-matrices G1, H1, G2, H2 (dicts on ``tree``), per-face eps1, eps2 and
    normals in face order; ``perm`` maps cluster positions to faces."""

    def __init__(self, tree, perm, G1, H1, G2, H2, k, eps1, eps2, nvec, htol=1e-6, kmax=4):
        self.t = tree
        self.perm = np.asarray(perm)
        self.k = k
        h = self.h = HArith(tree, htol, kmax)
        P = self.perm
        e1, e2 = np.asarray(eps1)[P], np.asarray(eps2)[P]
        nv = np.asarray(nvec)[P]
        self.eps1, self.eps2, self.nvec_f = np.asarray(eps1), np.asarray(eps2), np.asarray(nvec)
        self.G1i = h.lu(G1)
        self.G2i = h.lu(G2)
        self.Sigma1 = h.rsolve_lu(H1, self.G1i)
        Sigma2 = h.rsolve_lu(H2, self.G2i)
        self.Deltai = h.inv(h.add(self.Sigma1, h.uminus(Sigma2, 0, 0)))
        deps = e1 - e2
        # fun(Deltai, nvec): nvec1 D nvec1 + nvec2 D nvec2 + nvec3 D nvec3
        F = None
        for c in range(3):
            term = h.scale(h.scale(self.Deltai, nv[:, c], "L"), nv[:, c], "R")
            F = term if F is None else h.add(F, term)
        S = h.add(h.scale(self.Sigma1, e1, "L"), h.uminus(h.scale(Sigma2, e2, "L"), 0, 0))
        S = h.add(S, h.scale(h.scale(F, k ** 2 * deps, "L"), deps, "R"))
        self.Sigmai = h.lu(S)

    def _c(self, x):
        return x[self.perm]

    def _f(self, xc):
        out = np.empty_like(xc)
        out[self.perm] = xc
        return out

    def mul(self, A, x):
        sh = x.shape
        y = self.h.matvec(A, self._c(x).reshape(sh[0], -1))
        return self._f(y).reshape(sh)

    def sol(self, A, x):
        sh = x.shape
        y = self.h.solve(A, self._c(x).reshape(sh[0], -1))
        return self._f(y).reshape(sh)

    def apply(self, phi, a, De, alpha):
        """mfun.m:36-52 with matmul1 = H x, matmul2 = H-LU solve; phi, De
        [n, P], a, alpha [n, 3, P] (face order)"""
        k, nvec = self.k, self.nvec_f
        e1, e2 = self.eps1, self.eps2

        def outer(nv, s):
            return nv[:, :, None] * s[:, None, :]

        def inner(nv, v):
            return np.einsum("ik,ikp->ip", nv, v)
        alpha = alpha - self.mul(self.Sigma1, a) + 1j * k * outer(nvec, e1[:, None] * phi)
        De = De - e1[:, None] * self.mul(self.Sigma1, phi) + 1j * k * e1[:, None] * inner(nvec, a)
        sig2 = self.sol(self.Sigmai, De + 1j * k * (e1 - e2)[:, None] * inner(nvec, self.mul(self.Deltai, alpha)))
        h2 = self.mul(self.Deltai, 1j * k * outer(nvec, (e1 - e2)[:, None] * sig2) + alpha)
        sig1 = self.sol(self.G1i, sig2 + phi)
        h1 = self.sol(self.G1i, h2 + a)
        sig2 = self.sol(self.G2i, sig2)
        h2 = self.sol(self.G2i, h2)
        return sig1, h1, sig2, h2
