"""The H-matrix oracle (oracle/hlu_ref.py) pinned against dense linear algebra.

With truncation tight enough (htol 1e-12, kmax 100) the restated hlib
recursion must reproduce exact results: L U = A, X (L U) = B, A^-1 A = I,
sums, and the 'hmat' preconditioner of initprecond.m / mfun.m must equal the
dense chain of mldivide.m (the pinned BemRet oracle).  With the reference's
preconditioner options (kmax 4) the factors are approximations with
truncated blocks.  CPU only: a 284-face sphere with jittered vertices, leaves of
at most 16 faces (62 low-rank blocks).
"""
import numpy as np
import pytest

from oracle import hlu_ref as HL
from oracle import hmatrix_ref as HR
from oracle import mnpbem_ref as R


@pytest.fixture(scope="module")
def prob():
    from mnpbem_gb300 import shapes
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    v, f = shapes.trisphere(144, 20.0)
    rng = np.random.default_rng(2)
    v = v * (1 + 0.02 * rng.standard_normal((v.shape[0], 1)))
    cp = R.ComParticle([R.EpsConst(1.77), R.drude_eps()], [R.Particle(v, f, q)], [[2, 1]], [True])
    bem = R.BemRet(cp)
    bem.initmat(600.0)
    ct = HR.ClusterTree(cp.pos, np.zeros(cp.n, dtype=int), 16)
    full, low = ct.admissibility()
    T = HL.Tree(ct.son, ct.cind, full, low)
    P = ct.perm

    def hm(M):
        Mc = M[np.ix_(P, P)]
        vals = [Mc[T.rng(r), T.rng(c)] for r, c in full]
        ls, rs = [], []
        for r, c in low:
            L, Rr = HL.aca_full(Mc[T.rng(r), T.rng(c)], 1e-12, 100)
            ls.append(L)
            rs.append(Rr)
        return HL.from_blocks(T, full, low, vals, ls, rs), Mc
    mats = {k: hm(M) for k, M in (("G1", bem.G1), ("H1", bem.H1), ("G2", bem.G2), ("H2", bem.H2))}
    return {"cp": cp, "bem": bem, "T": T, "P": P, "mats": mats, "nlow": len(low)}


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_tree_has_low_rank_blocks(prob):
    assert prob["nlow"] > 10


def test_exact_arithmetic_at_tight_truncation(prob):
    h = HL.HArith(prob["T"], 1e-12, 100)
    G1, G1c = prob["mats"]["G1"]
    H1, H1c = prob["mats"]["H1"]
    n = G1c.shape[0]
    LU = h.lu(G1)
    F = h.full(LU)
    L, U = np.tril(F), np.triu(F, 1) + np.eye(n)
    assert rel(L @ U, G1c) < 1e-11
    X = h.rsolve_lu(H1, LU)
    assert rel(h.full(X) @ G1c, H1c) < 1e-11
    Gi = h.inv(G1)
    assert np.linalg.norm(h.full(Gi) @ G1c - np.eye(n)) / np.sqrt(n) < 1e-11
    b = np.random.default_rng(3).standard_normal((n, 2)) + 0j
    assert rel(G1c @ h.solve(LU, b), b) < 1e-11
    assert rel(h.full(h.add(G1, h.uminus(H1, 0, 0))), G1c - H1c) < 1e-12
    d = np.arange(1, n + 1) * (1 + 0.5j)
    assert rel(h.full(h.scale(G1, d, "L")), d[:, None] * G1c) < 1e-13
    assert rel(h.full(h.scale(G1, d, "R")), G1c * d[None, :]) < 1e-13


def test_preconditioner_equals_dense_chain(prob):
    """initprecond.m / mfun.m ('hmat') against mldivide.m's dense chain"""
    cp, bem, P = prob["cp"], prob["bem"], prob["P"]
    mats = [prob["mats"][k][0] for k in ("G1", "H1", "G2", "H2")]
    e1, e2 = cp.eps_faces(600.0, 0), cp.eps_faces(600.0, 1)
    pc = HL.HmatPrecond(prob["T"], P, *mats, bem.k, e1, e2, bem.nvec, htol=1e-12, kmax=100)
    rng = np.random.default_rng(4)
    n = cp.n
    c = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)
    phi, De, a, al = c(n, 1), c(n, 1), c(n, 3, 1), c(n, 3, 1)
    got = pc.apply(phi, a, De, al)
    want = bem.chain(phi, a, al, De)
    for k, g in zip(("sig1", "h1", "sig2", "h2"), got):
        assert rel(g, want[k]) < 1e-10, k


def test_reference_options_truncate(prob):
    """kmax 4: blocks formed by concatenation are truncated to rank 4 or less
    (blocks only solved against a leaf keep their rank, as in lu.h), and the
    factors are an approximation, not the exact ones"""
    h = HL.HArith(prob["T"], 1e-6, 4)
    G1, G1c = prob["mats"]["G1"]
    LU = h.lu(G1)
    inranks = {k: S.lhs.shape[1] for k, S in G1.items() if S.flag == HL.FLAG_RK}
    ranks = {k: S.lhs.shape[1] for k, S in LU.items() if S.flag == HL.FLAG_RK}
    assert any(ranks[k] <= 4 < inranks[k] for k in ranks)
    F = h.full(LU)
    n = G1c.shape[0]
    L, U = np.tril(F), np.triu(F, 1) + np.eye(n)
    e = rel(L @ U, G1c)
    assert 1e-12 < e < 1e-1


def test_lsolve_and_product_exact_at_tight_truncation(prob):
    h = HL.HArith(prob["T"], 1e-12, 100)
    G1, G1c = prob["mats"]["G1"]
    H1, H1c = prob["mats"]["H1"]
    X = h.lsolve_lu(H1, h.lu(G1))
    assert rel(G1c @ h.full(X), H1c) < 1e-11
    assert rel(h.full(h.mul(G1, H1)), G1c @ H1c) < 1e-11


def test_oracle_iterative_solver_with_hmat_preconditioner(prob):
    """bemretiter with precond='hmat' in the oracle: GMRES converges in a few
    steps (the preconditioner approximates the inverse to ~1e-3) and the
    charges approach the direct solve to the tolerances' order"""
    cp = prob["cp"]
    pw = R.PlaneWaveRet([[1, 0, 0]], [[0, 0, 1]], None)
    exc = pw.potential(cp, 600.0)
    it = HR.BemRetIter(cp, cleaf=16, precond="hmat", maxit=100)
    sig = it.solve(exc)
    assert it.flag == 0 and it.iter <= 10
    direct = R.BemRet(cp).solve(exc)
    for k in ("sig1", "sig2"):
        assert rel(sig[k], direct[k]) < 1e-3, k
    plain = HR.BemRetIter(cp, cleaf=16, precond=None, maxit=300)
    plain.solve(exc)
    assert plain.iter > it.iter


@pytest.mark.parametrize("cleaf", [16, 32])
def test_tree_views_agree(cleaf):
    """the library's tree arrays (treearrays, handed to mnpbem_hm_create) and
    the H-arithmetic oracle's Tree describe the same partition: the pair
    iterator below the root visits every leaf block once"""
    import mnpbem_gb300 as m
    from mnpbem_gb300.hmatrix import treearrays
    cp = m.comparticle([m.epsconst(1.77), m.epsconst(-8 + 1j)], [m.trisphere(256, 20.0)], [[2, 1]], 1)
    hp = m.hpartition(cp, cleaf)
    ta = treearrays.of(hp)
    assert ta.n == cp.n and ta.c.nfull == hp.full.shape[0] and ta.c.nlow == hp.low.shape[0]
    T = HL.Tree(ta.son, ta.cind, ta.full, ta.low)
    pairs = T.pairs(0, 0)
    blocks = {tuple(map(int, b)) for b in np.vstack([ta.full, ta.low])}
    assert len(pairs) == len(blocks) and set(pairs) == blocks
    assert sum(ta.rows(r) * ta.rows(c) for r, c in pairs) == cp.n ** 2
    for r, c in ta.full:
        assert T.leaf(int(r)) and T.leaf(int(c))
