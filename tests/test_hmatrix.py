"""Host side of the iterative solver (BEM/@bemretiter with H-matrices).

* the product's cluster tree and block partition (clustertree.m,
  bisection.m, admissibility.m) equal the oracle's, for one and two
  particles and several leaf sizes;
* the oracle's ACA (mex/hlib/aca.cpp) approximates the dense G1, H1, G2, H2
  to the order of htol (expanded H-matrices within 10 htol of the dense
  matrices in the Frobenius norm);
* the oracle's GMRES (with and without restarts), CGS and BiCGStab reproduce
  numpy's solve on random systems and converge in one iteration with an exact
  preconditioner, and the oracle's iterative BEM solve (preconditioned and
  plain) reaches the direct bemret solution within tol-scaled bounds.
"""
import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes
from oracle import hmatrix_ref as HR
from oracle import mnpbem_ref as R


def two_spheres():
    p1 = m.trisphere(400, 30.0)
    v, f = shapes.trisphere(144, 20.0)
    p2 = m.particle(v + np.array([45.0, 0.0, 0.0]), f)
    return m.comparticle([m.epsconst(1.77), m.epsconst(-8 + 1j)], [p1, p2], [[2, 1], [2, 1]], 1, 2), [p1, p2]


@pytest.mark.parametrize("cleaf", [16, 32, 64])
def test_cluster_tree_matches_oracle(cleaf):
    for cp, parts in ((m.comparticle([m.epsconst(1.77), m.epsconst(-8 + 1j)], [m.trisphere(400, 30.0)], [[2, 1]], 1),
                       None), two_spheres()):
        hp = m.hpartition(cp, cleaf)
        npart = 1 if parts is None else len(parts)
        counts = [cp.n] if parts is None else [q.n for q in parts]
        ot = HR.ClusterTree(cp.pos, np.repeat(np.arange(npart), counts), cleaf)
        of, ol = ot.admissibility()
        t = hp.tree
        for a, b in ((t.son, ot.son), (t.cind, ot.cind), (t.perm, ot.perm), (t.ipart, ot.ipart)):
            assert np.array_equal(a, b)
        assert np.array_equal(t.mid, ot.mid) and np.array_equal(t.rad, ot.rad)
        assert np.array_equal(hp.full, np.asarray(of).reshape(-1, 2))
        assert np.array_equal(hp.low, np.asarray(ol).reshape(-1, 2))
        # partition of the n x n matrix, leaves no larger than cleaf
        sz = t.cind[:, 1] - t.cind[:, 0] + 1
        area = np.sum(sz[hp.full[:, 0]] * sz[hp.full[:, 1]]) + np.sum(sz[hp.low[:, 0]] * sz[hp.low[:, 1]])
        assert area == cp.n ** 2
        assert np.all(sz[t.leaves] <= cleaf)
        if npart == 2:
            assert hp.low.shape[0] > 0 and np.all(t.ipart[hp.low] >= 0)


def oracle_sphere(nverts=400, diameter=30.0):
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    v, f = shapes.trisphere(nverts, diameter)
    return R.ComParticle([R.EpsConst(1.77), R.drude_eps()], [R.Particle(v, f, q)], [[2, 1]], [True])


def test_aca_approximates_dense_matrices():
    cp = oracle_sphere()
    it = HR.BemRetIter(cp, cleaf=32, htol=1e-6)
    it.initmat(600.0)
    b = it.bem
    assert len(it.H[0].low) > 100
    for H, D in zip(it.H, (b.G1, b.H1, b.G2, b.H2)):
        err = np.linalg.norm(H.full_matrix() - D) / np.linalg.norm(D)
        assert err < 1e-5, err
        assert 1 <= max(H.ranks()) <= 40


def test_aca_single_block_tolerance():
    # one admissible block of the exp(ikr)/r kernel: error tracks htol
    rng = np.random.default_rng(3)
    X = rng.random((300, 3))
    Y = rng.random((260, 3)) + np.array([3.0, 0.0, 0.0])
    k = 0.3 + 0.01j
    K = np.exp(1j * k * np.linalg.norm(X[:, None] - Y[None], axis=2)) / np.linalg.norm(X[:, None] - Y[None], axis=2)
    prev = None
    for tol in (1e-3, 1e-6, 1e-9):
        L, Rr = HR.aca(lambda i: K[i], lambda j: K[:, j], 300, 260, tol, 100)
        err = np.linalg.norm(L @ Rr.T - K) / np.linalg.norm(K)
        assert err < 30 * tol, (tol, err)
        if prev is not None:
            assert L.shape[1] >= prev
        prev = L.shape[1]


@pytest.mark.parametrize("restart", [None, 7])
def test_oracle_gmres_random_system(restart):
    rng = np.random.default_rng(5)
    n = 120
    A = np.eye(n) * 4 + (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    x, flag, relres, it = HR.gmres(lambda v: A @ v, b, tol=1e-10, maxit=200, restart=restart)
    assert flag == 0 and relres <= 1e-10
    assert np.linalg.norm(x - np.linalg.solve(A, b)) / np.linalg.norm(x) < 1e-8
    # a preconditioner that is the exact inverse converges in one step
    Ai = np.linalg.inv(A)
    x1, flag1, _, it1 = HR.gmres(lambda v: A @ v, b, tol=1e-10, maxit=20, restart=restart, mfun=lambda v: Ai @ v)
    assert flag1 == 0 and it1 == 1


def test_oracle_iterative_solve_matches_direct():
    cp = oracle_sphere()
    pw = R.PlaneWaveRet([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]], None)
    exc = pw.potential(cp, 600.0)
    direct = R.BemRet(cp).solve(exc)
    pre = HR.BemRetIter(cp, cleaf=32)
    s = pre.solve(exc)
    assert pre.flag == 0 and pre.iter <= 3
    plain = HR.BemRetIter(cp, cleaf=32, precond=None, maxit=300)
    s2 = plain.solve(exc)
    assert plain.flag == 0 and plain.iter > 20
    for k in ("sig1", "sig2", "h1", "h2"):
        scale = np.max(np.abs(direct[k]))
        assert np.max(np.abs(s[k] - direct[k])) / scale < 1e-5, k
        assert np.max(np.abs(s2[k] - direct[k])) / scale < 1e-3, k


@pytest.mark.parametrize("solver", ["cgs", "bicgstab"])
def test_oracle_cgs_bicgstab_random_system(solver):
    rng = np.random.default_rng(7)
    n = 120
    A = np.eye(n) * 4 + (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    fn = HR.cgs if solver == "cgs" else HR.bicgstab
    x, flag, relres, it = fn(lambda v: A @ v, b, tol=1e-10, maxit=200)
    assert flag == 0 and relres < 1e-9
    assert np.linalg.norm(x - np.linalg.solve(A, b)) / np.linalg.norm(x) < 1e-8
    # an exact preconditioner converges in one iteration
    Ai = np.linalg.inv(A)
    x1, flag1, _, it1 = fn(lambda v: A @ v, b, tol=1e-10, maxit=20, mfun=lambda v: Ai @ v)
    assert flag1 == 0 and it1 == 1
