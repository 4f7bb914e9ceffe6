"""FP64 NumPy adjoint gradient of the plane-wave extinction cross section.

Test infrastructure (the oracle): the reference (MNPBEM) has no gradients, so
this module restates the forward path of ``mnpbem_ref`` analytically
differentiated and is itself checked against central finite differences of
``mnpbem_ref``.  Scope: one closed particle (inside medium 2, outside medium 1
= excitation medium), flat faces, the derivative taken with the refinement
pattern held fixed.

Forward path (``BEM/@bemretiter/private/afun.m:6-35`` for the operator A,
``mldivide.m`` for its inverse, ``@planewaveret/extinction.m:12-16`` and
``@spectrumret/farfield.m:15-74`` for J):

    A x = b,   x = (sig1, h1, sig2, h2),  b = (phi, a, De, alpha)
    J = ext = 4 pi / k Im(pol* . e(dir)) = Re(w^T x)

Adjoint: A^T lam = w,  dJ = Re(lam^T (db - dA x)) + (dJ/dtheta at fixed x).
``lam^T dA x`` is the contraction of dG1, dH1, dG2, dH2 with the weight
matrices W (outer products of lam and x, see ``weights``) plus the explicit
normals / eps of the alpha and De rows.  The derivatives of the matrix
entries follow ``Greenfun/@greenret/private/eval1.m`` (far pairs), the
Taylor coefficients of ``greenret/private/init.m`` (near pairs, self
elements) and the closed-surface sum of ``compgreenret/private/initclosed.m``.
"""
import math

import numpy as np

from . import mnpbem_ref as R


def make_problem(verts, faces, quad, eps_out, eps_in, pattern=None, order=5):
    """ComParticle of one closed particle (inside eps_in, outside eps_out)."""
    p = R.Particle(verts, faces, quad)
    cp = R.ComParticle([R.EpsConst(eps_out), R.EpsConst(eps_in)], [p], [[2, 1]], [True])
    bem = R.BemRet(cp, order=order, pattern=pattern)
    return cp, bem


def extinction(verts, faces, quad, eps_out, eps_in, enei, pol, dirv, pattern=None):
    """J = ext for one polarisation (forward oracle)."""
    cp, bem = make_problem(verts, faces, quad, eps_out, eps_in, pattern)
    pw = R.PlaneWaveRet([pol], [dirv], None)
    sig = bem.solve(pw.potential(cp, enei))
    return float(pw.extinction(cp, sig)[0])


# --------------------------------------------------------------- operator
def afun_matrix(bem, enei):
    """Dense 8n x 8n matrix of afun.m (unknowns [sig1, h1, sig2, h2],
    equations [phi, a, De, alpha]; vector fields component-major [3][n])."""
    cp = bem.p
    n = cp.n
    k = 2 * np.pi / enei
    e1 = cp.eps_faces(enei, 0)
    e2 = cp.eps_faces(enei, 1)
    G1, H1, G2, H2 = bem.matrices(enei)
    nv = cp.nvec
    A = np.zeros((8 * n, 8 * n), dtype=complex)
    s1, h1, s2, h2 = 0, n, 4 * n, 5 * n          # unknown offsets
    ph, ea, de, al = 0, n, 4 * n, 5 * n          # equation offsets
    A[ph:ph + n, s1:s1 + n] = G1
    A[ph:ph + n, s2:s2 + n] = -G2
    for c in range(3):
        A[ea + c * n:ea + (c + 1) * n, h1 + c * n:h1 + (c + 1) * n] = G1
        A[ea + c * n:ea + (c + 1) * n, h2 + c * n:h2 + (c + 1) * n] = -G2
        A[al + c * n:al + (c + 1) * n, h1 + c * n:h1 + (c + 1) * n] = H1
        A[al + c * n:al + (c + 1) * n, h2 + c * n:h2 + (c + 1) * n] = -H2
        A[al + c * n:al + (c + 1) * n, s1:s1 + n] = -1j * k * (nv[:, c] * e1)[:, None] * G1
        A[al + c * n:al + (c + 1) * n, s2:s2 + n] = 1j * k * (nv[:, c] * e2)[:, None] * G2
        A[de:de + n, h1 + c * n:h1 + (c + 1) * n] = -1j * k * (nv[:, c] * e1)[:, None] * G1
        A[de:de + n, h2 + c * n:h2 + (c + 1) * n] = 1j * k * (nv[:, c] * e2)[:, None] * G2
    A[de:de + n, s1:s1 + n] = e1[:, None] * H1
    A[de:de + n, s2:s2 + n] = -e2[:, None] * H2
    return A


def pack_x(sig1, h1, sig2, h2):
    return np.concatenate([sig1, h1.T.ravel(), sig2, h2.T.ravel()])


def unpack_eq(v, n):
    """[phi, a (3n), De, alpha (3n)] -> phi [n], a [n,3], De [n], alpha [n,3]."""
    return v[:n], v[n:4 * n].reshape(3, n).T, v[4 * n:5 * n], v[5 * n:].reshape(3, n).T


def chain_transpose(bem, enei, gs1, gh1, gs2, gh2):
    """A^{-T} g through the transposed mldivide chain (the GPU algorithm):
    the steps of mldivide.m in reverse order with every matrix transposed.
    g = (gs1 [n], gh1 [n,3], gs2 [n], gh2 [n,3]) -> (lphi, la, lDe, lalpha)."""
    bem.initmat(enei)
    k, nv = bem.k, bem.nvec
    L1, L2 = bem.L1, bem.L2
    G1i, G2i, S1, Di, Si = bem.G1i, bem.G2i, bem.Sigma1, bem.Deltai, bem.Sigmai
    T = lambda M, v: M.T @ v
    gS2 = T(G2i, gs2)                         # sig2 = G2i s2
    gH2p = T(G2i, gh2)                        # h2 = G2i h2'
    t = T(G1i, gs1)                           # sig1 = G1i (s2 + phi)
    gS2 = gS2 + t
    gphi = t.copy()
    t = T(G1i, gh1)                           # h1 = G1i (h2' + a)
    gH2p = gH2p + t
    ga = t.copy()
    t = T(Di, gH2p)                           # h2' = Di (ik n x ((L1 - L2) s2) + alpha')
    gAl = t.copy()
    gS2 = gS2 + 1j * k * (L1 - L2) * np.sum(nv * t, 1)
    t = T(Si, gS2)                            # s2 = Si (De' + ik n . ((L1 - L2) Di alpha'))
    gDe = t.copy()
    gAl = gAl + T(Di, 1j * k * (L1 - L2) * nv * t[:, None])
    # De' = De - S1 L1 phi + ik n . (L1 a)
    gphi = gphi - L1 * T(S1, gDe)
    ga = ga + 1j * k * L1 * nv * gDe[:, None]
    # alpha' = alpha - S1 a + ik n x (L1 phi)
    ga = ga - T(S1, gAl)
    gphi = gphi + 1j * k * L1 * np.sum(nv * gAl, 1)
    return gphi, ga, gDe, gAl


# ------------------------------------------------------------ geometry
def _tri_area_grad(a, b, c, g_area):
    """Gradient of area = |(b - a) x (c - a)| / 2 onto (a, b, c)."""
    N = np.cross(b - a, c - a)
    nn = np.linalg.norm(N, axis=-1, keepdims=True)
    gN = 0.5 * g_area[..., None] * N / nn
    ge1 = np.cross(c - a, gN)
    ge2 = np.cross(gN, b - a)
    return -(ge1 + ge2), ge1, ge2


def _norm_flat_grad(p, g_pos, g_nvec, g_area, gv):
    """Chain rule of norm_flat.m: centroid, unit normal and area -> vertices.
    Quadrilaterals: area of both triangles, normal of the larger one."""
    v, f = p.verts, p.faces
    for i in range(p.n):
        idx = f[i][f[i] >= 0]
        gv[idx] += g_pos[i] / idx.size
        tris = [(idx[0], idx[1], idx[2])]
        if idx.size == 4:
            tris.append((idx[2], idx[3], idx[0]))
        areas = []
        for (i1, i2, i3) in tris:
            N = np.cross(v[i1] - v[i2], v[i3] - v[i2])
            areas.append(0.5 * np.linalg.norm(N))
        big = 1 if (len(tris) == 2 and areas[1] > areas[0]) else 0
        for t, (i1, i2, i3) in enumerate(tris):
            e1, e2 = v[i1] - v[i2], v[i3] - v[i2]
            N = np.cross(e1, e2)
            nN = np.linalg.norm(N)
            nh = N / nN
            gN = 0.5 * g_area[i] * nh
            if t == big:
                gn = g_nvec[i]
                gN = gN + (gn - nh * np.dot(nh, gn)) / nN
            ge1 = np.cross(e2, gN)
            ge2 = np.cross(gN, e1)
            gv[i1] += ge1
            gv[i3] += ge2
            gv[i2] -= ge1 + ge2


def _quad_points_faces(p, j):
    """Rule-18 points of face j: positions, weights, (triangle vertex ids, barycentric, rule weight)."""
    q = p.quad
    f = p.faces[j]
    idx = f[f >= 0]
    tris = [(idx[0], idx[1], idx[2])]
    if idx.size == 4:
        tris.append((idx[2], idx[3], idx[0]))
    out = []
    for (a, b, c) in tris:
        va, vb, vc = p.verts[a], p.verts[b], p.verts[c]
        area = 0.5 * np.linalg.norm(np.cross(vb - va, vc - va))
        bary = np.stack([q.x, q.y, 1 - q.x - q.y], 1)
        pts = bary @ np.stack([va, vb, vc])
        out.append(((a, b, c), bary, q.w, area, pts))
    return out


# ------------------------------------------------------------- gradient
def weights(cp, enei, lam, x):
    """Per-face factors of lam^T dA x (one polarisation).

    G1_ij weight = u1_i sig1_j + v1_i . h1_j,   G2_ij: -(u2_i sig2_j + v2_i . h2_j)
    H1_ij weight = lal_i . h1_j + e1 lDe_i sig1_j,  H2_ij: -(lal_i . h2_j + e2 lDe_i sig2_j)
    """
    lphi, la, lDe, lal = lam
    s1, h1, s2, h2 = x
    k = 2 * np.pi / enei
    nv = cp.nvec
    e1 = cp.eps_faces(enei, 0)
    e2 = cp.eps_faces(enei, 1)
    ln = np.sum(lal * nv, 1)
    u1 = lphi - 1j * k * e1 * ln
    v1 = la - 1j * k * (e1 * lDe)[:, None] * nv
    u2 = lphi - 1j * k * e2 * ln
    v2 = la - 1j * k * (e2 * lDe)[:, None] * nv
    WG1 = np.outer(u1, s1) + v1 @ h1.T
    WG2 = -(np.outer(u2, s2) + v2 @ h2.T)
    WH1 = lal @ h1.T + np.outer(e1 * lDe, s1)
    WH2 = -(lal @ h2.T + np.outer(e2 * lDe, s2))
    return WG1, WH1, WG2, WH2


def _fact(o):
    return float(math.factorial(o))


def ext_gradient(verts, faces, quad, eps_out, eps_in, enei, pol, dirv, order=5, check_chain=False):
    """Adjoint gradient of ext: returns (J, dJ/dverts [nv, 3], dJ/deps_in as
    dJ/dRe(eps) + i dJ/dIm(eps), dict of intermediate pieces)."""
    return cross_section_gradient(verts, faces, quad, eps_out, eps_in, enei, pol, dirv, "ext", None, order,
                                  check_chain)


def sca_rhs(cp, sig, pw, enei):
    """dJ/dx of the scattering cross section (scattering.m:14-31 with the far
    fields of farfield.m:15-74): J = sum_d c_d Re(n_d . (e_d x conj(h_d))),
    c_d = area_d / nb, e_d = sum_i Phi_di (i k0 h2_i - i k dir_d sig2_i),
    h_d = sum_i Phi_di i k dir_d x h2_i, Phi_di = exp(-i k dir_d . r_i) A_i.
    dJ = Re(g . dx) with g_h2_i = sum_d c_d Phi_di [i k0 (h_d* x n_d)
    + i k ((n_d x e_d*) x dir_d)], g_sig2_i = -i k sum_d c_d Phi_di dir_d . (h_d* x n_d).
    Returns (g_sig2, g_h2, dJ/dpos explicit, dJ/darea explicit)."""
    pinf = pw.pinfty
    dirs, ad = pinf.nvec, pinf.area
    e, h, k = pw.farfield(cp, sig, dirs)
    e, h = e[:, :, 0], h[:, :, 0]
    k0 = 2 * np.pi / enei
    nb = np.sqrt(cp.eps[0](enei)[0])
    c = ad / nb
    pos, area = cp.pos, cp.area
    Phi = np.exp(-1j * k * dirs @ pos.T) * area[None, :]          # [d, i]
    A1 = np.cross(np.conj(h), dirs)                              # h* x n
    A2 = np.cross(np.cross(dirs, np.conj(e)), dirs)              # (n x e*) x dir
    gh2 = np.einsum("d,di,dk->ik", c, Phi, 1j * k0 * A1 + 1j * k * A2)
    gs2 = -1j * k * np.einsum("d,di,d->i", c, Phi, np.sum(dirs * A1, 1))
    s2, h2 = sig["sig2"][:, 0], sig["h2"][:, :, 0]
    # explicit: Phi depends on r_i (phase) and A_i
    T = Phi * (np.einsum("dk,ik->di", A1, 1j * k0 * h2) - 1j * k * np.sum(dirs * A1, 1)[:, None] * s2[None, :]
               + np.einsum("dk,dik->di", np.cross(dirs, np.conj(e)), 1j * k * np.cross(dirs[:, None, :], h2[None, :, :])))
    gpos = np.real(np.einsum("d,di,dk->ik", c * (-1j * k), T, dirs))
    garea = np.real(np.einsum("d,di->i", c, T)) / area
    return gs2, gh2, gpos, garea


def cross_section_gradient(verts, faces, quad, eps_out, eps_in, enei, pol, dirv, which="ext", pinfty=None,
                           order=5, check_chain=False):
    """Adjoint gradient of ext or sca (one polarisation): returns (J, dJ/dverts
    [nv, 3], dJ/dRe(eps) + i dJ/dIm(eps) of the inside medium, intermediates)."""
    cp, bem = make_problem(verts, faces, quad, eps_out, eps_in, None, order)
    p = cp.pc
    n = cp.n
    pol = np.asarray(pol, dtype=float)
    dirv = np.asarray(dirv, dtype=float)
    pw = R.PlaneWaveRet([pol], [dirv], pinfty)
    exc = pw.potential(cp, enei)
    sig = bem.solve(exc)
    k0 = 2 * np.pi / enei
    kb = cp.eps[0](enei)[1]
    k1 = cp.eps[1](enei)[1]
    k2 = kb
    e1, e2 = complex(eps_in), complex(eps_out)
    pos, nv, area = cp.pos, cp.nvec, cp.area
    s1, hh1 = sig["sig1"][:, 0], sig["h1"][:, :, 0]
    s2, hh2 = sig["sig2"][:, 0], sig["h2"][:, :, 0]
    if which == "ext":
        J = float(pw.extinction(cp, sig)[0])
        # J = Re(ah . h2 + as . sig2) on faces outside in the excitation medium
        Phi = np.exp(-1j * kb * pos @ dirv) * area
        ah = (4 * np.pi * k0 / kb) * Phi[:, None] * pol[None, :]
        as_ = -4 * np.pi * Phi * np.dot(pol, dirv)
    else:
        J = float(pw.scattering(cp, sig)[0])
        as_, ah, gpos_sca, garea_sca = sca_rhs(cp, sig, pw, enei)
    # ---- adjoint solve A^T lam = w
    A = afun_matrix(bem, enei)
    w = pack_x(np.zeros(n), np.zeros((n, 3)), as_, ah)
    lam_v = np.linalg.solve(A.T, w)
    lam = unpack_eq(lam_v, n)
    lphi, la, lDe, lal = lam
    if check_chain:
        lc = chain_transpose(bem, enei, np.zeros(n), np.zeros((n, 3)), as_, ah)
        err = max(np.max(np.abs(a - b)) / np.max(np.abs(b)) for a, b in zip(lc, lam))
        assert err < 1e-9, err
    WG1, WH1, WG2, WH2 = weights(cp, enei, lam, (s1, hh1, s2, hh2))
    g_pos = np.zeros((n, 3))
    g_nv = np.zeros((n, 3))
    g_area = np.zeros(n)
    gv = np.zeros_like(p.verts)
    g_k1 = 0j                          # d(lam^T A x)/dk1 (holomorphic)
    # ---- explicit J dependence (farfield phase and area)
    if which == "ext":
        Jt = np.sum(ah * hh2, 1) + as_ * s2
        g_pos += np.real(-1j * kb * Jt)[:, None] * dirv[None, :]
        g_area += np.real(Jt / area)
    else:
        g_pos += gpos_sca
        g_area += garea_sca
    # ---- excitation b (planewaveret/potential.m + excitation.m), times lam
    ph = np.exp(1j * kb * pos @ dirv)
    la_p = la @ pol
    lal_p = lal @ pol
    npol_ = nv @ pol
    ndir = nv @ dirv
    # a = ph / (i k0) pol
    g_pos += np.real(la_p * ph * (kb / k0))[:, None] * dirv
    # De = -e2 (n . pol) ph
    g_nv += np.real(-e2 * lDe * ph)[:, None] * pol
    g_pos += np.real(-e2 * lDe * npol_ * 1j * kb * ph)[:, None] * dirv
    # alpha = (kb / k0) (n . dir) ph pol
    g_nv += np.real((kb / k0) * lal_p * ph)[:, None] * dirv
    g_pos += np.real((kb / k0) * ndir * lal_p * 1j * kb * ph)[:, None] * dirv
    # ---- explicit n and eps in the alpha / De rows of A (enters with minus)
    G1, H1, G2, H2 = bem.matrices(enei)
    Gs1, Gs2 = G1 @ s1, G2 @ s2
    Gh1, Gh2 = G1 @ hh1, G2 @ hh2
    Hs1 = H1 @ s1
    gn_expl = -1j * k0 * (lal * (e1 * Gs1 - e2 * Gs2)[:, None] + lDe[:, None] * (e1 * Gh1 - e2 * Gh2))
    g_nv -= np.real(gn_expl)
    deps1_expl = np.sum(-1j * k0 * np.sum(lal * nv, 1) * Gs1 + lDe * Hs1 - 1j * k0 * lDe * np.sum(nv * Gh1, 1))
    # ---- matrix entries
    gr = bem.g.g
    pat = gr.pattern
    media = ((k1, WG1, WH1), (k2, WG2, WH2))
    O = gr.order
    # far pairs
    far = (pat == 0)
    Rv = pos[:, None, :] - pos[None, :, :]
    d = np.sqrt(np.sum(Rv * Rv, 2))
    dsafe = np.where(far, d, 1.0)
    Rh = Rv / dsafe[:, :, None]
    nR = np.einsum("ik,ijk->ij", nv, Rv)
    for mi, (km, WG, WF) in enumerate(media):
        E = np.exp(1j * km * dsafe)
        G = area[None, :] * E / dsafe
        phi = (1j * km - 1 / dsafe) * E / dsafe ** 2
        dphi = E * (1 / dsafe ** 4 + (1j * km - 1 / dsafe) * (1j * km / dsafe ** 2 - 2 / dsafe ** 3))
        F = nR * phi * area[None, :]
        WGf = np.where(far, WG, 0)
        WFf = np.where(far, WF, 0)
        # d/dR
        cG = WGf * G * (1j * km - 1 / dsafe)                     # dG/dd
        cFd = WFf * nR * area[None, :] * dphi                    # dF/dd (at fixed n.R)
        vecR = (cG + cFd)[:, :, None] * Rh + (WFf * phi * area[None, :])[:, :, None] * nv[:, None, :]
        gR = np.real(vecR)
        g_pos -= gR.sum(1)
        g_pos += gR.sum(0)
        g_nv -= np.real(np.einsum("ij,ijk->ik", WFf * phi * area[None, :], Rv))
        g_area -= np.real(np.sum(WGf * E / dsafe + WFf * nR * phi, 0))
        if mi == 0:
            g_k1 += np.sum(WGf * 1j * dsafe * G + WFf * nR * area[None, :] * (-km * E / dsafe))
    # near off-diagonal pairs and self elements
    fr = lambda km: (1j * km) ** np.arange(O + 1)
    for e, (i, j) in enumerate(zip(gr.rows, gr.cols)):
        if i == j:
            continue
        Rij = pos[i] - pos[j]
        dij = np.linalg.norm(Rij)
        Rhij = Rij / dij
        for (tri, bary, qw, atri, pts) in _quad_points_faces(p, j):
            rho = pos[i] - pts
            r = np.linalg.norm(rho, axis=1)
            rh = rho / r[:, None]
            ww = qw * atri
            nrho = rho @ nv[i]
            dr = r - dij
            for mi, (km, WG, WF) in enumerate(media):
                c = fr(km)
                E = np.exp(1j * km * dij)
                Wg, Wf = WG[i, j], WF[i, j]
                # gamma = sum_w ww Gam, Gam = sum_o c_o (r - d)^o / (o! r)
                Gam = np.zeros_like(r, dtype=complex)
                Gr = np.zeros_like(r, dtype=complex)
                Gd = np.zeros_like(r, dtype=complex)
                Gk = np.zeros_like(r, dtype=complex)
                Psi = np.zeros_like(r, dtype=complex)
                Pr = np.zeros_like(r, dtype=complex)
                Pd = np.zeros_like(r, dtype=complex)
                Pk = np.zeros_like(r, dtype=complex)
                for o in range(O + 1):
                    fo = _fact(o)
                    Gam += c[o] * dr ** o / (fo * r)
                    Gr += c[o] * ((o * dr ** (o - 1) / r if o else 0) - dr ** o / r ** 2) / fo
                    Gd += -c[o] * (o * dr ** (o - 1) / r if o else 0) / fo
                    if o:
                        Gk += o * 1j * (1j * km) ** (o - 1) * dr ** o / (fo * r)
                    if o == 0:
                        psi, psr, psd = -1 / r ** 3, 3 / r ** 4, 0 * r
                    else:
                        fo1 = _fact(o - 1)
                        psi = -dr ** o / (r ** 3 * fo) + dr ** (o - 1) / (r ** 2 * fo1)
                        psr = (-(o * dr ** (o - 1) / r ** 3 - 3 * dr ** o / r ** 4) / fo
                               + (((o - 1) * dr ** (o - 2) if o > 1 else 0) / r ** 2
                                  - 2 * dr ** (o - 1) / r ** 3) / fo1)
                        psd = o * dr ** (o - 1) / (r ** 3 * fo) - (((o - 1) * dr ** (o - 2)) if o > 1 else 0) / (r ** 2 * fo1)
                        Pk += o * 1j * (1j * km) ** (o - 1) * psi
                    Psi += c[o] * psi
                    Pr += c[o] * psr
                    Pd += c[o] * psd
                gam = np.sum(ww * Gam)
                phn = np.sum(ww * nrho * Psi)
                # dG = E (dgam + gam ik dd), dF = E (dphn + phn ik dd)
                # d/dd (explicit d, incl. phase)
                cd = Wg * E * (np.sum(ww * Gd) + gam * 1j * km) + Wf * E * (np.sum(ww * nrho * Pd) + phn * 1j * km)
                # d/drho_w (per point)
                crho = (Wg * E * ww * Gr)[:, None] * rh + (Wf * E * ww)[:, None] * (nv[i][None, :] * Psi[:, None] + (nrho * Pr)[:, None] * rh)
                gi = np.real(crho.sum(0) + cd * Rhij)
                g_pos[i] -= gi
                g_pos[j] -= np.real(-cd * Rhij)
                g_nv[i] -= np.real(Wf * E * np.sum((ww * Psi)[:, None] * rho, 0))
                # points: rho = pos_i - x_w, x_w = bary @ tri vertices
                gx = -np.real(-crho)                   # gradient of J (minus sign of dA) wrt x_w
                tri_idx = np.array(tri)
                gv[tri_idx] += bary.T @ gx
                # weights ww = qw * atri
                gw = -np.real(Wg * E * Gam + Wf * E * nrho * Psi)
                ga_tri = np.sum(gw * qw)
                va, vb, vc = p.verts[tri_idx[0]], p.verts[tri_idx[1]], p.verts[tri_idx[2]]
                g1_, g2_, g3_ = _tri_area_grad(va, vb, vc, np.asarray(ga_tri))
                gv[tri_idx[0]] += g1_
                gv[tri_idx[1]] += g2_
                gv[tri_idx[2]] += g3_
                if mi == 0:
                    g_k1 += Wg * E * (np.sum(ww * Gk) + gam * 1j * dij) + Wf * E * (np.sum(ww * nrho * Pk) + phn * 1j * dij)
    # self elements: G_ii = sum_w ww sum_o c_o r^(o-1) / o! (polar points)
    q = p.quad
    for i in range(n):
        f = p.faces[i]
        idx = f[f >= 0]
        if idx.size == 3:
            bary = np.stack([q.x3, q.y3, 1 - q.x3 - q.y3], 1)
            coef = 1.0 / 3 - bary                   # rho = sum_a coef_wa v_a
            ww = q.w3 * area[i]
            wdep = "area"
        else:
            s_, sx, sy = R._quad_shape(q.x4, q.y4)
            coef = 0.25 - s_
            vv = p.verts[idx]
            px, py = sx @ vv, sy @ vv
            jac = np.cross(px, py)
            jn = np.linalg.norm(jac, axis=1)
            ww = q.w4 * jn
            wdep = "jac"
        rho = coef @ p.verts[idx]
        r = np.linalg.norm(rho, axis=1)
        rh = rho / r[:, None]
        for mi, (km, WG, WF) in enumerate(media):
            c = fr(km)
            Wg = WG[i, i]
            Gam = np.zeros_like(r, dtype=complex)
            Gr = np.zeros_like(r, dtype=complex)
            Gk = np.zeros_like(r, dtype=complex)
            for o in range(O + 1):
                fo = _fact(o)
                Gam += c[o] * r ** (o - 1) / fo
                Gr += c[o] * (o - 1) * r ** (o - 2) / fo
                if o:
                    Gk += o * 1j * (1j * km) ** (o - 1) * r ** (o - 1) / fo
            grho = -np.real(Wg * (ww * Gr)[:, None] * rh)
            gv[idx] += coef.T @ grho
            gw = -np.real(Wg * Gam)
            if wdep == "area":
                g_area[i] += np.sum(gw * q.w3)
            else:
                gj = (gw * q.w4)[:, None] * jac / jn[:, None]
                # jac = px x py with px = sx @ vv, py = sy @ vv
                gpx = np.cross(py, gj)
                gpy = np.cross(gj, px)
                gv[idx] += sx.T @ gpx + sy.T @ gpy
            if mi == 0:
                g_k1 += Wg * np.sum(ww * Gk)
    # closed-surface diagonal: F_bb = -2 pi - S_b, S_b = sum_{a != b} A_a F0_ab / A_b
    cb = np.array([WH1[b, b] + WH2[b, b] for b in range(n)])
    # far pairs (a row, b column): T_ab = -A_a n_a . R / d^3, R = r_a - r_b
    T = -area[:, None] * nR / dsafe ** 3
    CT = np.where(far, cb[None, :], 0)
    g_area += np.real(np.sum(CT * T, 1) / area)
    g_nv += np.real(np.einsum("ab,abk->ak", CT * (-area[:, None] / dsafe ** 3), Rv))
    gRt = np.real((CT * (-area[:, None]))[:, :, None] * (nv[:, None, :] / dsafe[:, :, None] ** 3
                                                        - 3 * nR[:, :, None] * Rv / dsafe[:, :, None] ** 5))
    g_pos += gRt.sum(1)
    g_pos -= gRt.sum(0)
    # near pairs: T_ab = -(A_a / A_b) sum_w ww (n_a . rho_w) / r_w^3, x_w on face b
    for e, (a, b) in enumerate(zip(gr.rows, gr.cols)):
        if a == b:
            continue
        for (tri, bary, qw, atri, pts) in _quad_points_faces(p, b):
            rho = pos[a] - pts
            r = np.linalg.norm(rho, axis=1)
            ww = qw * atri
            nrho = rho @ nv[a]
            fac = -area[a] / area[b]
            Tab = fac * np.sum(ww * nrho / r ** 3)
            cc = cb[b]
            g_area[a] += np.real(cc * Tab / area[a])
            g_area[b] -= np.real(cc * Tab / area[b])
            g_nv[a] += np.real(cc * fac * np.sum((ww / r ** 3)[:, None] * rho, 0))
            grho = np.real(cc * fac * ww[:, None] * (nv[a][None, :] / r[:, None] ** 3
                                                     - 3 * (nrho / r ** 5)[:, None] * rho))
            g_pos[a] += grho.sum(0)
            tri_idx = np.array(tri)
            gv[tri_idx] += bary.T @ (-grho)
            gw = np.real(cc * fac * nrho / r ** 3)
            va, vb, vc = p.verts[tri_idx[0]], p.verts[tri_idx[1]], p.verts[tri_idx[2]]
            g1_, g2_, g3_ = _tri_area_grad(va, vb, vc, np.asarray(np.sum(gw * qw)))
            gv[tri_idx[0]] += g1_
            gv[tri_idx[1]] += g2_
            gv[tri_idx[2]] += g3_
    # ---- faces -> vertices
    _norm_flat_grad(p, g_pos, g_nv, g_area, gv)
    # ---- eps of the inside medium: k1 = k0 sqrt(eps) and the explicit eps1
    dk1 = k1 / (2 * e1)
    g_eps = -(g_k1 * dk1 + deps1_expl)
    grad_eps = np.conj(g_eps)
    return J, gv, grad_eps, {"lam": lam, "x": (s1, hh1, s2, hh2)}


def scattering(verts, faces, quad, eps_out, eps_in, enei, pol, dirv, pinfty, pattern=None):
    """J = sca for one polarisation (forward oracle)."""
    cp, bem = make_problem(verts, faces, quad, eps_out, eps_in, pattern)
    pw = R.PlaneWaveRet([pol], [dirv], pinfty)
    sig = bem.solve(pw.potential(cp, enei))
    return float(pw.scattering(cp, sig)[0])


def fd_gradient(verts, faces, quad, eps_out, eps_in, enei, pol, dirv, coords, h=1e-4, which="ext",
                pinfty=None):
    """Central finite differences of J at fixed refinement pattern for the
    vertex coordinates ``coords`` [(vertex, axis)] and for eps_in (Re, Im)."""
    cp, bem = make_problem(verts, faces, quad, eps_out, eps_in)
    pat = bem.g.g.pattern

    def J(v, e):
        if which == "sca":
            return scattering(v, faces, quad, eps_out, e, enei, pol, dirv, pinfty, pattern=pat)
        return extinction(v, faces, quad, eps_out, e, enei, pol, dirv, pattern=pat)
    out = []
    for (iv, ax) in coords:
        vp = verts.copy()
        vp[iv, ax] += h
        vm = verts.copy()
        vm[iv, ax] -= h
        out.append((J(vp, eps_in) - J(vm, eps_in)) / (2 * h))
    he = 1e-6 * abs(eps_in)
    de_re = (J(verts, eps_in + he) - J(verts, eps_in - he)) / (2 * he)
    de_im = (J(verts, eps_in + 1j * he) - J(verts, eps_in - 1j * he)) / (2 * he)
    return np.array(out), de_re + 1j * de_im
