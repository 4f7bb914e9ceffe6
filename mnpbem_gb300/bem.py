"""MNPBEM's calling surface for the retarded BEM path, backed by the GPU library.

    op  = bemoptions(sim='ret', interp='flat')
    p   = comparticle(epstab, [trisphere(256, 20)], [[2, 1]], 1, op=op)
    bem = bemsolver(p, op)                   # Base/bemsolver.m -> bemret
    exc = planewave([1, 0, 0], [0, 0, 1], op)
    sig = bem.mldivide(exc(p, enei))         # sig = bem \\ exc(p, enei)
    ext, sca = exc.ext(sig), exc.sca(sig)

``bem.spectrum(exc, enei)`` runs a whole wavelength sweep in one library call.
``op['precision']`` selects ``'mixed'`` (complex64 TF32 tensor-core inversion
plus FP64 refinement, default) or ``'fp64'``.
"""
import ctypes

import numpy as np

from . import _lib
from .particles import comparticle, trisphere


def bemoptions(op=None, **kw):
    """Default options (Misc/bemoptions.m:16-25) updated by keyword pairs."""
    base = {"sim": "ret", "waitbar": 0, "RelCutoff": 3, "order": 5, "interp": "flat"}
    if op:
        base.update(op)
    base.update(kw)
    return base


class compstruct:
    """Structure holding particle, wavelength and named fields (@compstruct)."""

    def __init__(self, p, enei, **fields):
        self.p, self.enei = p, enei
        self.__dict__.update(fields)

    def __repr__(self):
        keys = [k for k in self.__dict__ if k not in ("p", "enei")]
        return "compstruct(enei=%r, fields=%s)" % (self.enei, keys)

    def _fields(self):
        return {k: v for k, v in self.__dict__.items() if k not in ("p", "enei")}

    @staticmethod
    def _numeric(v):
        return isinstance(v, (np.ndarray, int, float, complex, np.number))

    def __add__(self, other):
        """Field-wise sum (@compstruct/plus.m): fields of both are added,
        fields of one are kept; non-numeric fields keep the left operand's."""
        out = compstruct(self.p, self.enei, **self._fields())
        for k, v in other._fields().items():
            mine = out.__dict__.get(k)
            if mine is None:
                setattr(out, k, v)
            elif self._numeric(mine) and self._numeric(v):
                setattr(out, k, mine + v)
        return out

    def __neg__(self):
        """@compstruct/uminus.m on the numeric fields."""
        return compstruct(self.p, self.enei, **{k: (-v if self._numeric(v) else v)
                                                for k, v in self._fields().items()})

    def __sub__(self, other):
        """@compstruct/minus.m: self + (-other)."""
        return self + (-other)

    def __mul__(self, val):
        """@compstruct/mtimes.m: every numeric field times a scalar."""
        return compstruct(self.p, self.enei, **{k: (val * v if self._numeric(v) else v)
                                                for k, v in self._fields().items()})

    __rmul__ = __mul__


class spectrumret:
    """Unit sphere at infinity used for far fields (@spectrumret)."""

    def __init__(self, pinfty=None, medium=1):
        self.pinfty = pinfty if pinfty is not None else trisphere(256, 2)
        self.medium = medium

    def farfield(self, bem, sig, dir=None):
        """Far fields of ``sig = bem \\ exc`` in the unit directions ``dir
        [ndir, 3]`` (default: the normals of the sphere at infinity), in this
        spectrum's medium (@spectrumret/farfield.m:15-74), by
        ``mnpbem_farfield``; ``bem`` is the solver that holds the particle.
        Returns ``compstruct`` with ``e, h [ndir, 3, npol]``."""
        dirs = np.ascontiguousarray(self.nvec if dir is None else np.atleast_2d(dir), dtype=np.float64)
        enei = float(sig.enei)
        em = np.ascontiguousarray(bem.p.eps_media(enei)[0])
        parts = [np.ascontiguousarray(getattr(sig, k), dtype=np.complex128) for k in ("sig1", "sig2", "h1", "h2")]
        P = parts[0].shape[1]
        nd = dirs.shape[0]
        e = np.zeros((nd, 3, P), np.complex128)
        h = np.zeros((nd, 3, P), np.complex128)
        for c0 in range(0, P, 4):        # up to four columns per call
            cols = slice(c0, min(P, c0 + 4))
            w = cols.stop - cols.start
            cin = [np.ascontiguousarray(a[..., cols]) for a in parts]
            ec = np.zeros((nd, 3, w), np.complex128)
            hc = np.zeros((nd, 3, w), np.complex128)
            _lib.check(bem._lib.mnpbem_farfield(
                bem._h, enei, em.view(np.float64).ctypes.data_as(_lib.c_double_p), em.size, self.medium, nd,
                _lib.dptr(dirs), w, *[a.ctypes.data for a in cin], ec.ctypes.data, hc.ctypes.data))
            e[..., cols], h[..., cols] = ec, hc
        return compstruct(bem.p, enei, e=e, h=h)

    @property
    def nvec(self):
        return np.ascontiguousarray(self.pinfty.nvec, dtype=np.float64)

    @property
    def area(self):
        return np.ascontiguousarray(self.pinfty.area, dtype=np.float64)


class planewaveret:
    """Plane-wave excitation for the retarded solver (@planewaveret)."""

    name = "planewave"
    needs = [{"sim": "ret"}]

    def __init__(self, pol, dir, op=None, medium=None, pinfty=None):
        op = op or {}
        self.pol = np.ascontiguousarray(np.atleast_2d(np.asarray(pol, dtype=np.float64)))
        self.dir = np.ascontiguousarray(np.atleast_2d(np.asarray(dir, dtype=np.float64)))
        if self.pol.shape != self.dir.shape or self.pol.shape[1] != 3:
            raise ValueError("pol and dir must both be [npol, 3]")
        if np.any(np.sum(self.pol * self.dir, 1) != 0):
            raise ValueError("polarisation and propagation direction must be orthogonal")
        self.medium = int(medium if medium is not None else op.get("medium", 1))
        self.spec = spectrumret(pinfty if pinfty is not None else op.get("pinfty"), self.medium)

    @property
    def npol(self):
        return self.pol.shape[0]

    def __call__(self, p, enei):
        """External potential for bemret at wavelength enei (potential.m)."""
        return compstruct(p, float(enei), exc=self)

    def _struct(self):
        pw = _lib.PlaneWave()
        pw.npol = self.npol
        pw.pol = _lib.dptr(self.pol)
        pw.dir = _lib.dptr(self.dir)
        pw.medium = self.medium
        self._nv, self._ar = self.spec.nvec, self.spec.area
        pw.ninf = self._nv.shape[0]
        pw.inf_nvec = _lib.dptr(self._nv)
        pw.inf_area = _lib.dptr(self._ar)
        return pw

    def field(self, p, enei, inout=1):
        """Incoming fields at the positions of ``p`` (Simulation/retarded/
        @planewaveret/field.m): a comparticle (its faces, medium column
        ``inout`` of the faces' media) or a meshfield (its points and their
        media).  Positions in the excitation medium get
        e = pol exp(i k dir . r), h = nb dir x e; the others zero.  Returns
        ``compstruct`` with ``e, h [m, 3, npol]`` (closed form, on the host)."""
        enei = float(enei)
        if isinstance(p, meshfield):
            pos, med, eps = p.pts, p.medium, p.bem.p.eps_media(enei)[0]
        else:
            pos = p.pos
            med = np.repeat(np.asarray(p.inout)[:, inout - 1], [q.n for q in p.p])
            eps = p.eps_media(enei)[0]
        nb = np.sqrt(eps[self.medium - 1])
        k0 = 2 * np.pi / enei
        k = k0 * nb
        m, P = pos.shape[0], self.npol
        e = np.zeros((m, 3, P), np.complex128)
        h = np.zeros((m, 3, P), np.complex128)
        ind = np.nonzero(med == self.medium)[0]
        for i in range(P):
            ph = np.exp(1j * k * pos[ind] @ self.dir[i])
            e[ind, :, i] = ph[:, None] * self.pol[i][None, :]
            h[:, :, i] = nb * np.cross(np.broadcast_to(self.dir[i], (m, 3)), e[:, :, i])
        return compstruct(p, enei, e=e, h=h)

    def extinction(self, sig):
        return sig.ext

    def scattering(self, sig):
        return sig.sca

    def dscattering(self, bem, sig):
        """``sca, dsca`` as ``[sca, dsca] = scattering(exc, sig)``
        (@planewaveret/scattering.m, Simulation/retarded/scattering.m): the
        Poynting flux 0.5 Re(n . (e x conj h)) of the charges' far fields on
        the sphere at infinity (``mnpbem_farfield``) per direction, divided by
        0.5 nb of medium 1 (``dsca [ninf, npol]``), and its area-weighted sum
        ``sca [npol]``."""
        ff = self.spec.farfield(bem, sig)
        nv = self.spec.nvec
        flux = 0.5 * np.real(np.einsum("dc,dcp->dp", nv, np.cross(ff.e, np.conj(ff.h), axis=1)))
        nb = np.sqrt(bem.p.eps_media(float(sig.enei))[0][0])
        dsca = np.real(flux / (0.5 * nb))
        sca = self.spec.area @ dsca
        return sca, compstruct(self.spec.pinfty, sig.enei, dsca=dsca)

    ext = extinction
    sca = scattering

    def absorption(self, sig):
        return sig.ext - sig.sca


def planewave(pol, dir, op=None, **kw):
    """Factory of Base/planewave.m for sim = 'ret'."""
    op = bemoptions(op)
    if op.get("sim", "ret") != "ret":
        raise NotImplementedError("only the retarded plane-wave excitation is implemented")
    return planewaveret(pol, dir, op, **kw)


class bemret:
    """Retarded BEM solver on one GPU (BEM/@bemret).

    Construction builds the composite Green function on the GPU: geometry,
    refinement pattern, Taylor coefficients of the near elements and the
    closed-surface sum rule (compgreenret(p, p, op)).
    """

    name = "bemsolver"
    needs = [{"sim": "ret"}]

    def __init__(self, p, op=None):
        if not isinstance(p, comparticle):
            raise TypeError("bemret needs a comparticle")
        self.p = p
        self.op = bemoptions(op)
        prec = self.op.get("precision", "mixed")
        if prec not in ("mixed", "fp64"):
            raise ValueError("precision must be 'mixed' or 'fp64'")
        self.precision = _lib.MIXED if prec == "mixed" else _lib.FP64
        self.refine_iters = int(self.op.get("refine_iters", 10))
        self.refine_tol = float(self.op.get("refine_tol", 1e-10))
        lib = _lib.load()
        q = p.quad
        self._quad_arrays = [np.ascontiguousarray(a, dtype=np.float64)
                             for a in (q.x, q.y, q.w, q.x3, q.y3, q.w3, q.x4, q.y4, q.w4)]
        qa = self._quad_arrays
        quad = _lib.Quad(qa[0].size, _lib.dptr(qa[0]), _lib.dptr(qa[1]), _lib.dptr(qa[2]),
                         qa[3].size, _lib.dptr(qa[3]), _lib.dptr(qa[4]), _lib.dptr(qa[5]),
                         qa[6].size, _lib.dptr(qa[6]), _lib.dptr(qa[7]), _lib.dptr(qa[8]))
        opts = _lib.Options(float(self.op.get("RelCutoff", 3)), float(self.op.get("AbsCutoff", 0)),
                            int(self.op.get("order", 5)), int(self.op.get("device", 0)))
        part_n = np.ascontiguousarray([q.n for q in p.p], dtype=np.int64)
        inout = np.ascontiguousarray(p.inout, dtype=np.int32)
        closed = np.ascontiguousarray(p.closed, dtype=np.int32)
        h = ctypes.c_void_p()
        if getattr(p, "curved", False):
            # curved boundary elements (interp = 'curv')
            _lib.check(lib.mnpbem_geom_create_curved(
                _lib.dptr(p.verts2), p.verts2.shape[0], p.faces2.ctypes.data_as(_lib.c_int64_p), p.n,
                len(p.p), part_n.ctypes.data_as(_lib.c_int64_p), inout.ctypes.data_as(_lib.c_int32_p),
                closed.ctypes.data_as(_lib.c_int32_p), ctypes.byref(quad), ctypes.byref(opts),
                ctypes.byref(h)))
        else:
            _lib.check(lib.mnpbem_geom_create(
                _lib.dptr(p.verts), p.verts.shape[0], p.faces.ctypes.data_as(_lib.c_int64_p), p.n,
                len(p.p), part_n.ctypes.data_as(_lib.c_int64_p), inout.ctypes.data_as(_lib.c_int32_p),
                closed.ctypes.data_as(_lib.c_int32_p), ctypes.byref(quad), ctypes.byref(opts),
                ctypes.byref(h)))
        self._h = h
        self._lib = lib
        if self.op.get("tuned", True):
            from . import autotune
            for key, val in autotune.settings_for(p.n, prec).items():
                self.set_option(key, val)
        if self.op.get("lanes"):          # 0 / None: the tuned or automatic lane count
            self.set_lanes(int(self.op["lanes"]))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.mnpbem_geom_destroy(h)
            except Exception:
                pass
            self._h = None

    def set_option(self, key, value):
        """Tuning option of the handle (``mnpbem_geom_set_option``)."""
        _lib.check(self._lib.mnpbem_geom_set_option(self._h, key.encode(), int(value)))

    def set_lanes(self, lanes):
        """Wavelengths kept in flight at once by ``spectrum`` (0 = automatic)."""
        _lib.check(self._lib.mnpbem_geom_set_lanes(self._h, int(lanes)))

    def stat(self, key):
        """Statistic of the handle (``mnpbem_geom_stat``): 'block_cond_max'
        (largest condition proxy of the diagonal blocks factored since the
        last 'block_cond_reset'), 'g1_blocks'."""
        v = ctypes.c_double()
        _lib.check(self._lib.mnpbem_geom_stat(self._h, key.encode(), ctypes.byref(v)))
        return v.value

    # ----------------------------------------------------------- queries
    @property
    def handle(self):
        return self._h

    def sizes(self):
        n, nref = ctypes.c_int64(), ctypes.c_int64()
        _lib.check(self._lib.mnpbem_geom_size(self._h, ctypes.byref(n), ctypes.byref(nref)))
        return n.value, nref.value

    def refinement(self):
        """Geometry and greenret refinement data (pos, nvec, ..., ind, g, f)."""
        n, nref = self.sizes()
        O = int(self.op.get("order", 5))
        out = {k: np.zeros((n, 3)) for k in ("pos", "nvec", "tvec1", "tvec2")}
        out["area"] = np.zeros(n)
        out["row"] = np.zeros(nref, dtype=np.int64)
        out["col"] = np.zeros(nref, dtype=np.int64)
        out["g"] = np.zeros((nref, O + 1))
        out["f"] = np.zeros((nref, 3, O + 1))
        _lib.check(self._lib.mnpbem_geom_export(
            self._h, *[_lib.vptr(out[k]) for k in ("pos", "nvec", "tvec1", "tvec2", "area", "row",
                                                   "col", "g", "f")]))
        return out

    def _eps(self, enei):
        em = np.ascontiguousarray(self.p.eps_media(enei), dtype=np.complex128)
        return em

    def matrices(self, enei, precision="fp64"):
        """G1, H1, G2, H2 of initmat.m:27-31 at wavelength enei (host arrays)."""
        em = self._eps(enei)[0]
        k = np.ascontiguousarray(2 * np.pi / enei * np.sqrt(em))
        n = self.p.n
        dt = np.complex64 if precision == "fp32" else np.complex128
        code = {"fp64": _lib.FP64, "fp32": _lib.FP32, "mixed": _lib.MIXED}[precision]
        mats = [np.zeros((n, n), dtype=dt) for _ in range(4)]
        _lib.check(self._lib.mnpbem_assemble(self._h, k.view(np.float64).ctypes.data_as(_lib.c_double_p),
                                             k.size, code, *[_lib.vptr(m) for m in mats]))
        return tuple(mats)

    def bem_matrices(self, enei, precision=None):
        """G1i, G2i, Sigma1, Deltai, Sigmai (initmat.m:27-72) as complex128."""
        prec = self.precision if precision is None else (_lib.MIXED if precision == "mixed" else _lib.FP64)
        em = np.ascontiguousarray(self._eps(enei)[0])
        n = self.p.n
        mats = [np.zeros((n, n), dtype=np.complex128) for _ in range(5)]
        _lib.check(self._lib.mnpbem_bem_matrices(self._h, float(enei),
                                                 em.view(np.float64).ctypes.data_as(_lib.c_double_p),
                                                 em.size, prec, *[_lib.vptr(m) for m in mats]))
        return dict(zip(("G1i", "G2i", "Sigma1", "Deltai", "Sigmai"), mats))

    # ------------------------------------------------------------- solves
    def _sweep_args(self, exc, enei, fields, out):
        """Arrays and C structures of one sweep (kept alive by the caller)."""
        enei = np.ascontiguousarray(np.atleast_1d(np.asarray(enei, dtype=np.float64)))
        nw, P, n = enei.size, exc.npol, self.p.n
        em = np.ascontiguousarray(self._eps(enei))
        pw = exc._struct()
        shapes_ = {"ext": ((nw, P), np.float64), "sca": ((nw, P), np.float64),
                   "sig1": ((nw, n, P), np.complex128), "sig2": ((nw, n, P), np.complex128),
                   "h1": ((nw, n, 3, P), np.complex128), "h2": ((nw, n, 3, P), np.complex128)}
        given = out or {}
        res = {"ir_iters": np.zeros(nw, dtype=np.int32), "ir_resid": np.zeros(nw)}
        for key, (shp, dt) in shapes_.items():
            if key in ("sig1", "sig2", "h1", "h2") and not fields:
                continue
            if key in given:
                arr = given[key]
                if arr.shape != shp or arr.dtype != dt or not arr.flags["C_CONTIGUOUS"]:
                    raise ValueError("out[%r] must be a C-contiguous %s array of shape %s" % (key, dt, shp))
                res[key] = arr
            else:
                res[key] = np.zeros(shp, dtype=dt)
        sol = _lib.Solution()
        for key in ("ext", "sca", "sig1", "sig2", "h1", "h2", "ir_iters", "ir_resid"):
            if key in res:
                setattr(sol, key, res[key].ctypes.data)
        sol.outputs_on_device = 0
        return {"enei": enei, "em": em, "pw": pw, "sol": sol, "exc": exc, "res": res}

    def spectrum(self, exc, enei, fields=False, out=None):
        """Wavelength sweep: returns dict with ext, sca [nenei, npol] (+ fields).

        ``out`` may supply preallocated (e.g. pinned) C-contiguous host arrays
        for any of ext, sca, sig1, sig2, h1, h2 with the shapes below.
        """
        a = self._sweep_args(exc, enei, fields, out)
        ref = _lib.Refine(self.refine_iters, self.refine_tol)
        _lib.check(self._lib.mnpbem_solve(self._h, ctypes.byref(a["pw"]), a["enei"].size, _lib.dptr(a["enei"]),
                                          a["em"].view(np.float64).ctypes.data_as(_lib.c_double_p),
                                          a["em"].shape[1], self.precision, ctypes.byref(ref),
                                          ctypes.byref(a["sol"])))
        return a["res"]

    def ext_gradient(self, exc, enei, ipol=0):
        """Extinction of polarisation ``ipol`` at ``enei`` and its gradient
        (adjoint method, FP64): returns ``(ext, dext/dverts [nverts, 3],
        dext/deps)`` with ``dext/deps = dext/dRe(eps) + 1j dext/dIm(eps)`` of
        the medium inside the particle.  One closed particle excited from its
        outside medium; the refinement pattern is held fixed."""
        return self.cross_section_gradient(exc, enei, ipol, "ext")

    def cross_section_gradient(self, exc, enei, ipol=0, which="ext", precision="fp64"):
        """``which`` = 'ext' or 'sca': the cross section and its gradient
        (see ``ext_gradient``); 'sca' integrates over ``exc``'s sphere at
        infinity as ``scattering.m``.  ``precision`` 'mixed': complex64
        forward and transposed solves with FP64-class refinement."""
        em = np.ascontiguousarray(self._eps(float(enei))[0])
        pw = exc._struct()
        val = np.zeros(1)
        gv = np.zeros((self.p.verts.shape[0], 3))
        ge = np.zeros(2)
        _lib.check(self._lib.mnpbem_cross_section_gradient(
            self._h, ctypes.byref(pw), int(ipol), {"ext": 0, "sca": 1}[which], float(enei),
            em.view(np.float64).ctypes.data_as(_lib.c_double_p), em.size,
            _lib.MIXED if precision == "mixed" else _lib.FP64,
            _lib.vptr(val), _lib.vptr(gv), _lib.vptr(ge)))
        return float(val[0]), gv, complex(ge[0], ge[1])

    def mldivide(self, exc):
        """sig = bem \\ exc(p, enei): surface charges and currents (mldivide.m).

        ``exc`` from a plane wave (``planewave(...)(p, enei)``) or with
        external potentials ``phi1, phi1p, phi2, phi2p [n, P]``, ``a1, a1p, a2,
        a2p [n, 3, P]`` (e.g. ``dipoleret.potential``), solved in groups of at
        most four columns by ``mnpbem_solve_potentials``."""
        if not hasattr(exc, "exc"):
            return self._solve_potentials(exc)
        pw = exc.exc
        r = self.spectrum(pw, exc.enei, fields=True)
        return compstruct(self.p, exc.enei, sig1=r["sig1"][0], sig2=r["sig2"][0], h1=r["h1"][0],
                          h2=r["h2"][0], ext=r["ext"][0], sca=r["sca"][0],
                          ir_iters=int(r["ir_iters"][0]), ir_resid=float(r["ir_resid"][0]))

    solve = mldivide

    def _surface(self, sig, inout, want):
        if inout not in (1, 2):
            raise ValueError("inout must be 1 (inside) or 2 (outside)")
        enei = float(sig.enei)
        em = np.ascontiguousarray(self.p.eps_media(enei)[0])
        parts = [np.ascontiguousarray(getattr(sig, k), dtype=np.complex128) for k in ("sig1", "sig2", "h1", "h2")]
        n, P = parts[0].shape
        dims = {"e": (n, 3, P), "h": (n, 3, P), "phi": (n, P), "phip": (n, P), "a": (n, 3, P), "ap": (n, 3, P)}
        out = {k: np.zeros(dims[k], np.complex128) for k in want}
        for c0 in range(0, P, 4):        # mnpbem_surface_fields takes up to four columns per call
            cols = slice(c0, min(P, c0 + 4))
            w = cols.stop - cols.start
            cin = [np.ascontiguousarray(a[..., cols]) for a in parts]
            cout = {k: np.zeros(dims[k][:-1] + (w,), np.complex128) for k in want}
            ptr = [cout[k].ctypes.data if k in cout else None for k in ("e", "h", "phi", "phip", "a", "ap")]
            _lib.check(self._lib.mnpbem_surface_fields(
                self._h, enei, em.view(np.float64).ctypes.data_as(_lib.c_double_p), em.size, w, inout,
                *[a.ctypes.data for a in cin], *ptr))
            for k in want:
                out[k][..., cols] = cout[k]
        return out

    def field(self, sig, inout=2):
        """Electric and magnetic fields at the face centroids on side
        ``inout`` (1 inside, 2 outside, the default of BEM/@bemret/field.m),
        from ``sig = bem \\ exc``: compgreenret field.m on the particle itself,
        by ``mnpbem_surface_fields``.  Returns ``compstruct(p, enei, e=[n, 3,
        npol], h=[n, 3, npol])``; the incoming field is not included."""
        r = self._surface(sig, inout, ("e", "h"))
        return compstruct(self.p, sig.enei, e=r["e"], h=r["h"])

    def potential(self, sig, inout=2):
        """Scalar and vector potentials and their surface derivatives at the
        faces on side ``inout`` (BEM/@bemret/potential.m -> compgreenret
        potential.m:16-48): ``compstruct`` with ``phi1, phi1p, a1, a1p``
        (inout = 1) or ``phi2, phi2p, a2, a2p`` (inout = 2)."""
        r = self._surface(sig, inout, ("phi", "phip", "a", "ap"))
        s = str(inout)
        return compstruct(self.p, sig.enei, **{"phi" + s: r["phi"], "phi" + s + "p": r["phip"],
                                               "a" + s: r["a"], "a" + s + "p": r["ap"]})

    def mtimes(self, sig):
        """phi = bem * sig (BEM/@bemret/mtimes.m): the potentials of both
        sides, ``compstruct`` with phi1, phi1p, a1, a1p, phi2, phi2p, a2, a2p."""
        p1, p2 = self.potential(sig, 1), self.potential(sig, 2)
        fields = {k: v for q in (p1, p2) for k, v in q.__dict__.items() if k not in ("p", "enei")}
        return compstruct(self.p, sig.enei, **fields)

    __mul__ = mtimes

    def _solve_potentials(self, exc):
        enei = float(exc.enei)
        n = self.p.n
        keys1, keys3 = ("phi1", "phi1p", "phi2", "phi2p"), ("a1", "a1p", "a2", "a2p")
        P = next(np.asarray(getattr(exc, k)).shape[-1] for k in keys1 + keys3 if hasattr(exc, k))
        em = np.ascontiguousarray(self.p.eps_media(enei)[0])
        out = {k: np.zeros((n, P), np.complex128) for k in ("sig1", "sig2")}
        out.update({k: np.zeros((n, 3, P), np.complex128) for k in ("h1", "h2")})
        iters = []
        for c0 in range(0, P, 4):
            cols = slice(c0, min(P, c0 + 4))
            w = cols.stop - cols.start
            keep = []
            pot = _lib.Potentials()
            pot.npol = w
            for k in keys1 + keys3:
                if hasattr(exc, k):
                    arr = np.ascontiguousarray(np.asarray(getattr(exc, k))[..., cols], dtype=np.complex128)
                    keep.append(arr)
                    setattr(pot, k, arr.ctypes.data)
            part = {k: np.zeros((n, w) if k.startswith("sig") else (n, 3, w), np.complex128)
                    for k in ("sig1", "sig2", "h1", "h2")}
            it, res = np.zeros(1, np.int32), np.zeros(1)
            sol = _lib.Solution()
            sol.sig1, sol.sig2 = part["sig1"].ctypes.data, part["sig2"].ctypes.data
            sol.h1, sol.h2 = part["h1"].ctypes.data, part["h2"].ctypes.data
            sol.ir_iters, sol.ir_resid = it.ctypes.data, res.ctypes.data
            ref = _lib.Refine(self.refine_iters, self.refine_tol)
            _lib.check(self._lib.mnpbem_solve_potentials(
                self._h, ctypes.byref(pot), enei, em.view(np.float64).ctypes.data_as(_lib.c_double_p), em.size,
                self.precision, ctypes.byref(ref), ctypes.byref(sol)))
            for k in part:
                out[k][..., cols] = part[k]
            iters.append(int(it[0]))
        return compstruct(self.p, enei, ir_iters=max(iters), **out)


class dipoleret:
    """Oscillating dipoles for the retarded solver (Simulation/retarded/@dipoleret).

    ``dipoleret(p, pos, dip=None)``: dipoles at ``pos [npt, 3]`` near the
    comparticle ``p`` with moments ``dip`` ([3] or [ndip, 3] for every
    position, default the unit vectors; ``[npt, 3, ndip]`` with ``full=True``).
    The media of the positions follow compoint (``medium`` overrides them).
    ``exc = dip(p, enei)`` holds the potentials of potential.m:14-117 (columns
    = (position, orientation), position-major); ``sig = bem \\ exc``;
    ``tot, rad, rad0 = dip.decayrate(bem, sig)`` (decayrate.m:13-62): the
    induced field at the dipoles comes from ``mnpbem_fields``, the radiated
    power from the far fields of the charges (spectrumret/farfield.m) and of
    the dipoles (farfield.m:11-55) on the unit sphere at infinity.
    """

    def __init__(self, p, pos, dip=None, full=False, medium=None, pinfty=None, spec_medium=1):
        self.p = p
        self.pos = np.ascontiguousarray(np.asarray(pos, dtype=np.float64).reshape(-1, 3))
        npt = self.pos.shape[0]
        if full:
            d = np.asarray(dip, dtype=np.float64)
            self.dip = d.reshape(npt, 3, -1)
        else:
            d = np.eye(3) if dip is None else np.atleast_2d(np.asarray(dip, dtype=np.float64))
            self.dip = np.repeat(d.T[None, :, :], npt, axis=0)       # [npt, 3, ndip]
        self.medium = (point_media(p, self.pos) if medium is None
                       else np.ascontiguousarray(np.broadcast_to(medium, npt), dtype=np.int32))
        self.spec = spectrumret(pinfty, spec_medium)

    @property
    def ncol(self):
        return self.dip.shape[0] * self.dip.shape[2]

    def __call__(self, p, enei):
        return self.potential(p, enei)

    def potential(self, p, enei):
        """Potentials at the faces (potential.m:14-117)."""
        enei = float(enei)
        npt, ndip = self.dip.shape[0], self.dip.shape[2]
        n, P = p.n, self.ncol
        f = {k: np.zeros((n, P), np.complex128) for k in ("phi1", "phi1p", "phi2", "phi2p")}
        f.update({k: np.zeros((n, 3, P), np.complex128) for k in ("a1", "a1p", "a2", "a2p")})
        fmed = np.repeat(p.inout, [q.n for q in p.p], axis=0)
        eps = p.eps_media(enei)[0]
        k0 = 2 * np.pi / enei
        for ipt in range(npt):
            mm = int(self.medium[ipt])
            e = eps[mm - 1]
            k = k0 * np.sqrt(e)
            for side, sfx in ((0, "1"), (1, "2")):
                ind = np.nonzero(fmed[:, side] == mm)[0]
                if ind.size == 0:
                    continue
                v = p.pos[ind] - self.pos[ipt][None, :]
                r = np.sqrt(np.sum(v * v, 1))
                u = v / r[:, None]
                G = np.exp(1j * k * r) / r
                F = (1j * k - 1 / r) * G
                nv = p.nvec[ind]
                en = np.sum(nv * u, 1)
                for idip in range(ndip):
                    d = self.dip[ipt, :, idip]
                    col = ipt * ndip + idip
                    ep, npd = u @ d, nv @ d
                    f["phi" + sfx][ind, col] = -ep * F / e
                    f["phi" + sfx + "p"][ind, col] = ((npd - 3 * en * ep) / r ** 2 * (1 - 1j * k * r) * G / e
                                                       + k ** 2 * ep * en * G / e)
                    f["a" + sfx][ind, :, col] = -1j * k0 * d[None, :] * G[:, None]
                    f["a" + sfx + "p"][ind, :, col] = -1j * k0 * d[None, :] * (en * F)[:, None]
        return compstruct(p, enei, **f)

    def _farfields(self, bem, sig):
        """Far fields of the induced charges (``mnpbem_farfield``) and of the
        dipoles themselves (farfield.m:11-55, closed form) on the unit sphere
        at infinity."""
        p = bem.p
        enei = float(sig.enei)
        dirs, med = self.spec.nvec, self.spec.medium
        eps = p.eps_media(enei)[0][med - 1]
        k0 = 2 * np.pi / enei
        k = k0 * np.sqrt(eps)
        ff = self.spec.farfield(bem, sig)
        e, h = ff.e, ff.h
        npt, ndip = self.dip.shape[0], self.dip.shape[2]
        for ipt in range(npt):
            if self.medium[ipt] != med:
                continue
            g = np.exp(-1j * k * dirs @ self.pos[ipt])
            for idip in range(ndip):
                hh = np.cross(dirs, self.dip[ipt, :, idip][None, :]) * g[:, None]
                col = ipt * ndip + idip
                e[:, :, col] += k ** 2 * np.cross(hh, dirs) / eps
                h[:, :, col] += k ** 2 * hh / np.sqrt(eps)
        return e, h

    def decayrate(self, bem, sig):
        """``tot, rad, rad0 [npt, ndip]``: total and radiative decay rates in
        units of the free-space rate, and the free-space rate nb * 4/3 k0^3."""
        p = self.p
        enei = float(sig.enei)
        k0 = 2 * np.pi / enei
        gamma = 4.0 / 3.0 * k0 ** 3
        e, _ = meshfield(bem, self.pos, medium=self.medium)(sig)              # [npt, 3, P]
        ef, hf = self._farfields(bem, sig)
        flux = 0.5 * np.real(np.einsum("dc,dcp->dp", self.spec.nvec, np.cross(ef, np.conj(hf), axis=1)))
        sca = self.spec.area @ flux
        npt, ndip = self.dip.shape[0], self.dip.shape[2]
        eps = p.eps_media(enei)[0]
        tot, rad, rad0 = np.zeros((npt, ndip)), np.zeros((npt, ndip)), np.zeros((npt, ndip))
        for ipt in range(npt):
            nb = np.sqrt(eps[int(self.medium[ipt]) - 1]).real
            for idip in range(ndip):
                col = ipt * ndip + idip
                tot[ipt, idip] = 1 + np.imag(e[ipt, :, col] @ np.conj(self.dip[ipt, :, idip])) / (0.5 * nb * gamma)
                rad[ipt, idip] = sca[col] / (2 * np.pi * k0) / (0.5 * nb * gamma)
                rad0[ipt, idip] = nb * gamma
        return tot, rad, rad0


def point_media(p, pts):
    """Medium of each point (compoint, Particles/@compoint/init.m:20-35): the
    point is inside (outside) the face nearest to it when it lies behind (in
    front of) that face's plane, and takes the face's inside (outside) medium.
    The nearest face is the one with the nearest centroid (compoint measures
    the distance to the element itself; the two agree away from the surface)."""
    pts = np.asarray(pts, dtype=np.float64).reshape(-1, 3)
    med = np.zeros(pts.shape[0], dtype=np.int32)
    fmed = np.repeat(p.inout, [q.n for q in p.p], axis=0)
    for s0 in range(0, pts.shape[0], 2048):
        q = pts[s0:s0 + 2048]
        d2 = np.sum((q[:, None, :] - p.pos[None, :, :]) ** 2, 2)
        j = np.argmin(d2, 1)
        side = np.sum((q - p.pos[j]) * p.nvec[j], 1) >= 0
        med[s0:s0 + 2048] = np.where(side, fmed[j, 1], fmed[j, 0])
    return med


class meshfield:
    """Electric and magnetic fields on a set of points (Simulation/misc/@meshfield).

    ``meshfield(bem, x, y, z)`` with arrays of equal shape (or ``pts [m, 3]``
    as ``x``); ``e, h = emesh(sig)`` for surface charges ``sig`` from
    ``bem.mldivide`` (or ``bem \\ exc``), each shaped ``x.shape + (3, npol)``.
    ``medium`` overrides the media of the points (1-based, compoint's inout).
    Computed by ``mnpbem_fields`` on the GPU.
    """

    def __init__(self, bem, x, y=None, z=None, medium=None):
        self.bem = bem
        if y is None:
            pts = np.asarray(x, dtype=np.float64).reshape(-1, 3)
            self.shape = pts.shape[:1]
        else:
            x, y, z = np.broadcast_arrays(np.asarray(x, float), np.asarray(y, float), np.asarray(z, float))
            self.shape = x.shape
            pts = np.stack([x.ravel(), y.ravel(), z.ravel()], 1)
        self.pts = np.ascontiguousarray(pts)
        self.medium = (point_media(bem.p, self.pts) if medium is None
                       else np.ascontiguousarray(np.broadcast_to(medium, self.pts.shape[0]), dtype=np.int32))

    def __call__(self, sig):
        if hasattr(sig, "e") and not hasattr(sig, "sig1"):
            # fields already at the points (e.g. exc.field(emesh, enei)): reshape only
            P = sig.e.shape[-1]
            return sig.e.reshape(self.shape + (3, P)), sig.h.reshape(self.shape + (3, P))
        b = self.bem
        enei = float(sig.enei)
        em = np.ascontiguousarray(b.p.eps_media(enei)[0])
        s1 = np.ascontiguousarray(sig.sig1, dtype=np.complex128)
        P = s1.shape[1]
        s2 = np.ascontiguousarray(sig.sig2, dtype=np.complex128)
        q1 = np.ascontiguousarray(sig.h1, dtype=np.complex128)
        q2 = np.ascontiguousarray(sig.h2, dtype=np.complex128)
        m = self.pts.shape[0]
        e = np.zeros((m, 3, P), np.complex128)
        h = np.zeros((m, 3, P), np.complex128)
        for c0 in range(0, P, 4):        # mnpbem_fields takes up to four columns per call
            cols = slice(c0, min(P, c0 + 4))
            w = cols.stop - cols.start
            part = [np.ascontiguousarray(a[..., cols]) for a in (s1, s2, q1, q2)]
            ec = np.zeros((m, 3, w), np.complex128)
            hc = np.zeros((m, 3, w), np.complex128)
            _lib.check(b._lib.mnpbem_fields(
                b._h, m, _lib.dptr(self.pts), self.medium.ctypes.data_as(_lib.c_int32_p), enei,
                em.view(np.float64).ctypes.data_as(_lib.c_double_p), em.size, w,
                part[0].ctypes.data, part[1].ctypes.data, part[2].ctypes.data, part[3].ctypes.data,
                ec.ctypes.data, hc.ctypes.data))
            e[..., cols], h[..., cols] = ec, hc
        return e.reshape(self.shape + (3, P)), h.reshape(self.shape + (3, P))


def spectrum_batch(items, fields=False):
    """Sweeps of several particles in one library call (``mnpbem_solve_batch``).

    ``items``: sequence of ``(bem, exc, enei)`` with distinct solvers of one
    precision; returns one result dict per item, as ``bemret.spectrum``.  The
    reference loops over particles in user code; here the wavelengths of all
    particles share the GPU at once.
    """
    items = list(items)
    if not items:
        return []
    prec = {b.precision for b, _, _ in items}
    if len(prec) != 1:
        raise ValueError("spectrum_batch: all solvers must use one precision")
    args = [b._sweep_args(e, w, fields, None) for b, e, w in items]
    jobs = (_lib.Job * len(items))()
    for k, ((b, _, _), a) in enumerate(zip(items, args)):
        jobs[k].g = b.handle.value
        jobs[k].exc = ctypes.pointer(a["pw"])
        jobs[k].nenei = a["enei"].size
        jobs[k].enei = _lib.dptr(a["enei"])
        jobs[k].eps_media = a["em"].view(np.float64).ctypes.data_as(_lib.c_double_p)
        jobs[k].nmed = a["em"].shape[1]
        jobs[k].out = ctypes.pointer(a["sol"])
    b0 = items[0][0]
    ref = _lib.Refine(b0.refine_iters, b0.refine_tol)
    _lib.check(b0._lib.mnpbem_solve_batch(jobs, len(items), b0.precision, ctypes.byref(ref)))
    return [a["res"] for a in args]


def bemiter_options(**kw):
    """Options of the iterative solver (BEM/@bemiter/options.m:19-44)."""
    op = {"solver": "gmres", "tol": 1e-6, "maxit": 100, "restart": None, "precond": "full", "output": 0,
          "cleaf": 200, "htol": 1e-6, "kmax": [4, 100], "eta": 2.5, "reuse_precond": False,
          "refresh_steps": 0}
    op.update(kw)
    return op


class bemretiter(bemret):
    """Iterative retarded solver (BEM/@bemretiter) on one GPU.

    H-matrices of G1, H1, G2, H2 on a cluster tree of the faces: full blocks
    hold the complete Green function (refinement included), far blocks are
    compressed by adaptive cross approximation (tolerance ``htol``, rank at
    most ``max(kmax)``).  ``sig = bem.mldivide(exc(p, enei))`` runs GMRES on
    the operator of afun.m with H-matrix products, preconditioned by the dense
    inverses of bemret (``precond='full'``, in the solver's precision), by
    H-matrix LU factors (``precond='hmat'``: initprecond.m with the H-matrix
    arithmetic of hlib on the GPU, FP64, truncation with ``max(htol)`` and
    ``min(kmax)``) or not at all (``precond=None``).  After a solve ``bem.info`` holds flag, iter,
    relres, true_relres, rank_max, rank_mean, compression and precond_enei.
    ``reuse_precond=True`` (not in the reference) keeps the preconditioner of
    an earlier wavelength (rebuilt when a solve needed more than
    ``refresh_steps`` GMRES steps): a sweep then pays the dense inversion
    once instead of at every wavelength, with the same solutions to ``tol``.

    Solvers 'gmres', 'cgs' and 'bicgstab' (@bemiter/solve.m).
    """

    def __init__(self, p, op=None):
        op = bemoptions(op)
        it = bemiter_options(**op.get("iter", {}))
        for k in ("solver", "tol", "maxit", "restart", "precond", "cleaf", "htol", "kmax", "eta", "reuse_precond",
                  "refresh_steps"):
            if k in op:
                it[k] = op[k]
        if it["solver"] not in ("gmres", "cgs", "bicgstab"):
            raise ValueError("solver must be 'gmres', 'cgs' or 'bicgstab'")
        if it["precond"] not in ("full", "hmat", None, ""):
            raise ValueError("precond must be 'full', 'hmat' or None")
        super().__init__(p, op)
        from .hmatrix import hpartition
        self.iter_op = it
        self.hpart = hpartition(p, it["cleaf"], it["eta"])
        self.info = None

    def _opts(self, reuse=None):
        it = dict(self.iter_op)
        if reuse is not None:
            it["reuse_precond"] = reuse
        o = _lib.IterOptions()
        o.solver = ("gmres", "cgs", "bicgstab").index(it["solver"])
        o.tol = float(it["tol"])
        o.maxit = int(it["maxit"])
        o.restart = int(it["restart"] or 0)
        o.precond = {"full": 1, "hmat": 2}.get(it["precond"], 0)
        o.htol = float(np.min(it["htol"]))
        o.kmax = int(np.max(it["kmax"]))
        o.kmax_precond = int(np.min(it["kmax"]))
        o.htol_precond = float(np.max(it["htol"]))
        o.reuse_precond = int(bool(it["reuse_precond"]))
        o.refresh_steps = int(it["refresh_steps"] or 0)
        return o

    def hmat_full(self, enei, which):
        """H-matrix ``which`` ('G1', 'H1', 'G2', 'H2') expanded to a dense
        [n, n] array (@hmatrix/full.m) and the ACA ranks [4, nlow]."""
        q = ("G1", "H1", "G2", "H2").index(which)
        em = np.ascontiguousarray(self._eps(float(enei))[0])
        n = self.p.n
        out = np.zeros((n, n), np.complex128)
        ranks = np.zeros((4, max(1, self.hpart.low.shape[0])), np.int32)
        o = self._opts()
        _lib.check(self._lib.mnpbem_hmat_full(
            self._h, ctypes.byref(self.hpart.c), ctypes.byref(o), float(enei),
            em.view(np.float64).ctypes.data_as(_lib.c_double_p), em.size, q, out.ctypes.data, ranks.ctypes.data))
        return out, ranks[:, :self.hpart.low.shape[0]]

    def mldivide(self, exc, reuse=None):
        """sig = bem \\ exc(p, enei) with preconditioned GMRES (bemretiter/solve.m);
        ``reuse`` overrides the ``reuse_precond`` option for this call."""
        enei = float(exc.enei)
        n = self.p.n
        em = np.ascontiguousarray(self._eps(enei)[0])
        o = self._opts(reuse)
        info = _lib.IterInfo()
        keep = []
        if hasattr(exc, "exc"):
            pw = exc.exc._struct()
            P = exc.exc.npol
            pot_ptr = None
        else:
            keys1, keys3 = ("phi1", "phi1p", "phi2", "phi2p"), ("a1", "a1p", "a2", "a2p")
            P = next(np.asarray(getattr(exc, k)).shape[-1] for k in keys1 + keys3 if hasattr(exc, k))
            if P > 4:
                raise ValueError("bemretiter: at most 4 excitation columns per solve")
            pot = _lib.Potentials()
            pot.npol = P
            for k in keys1 + keys3:
                if hasattr(exc, k):
                    arr = np.ascontiguousarray(np.asarray(getattr(exc, k)), dtype=np.complex128)
                    keep.append(arr)
                    setattr(pot, k, arr.ctypes.data)
            pw = None
            pot_ptr = ctypes.byref(pot)
        sig = {k: np.zeros((n, P) if k.startswith("sig") else (n, 3, P), np.complex128)
               for k in ("sig1", "sig2", "h1", "h2")}
        ext, sca = np.zeros(P), np.zeros(P)
        it, res = np.zeros(1, np.int32), np.zeros(1)
        sol = _lib.Solution()
        sol.sig1, sol.sig2 = sig["sig1"].ctypes.data, sig["sig2"].ctypes.data
        sol.h1, sol.h2 = sig["h1"].ctypes.data, sig["h2"].ctypes.data
        sol.ir_iters, sol.ir_resid = it.ctypes.data, res.ctypes.data
        if pw is not None:
            sol.ext, sol.sca = ext.ctypes.data, sca.ctypes.data
        _lib.check(self._lib.mnpbem_solve_iter(
            self._h, ctypes.byref(self.hpart.c), ctypes.byref(o), ctypes.byref(pw) if pw is not None else None,
            pot_ptr, enei, em.view(np.float64).ctypes.data_as(_lib.c_double_p), em.size, self.precision, ctypes.byref(sol),
            ctypes.byref(info)))
        self.info = {k: getattr(info, k) for k, _ in _lib.IterInfo._fields_}
        extra = {"ext": ext, "sca": sca} if pw is not None else {}
        return compstruct(self.p, enei, iter=int(it[0]), relres=float(res[0]), **sig, **extra)

    solve = mldivide

    def spectrum(self, exc, enei, fields=False, out=None):
        """Wavelength sweep through the iterative solver (one mnpbem_solve_iter
        call per wavelength): dict with ext, sca [nenei, npol], GMRES steps
        ``ir_iters`` and true relative residuals ``ir_resid`` [nenei] (+ sig1,
        sig2, h1, h2 with ``fields``).  With ``reuse_precond`` the preconditioner
        is built at the first wavelength and reused (rebuilt when a solve needed
        more than ``refresh_steps`` steps).  ``out`` is not used."""
        eneis = np.atleast_1d(np.asarray(enei, dtype=np.float64))
        # a sweep builds its preconditioner at its first wavelength
        sigs, self.sweep_info = [], []
        for i, e in enumerate(eneis):
            sigs.append(self.mldivide(exc(self.p, float(e)), reuse=False if i == 0 else None))
            self.sweep_info.append(dict(self.info))
        res = {"ext": np.array([s.ext for s in sigs]), "sca": np.array([s.sca for s in sigs]),
               "ir_iters": np.array([s.iter for s in sigs], dtype=np.int32),
               "ir_resid": np.array([s.relres for s in sigs])}
        if fields:
            for k in ("sig1", "sig2", "h1", "h2"):
                res[k] = np.array([getattr(s, k) for s in sigs])
        return res


def bemsolver(p, op=None, **kw):
    """Factory of Base/bemsolver.m: picks the solver class whose needs match op
    (``'iter'`` in the options selects bemretiter, as its needs = {'iter'})."""
    op = bemoptions(op, **kw)
    if op.get("sim", "ret") != "ret":
        raise NotImplementedError("only the retarded solver (sim='ret') is implemented")
    if "iter" in op:
        return bemretiter(p, op)
    return bemret(p, op)
