"""torch.autograd wrappers of the adjoint cross-section gradients
(mnpbem_cross_section_gradient).

``extinction(verts, eps, faces, enei, pol, dir, eps_out)`` and
``scattering(...)`` return the extinction / scattering cross section of one
closed particle as a differentiable function of the vertex coordinates
``verts`` (float64 [nverts, 3]) and of the complex dielectric function ``eps``
of the particle, passed as a real tensor ``[Re eps, Im eps]``.  The forward
pass builds the geometry and solves on the GPU in FP64; the backward pass
returns the adjoint gradient computed with it, so ``torch.autograd.gradcheck``
compares the adjoint with central finite differences of the same library.
The scattering cross section integrates over the plane wave's sphere at
infinity (scattering.m).
"""
import numpy as np

from . import bem as _bem
from .materials import epsconst
from .particles import comparticle, particle


def _solve(verts, eps, faces, enei, pol, dirv, eps_out, device, which):
    p = particle(verts, faces)
    cp = comparticle([epsconst(eps_out), epsconst(eps)], [p], [[2, 1]], 1)
    solver = _bem.bemsolver(cp, _bem.bemoptions(precision="fp64", device=device))
    exc = _bem.planewave([pol], [dirv])
    return solver.cross_section_gradient(exc, enei, 0, which)


def _function():
    import torch

    class CrossSectionFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, verts, eps_ri, faces, enei, pol, dirv, eps_out, device, which):
            v = verts.detach().cpu().numpy().astype(np.float64)
            e = complex(float(eps_ri[0]), float(eps_ri[1]))
            ext, gv, ge = _solve(v, e, faces, enei, pol, dirv, eps_out, device, which)
            ctx.save_for_backward(torch.as_tensor(gv, dtype=verts.dtype, device=verts.device),
                                  torch.tensor([ge.real, ge.imag], dtype=eps_ri.dtype, device=eps_ri.device))
            return torch.tensor(ext, dtype=verts.dtype, device=verts.device)

        @staticmethod
        def backward(ctx, grad_out):
            gv, ge = ctx.saved_tensors
            return grad_out * gv, grad_out * ge, None, None, None, None, None, None, None

    return CrossSectionFn


_FN = None


def _apply(which, verts, eps_ri, faces, enei, pol, dir, eps_out, device):
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(verts, eps_ri, np.asarray(faces), float(enei), tuple(pol), tuple(dir), float(eps_out),
                     int(device), which)


def extinction(verts, eps_ri, faces, enei, pol=(1.0, 0.0, 0.0), dir=(0.0, 0.0, 1.0), eps_out=1.77, device=0):
    """Differentiable extinction cross section (see module docstring)."""
    return _apply("ext", verts, eps_ri, faces, enei, pol, dir, eps_out, device)


def scattering(verts, eps_ri, faces, enei, pol=(1.0, 0.0, 0.0), dir=(0.0, 0.0, 1.0), eps_out=1.77, device=0):
    """Differentiable scattering cross section (see module docstring)."""
    return _apply("sca", verts, eps_ri, faces, enei, pol, dir, eps_out, device)
