"""CPU FP64 oracle for the MNPBEM retarded BEM path — TEST INFRASTRUCTURE ONLY.

This package restates, in NumPy/SciPy FP64, the reference MATLAB code of the
path (geometry -> near-field refinement -> compgreenret assembly -> bemret
solve -> plane-wave spectra, plus Mie theory).  Every function cites the
reference file:line it follows (paths relative to the MNPBEM17 checkout).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg (and its ``--impl reference`` arm) may import this package, and only as
the checker / the timed CPU baseline.  The product path (``mnpbem_gb300``)
never imports it.

Parity status: **parity unpinned**.  MNPBEM ships no tests, golden vectors or
stored outputs for this path, and MATLAB/Octave are not available to run the
reference, so no output of the reference itself pins this restatement.  The
restatement is instead checked against independent known answers: exactness
of the quadrature rules, the Fuchs-Liu closed-surface sum rule, consistency of
the direct solve with the full BEM operator (``afun``), and Mie theory for
spheres (a physics check with a stated discretisation error).
"""
from .mnpbem_ref import *  # noqa: F401,F403
