"""GB300-native retarded BEM hot path of MNPBEM.

compgreenret assembly (G, F -> G1, H1, G2, H2 with near-field refinement),
the bemret solve (Garcia de Abajo & Howie) and plane-wave extinction /
scattering spectra run in ``libmnpbem_gpu.so`` (hand-written CUDA for
sm_103a, C ABI in ``include/mnpbem_gpu.h``).  This package mirrors MNPBEM's
MATLAB calling surface on top of that library.
"""
from .materials import EV2NM, epsconst, epsdrude, epsfun, epstable  # noqa: F401
from .particles import (comparticle, curved, lglnodes, particle, quadface, tricube, trirod,  # noqa: F401
                        trisphere, trispheresegment)
from .bem import (bemiter_options, bemoptions, bemret, bemretiter, bemsolver, compstruct, dipoleret,  # noqa: F401
                  meshfield, planewave, planewaveret, point_media, spectrum_batch, spectrumret)
from .hmatrix import clustertree, hmatrix_blocks, hpartition  # noqa: F401
from .mie import mieret, miesolver  # noqa: F401

__version__ = "0.1.0"
