"""ctypes binding of ``libmnpbem_gpu.so`` (declared in ``include/mnpbem_gpu.h``).

The library is the only compute path of this package: if it cannot be loaded
the import of the solver fails with an error, there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmnpbem_gpu.so")

MNPBEM_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "CUDA", 3: "OUT_OF_MEMORY", 4: "SINGULAR",
                5: "NOT_CONVERGED", 6: "TIMEOUT", 7: "UNSUPPORTED"}
FP64, MIXED, FP32 = 0, 1, 2

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_int32_p = ctypes.POINTER(ctypes.c_int32)


class MnpbemError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("mnpbem status %s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


class Quad(ctypes.Structure):
    _fields_ = [("n_tri", ctypes.c_int32), ("x", c_double_p), ("y", c_double_p), ("w", c_double_p),
                ("n_pol3", ctypes.c_int32), ("x3", c_double_p), ("y3", c_double_p), ("w3", c_double_p),
                ("n_pol4", ctypes.c_int32), ("x4", c_double_p), ("y4", c_double_p), ("w4", c_double_p)]


class Options(ctypes.Structure):
    _fields_ = [("rel_cutoff", ctypes.c_double), ("abs_cutoff", ctypes.c_double),
                ("order", ctypes.c_int32), ("device", ctypes.c_int32)]


class PlaneWave(ctypes.Structure):
    _fields_ = [("npol", ctypes.c_int32), ("pol", c_double_p), ("dir", c_double_p),
                ("medium", ctypes.c_int32), ("ninf", ctypes.c_int32), ("inf_nvec", c_double_p),
                ("inf_area", c_double_p)]


class Solution(ctypes.Structure):
    _fields_ = [("ext", ctypes.c_void_p), ("sca", ctypes.c_void_p), ("sig1", ctypes.c_void_p),
                ("sig2", ctypes.c_void_p), ("h1", ctypes.c_void_p), ("h2", ctypes.c_void_p),
                ("ir_iters", ctypes.c_void_p), ("ir_resid", ctypes.c_void_p),
                ("outputs_on_device", ctypes.c_int32)]


class Potentials(ctypes.Structure):
    _fields_ = [("npol", ctypes.c_int32)] + [(k, ctypes.c_void_p) for k in
                                             ("phi1", "phi1p", "phi2", "phi2p", "a1", "a1p", "a2", "a2p")]


class ClusterTree(ctypes.Structure):
    _fields_ = [("ncluster", ctypes.c_int32), ("son", ctypes.c_void_p), ("cind", ctypes.c_void_p),
                ("ipart", ctypes.c_void_p), ("perm", ctypes.c_void_p), ("nfull", ctypes.c_int32),
                ("full", ctypes.c_void_p), ("nlow", ctypes.c_int32), ("low", ctypes.c_void_p)]


class IterOptions(ctypes.Structure):
    _fields_ = [("solver", ctypes.c_int32), ("tol", ctypes.c_double), ("maxit", ctypes.c_int32),
                ("restart", ctypes.c_int32), ("precond", ctypes.c_int32), ("htol", ctypes.c_double),
                ("kmax", ctypes.c_int32), ("reuse_precond", ctypes.c_int32), ("refresh_steps", ctypes.c_int32),
                ("kmax_precond", ctypes.c_int32), ("htol_precond", ctypes.c_double)]


class IterInfo(ctypes.Structure):
    _fields_ = [("flag", ctypes.c_int32), ("iter", ctypes.c_int32), ("relres", ctypes.c_double),
                ("true_relres", ctypes.c_double), ("rank_max", ctypes.c_int32), ("rank_mean", ctypes.c_double),
                ("compression", ctypes.c_double), ("precond_enei", ctypes.c_double)]


class Refine(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_int32), ("tol", ctypes.c_double)]


class Job(ctypes.Structure):
    _fields_ = [("g", ctypes.c_void_p), ("exc", ctypes.POINTER(PlaneWave)), ("nenei", ctypes.c_int32),
                ("enei", c_double_p), ("eps_media", c_double_p), ("nmed", ctypes.c_int32),
                ("out", ctypes.POINTER(Solution))]


# name -> (restype, argtypes)
SIGNATURES = {
    "mnpbem_geom_create": (ctypes.c_int, [c_double_p, ctypes.c_int64, c_int64_p, ctypes.c_int64,
                                          ctypes.c_int32, c_int64_p, c_int32_p, c_int32_p,
                                          ctypes.POINTER(Quad), ctypes.POINTER(Options),
                                          ctypes.POINTER(ctypes.c_void_p)]),
    "mnpbem_geom_create_curved": (ctypes.c_int, [c_double_p, ctypes.c_int64, c_int64_p, ctypes.c_int64,
                                                 ctypes.c_int32, c_int64_p, c_int32_p, c_int32_p,
                                                 ctypes.POINTER(Quad), ctypes.POINTER(Options),
                                                 ctypes.POINTER(ctypes.c_void_p)]),
    "mnpbem_geom_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "mnpbem_solve_potentials": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Potentials), ctypes.c_double,
                                               c_double_p, ctypes.c_int32, ctypes.c_int32,
                                               ctypes.POINTER(Refine), ctypes.POINTER(Solution)]),
    "mnpbem_solve_iter": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ClusterTree), ctypes.POINTER(IterOptions),
                                         ctypes.POINTER(PlaneWave), ctypes.POINTER(Potentials), ctypes.c_double,
                                         c_double_p, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(Solution),
                                         ctypes.POINTER(IterInfo)]),
    "mnpbem_hmat_full": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ClusterTree), ctypes.POINTER(IterOptions),
                                        ctypes.c_double, c_double_p, ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_void_p, ctypes.c_void_p]),
    "mnpbem_fields": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, c_double_p, c_int32_p, ctypes.c_double,
                                     c_double_p, ctypes.c_int32, ctypes.c_int32] + [ctypes.c_void_p] * 6),
    "mnpbem_surface_fields": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, c_double_p, ctypes.c_int32,
                                             ctypes.c_int32, ctypes.c_int32] + [ctypes.c_void_p] * 10),
    "mnpbem_farfield": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, c_double_p, ctypes.c_int32,
                                       ctypes.c_int32, ctypes.c_int64, c_double_p, ctypes.c_int32]
                        + [ctypes.c_void_p] * 6),
    "mnpbem_geom_size": (ctypes.c_int, [ctypes.c_void_p, c_int64_p, c_int64_p]),
    "mnpbem_geom_export": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.c_void_p] * 9),
    "mnpbem_assemble": (ctypes.c_int, [ctypes.c_void_p, c_double_p, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p]),
    "mnpbem_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(PlaneWave), ctypes.c_int32,
                                    c_double_p, c_double_p, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.POINTER(Refine), ctypes.POINTER(Solution)]),
    "mnpbem_solve_batch": (ctypes.c_int, [ctypes.POINTER(Job), ctypes.c_int32, ctypes.c_int32,
                                          ctypes.POINTER(Refine)]),
    "mnpbem_ext_gradient": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(PlaneWave), ctypes.c_int32,
                                           ctypes.c_double, c_double_p, ctypes.c_int32, ctypes.c_int32,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "mnpbem_cross_section_gradient": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(PlaneWave), ctypes.c_int32,
                                                     ctypes.c_int32, ctypes.c_double, c_double_p, ctypes.c_int32,
                                                     ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                                     ctypes.c_void_p]),
    "mnpbem_bem_matrices": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, c_double_p,
                                           ctypes.c_int32, ctypes.c_int32] + [ctypes.c_void_p] * 5),
    "mnpbem_profile_enable": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "mnpbem_profile_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "mnpbem_profile_read": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, c_double_p, c_double_p,
                                           c_double_p, c_int64_p]),
    "mnpbem_gemm_c64": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, ctypes.c_int64,
                                       ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                       ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_int64]),
    "mnpbem_cross_sections_noalloc": (ctypes.c_int, [ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64,
                                                     ctypes.c_int32] + [ctypes.c_void_p] * 10
                                                    + [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                                       ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                                       ctypes.c_void_p, ctypes.c_void_p]),
    "mnpbem_geom_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "mnpbem_geom_set_lanes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "mnpbem_geom_set_option": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int32]),
    "mnpbem_geom_stat": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, c_double_p]),
    "mnpbem_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32]),
    # H-matrix arithmetic (handles are void*)
    "mnpbem_hm_create": (ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(ClusterTree), ctypes.c_double, ctypes.c_int32,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "mnpbem_hm_set_options": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int32]),
    "mnpbem_hm_lu": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "mnpbem_hm_rsolve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "mnpbem_hm_inv": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "mnpbem_hm_lsolve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "mnpbem_hm_matmul": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "mnpbem_hm_add": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                     ctypes.POINTER(ctypes.c_void_p)]),
    "mnpbem_hm_scale": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char,
                                       ctypes.POINTER(ctypes.c_void_p)]),
    "mnpbem_hm_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char, ctypes.c_void_p, ctypes.c_int32]),
    "mnpbem_hm_mul": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "mnpbem_hm_full": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "mnpbem_hm_sizes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_int64)]),
    "mnpbem_hm_export": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p]),
    "mnpbem_hm_free": (None, [ctypes.c_void_p]),
    "mnpbem_last_error": (ctypes.c_char_p, []),
    "mnpbem_version": (ctypes.c_char_p, []),
}

_LIB = None


def load(path=None):
    """Load the library (once).  Raises if it is missing: no CPU fallback."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError("libmnpbem_gpu.so not found at %s; run mnpbem_gb300.build.build() "
                          "(nvcc, sm_103a) first" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status):
    if status != MNPBEM_OK:
        msg = load().mnpbem_last_error()
        raise MnpbemError(status, msg.decode() if msg else "")


def dptr(a):
    """double* of a C-contiguous float64/complex128 numpy array."""
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(c_double_p)


def vptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)
