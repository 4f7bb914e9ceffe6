#!/usr/bin/env python
"""Throughput of the retarded BEM path: wavelength-solves/s on GB300.

One wavelength-solve = assembly of G1, H1, G2, H2 (with near-field
refinement), the bemret factorisations and products, the mldivide chain for
all polarisations, FP64-class iterative refinement (mixed precision), and the
extinction and scattering cross sections.  The per-geometry set-up
(refinement coefficients, closed-surface sum rule) runs once before timing,
like ``bem = bemsolver(p, op)`` in MNPBEM.

Default workload (synthetic, deterministic; the configuration the metric's
target is stated on): a dimer of two d = 50 nm spheres with a 2 nm gap,
12 000 flat faces each, Drude metal eps(w) = 10 - 9.065^2 / (w (w + 0.0708 i))
(w in eV) in eps = 1.77, plane wave polarised along the dimer axis (x)
travelling along +z, wavelengths on the 32-point grid 500..900 nm.  A step is
one batch of ``--batch`` wavelengths per GPU, which the library runs as one
CUDA graph (its lanes take the wavelengths from a device-side queue and decide
the refinement steps on the device; ``MNPBEM_SWEEP_GRAPH=0`` selects the
host-polled scheduler, same results); with N GPUs rank r takes its own
wavelengths (weak scaling, no collective on the data path).  The line also
carries the plain FP64 GPU path on one wavelength of the same workload, the
CPU oracle on the same geometry at a smaller size (extrapolated), the GPU
results against that oracle, and a short run of the 4000-face sphere.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--workload ...]
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "wavelength-solves/s at N faces: mixed+batched vs FP64 GPU, ext err ≤1e-6"
UNIT = "wavelength-solves/s"
DRUDE = (10.0, 9.065, 0.0708)

# Workloads.  dimer24k is the configuration the metric's target is stated on:
# two d = 50 nm spheres with a 2 nm gap, 12 000 flat faces each (separate
# media, so G1 and H1 are block-diagonal), x-polarised (along the dimer axis)
# along +z, 32 wavelengths 500-900 nm.  sphere4000: one d = 50 nm sphere with
# 4000 faces, 60 wavelengths 450-750 nm.
WORKLOADS = {
    "dimer24k": {"faces": 24000, "grid": (500.0, 900.0, 32), "batch": 3, "dimer": True},
    "sphere4000": {"faces": 4000, "grid": (450.0, 750.0, 60), "batch": 20, "dimer": False},
}
# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of the dominant
# tensor-core launch of each workload, from one ncu capture (filled per workload
# once captured; None: not captured)
TC_TRAFFIC = {
    "dimer24k": {"bytes": 9.9e9,
                 "note": "dram__bytes_read.sum + dram__bytes_write.sum of one scaled-FP16 rank-1024 update captured "
                         "at M = N = 5888 (652 MB measured against 627 MB algorithmic), scaled by the C tile count "
                         "to the first trailing update of the 24 000-face G2 (M = N = 22 976); the capture of the "
                         "full-size launch exceeds the profiler's memory rule"},
}
# faces of the CPU sample (the oracle) for each workload: the same geometry at
# a size the oracle solves in seconds
CPU_FACES = {"dimer24k": 4000, "sphere4000": 4000}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dimer24k",
                    choices=["dimer24k", "sphere4000", "batch3", "iter24k", "gemm_rank1024"],
                    help="dimer24k: two 12000-face spheres, 32 wavelengths (the headline); sphere4000: one "
                         "4000-face sphere, 60 wavelengths; batch3: three particles of uneven size, 128 "
                         "wavelengths, two polarisations; iter24k: the dimer through the iterative H-matrix solver; "
                         "gemm_rank1024: one rank-1024 trailing update of the factorisations (5888 x 5888 complex "
                         "C, device-resident) on the TF32 and the scaled-FP16 tensor-core paths")
    ap.add_argument("--faces", type=int, default=0, help="faces of the workload (0: its own)")
    ap.add_argument("--batch", type=int, default=0, help="wavelengths per step per GPU (0: the workload's)")
    ap.add_argument("--lanes", type=int, default=0, help="wavelengths in flight at once (0: library default)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--refine-tol", type=float, default=1e-8,
                    help="mixed precision: refinement stops at ||dx|| <= tol ||x|| (the metric asks for an "
                         "extinction error <= 1e-6 against FP64; the library default is 1e-10)")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true", help="skip the FP64 GPU wavelength at full size")
    ap.add_argument("--skip-c2", action="store_true", help="skip the side runs of configurations 2, 3 and 4")
    ap.add_argument("--cpu-faces", type=int, default=0, help="faces of the CPU sample (0: the workload's)")
    ap.add_argument("--profile-steps", type=int, default=3, help="steps of the profiled repeat")
    ap.add_argument("--iter-precond", choices=("full", "hmat"), default="full",
                    help="preconditioner of --workload iter24k: the dense inverses ('full') or H-matrix LU ('hmat')")
    ap.add_argument("--iter-faces", type=int, default=24000,
                    help="iter24k: total faces of the dimer (smaller sizes for profiling runs)")
    a = ap.parse_args()
    if a.workload in WORKLOADS:
        w = WORKLOADS[a.workload]
        a.faces = a.faces or w["faces"]
        a.batch = a.batch or w["batch"]
        a.cpu_faces = a.cpu_faces or CPU_FACES[a.workload]
    return a


def grid(a):
    lo, hi, num = WORKLOADS[a.workload]["grid"]
    return np.linspace(lo, hi, num)


def step_wavelengths(a, step, rank, world, batch):
    g = grid(a)
    base = (step * world + rank) * batch
    return g[(base + np.arange(batch)) % g.size]


def max_over_ranks(dist, values, device, torch):
    """Per-rank timings reduced to their maximum over ranks (the slowest rank
    sets the whole job's time); unchanged without a process group."""
    if dist is None:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def workload_desc(a, faces=None, batch=None):
    faces = faces or a.faces
    lo, hi, num = WORKLOADS[a.workload]["grid"]
    tail = ", Drude eps_inf=10 wp=9.065 eV gamma=0.0708 eV in eps=1.77, x-pol along +z, %d-point wavelength " \
           "grid %g-%g nm" % (num, lo, hi)
    if batch:
        tail += ", %d wavelengths per step per GPU" % batch
    if WORKLOADS[a.workload]["dimer"]:
        return "dimer of two d=50 nm spheres, 2 nm gap, 2 x %d flat faces (separate media)" % (faces // 2) + tail
    return "sphere d=50 nm, %d flat faces" % faces + tail


# --------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------- our arm
def drude():
    import mnpbem_gb300 as m
    e0, wp, g = DRUDE
    return m.epsfun(lambda w: e0 - wp ** 2 / (w * (w + 1j * g)), "eV")


def geometry(faces, dimer):
    """(particles, inout, closed) of the workload's geometry at ``faces`` faces."""
    import mnpbem_gb300 as m
    from mnpbem_gb300 import shapes
    if dimer:
        nf = faces // 2
        v1, f1 = shapes.fibsphere(nf, 50.0, center=(-26.0, 0.0, 0.0))
        v2, f2 = shapes.fibsphere(nf, 50.0, center=(26.0, 0.0, 0.0))
        return [(v1, f1), (v2, f2)], [[2, 1], [3, 1]]
    v, f = shapes.fibsphere(faces, 50.0)
    return [(v, f)], [[2, 1]]


def make_solver(faces, dimer, device, precision, lanes=0, refine_tol=1e-8):
    import mnpbem_gb300 as m
    parts, inout = geometry(faces, dimer)
    eps = [m.epsconst(1.77)] + [drude() for _ in parts]
    cp = m.comparticle(eps, [m.particle(v, f) for v, f in parts], inout, *range(1, len(parts) + 1))
    bem = m.bemsolver(cp, m.bemoptions(precision=precision, device=device, lanes=lanes))
    bem.refine_iters = 20
    bem.refine_tol = refine_tol
    return cp, bem


def make_problem(a, device, precision):
    import mnpbem_gb300 as m
    cp, bem = make_solver(a.faces, WORKLOADS[a.workload]["dimer"], device, precision, a.lanes, a.refine_tol)
    exc = m.planewave([1, 0, 0], [0, 0, 1])
    return cp, bem, exc


class DeviceSweep:
    """Direct C-ABI call with device-resident outputs (the ``value`` path)."""

    def __init__(self, bem, exc, batch, torch):
        from mnpbem_gb300 import _lib
        self._lib, self.bem, self.exc, self.batch = _lib, bem, exc, batch
        n, P = bem.p.n, exc.npol
        dev = torch.device("cuda", torch.cuda.current_device())
        self.ext = torch.empty((batch, P), dtype=torch.float64, device=dev)
        self.sca = torch.empty((batch, P), dtype=torch.float64, device=dev)
        self.sig1 = torch.empty((batch, n, P, 2), dtype=torch.float64, device=dev)
        self.sig2 = torch.empty((batch, n, P, 2), dtype=torch.float64, device=dev)
        self.h1 = torch.empty((batch, n, 3, P, 2), dtype=torch.float64, device=dev)
        self.h2 = torch.empty((batch, n, 3, P, 2), dtype=torch.float64, device=dev)
        self.iters = np.zeros(batch, dtype=np.int32)
        self.resid = np.zeros(batch)
        self.pw = exc._struct()
        self.ref = _lib.Refine(bem.refine_iters, bem.refine_tol)

    def run(self, enei):
        _lib = self._lib
        enei = np.ascontiguousarray(enei, dtype=np.float64)
        em = np.ascontiguousarray(self.bem.p.eps_media(enei))
        sol = _lib.Solution()
        sol.ext, sol.sca = self.ext.data_ptr(), self.sca.data_ptr()
        sol.sig1, sol.sig2 = self.sig1.data_ptr(), self.sig2.data_ptr()
        sol.h1, sol.h2 = self.h1.data_ptr(), self.h2.data_ptr()
        sol.ir_iters, sol.ir_resid = self.iters.ctypes.data, self.resid.ctypes.data
        sol.outputs_on_device = 1
        _lib.check(self.bem._lib.mnpbem_solve(
            self.bem.handle, ctypes.byref(self.pw), enei.size, _lib.dptr(enei),
            em.view(np.float64).ctypes.data_as(_lib.c_double_p), em.shape[1], self.bem.precision,
            ctypes.byref(self.ref), ctypes.byref(sol)))


def lib_stream(bem, torch):
    from mnpbem_gb300 import _lib
    s = ctypes.c_void_p()
    _lib.check(bem._lib.mnpbem_geom_stream(bem.handle, ctypes.byref(s)))
    return torch.cuda.ExternalStream(s.value)


def tuned_lanes(n, precision):
    """Lane count the library uses when none is given: the tuned table's entry
    for this size, else its automatic default."""
    from mnpbem_gb300 import autotune
    lanes = autotune.settings_for(n, precision).get("lanes")
    return "tuned: %d" % lanes if lanes else "auto"


def read_profile(bem):
    from mnpbem_gb300 import _lib
    names = ["assembly", "gemm_n3", "gemm_thin", "block_inverse", "elementwise", "spectra", "geometry",
             "hmat_build", "hmat_matvec"]
    out = {}
    for ph, nm in enumerate(names):
        ms, fl, by = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        nl = ctypes.c_int64()
        _lib.check(bem._lib.mnpbem_profile_read(bem.handle, ph, ctypes.byref(ms), ctypes.byref(fl),
                                                ctypes.byref(by), ctypes.byref(nl)))
        out[nm] = {"ms": ms.value, "flops": fl.value, "bytes": by.value, "launches": nl.value}
    return out


def peaks():
    """(HBM GB/s, bf16 TFLOP/s burst, bf16 TFLOP/s sustained, source)."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return d["hbm_gbs"], d["bf16_tflops"], d.get("bf16_tflops_sustained", d["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, 1700.0, "fallback"


def solve_flops(n, dimer):
    """Real FLOP of the n^3 work of one wavelength as the library factors it:
    block LU of G1 (per particle block), of G2 and of Sigma (8/3 n^3 each),
    Sigma1 = H1 G1^-1 and Sigma2 = H2 G2^-1 by two triangular solves each
    (8 n^3, per block for G1), Deltai by Gauss-Jordan inversion (8 n^3)."""
    nb = n / 2 if dimer else n
    nblk = 2 if dimer else 1
    g1 = nblk * (8.0 / 3.0 + 8.0) * nb ** 3
    return g1 + (8.0 / 3.0 + 8.0 + 8.0 + 8.0 / 3.0) * n ** 3


def run_ours(a, rank, world, dist, torch):
    device = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    cp, bem, exc = make_problem(a, device, a.precision)
    sweep = DeviceSweep(bem, exc, a.batch, torch)
    stream = lib_stream(bem, torch)
    n, P = cp.n, exc.npol
    sw = lambda s: step_wavelengths(a, s, rank, world, a.batch)

    def barrier():
        if dist is not None:
            dist.barrier()

    bem_lib = bem._lib
    for s in range(a.warmup):
        sweep.run(sw(s))
    # ---------------- timed region (device-resident outputs, no per-launch events)
    bem_lib.mnpbem_profile_reset(bem.handle)
    clocks = ClockSampler(device)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    torch.cuda.nvtx.range_push("timed")          # for launch lists of the timed steps (ncu --nvtx)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for s in range(a.steps):
        sweep.run(sw(a.warmup + s))
    e1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    launches_timed = read_profile(bem)
    block_cond = bem.stat("block_cond_max")
    iters = sweep.iters.copy()
    ext_timed = sweep.ext.cpu().numpy().copy()
    # ---------------- profiled repeat of a few of the same steps: CUDA events on
    # the library stream around every launch give per-kernel-class durations
    bem_lib.mnpbem_profile_enable(bem.handle, 1)
    sweep.run(sw(a.warmup))      # captures graphs with event nodes
    bem_lib.mnpbem_profile_reset(bem.handle)
    nprof = max(1, min(a.profile_steps, a.steps))
    for s in range(nprof):
        sweep.run(sw(a.warmup + s))
    torch.cuda.synchronize()
    bem_lib.mnpbem_profile_enable(bem.handle, 0)
    prof = read_profile(bem)
    # ---------------- e2e: public API, host (pinned) outputs, copies inside the region
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    host = {"ext": pin((a.batch, P), torch.float64), "sca": pin((a.batch, P), torch.float64),
            "sig1": pin((a.batch, n, P), torch.complex128), "sig2": pin((a.batch, n, P), torch.complex128),
            "h1": pin((a.batch, n, 3, P), torch.complex128), "h2": pin((a.batch, n, 3, P), torch.complex128)}
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for s in range(a.steps):
        bem.spectrum(exc, sw(a.warmup + a.steps + s), fields=True, out=host)
    f1.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = f0.elapsed_time(f1)
    e2e_wall = (time.perf_counter() - t0) * 1e3
    nmed = len(cp.eps)
    h2d = a.batch * (8 + 16 * nmed + 32 * n) + 48 * P + 32 * exc.spec.pinfty.n + 2 * n
    d2h = a.batch * (16 * P * 8 * n + 16 * P + 16)
    # ---------------- max over ranks
    ms, e2e_ms = max_over_ranks(dist, [ms, e2e_ms], "cuda", torch)
    total = a.batch * a.steps * world
    value = total / (ms / 1e3)
    e2e_value = total / (e2e_ms / 1e3)
    # ---------------- roofline: the tensor-core GEMMs (the dominant kernel class in
    # FLOPs and device time); timed inside seconds-long steps, so the reference
    # peak is the sustained bf16 rate
    hbm, bf16, bf16_sus, src = peaks()
    timing = ("CUDA events on the library stream around each launch, over a profiled repeat of %d of "
              "the timed steps" % nprof)
    d = prof["gemm_n3"]
    achieved = d["flops"] / (d["ms"] / 1e3) / 1e12 if d["ms"] > 0 else 0.0
    traffic = TC_TRAFFIC.get(a.workload)
    roof = {"kernel": "k_tc_gemm (tcgen05; kind::f16 on scaled FP16 operands for the rank-512/1024 updates, "
                      "kind::tf32 for the 256-wide panel products; all tensor-core GEMM launches)",
            "bound": "tensor", "achieved": achieved, "peak": bf16_sus, "unit": "TFLOP/s", "frac": achieved / bf16_sus,
            "peak_source": src + " sustained dense bf16 (FP16 MMAs issue at the bf16 rate; the kernel is timed "
                                 "inside seconds-long steps)",
            "traffic": traffic["bytes"] if traffic else None,
            "traffic_note": traffic["note"] if traffic else "no ncu capture of this configuration",
            "launches": d["launches"], "ms": d["ms"], "timing": timing,
            "flops_per_wavelength_n3": solve_flops(n, WORKLOADS[a.workload]["dimer"])}
    phases_roof = {}
    for k, v in prof.items():
        if v["ms"] <= 0 or k == "geometry":
            continue
        phases_roof[k] = {"ms": round(v["ms"], 3), "launches": v["launches"],
                          "GB/s": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1) if v["bytes"] else None,
                          "hbm_frac": round(v["bytes"] / (v["ms"] / 1e3) / 1e9 / hbm, 4) if v["bytes"] else None,
                          "TFLOP/s": round(v["flops"] / (v["ms"] / 1e3) / 1e12, 2) if v["flops"] else None}
    asm = prof["assembly"]
    nsol_prof = a.batch * nprof
    extra = {"phases_ms_per_wavelength": {k: round(v["ms"] / nsol_prof, 3) for k, v in prof.items()},
             "phases_roofline": phases_roof,
             "assembly_hbm_gbs": asm["bytes"] / (asm["ms"] / 1e3) / 1e9 if asm["ms"] > 0 else None,
             "assembled_pairs_per_s": (n * n * nsol_prof) / (asm["ms"] / 1e3) if asm["ms"] > 0 else None,
             "refinement_iterations": iters.tolist(),
             "pivot_stat": {"block_cond_max": block_cond, "g1_blocks": int(bem.stat("g1_blocks")),
                            "note": "largest max|A_kk| * max|inv(A_kk)| over the diagonal blocks of the LDU "
                                    "factorisations (G1, G2, Sigma) and of the Gauss-Jordan inverse of Delta, "
                                    "warm-up and timed steps; 1e6 fails the solve in complex64"},
             "launches_per_wavelength": sum(v["launches"] for k, v in launches_timed.items() if k != "geometry")
                                        / float(a.batch * a.steps)}
    launches = int(sum(v["launches"] for k, v in launches_timed.items() if k != "geometry"))
    out = {"value": value, "ms": ms, "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                                             "d2h_bytes_per_step": int(d2h), "ms": e2e_ms,
                                             "wall_ms": e2e_wall},
           "roofline": roof, "gpu_launches": launches, "clocks": clk, "extra": extra,
           "bem": bem, "exc": exc, "cp": cp, "ext_timed": ext_timed}
    return out


def fp64_full(a, torch, mixed):
    """The plain FP64 GPU path on one wavelength of the full workload, and the
    mixed path's error against it there.  The mixed handle is released first
    (both do not fit in device memory at 24 000 faces)."""
    import gc
    lam = 700.0
    bem, exc = mixed["bem"], mixed["exc"]
    rmx = bem.spectrum(exc, [lam])
    mixed["bem"] = None
    del bem
    gc.collect()
    torch.cuda.synchronize()
    device = torch.cuda.current_device()
    cp64, b64 = make_solver(a.faces, WORKLOADS[a.workload]["dimer"], device, "fp64", 1)
    r64, t64 = _timed(lambda: b64.spectrum(exc, [lam]), torch)
    del b64
    gc.collect()
    err_ext = float(np.max(np.abs(rmx["ext"][0] - r64["ext"][0]) / np.abs(r64["ext"][0])))
    err_sca = float(np.max(np.abs(rmx["sca"][0] - r64["sca"][0]) / np.abs(r64["sca"][0])))
    return {"value": 1.0 / t64, "unit": UNIT, "seconds": t64,
            "sample": "1 wavelength (%g nm) of the same %d-face workload through the FP64 path (block LU + "
                      "triangular solves + Gauss-Jordan inverse on CUDA-core FP64 GEMMs), host wall clock "
                      "around bemsolver.spectrum" % (lam, a.faces),
            "ext_rel_err_mixed_vs_fp64": err_ext, "sca_rel_err_mixed_vs_fp64": err_sca,
            "mixed_refine_tol": a.refine_tol}


# ------------------------------------------------- secondary workloads
def _timed(fn, torch):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def run_batch3(a, torch):
    """Three particles of uneven size (sphere d = 30 nm / 1000 faces, capped rod
    10 x 40 nm / 2500 quadrilaterals, cube 40 nm with 4 nm edge rounding / 2904
    faces), 128 wavelengths 400-900 nm, x and y polarisation along +z, solved
    together by mnpbem_solve_batch; one wavelength-solve = one particle at one
    wavelength (both polarisations)."""
    import mnpbem_gb300 as m
    from mnpbem_gb300 import shapes
    dev = torch.cuda.current_device()
    geo = [shapes.fibsphere(1000, 30.0), shapes.trirod(10.0, 40.0, (51, 11, 31)),
           shapes.tricube(23, 40.0, shapes.rounding_to_e(40.0, 4.0))]
    exc = m.planewave([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]])
    enei = np.linspace(400.0, 900.0, 128)

    def solvers(prec, lanes):
        out = []
        for v, f in geo:
            cp = m.comparticle([m.epsconst(1.77), drude()], [m.particle(v, f)], [[2, 1]], 1)
            out.append(m.bemsolver(cp, m.bemoptions(precision=prec, device=dev, lanes=lanes)))
            if prec == "mixed":
                out[-1].refine_tol = a.refine_tol
        return out
    bems = solvers("mixed", a.lanes)
    for _ in range(max(1, a.warmup)):
        m.spectrum_batch([(b, exc, enei) for b in bems])
    times = []
    for _ in range(a.steps):
        res, dt = _timed(lambda: m.spectrum_batch([(b, exc, enei) for b in bems]), torch)
        times.append(dt)
    nsol = len(bems) * enei.size
    value = nsol * a.steps / sum(times)
    # FP64 GPU on two wavelengths per particle, and the accuracy of the mixed results there
    b64 = solvers("fp64", 1)
    lam = enei[[20, 90]]
    m.spectrum_batch([(b, exc, lam[:1]) for b in b64])
    r64, t64 = _timed(lambda: m.spectrum_batch([(b, exc, lam) for b in b64]), torch)
    idx = [20, 90]
    err = max(float(np.max(np.abs(res[k]["ext"][idx] - r64[k]["ext"]) / np.abs(r64[k]["ext"]))) for k in range(3))
    v64 = 3 * lam.size / t64
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * sum(times) / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64(fp16/tf32)+f64", "data": "synthetic",
            "config": {"workload": "batch of 3 particles (sphere d=30 nm 1000 faces, capped rod 10x40 nm 2500 "
                                   "quadrilaterals, rounded cube 40 nm / 4 nm rounding 2904 faces), Drude metal in "
                                   "eps=1.77, x and y polarisation along +z, 128 wavelengths 400-900 nm per particle",
                       "faces": [int(b.p.n) for b in bems], "wavelength_solves_per_step": nsol,
                       "timing": "host wall clock around mnpbem_solve_batch (public API, ext/sca to host)",
                       "refine_tol": a.refine_tol},
            "fp64_gpu": {"value": v64, "unit": UNIT, "sample": "2 wavelengths x 3 particles, FP64 path"},
            "speedup_vs_fp64_gpu": value / v64, "ext_rel_err_mixed_vs_fp64": err,
            "refinement_iterations_max": int(max(int(r["ir_iters"].max()) for r in res)),
            "refinement_final_residual_max": float(max(float(r["ir_resid"].max()) for r in res))}


def run_iter(a, torch):
    """Iterative solver (bemretiter) on the 2 nm-gap dimer (--iter-faces,
    default 24000 faces): H-matrices of G1, H1, G2, H2 (leaves of at most 200
    faces, htol 1e-6, kmax 100), GMRES (tol 1e-6) preconditioned by the
    complex64 tensor-core inverses (--iter-precond full) or by H-matrix LU
    factors (hmat: no dense matrix).  Timed: a sweep of 8 wavelengths 600-740 nm
    that builds the preconditioner at its first wavelength and keeps it while
    GMRES needs at most 30 steps (reuse_precond), after a warm-up sweep of two
    wavelengths; then a profiled repeat at 600 nm (preconditioner rebuilt) for
    the H-matrix phases.  The extinction is compared with the direct mixed
    solve of the same handle at 600 and 740 nm."""
    import mnpbem_gb300 as m
    from mnpbem_gb300 import shapes
    dev = torch.cuda.current_device()
    nf = a.iter_faces // 2
    v1, f1 = shapes.fibsphere(nf, 50.0, center=(-26.0, 0.0, 0.0))
    v2, f2 = shapes.fibsphere(nf, 50.0, center=(26.0, 0.0, 0.0))
    cp = m.comparticle([m.epsconst(1.77), drude(), drude()], [m.particle(v1, f1), m.particle(v2, f2)],
                       [[2, 1], [3, 1]], 1, 2)
    bem = m.bemsolver(cp, m.bemoptions(precision="mixed", device=dev, lanes=1,
                                       iter=m.bemiter_options(cleaf=200, htol=1e-6, kmax=[4, 100],
                                                              precond=a.iter_precond, reuse_precond=True,
                                                              refresh_steps=30)))
    exc = m.planewave([1, 0, 0], [0, 0, 1])
    bem.spectrum(exc, [650.0, 660.0])
    eneis = np.linspace(600.0, 740.0, 8)
    res, dt = _timed(lambda: bem.spectrum(exc, eneis), torch)
    infos = bem.sweep_info
    lib = bem._lib
    lib.mnpbem_profile_enable(bem.handle, 1)
    lib.mnpbem_profile_reset(bem.handle)
    bem.mldivide(exc(cp, 600.0), reuse=False)
    lib.mnpbem_profile_enable(bem.handle, 0)
    prof = read_profile(bem)
    direct = bemret_spectrum(bem, exc, [600.0, 740.0])
    err = [abs(res["ext"][0, 0] - direct["ext"][0, 0]) / abs(direct["ext"][0, 0]),
           abs(res["ext"][-1, 0] - direct["ext"][1, 0]) / abs(direct["ext"][1, 0])]
    hbm, _, _, src = peaks()
    mv, hb = prof["hmat_matvec"], prof["hmat_build"]
    gbs = mv["bytes"] / (mv["ms"] * 1e-3) / 1e9 if mv["ms"] > 0 else None
    return {"metric": METRIC, "value": eneis.size / dt, "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": 1e3 * dt, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64-class H-matrix operator (double-single) + " + (
                "c64(tf32) dense preconditioner" if a.iter_precond == "full" else
                "f64 H-matrix LU preconditioner (hmat, kmax 4)"), "data": "synthetic",
            "config": {"workload": "iterative solver (bemretiter, H-matrices + GMRES) on the dimer of two d=50 nm "
                                   "spheres, 2 nm gap, 2 x %d faces, x-pol along +z, 8 wavelengths 600-740 nm" % nf,
                       "faces": 2 * nf, "cleaf": 200, "htol": 1e-6, "kmax": 100, "gmres_tol": 1e-6,
                       "precond": a.iter_precond,
                       "reuse_precond": True, "refresh_steps": 30,
                       "timing": "host wall clock around bemretiter.spectrum (public API, one mnpbem_solve_iter "
                                 "per wavelength, charges and ext/sca to host)"},
            "gmres_steps": [i["iter"] for i in infos], "precond_built_at": [i["precond_enei"] for i in infos],
            "true_relres": [i["true_relres"] for i in infos], "rank_max": infos[0]["rank_max"],
            "rank_mean": infos[0]["rank_mean"], "compression": infos[0]["compression"],
            "dense_fraction": bem.hpart.dense_fraction(), "low_rank_blocks": int(bem.hpart.low.shape[0]),
            "full_blocks": int(bem.hpart.full.shape[0]),
            "ext_rel_err_vs_direct_600_740": err,
            "phases_ms_600nm_rebuilt": {k: round(v["ms"], 3) for k, v in prof.items() if v["ms"] > 0},
            "hmat_matvec": {"launches": mv["launches"], "ms": mv["ms"], "GB/s": gbs,
                            "hbm_frac": gbs / hbm if gbs else None, "peak_source": src,
                            "bytes_note": "stored entries of the four H-matrices (full blocks + used factor "
                                          "columns, 16 B each) + vectors, per product"},
            "hmat_build_ms": hb["ms"]}


def run_gemm(a, torch):
    """The building block of the factorisations on its own: C -= A B with
    M = N = 5888 complex (C 277 MB, larger than L2) and K = 1024, the rank of
    the 24 000-face dimer's trailing updates, through mnpbem_gemm_c64 on
    device-resident operands: path 1 (TF32 operands) and path 4 (FP16 operands
    scaled per row / column).  Each step is one product per path; CUDA events
    on the default stream."""
    from mnpbem_gb300 import _lib
    lib = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    M = N = 5888
    K = 1024
    g = torch.Generator(device=dev).manual_seed(1)
    A = torch.randn((M, K), dtype=torch.complex64, device=dev, generator=g)
    B = torch.randn((K, N), dtype=torch.complex64, device=dev, generator=g)
    C0 = torch.randn((M, N), dtype=torch.complex64, device=dev, generator=g)
    al = np.array([-1.0, 0.0], dtype=np.float32)
    be = np.array([1.0, 0.0], dtype=np.float32)
    ref = (C0[:64].to(torch.complex128) - A[:64].to(torch.complex128) @ B.to(torch.complex128))
    out = {}
    flops = 8.0 * M * N * K
    for path, name in ((1, "tf32"), (4, "fp16_scaled")):
        C = C0.clone()
        run = lambda: _lib.check(lib.mnpbem_gemm_c64(0, path, M, N, K, al.ctypes.data, A.data_ptr(), K,
                                                     B.data_ptr(), N, be.ctypes.data, C.data_ptr(), N))
        run()
        torch.cuda.synchronize()
        err = float((C[:64].to(torch.complex128) - ref).abs().max() / ref.abs().max())
        for _ in range(max(0, a.warmup - 1)):
            run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(a.steps):
            run()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / a.steps
        out[name] = {"ms": ms, "TFLOP/s": flops / (ms / 1e3) / 1e12, "rel_err_first_64_rows": err}
    hbm, bf16, bf16_sus, src = peaks()
    best = out["fp16_scaled"]["TFLOP/s"]
    return {"metric": "TFLOP/s of one complex rank-1024 update (5888 x 5888 x 1024)", "value": best,
            "unit": "TFLOP/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": out["fp16_scaled"]["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f16 (scaled) / tf32 operands, f32 accumulation", "data": "synthetic",
            "config": {"workload": "gemm_rank1024: C -= A B, M = N = 5888, K = 1024 complex64, device-resident",
                       "l2": "C (277 MB) larger than the 129 MB L2"},
            "paths": out, "frac_of_bf16_burst": best / bf16, "peak_source": src}


def bemret_spectrum(bem, exc, eneis):
    """Direct (bemret) sweep on a bemretiter's handle (the parent class's
    spectrum runs mnpbem_solve)."""
    import mnpbem_gb300 as m
    return m.bemret.spectrum(bem, exc, eneis)


# ---------------------------------------------------------- CPU / reference
def cpu_problem(faces, dimer):
    """The workload's geometry at ``faces`` faces as an oracle problem."""
    from mnpbem_gb300 import shapes
    from oracle import mnpbem_ref as R
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    parts, inout = geometry(faces, dimer)
    eps = [R.EpsConst(1.77)] + [R.drude_eps(*DRUDE) for _ in parts]
    cp = R.ComParticle(eps, [R.Particle(v, f, q) for v, f in parts], inout, [True] * len(parts))
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([1, 0, 0], [0, 0, 1], R.Particle(vi, fi, q))
    return R, cp, pw


def cpu_solve_phases(bem, cp, pw, enei):
    """One oracle wavelength-solve split into its O(n^2) and O(n^3) parts:
    returns (ext, sca, seconds of the assembly, of the inversions and
    products of initmat, of the excitation + mldivide + cross sections)."""
    bem.enei = None
    t0 = time.perf_counter()
    bem.matrices(enei)
    t1 = time.perf_counter()
    bem.initmat(enei)                      # assembles again, then inverts
    t2 = time.perf_counter()
    sig = bem.solve(pw.potential(cp, enei))
    ext, sca = pw.extinction(cp, sig), pw.scattering(cp, sig)
    t3 = time.perf_counter()
    t_asm = t1 - t0
    return ext, sca, t_asm, max(0.0, (t2 - t1) - t_asm), t3 - t2


def extrapolate(a, t_asm, t_n3, t_rest):
    """Seconds per wavelength-solve at the workload's size from a sample at
    a.cpu_faces: the inversions and products scale as n^3, the rest as n^2."""
    r = a.faces / float(a.cpu_faces)
    return t_n3 * r ** 3 + (t_asm + t_rest) * r ** 2


def cpu_sample_desc(a, nsolves):
    cores = os.cpu_count()
    extr = "" if a.cpu_faces == a.faces else (
        "; extrapolated to %d faces: initmat's inversions and products (measured apart) scaled by (n/%d)^3, "
        "assembly, excitation, mldivide and cross sections by (n/%d)^2" % (a.faces, a.cpu_faces, a.cpu_faces))
    return ("%d wavelength-solve(s) of the NumPy/SciPy FP64 oracle (restatement of the reference CPU path: "
            "initmat with explicit inverses, mldivide, ext, sca; set-up excluded) on the same geometry at %d "
            "faces, OpenBLAS on all %d host threads%s" % (nsolves, a.cpu_faces, cores, extr))


def cpu_baseline(a, nsolves=1):
    R, cp, pw = cpu_problem(a.cpu_faces, WORKLOADS[a.workload]["dimer"])
    bem = R.BemRet(cp)              # set-up (refinement, sum rule) is not timed
    t = np.zeros(3)
    lams = [float(grid(a)[(7 * i + 3) % grid(a).size]) for i in range(nsolves)]
    res = []
    for lam in lams:
        ext, sca, *ph = cpu_solve_phases(bem, cp, pw, lam)
        t += ph
        res.append((lam, ext, sca))
    t /= nsolves
    sec = extrapolate(a, *t)
    return {"value": 1.0 / sec, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": cpu_sample_desc(a, nsolves),
            "seconds_per_solve_at_sample": float(t.sum()), "phases_s_at_sample": [float(x) for x in t],
            "extrapolated": a.cpu_faces != a.faces}, res


def parity_at_sample(a, torch, oracle_res):
    """GPU solves (mixed and FP64) of the CPU sample's problem at the oracle's
    wavelengths against the oracle's cross sections."""
    import mnpbem_gb300 as m
    dev = torch.cuda.current_device()
    exc = m.planewave([1, 0, 0], [0, 0, 1])
    out = {"faces": a.cpu_faces, "geometry": WORKLOADS[a.workload]["dimer"] and "dimer" or "sphere"}
    for prec in ("mixed", "fp64"):
        cp, bem = make_solver(a.cpu_faces, WORKLOADS[a.workload]["dimer"], dev, prec, 1, a.refine_tol)
        lams = [r[0] for r in oracle_res]
        r = bem.spectrum(exc, lams)
        e_ext = max(float(np.max(np.abs(r["ext"][i] - o[1]) / np.abs(o[1]))) for i, o in enumerate(oracle_res))
        e_sca = max(float(np.max(np.abs(r["sca"][i] - o[2]) / np.abs(o[2]))) for i, o in enumerate(oracle_res))
        out[prec] = {"ext_rel_err_vs_oracle": e_ext, "sca_rel_err_vs_oracle": e_sca,
                     "refine_tol": a.refine_tol if prec == "mixed" else None}
        del bem
    out["wavelengths"] = [r[0] for r in oracle_res]
    return out


def run_c2(torch, device):
    """Short device-timed sweep of the 4000-face sphere (configuration 2)."""
    import argparse as _ap
    b = _ap.Namespace(workload="sphere4000", faces=4000, batch=20, lanes=0, refine_tol=1e-8)
    cp, bem, exc = make_problem(b, device, "mixed")
    sweep = DeviceSweep(bem, exc, b.batch, torch)
    stream = lib_stream(bem, torch)
    for s in range(2):
        sweep.run(step_wavelengths(b, s, 0, 1, b.batch))
    bem._lib.mnpbem_profile_reset(bem.handle)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    steps = 3
    for s in range(steps):
        sweep.run(step_wavelengths(b, 2 + s, 0, 1, b.batch))
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    lt = read_profile(bem)
    launches = sum(v["launches"] for k, v in lt.items() if k != "geometry")
    return {"workload": workload_desc(b, batch=b.batch), "value": steps * b.batch / (ms / 1e3), "unit": UNIT,
            "steps": steps, "ms_per_step": ms / steps, "launches_per_wavelength": launches / float(steps * b.batch),
            "refinement_iterations": sweep.iters.tolist(), "refine_tol": b.refine_tol}


def run_c4(torch, device):
    """Configuration 4: adjoint gradients of the extinction on the capped rod
    (10 x 40 nm, 2016 triangles, polarisation along the axis, 650 nm) with
    respect to every vertex coordinate and eps, FP64 and mixed precision; host
    wall clock around each call after a warm-up call."""
    import mnpbem_gb300 as m
    from mnpbem_gb300 import shapes
    v, f = shapes.trirod(10.0, 40.0, (25, 7, 32), triangles=True)
    cp = m.comparticle([m.epsconst(1.77), drude()], [m.particle(v, f)], [[2, 1]], 1)
    bem = m.bemsolver(cp, m.bemoptions(precision="fp64", device=device, lanes=1))
    exc = m.planewave([[0, 0, 1.0]], [[1.0, 0, 0]])
    out = {"faces": int(cp.n), "vertices": int(v.shape[0]), "enei": 650.0}
    res = {}
    for prec in ("fp64", "mixed"):
        bem.cross_section_gradient(exc, 650.0, 0, "ext", prec)
        r, dt = _timed(lambda: bem.cross_section_gradient(exc, 650.0, 0, "ext", prec), torch)
        res[prec] = r
        out[prec] = {"seconds": dt, "ext": r[0]}
    out["grad_rel_diff_mixed_vs_fp64"] = float(np.max(np.abs(res["mixed"][1] - res["fp64"][1])) /
                                               np.max(np.abs(res["fp64"][1])))
    return out


def run_reference(a, rank, world):
    if rank != 0:
        return None
    dimer = WORKLOADS[a.workload]["dimer"]
    # warm-up: small solves (NumPy/BLAS thread pools, page-in)
    R, cps, pws = cpu_problem(284, False)
    bs = R.BemRet(cps)
    for s in range(a.warmup):
        cpu_solve_phases(bs, cps, pws, 500.0)
    R, cp, pw = cpu_problem(a.cpu_faces, dimer)
    bem = R.BemRet(cp)
    ph = np.zeros(3)
    wall = 0.0
    for s in range(a.steps):
        lam = float(step_wavelengths(a, s, 0, 1, 1)[0])
        t0 = time.perf_counter()
        _, _, *t = cpu_solve_phases(bem, cp, pw, lam)
        wall += time.perf_counter() - t0
        ph += t
    ph /= a.steps
    sec = extrapolate(a, *ph)
    value = 1.0 / sec
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * wall / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": workload_desc(a), "faces": a.faces, "wavelengths_per_step": 1,
                       "l2": "working set of dense n x n complex128 matrices > L2"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "sample": cpu_sample_desc(a, 1) + " per step",
                             "phases_s_at_sample": [float(x) for x in ph],
                             "extrapolated": a.cpu_faces != a.faces},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------- main
def main():
    a = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if a.impl == "reference":
        if a.workload not in WORKLOADS:
            print(json.dumps({"impl": "reference", "unavailable": "reference arm is defined for dimer24k and "
                                                                   "sphere4000 only"}))
            return
        line = run_reference(a, rank, world)
        if line is not None:
            print(json.dumps(line))
        return
    import torch
    if a.workload not in WORKLOADS:
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        line = {"batch3": run_batch3, "iter24k": run_iter, "gemm_rank1024": run_gemm}[a.workload](a, torch)
        if rank == 0:
            print(json.dumps(line))
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    r = run_ours(a, rank, world, dist, torch)
    device = torch.cuda.current_device()
    fp64 = cpu = parity = c2 = None
    if rank == 0 and not a.skip_fp64 and a.precision == "mixed":
        fp64 = fp64_full(a, torch, r)
    r["bem"] = None
    import gc
    gc.collect()
    if rank == 0 and not a.skip_cpu:
        cpu, ores = cpu_baseline(a)
        parity = parity_at_sample(a, torch, ores)
    c3 = c4 = None
    if rank == 0 and not a.skip_c2 and a.workload != "sphere4000":
        c2 = run_c2(torch, device)
        import argparse as _ap
        b3 = run_batch3(_ap.Namespace(lanes=0, refine_tol=a.refine_tol, warmup=1, steps=1), torch)
        c3 = {k: b3[k] for k in ("value", "unit", "ms_per_step", "speedup_vs_fp64_gpu", "ext_rel_err_mixed_vs_fp64",
                                 "refinement_iterations_max")}
        c3["workload"] = b3["config"]["workload"]
        c3["timing"] = b3["config"]["timing"]
        c4 = run_c4(torch, device)
    if dist is not None:
        dist.barrier()
    if rank == 0:
        n = r["cp"].n
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": r["ms"] / a.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "c64(fp16/tf32)+f64" if a.precision == "mixed" else "f64", "data": "synthetic",
                "config": {"workload": workload_desc(a, batch=a.batch), "faces": n, "wavelengths_per_step": a.batch,
                           "precision": a.precision, "lanes": a.lanes or tuned_lanes(n, a.precision),
                           "refine_tol": a.refine_tol if a.precision == "mixed" else None,
                           "l2": "no flush: the working set of one wavelength (%.1f GB of dense matrices) is "
                                 "far larger than the 129 MB L2" % ((5 * 8 + 4 * 16) * n * n / 1e9)},
                "e2e": r["e2e"], "gpu_launches": r["gpu_launches"], "roofline": r["roofline"],
                "cpu_baseline": cpu, "clocks": r["clocks"], "fp64_gpu": fp64, "parity_vs_oracle": parity,
                "c2_sphere4000": c2, "c3_batch3": c3, "c4_gradient": c4}
        if fp64:
            line["speedup_vs_fp64_gpu"] = r["value"] / fp64["value"]
        line.update(r["extra"])
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
