#!/usr/bin/env python
"""Throughput of the retarded BEM path: wavelength-solves/s on GB300.

One wavelength-solve = assembly of G1, H1, G2, H2 (with near-field
refinement), the bemret inversions and products, the mldivide chain for all
polarisations, FP64 iterative refinement (mixed precision), and the extinction
and scattering cross sections.  The per-geometry set-up (refinement
coefficients, closed-surface sum rule) runs once before timing, like
``bem = bemsolver(p, op)`` in MNPBEM.

Workload (synthetic, deterministic): sphere of diameter 50 nm with 4000 flat
faces, Drude metal eps(w) = 10 - 9.065^2 / (w (w + 0.0708 i)) (w in eV) in
eps = 1.77, x-polarised plane wave along +z, wavelengths on the 60-point grid
450..750 nm.  A step is one batch of ``--batch`` wavelengths per GPU; with N
GPUs rank r takes its own wavelengths (weak scaling, no collective on the
data path).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]
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
NGRID = 60
# DRAM bytes (read + write) of one full-size rank-256 Gauss-Jordan update of the
# 4000-face workload, from one ncu capture (profiles/tc_gemm_rank256_update_sphere4000.md)
TC_TRAFFIC_PER_LAUNCH = 152.7e6 + 67.5e6
TC_TRAFFIC_NOTE = ("dram__bytes_read.sum + dram__bytes_write.sum of the full-size rank-256 update "
                   "(4000 x 8000 x 512 real) from one ncu capture; algorithmic bytes of that launch 280 MB")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--faces", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=20, help="wavelengths per step per GPU")
    ap.add_argument("--lanes", type=int, default=0, help="wavelengths in flight at once (0: library default)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--refine-tol", type=float, default=1e-8,
                    help="mixed precision: refinement stops at ||dx|| <= tol ||x|| (the metric asks for an "
                         "extinction error <= 1e-6 against FP64; the library default is 1e-10)")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--cpu-faces", type=int, default=0, help="faces of the CPU sample (default: workload)")
    ap.add_argument("--workload", default="sphere4000", choices=["sphere4000", "batch3", "dimer24k", "iter24k"],
                    help="sphere4000: the headline sweep; batch3: three particles of uneven size, 128 "
                         "wavelengths, two polarisations; dimer24k: two 12000-face spheres, 32 wavelengths; "
                         "iter24k: the same dimer through the iterative H-matrix solver")
    ap.add_argument("--iter-faces", type=int, default=24000,
                    help="iter24k: total faces of the dimer (smaller sizes for profiling runs)")
    ap.add_argument("--fp64-faces", type=int, default=12000,
                    help="dimer24k: total faces of the FP64 timing sample (scaled by n^3 to 24000)")
    return ap.parse_args()


def grid():
    return np.linspace(450.0, 750.0, NGRID)


def step_wavelengths(step, rank, world, batch):
    base = (step * world + rank) * batch
    return grid()[(base + np.arange(batch)) % NGRID]


def max_over_ranks(dist, values, device, torch):
    """Per-rank timings reduced to their maximum over ranks (the slowest rank
    sets the whole job's time); unchanged without a process group."""
    if dist is None:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def workload_desc(a):
    return ("sphere d=50 nm, %d flat faces, Drude eps_inf=10 wp=9.065 eV gamma=0.0708 eV in eps=1.77, "
            "x-pol along +z, %d-point wavelength grid 450-750 nm, %d wavelengths per step per GPU"
            % (a.faces, NGRID, a.batch))


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


def make_problem(a, device, precision):
    import mnpbem_gb300 as m
    from mnpbem_gb300 import shapes
    v, f = shapes.fibsphere(a.faces, 50.0)
    p = m.particle(v, f)
    cp = m.comparticle([m.epsconst(1.77), drude()], [p], [[2, 1]], 1)
    bem = m.bemsolver(cp, m.bemoptions(precision=precision, device=device, lanes=a.lanes))
    bem.refine_tol = a.refine_tol
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
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def run_ours(a, rank, world, dist, torch):
    device = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    cp, bem, exc = make_problem(a, device, a.precision)
    sweep = DeviceSweep(bem, exc, a.batch, torch)
    stream = lib_stream(bem, torch)
    n, P = cp.n, exc.npol

    def barrier():
        if dist is not None:
            dist.barrier()

    bem_lib = bem._lib
    for s in range(a.warmup):
        sweep.run(step_wavelengths(s, rank, world, a.batch))
    # ---------------- timed region (device-resident outputs, no per-launch events)
    bem_lib.mnpbem_profile_reset(bem.handle)
    clocks = ClockSampler(device)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for s in range(a.steps):
        sweep.run(step_wavelengths(a.warmup + s, rank, world, a.batch))
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    launches_timed = read_profile(bem)
    iters = sweep.iters.copy()
    # ---------------- the same steps at the library's default tolerance (1e-10)
    tol_default = None
    if a.precision == "mixed" and a.refine_tol != 1e-10:
        from mnpbem_gb300 import _lib as L_
        sweep_d = DeviceSweep(bem, exc, a.batch, torch)
        sweep_d.ref = L_.Refine(bem.refine_iters, 1e-10)
        sweep_d.run(step_wavelengths(0, rank, world, a.batch))
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        for s in range(a.steps):
            sweep_d.run(step_wavelengths(a.warmup + s, rank, world, a.batch))
        g1.record(stream)
        torch.cuda.synchronize()
        tol_default = {"refine_tol": 1e-10, "value": a.batch * a.steps / (g0.elapsed_time(g1) / 1e3),
                       "refinement_iterations": sweep_d.iters.tolist()}
    # ---------------- profiled repeat of the same steps: CUDA events on the
    # library stream around every launch give per-kernel-class durations
    bem_lib.mnpbem_profile_enable(bem.handle, 1)
    sweep.run(step_wavelengths(a.warmup, rank, world, a.batch))      # captures graphs with event nodes
    bem_lib.mnpbem_profile_reset(bem.handle)
    for s in range(a.steps):
        sweep.run(step_wavelengths(a.warmup + s, rank, world, a.batch))
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
        r = bem.spectrum(exc, step_wavelengths(a.warmup + a.steps + s, rank, world, a.batch),
                         fields=True, out=host)
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
    # ---------------- roofline: the tensor-core GEMMs (the dominant kernel class
    # in FLOPs and, with several wavelengths in flight, in device time; the
    # pivot-block inversions run on one 8-CTA cluster each and overlap other
    # wavelengths' GEMMs); every other kernel class is listed in phases_roofline
    hbm, bf16, src = peaks()
    timing = ("CUDA events on the library stream around each launch, over a profiled repeat of "
              "the %d timed steps (one wavelength in flight)" % a.steps)
    d = prof["gemm_n3"]
    achieved = d["flops"] / (d["ms"] / 1e3) / 1e12 if d["ms"] > 0 else 0.0
    roof = {"kernel": "k_tc_gemm (tcgen05 kind::tf32, all tensor-core GEMM launches)", "bound": "tensor",
            "achieved": achieved, "peak": bf16, "unit": "TFLOP/s", "frac": achieved / bf16,
            "peak_source": src + " dense bf16 (TF32 runs at half the bf16 rate: frac of the TF32 rate = %.3f)"
                           % (2 * achieved / bf16),
            "traffic": TC_TRAFFIC_PER_LAUNCH, "traffic_note": TC_TRAFFIC_NOTE,
            "launches": d["launches"], "ms": d["ms"], "timing": timing}
    phases_roof = {}
    for k, v in prof.items():
        if v["ms"] <= 0 or k == "geometry":
            continue
        phases_roof[k] = {"ms": round(v["ms"], 3), "launches": v["launches"],
                          "GB/s": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1) if v["bytes"] else None,
                          "hbm_frac": round(v["bytes"] / (v["ms"] / 1e3) / 1e9 / hbm, 4) if v["bytes"] else None,
                          "TFLOP/s": round(v["flops"] / (v["ms"] / 1e3) / 1e12, 2) if v["flops"] else None}
    asm = prof["assembly"]
    extra = {"phases_ms": {k: round(v["ms"], 3) for k, v in prof.items()}, "phases_roofline": phases_roof,
             "assembly_hbm_gbs": asm["bytes"] / (asm["ms"] / 1e3) / 1e9 if asm["ms"] > 0 else None,
             "assembled_pairs_per_s": (n * n * a.batch * a.steps) / (asm["ms"] / 1e3) if asm["ms"] > 0 else None,
             "refinement_iterations": iters.tolist(), "at_default_tolerance": tol_default}
    launches = int(sum(v["launches"] for k, v in launches_timed.items() if k != "geometry"))
    out = {"value": value, "ms": ms, "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                                             "d2h_bytes_per_step": int(d2h), "ms": e2e_ms,
                                             "wall_ms": e2e_wall},
           "roofline": roof, "gpu_launches": launches, "clocks": clk, "extra": extra,
           "bem": bem, "exc": exc, "cp": cp, "sweep": sweep}
    return out


def fp64_comparison(a, cp, exc, torch, mixed_bem):
    """Plain FP64 GPU path on one wavelength + accuracy of the mixed path."""
    import mnpbem_gb300 as m
    device = torch.cuda.current_device()
    bem64 = m.bemsolver(cp, m.bemoptions(precision="fp64", device=device))
    lam = [450.0, 600.0, 750.0]
    bem64.spectrum(exc, [500.0])          # warm-up (kernel loading)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r64 = bem64.spectrum(exc, lam)
    torch.cuda.synchronize()
    t64 = (time.perf_counter() - t0) / len(lam)
    rmx = mixed_bem.spectrum(exc, lam)
    err_ext = float(np.max(np.abs(rmx["ext"] - r64["ext"]) / np.abs(r64["ext"])))
    err_sca = float(np.max(np.abs(rmx["sca"] - r64["sca"]) / np.abs(r64["sca"])))
    return {"value": 1.0 / t64, "unit": UNIT, "sample": "3 wavelengths (450, 600, 750 nm), same workload",
            "ext_rel_err_mixed_vs_fp64": err_ext, "sca_rel_err_mixed_vs_fp64": err_sca,
            "mixed_refine_tol": mixed_bem.refine_tol}


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
            "scaling": "weak", "vs_baseline": None, "dtype": "c64(tf32)+f64", "data": "synthetic",
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


def dimer_problem(faces_total, precision, dev, lanes):
    import mnpbem_gb300 as m
    from mnpbem_gb300 import shapes
    nf = faces_total // 2
    v1, f1 = shapes.fibsphere(nf, 50.0, center=(-26.0, 0.0, 0.0))
    v2, f2 = shapes.fibsphere(nf, 50.0, center=(26.0, 0.0, 0.0))
    cp = m.comparticle([m.epsconst(1.77), drude(), drude()], [m.particle(v1, f1), m.particle(v2, f2)],
                       [[2, 1], [3, 1]], 1, 2)
    return m.bemsolver(cp, m.bemoptions(precision=precision, device=dev, lanes=lanes))


def run_dimer(a, torch):
    """Two spheres d = 50 nm, 2 nm gap, 12000 faces each (separate media: G1
    block-diagonal, factored as a full matrix), x-polarised along +z, 32
    wavelengths 500-900 nm, mixed precision; the FP64 path is timed on one
    wavelength of a dimer with --fp64-faces faces and scaled by n^3."""
    import mnpbem_gb300 as m
    dev = torch.cuda.current_device()
    exc = m.planewave([1, 0, 0], [0, 0, 1])
    enei = np.linspace(500.0, 900.0, 32)
    bem = dimer_problem(24000, "mixed", dev, a.lanes)
    bem.refine_iters = 20
    bem.refine_tol = a.refine_tol
    bem.spectrum(exc, enei[:max(1, a.lanes or 3)])        # warm-up: sizes and captures every lane
    res, dt = _timed(lambda: bem.spectrum(exc, enei), torch)
    value = enei.size / dt
    b64 = dimer_problem(a.fp64_faces, "fp64", dev, 1)
    b64.spectrum(exc, [700.0])
    r64, t64 = _timed(lambda: b64.spectrum(exc, [700.0]), torch)
    bmx = dimer_problem(a.fp64_faces, "mixed", dev, 1)
    bmx.refine_iters, bmx.refine_tol = 20, a.refine_tol
    rmx = bmx.spectrum(exc, [700.0])
    err = float(abs(rmx["ext"][0, 0] - r64["ext"][0, 0]) / abs(r64["ext"][0, 0]))
    scale = (24000.0 / a.fp64_faces) ** 3
    v64 = 1.0 / (t64 * scale)
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": 1e3 * dt, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64(tf32)+f64", "data": "synthetic",
            "config": {"workload": "dimer of two d=50 nm spheres, 2 nm gap, 2 x 12000 faces, Drude metal in "
                                   "eps=1.77, x-pol along +z, 32 wavelengths 500-900 nm", "faces": 24000,
                       "timing": "host wall clock around bemsolver.spectrum (public API, ext/sca to host)",
                       "refine_tol": a.refine_tol},
            "fp64_gpu": {"value": v64, "unit": UNIT,
                         "sample": "1 wavelength (700 nm) of a %d-face dimer, %.3f s, scaled by (24000/%d)^3"
                                   % (a.fp64_faces, t64, a.fp64_faces)},
            "speedup_vs_fp64_gpu": value / v64,
            "ext_rel_err_mixed_vs_fp64": err, "ext_err_sample": "%d-face dimer at 700 nm" % a.fp64_faces,
            "refinement_iterations": res["ir_iters"].tolist(),
            "refinement_final_residual_max": float(np.max(res["ir_resid"]))}


def run_iter(a, torch):
    """Iterative solver (bemretiter) on the dimer of run_dimer (--iter-faces,
    default 24000 faces): H-matrices of G1, H1, G2, H2 (leaves of at most 200
    faces, htol 1e-6, kmax 100), GMRES (tol 1e-6) preconditioned by the
    complex64 tensor-core inverses.  Timed: a sweep of 8 wavelengths 600-740 nm
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
                                                              reuse_precond=True, refresh_steps=30)))
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
    hbm, _, src = peaks()
    mv, hb = prof["hmat_matvec"], prof["hmat_build"]
    gbs = mv["bytes"] / (mv["ms"] * 1e-3) / 1e9 if mv["ms"] > 0 else None
    return {"metric": METRIC, "value": eneis.size / dt, "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": 1e3 * dt, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64-class H-matrix operator (double-single) + c64(tf32) preconditioner", "data": "synthetic",
            "config": {"workload": "iterative solver (bemretiter, H-matrices + GMRES) on the dimer of two d=50 nm "
                                   "spheres, 2 nm gap, 2 x %d faces, x-pol along +z, 8 wavelengths 600-740 nm" % nf,
                       "faces": 2 * nf, "cleaf": 200, "htol": 1e-6, "kmax": 100, "gmres_tol": 1e-6,
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


def bemret_spectrum(bem, exc, eneis):
    """Direct (bemret) sweep on a bemretiter's handle (the parent class's
    spectrum runs mnpbem_solve)."""
    import mnpbem_gb300 as m
    return m.bemret.spectrum(bem, exc, eneis)


# ---------------------------------------------------------- CPU / reference
def cpu_problem(faces):
    from mnpbem_gb300 import shapes
    from oracle import mnpbem_ref as R
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    v, f = shapes.fibsphere(faces, 50.0)
    cp = R.ComParticle([R.EpsConst(1.77), R.drude_eps(*DRUDE)], [R.Particle(v, f, q)], [[2, 1]], [True])
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([1, 0, 0], [0, 0, 1], R.Particle(vi, fi, q))
    return R, cp, pw


def cpu_solve_one(R, bem, cp, pw, enei):
    bem.enei = None
    sig = bem.solve(pw.potential(cp, enei))
    return pw.extinction(cp, sig), pw.scattering(cp, sig)


def cpu_baseline(a, nsolves=1):
    faces = a.cpu_faces or a.faces
    R, cp, pw = cpu_problem(faces)
    bem = R.BemRet(cp)              # set-up (refinement, sum rule) is not timed
    t0 = time.perf_counter()
    for i in range(nsolves):
        cpu_solve_one(R, bem, cp, pw, float(grid()[(7 * i + 3) % NGRID]))
    dt = time.perf_counter() - t0
    cores = os.cpu_count()
    scale = (faces / a.faces) ** 3
    return {"value": nsolves / dt * scale, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d wavelength-solve(s) of the NumPy/SciPy FP64 oracle at %d faces "
                      "(initmat with explicit inverses + mldivide + ext + sca; set-up excluded), "
                      "OpenBLAS on all %d host threads%s" % (
                          nsolves, faces, cores,
                          "" if faces == a.faces else ", scaled by (n/%d)^3" % a.faces),
            "seconds": dt}


def run_reference(a, rank, world):
    if rank != 0:
        return None
    # warm-up: small solves (NumPy/BLAS thread pools, page-in)
    R, cps, pws = cpu_problem(284)
    bs = R.BemRet(cps)
    for s in range(a.warmup):
        cpu_solve_one(R, bs, cps, pws, 500.0)
    faces = a.cpu_faces or a.faces
    R, cp, pw = cpu_problem(faces)
    bem = R.BemRet(cp)
    times = []
    for s in range(a.steps):
        lam = float(step_wavelengths(s, 0, 1, 1)[0])
        t0 = time.perf_counter()
        cpu_solve_one(R, bem, cp, pw, lam)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.sum(times))
    scale = (faces / a.faces) ** 3
    value = a.steps / (ms / 1e3) * scale
    cores = os.cpu_count()
    sample = ("1 wavelength-solve per step of the NumPy/SciPy FP64 oracle (restatement of the "
              "reference CPU path) at %d faces, OpenBLAS on all %d host threads%s"
              % (faces, cores, "" if faces == a.faces else ", scaled by (n/%d)^3" % a.faces))
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": workload_desc(a), "faces": a.faces, "wavelengths_per_step": 1,
                       "l2": "working set of dense n x n complex128 matrices > L2"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------- main
def main():
    a = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if a.impl == "reference":
        line = run_reference(a, rank, world)
        if line is not None:
            print(json.dumps(line))
        return
    import torch
    if a.workload != "sphere4000":
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        line = {"batch3": run_batch3, "dimer24k": run_dimer, "iter24k": run_iter}[a.workload](a, torch)
        if rank == 0:
            print(json.dumps(line))
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    r = run_ours(a, rank, world, dist, torch)
    fp64 = None
    if rank == 0 and not a.skip_fp64:
        fp64 = fp64_comparison(a, r["cp"], r["exc"], torch, r["bem"])
    cpu = None
    if rank == 0 and not a.skip_cpu:
        cpu = cpu_baseline(a)
    if dist is not None:
        dist.barrier()
    if rank == 0:
        n = r["cp"].n
        wset = (5 * 8 + 4 * 16) * n * n
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": r["ms"] / a.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "c64(tf32)+f64" if a.precision == "mixed" else "f64", "data": "synthetic",
                "config": {"workload": workload_desc(a), "faces": n, "wavelengths_per_step": a.batch,
                           "precision": a.precision, "lanes": a.lanes or tuned_lanes(n, a.precision),
                           "refine_tol": a.refine_tol if a.precision == "mixed" else None,
                           "l2": "no flush: per-wavelength working set %.2f GB > 129 MB L2" % (wset / 1e9)},
                "e2e": r["e2e"], "gpu_launches": r["gpu_launches"], "roofline": r["roofline"],
                "cpu_baseline": cpu, "clocks": r["clocks"], "fp64_gpu": fp64}
        if fp64:
            line["speedup_vs_fp64_gpu"] = r["value"] / fp64["value"]
        line.update(r["extra"])
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
