"""Autotuner of the mixed-precision sweep: tile / pipeline / concurrency choices.

For a problem size it times short wavelength sweeps on the GPU over the
options of ``mnpbem_geom_set_option`` -- the tensor-core GEMM's TMA pipeline
depth (3 or 4 stages of 128 x 256 x 32 tiles), the Gauss-Jordan step width
of the tensor-core inversion of Delta (256 or 512: the K extent of its
rank-nb updates and the size of its pivot blocks), the number of 256-row LDU
steps gathered into one trailing update of the factorisations (1, 2, 4: rank
256, 512, 1024), the number of wavelengths in flight (lanes) -- and stores
the fastest combination in ``data/tuned.json``
keyed by the face count.  ``bemsolver`` applies the entry whose face count is
closest (within a factor of 2) when it creates a mixed-precision solver.

    python -m mnpbem_gb300.autotune --faces 4000 [--device 0]
"""
import argparse
import itertools
import json
import os
import time

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
TUNED = os.path.join(_HERE, "data", "tuned.json")
GRID = {"tc_stages": (3, 4), "gj_block": (256, 512), "lu_steps": (1, 2, 4), "lanes": (2, 4, 6, 8)}


def load():
    try:
        with open(TUNED) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def settings_for(nfaces, precision):
    """Stored settings for the closest tuned face count (mixed precision only)."""
    if precision != "mixed":
        return {}
    table = load()
    best, dist = None, None
    for key, val in table.items():
        try:
            nf = int(key)
        except ValueError:
            continue
        r = max(nf, nfaces) / max(1, min(nf, nfaces))
        if r <= 2.0 and (dist is None or r < dist):
            best, dist = val, r
    return dict(best["options"]) if best else {}


def _problem(faces, device):
    from . import bem as B
    from .materials import epsconst, epsfun
    from .particles import comparticle, particle
    from . import shapes
    v, f = shapes.fibsphere(faces, 50.0)
    drude = epsfun(lambda w: 10 - 9.065 ** 2 / (w * (w + 0.0708j)), "eV")
    cp = comparticle([epsconst(1.77), drude], [particle(v, f)], [[2, 1]], 1)
    return B, cp


def tune(faces, device=0, nw=16, repeats=2):
    """Time every option combination on a sweep of ``nw`` wavelengths."""
    import torch
    B, cp = _problem(faces, device)
    exc = B.planewave([1, 0, 0], [0, 0, 1])
    enei = np.linspace(450.0, 750.0, nw)
    results = []
    for combo in itertools.product(*GRID.values()):
        opts = dict(zip(GRID.keys(), combo))
        solver = B.bemsolver(cp, B.bemoptions(precision="mixed", device=device, tuned=False))
        for k, v in opts.items():
            solver.set_option(k, v)
        solver.spectrum(exc, enei)                      # sizes buffers, captures graphs
        best = None
        for _ in range(repeats):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            solver.spectrum(exc, enei)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        results.append({"options": opts, "wavelength_solves_per_s": nw / best})
        del solver
    results.sort(key=lambda r: -r["wavelength_solves_per_s"])
    return results


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--faces", type=int, default=4000)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--wavelengths", type=int, default=16)
    a = ap.parse_args()
    res = tune(a.faces, a.device, a.wavelengths)
    table = load()
    table[str(a.faces)] = {"options": res[0]["options"], "wavelength_solves_per_s": res[0]["wavelength_solves_per_s"],
                           "all": res}
    os.makedirs(os.path.dirname(TUNED), exist_ok=True)
    with open(TUNED, "w") as f:
        json.dump(table, f, indent=1)
    for r in res:
        print(json.dumps(r))


if __name__ == "__main__":
    main()
