"""Regenerate ``tables.npz`` — the two numeric tables the retarded BEM path reads.

Both tables are published data that MNPBEM ships as inputs, not code:

* the stored minimum-energy point sets on the unit sphere that ``trisphere``
  triangulates (``Particles/particleshapes/trisphere.mat``; 24 sets of
  32 ... 1444 points, float32), and
* the 28-point, degree-11 triangle rule of Lyness and Jespersen that
  ``quadface`` uses by default (``rule = 18`` in
  ``Misc/integration/@quadface/private/triangle_unit_set.m:471-505``).

The script reads them out of a MNPBEM checkout (path given on the command
line) and writes them unchanged into ``tables.npz`` beside this file.  It also
writes ``epstables.npz``: the tabulated optical constants that ``epstable``
reads (``Material/@epstable/*.dat``: photon energy in eV, n, k per row; gold
and silver of Johnson and Christy, gold, silver and copper of Palik), one
``[m, 3]`` float64 array per file, keyed by the file name without ``.dat``.  The
rule is read by evaluating the scalar assignments and the three vector
assignments of the ``rule == 18`` branch; nothing else of that file is used.

Usage:  python make_tables.py <path-to-MNPBEM-checkout>
"""
import os
import re
import sys

import numpy as np


def _read_rule18(path):
    src = open(path).read()
    start = src.index("elseif ( rule == 18 )")
    stop = src.index("elseif ( rule == 19 )")
    block = src[start:stop]
    env = {}
    # scalar assignments  "a = 0.123E+00;"  or  "a = 1.0E+00 / 3.0E+00;"
    for name, expr in re.findall(r"^\s*(\w+)\s*=\s*([0-9.E+\-/ ]+);", block, re.M):
        env[name] = float(eval(expr.replace("E", "e"), {}, {}))
    out = {}
    for key in ("xtab", "ytab", "weight"):
        m = re.search(key + r"\(1:28\)\s*=\s*\[(.*?)\];", block, re.S)
        names = [t.strip() for t in m.group(1).replace("...", " ").replace("\n", " ").split(",")]
        out[key] = np.array([env[t] for t in names if t], dtype=np.float64)
        assert out[key].size == 28, key
    return out["xtab"], out["ytab"], out["weight"]


def _read_spheres(path):
    import scipy.io
    d = scipy.io.loadmat(path)
    sets = {}
    for key, val in d.items():
        if not key.startswith("sphere"):
            continue
        n = int(key[len("sphere"):])
        xyz = np.hstack([np.asarray(val["x"][0, 0]), np.asarray(val["y"][0, 0]),
                         np.asarray(val["z"][0, 0])]).astype(np.float32)
        sets[n] = xyz
    return sets


def read_eps_file(path):
    """Rows of an ``ene n k`` table; ``%`` starts a comment (the 'matlab'
    comment style of epstable.m's textread)."""
    rows = []
    for line in open(path):
        line = line.split("%")[0].strip()
        if line:
            rows.append([float(t) for t in line.split()[:3]])
    return np.asarray(rows, dtype=np.float64).reshape(-1, 3)


def _write_epstables(root):
    folder = os.path.join(root, "Material", "@epstable")
    tabs = {f[:-4]: read_eps_file(os.path.join(folder, f))
            for f in sorted(os.listdir(folder)) if f.endswith(".dat")}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "epstables.npz")
    np.savez_compressed(dst, **tabs)
    print("wrote", dst, {k: v.shape for k, v in tabs.items()})


def main(root):
    x, y, w = _read_rule18(os.path.join(
        root, "Misc", "integration", "@quadface", "private", "triangle_unit_set.m"))
    spheres = _read_spheres(os.path.join(root, "Particles", "particleshapes", "trisphere.mat"))
    arrays = {"rule18_x": x, "rule18_y": y, "rule18_w": w,
              "sphere_sizes": np.array(sorted(spheres), dtype=np.int64)}
    for n, xyz in spheres.items():
        arrays["sphere%d" % n] = xyz
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tables.npz")
    np.savez_compressed(dst, **arrays)
    print("wrote", dst, "rule weight sum", w.sum(), "sphere sets", sorted(spheres))
    _write_epstables(root)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_tables.py <path of an MNPBEM checkout>")
    main(sys.argv[1])
