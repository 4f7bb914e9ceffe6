"""One-graph sweeps (device-side wavelength queue and refinement decisions)
against the host scheduler: bit-identical charges, cross sections and
refinement counts, for one handle with several lanes and for a batch of
uneven particles (mnpbem_solve_batch).  The reported refinement residual
(a diagnostic, sqrt of a ratio of two norms) is formed on the device in the
graph and on the host otherwise: equal to 1e-12."""
import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes

from test_gpu_parity import drude

pytestmark = pytest.mark.gpu


def sphere(nv, d=20.0):
    return m.comparticle([m.epsconst(1.77), drude()], [m.trisphere(nv, d)], [[2, 1]], 1)


def solve(cp, graph, enei, lanes=3, precision="mixed"):
    bem = m.bemsolver(cp, m.bemoptions(precision=precision, lanes=lanes))
    bem.set_option("sweep_graph", 1 if graph else 0)
    exc = m.planewave([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]])
    r = bem.spectrum(exc, enei, fields=True)
    # the graph ran (or, switched off, did not)
    assert bem.stat("sweep_graph_error") == 0
    assert (bem.stat("sweep_graph_runs") > 0) == (graph and bem.stat("stage_graphs") > 0), \
        (bem.stat("sweep_graph_runs"), bem.stat("stage_graphs"))
    return r


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_sweep_graph_bit_identical(precision):
    cp = sphere(400)
    enei = np.linspace(450.0, 750.0, 11)
    a = solve(cp, True, enei, precision=precision)
    b = solve(cp, False, enei, precision=precision)
    for k in ("ext", "sca", "sig1", "sig2", "h1", "h2", "ir_iters"):
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k
    assert np.allclose(a["ir_resid"], b["ir_resid"], rtol=1e-12, atol=0)
    # repeated call reuses the graph
    c = solve(cp, True, enei, precision=precision)
    assert np.array_equal(c["ext"], a["ext"])


def test_batch_graph_bit_identical():
    parts = [sphere(256, 20.0), sphere(400, 30.0), m.comparticle([m.epsconst(1.77), drude()],
                                                                  [m.trirod(10.0, 40.0, (15, 15, 20))],
                                                                  [[2, 1]], 1)]
    enei = np.linspace(500.0, 800.0, 9)
    exc = m.planewave([[1, 0, 0]], [[0, 0, 1]])
    out = []
    for graph in (1, 0):
        items = []
        for cp in parts:
            bem = m.bemsolver(cp, m.bemoptions(precision="mixed", lanes=2))
            bem.set_option("sweep_graph", graph)
            items.append((bem, exc, enei))
        out.append(m.spectrum_batch(items))
        assert all((b.stat("sweep_graph_runs") > 0) == bool(graph) for b, _, _ in items)
    for ra, rb in zip(*out):
        for k in ("ext", "sca", "ir_iters"):
            assert np.array_equal(ra[k], rb[k]), k
        assert np.allclose(ra["ir_resid"], rb["ir_resid"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("iters", [0, 1, 2])
def test_sweep_graph_refinement_limits(iters):
    """the device-side stop rule at small refinement limits (0: the
    library's default limit, 10)"""
    cp = sphere(256)
    enei = np.linspace(500.0, 700.0, 7)
    res = []
    for graph in (True, False):
        bem = m.bemsolver(cp, m.bemoptions(precision="mixed", lanes=2))
        bem.set_option("sweep_graph", 1 if graph else 0)
        bem.refine_iters = iters
        exc = m.planewave([[1, 0, 0]], [[0, 0, 1]])
        res.append(bem.spectrum(exc, enei, fields=True))
    a, b = res
    for k in ("ext", "sca", "sig2", "h2", "ir_iters"):
        assert np.array_equal(a[k], b[k]), k
    assert np.all(a["ir_iters"] <= (iters if iters > 0 else 10))


def test_sweep_graph_page_locked_outputs():
    """results written by the graph straight into page-locked host buffers
    equal those staged for pageable buffers"""
    torch = pytest.importorskip("torch")
    cp = sphere(256)
    enei = np.linspace(500.0, 700.0, 7)
    exc = m.planewave([[1, 0, 0]], [[0, 0, 1]])
    bem = m.bemsolver(cp, m.bemoptions(precision="mixed", lanes=2))
    ref = bem.spectrum(exc, enei, fields=True)
    n = cp.n
    out = {k: torch.zeros(shape, dtype=dt, pin_memory=True).numpy() for k, shape, dt in (
        ("ext", (7, 1), torch.float64), ("sca", (7, 1), torch.float64),
        ("sig2", (7, n, 1), torch.complex128), ("h2", (7, n, 3, 1), torch.complex128))}
    got = bem.spectrum(exc, enei, fields=True, out=out)
    assert bem.stat("sweep_graph_runs") > 0
    for k in ("ext", "sca", "sig2", "h2"):
        assert np.array_equal(np.asarray(got[k]).reshape(ref[k].shape), ref[k]), k
