"""GPU test of mnpbem_cross_sections_noalloc, the entry point for callers that
cannot allocate GPU memory (for example a MEX gateway inside a MATLAB session
whose GPU memory belongs to MATLAB, or a plugin whose host application owns
all device memory): it receives only caller-owned device buffers and keeps its
scratch in a fixed array inside the library.

Here the test itself plays the caller that owns the buffers (allocated with
torch).  The cross sections must equal those of the regular entry point
(mnpbem_solve) on the same surface charges within the FP64 tolerance of the
parity tests (1e-10), on two calls in a row with different inputs, so that
the shared scratch carries nothing from one call to the next.  The file is
named to be collected last, and it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import mnpbem_gb300 as m

pytestmark = pytest.mark.gpu


def test_cross_sections_noalloc_matches_solve(gpu_lib):
    torch = pytest.importorskip("torch")
    from mnpbem_gb300 import _lib

    drude = m.epsfun(lambda w: 10 - 9.065 ** 2 / (w * (w + 0.0708j)), "eV")
    p = m.trisphere(144, 30.0)
    cp = m.comparticle([m.epsconst(1.77), drude], [p], [[2, 1]], 1)
    bem = m.bemsolver(cp, m.bemoptions(precision="fp64"))
    exc = m.planewave([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]])
    lams = [480.0, 600.0]
    ref = bem.spectrum(exc, lams, fields=True)          # the regular entry point
    n, P = cp.n, exc.npol

    dev = torch.device("cuda", 0)

    def d(a, dtype=torch.float64):
        return torch.as_tensor(np.ascontiguousarray(a)).to(dtype=dtype, device=dev).contiguous()

    media = np.repeat(cp.inout, [q.n for q in cp.p], axis=0)
    pos, area = d(cp.pos), d(cp.area)
    exc_in = d(media[:, 0] == exc.medium, torch.uint8)
    exc_out = d(media[:, 1] == exc.medium, torch.uint8)
    pol, dirs = d(exc.pol), d(exc.dir)
    inf_nvec, inf_area = d(exc.spec.nvec), d(exc.spec.area)
    ext = torch.zeros(P, dtype=torch.float64, device=dev)
    sca = torch.zeros(P, dtype=torch.float64, device=dev)

    def ptr(t):
        return ctypes.c_void_p(t.data_ptr())

    for w, lam in enumerate(lams):                      # two calls in a row
        fields = {k: d(ref[k][w].view(np.float64)) for k in ("sig1", "h1", "sig2", "h2")}
        eps = cp.eps_media([lam])[0]
        eps_exc = np.array([eps[exc.medium - 1].real, eps[exc.medium - 1].imag])
        eps_1 = np.array([eps[0].real, eps[0].imag])
        ext.fill_(float("nan"))
        sca.fill_(float("nan"))
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(0)[0]
        st = gpu_lib.mnpbem_cross_sections_noalloc(
            0, None, n, P, ptr(pos), ptr(area), ptr(exc_in), ptr(exc_out), ptr(fields["sig1"]),
            ptr(fields["h1"]), ptr(fields["sig2"]), ptr(fields["h2"]), ptr(pol), ptr(dirs),
            inf_nvec.shape[0], ptr(inf_nvec), ptr(inf_area), lam, eps_exc.ctypes.data,
            eps_1.ctypes.data, ptr(ext), ptr(sca))
        _lib.check(st)
        torch.cuda.synchronize()
        if w > 0:
            # after the first call (which loads the module) no device memory is taken
            assert torch.cuda.mem_get_info(0)[0] == free0
        got_ext, got_sca = ext.cpu().numpy(), sca.cpu().numpy()
        e_ext = np.max(np.abs(got_ext - ref["ext"][w]) / np.abs(ref["ext"][w]))
        e_sca = np.max(np.abs(got_sca - ref["sca"][w]) / np.abs(ref["sca"][w]))
        assert e_ext < 1e-10 and e_sca < 1e-10, (lam, e_ext, e_sca)

    # sizes beyond the fixed scratch are rejected with a clear error
    big = gpu_lib.mnpbem_cross_sections_noalloc(
        0, None, n, P, ptr(pos), ptr(area), ptr(exc_in), ptr(exc_out), ptr(pos), ptr(pos), ptr(pos),
        ptr(pos), ptr(pol), ptr(dirs), 5000, ptr(inf_nvec), ptr(inf_area), 500.0,
        eps_exc.ctypes.data, eps_1.ctypes.data, ptr(ext), ptr(sca))
    assert big == 1 and b"exceed the maximum" in gpu_lib.mnpbem_last_error()
    # more polarisations than the scratch holds are rejected too
    many = gpu_lib.mnpbem_cross_sections_noalloc(
        0, None, n, 5, ptr(pos), ptr(area), ptr(exc_in), ptr(exc_out), ptr(pos), ptr(pos), ptr(pos),
        ptr(pos), ptr(pol), ptr(dirs), 10, ptr(inf_nvec), ptr(inf_area), 500.0,
        eps_exc.ctypes.data, eps_1.ctypes.data, ptr(ext), ptr(sca))
    assert many == 1 and b"exceeds the maximum" in gpu_lib.mnpbem_last_error()
