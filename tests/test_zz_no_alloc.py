"""rp_zinv_batched_noalloc: the dielectric-matrix inverse that allocates no
device memory.  Its results are checked against rp_epsinv_q, the context entry
point whose Gauss-Jordan inversion it mirrors, on two calls in a row.  This
file is collected last so that it also runs after every other GPU test in the
same process."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

from respackdev_gb300 import chiqw as rp
from respackdev_gb300 import synth
from tests.helpers import EM_TEST, normwise_err, run_params


def _lib():
    L = rp.load()
    L.rp_zinv_batched_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.rp_zinv_batched_noalloc.restype = C.c_int
    return L


def test_noalloc_rejects_sizes_beyond_scratch():
    """Requests larger than the fixed scratch, or empty ones, fail with code 1
    before any device work (the pointers are never touched)."""
    L = _lib()
    fake = C.c_void_p(4096)
    assert L.rp_zinv_batched_noalloc(fake, fake, 1000, 1000, None) == 1
    assert b"exceeds the fixed scratch" in L.rp_last_error(None)
    assert L.rp_zinv_batched_noalloc(fake, fake, 8, 2000, None) == 1
    assert L.rp_zinv_batched_noalloc(fake, fake, 0, 4, None) == 1
    assert L.rp_zinv_batched_noalloc(None, fake, 4, 4, None) == 1
    assert b"null pointer" in L.rp_last_error(None)
    # a partial overlap of input and output is rejected (4x4 complex = 256 bytes)
    assert L.rp_zinv_batched_noalloc(fake, C.c_void_p(4096 + 128), 4, 1, None) == 1
    assert b"overlap" in L.rp_last_error(None)


def _eps_from_chi(chi: np.ndarray, ql: np.ndarray) -> np.ndarray:
    """1 - 2 * 4 pi chi / (|q+G||q+G'|) for q != 0 (calc_eps_rpa, chiqw_sub.F:386-440)."""
    ng = chi.shape[0]
    v = 4.0 * np.pi / np.outer(ql, ql)
    return np.eye(ng)[:, :, None] - 2.0 * chi * v[:, :, None]


def _to_device(a_cm: np.ndarray, torch):
    """(ng, ng, nmat) column-major complex -> contiguous device buffer of nmat
    column-major matrices."""
    host = np.ascontiguousarray(a_cm.transpose(2, 1, 0))       # (nmat, col, row)
    return torch.from_numpy(host.view(np.float64).copy()).cuda()


def _from_device(t, ng: int, nmat: int) -> np.ndarray:
    host = t.cpu().numpy().view(np.complex128).reshape(nmat, ng, ng)
    return host.transpose(2, 1, 0)


@pytest.mark.gpu
def test_noalloc_reports_singular_input():
    """A matrix with a zero column gives code 3; the next call works again."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = _lib()
    n, nmat = 6, 2
    rng = np.random.default_rng(3)
    m = rng.standard_normal((n, n, nmat)) + 1j * rng.standard_normal((n, n, nmat))
    bad = m.copy()
    bad[:, 2, 1] = 0.0
    a = _to_device(bad, torch)
    out = torch.empty_like(a)
    stream = torch.cuda.current_stream().cuda_stream
    assert L.rp_zinv_batched_noalloc(a.data_ptr(), out.data_ptr(), n, nmat, stream) == 3
    assert b"singular" in L.rp_last_error(None)
    a = _to_device(m, torch)
    assert L.rp_zinv_batched_noalloc(a.data_ptr(), out.data_ptr(), n, nmat, stream) == 0
    got = _from_device(out, n, nmat)
    for e in range(nmat):
        np.testing.assert_allclose(got[:, :, e], np.linalg.inv(m[:, :, e]), rtol=0, atol=1e-12 * np.abs(
            np.linalg.inv(m[:, :, e])).max())


@pytest.mark.gpu
def test_noalloc_matches_epsinv_q_two_calls(case_dir, fresh_copy):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = _lib()
    root = fresh_copy(case_dir("tiny"))
    bvec = synth.generate(synth.CASES["tiny"]).bvec
    kw = run_params("tiny")
    stream = torch.cuda.current_stream()
    with rp.Context(root, rp.default_params(precision=rp.PREC_FP64, **kw), EM_TEST) as ctx:
        for call, iq in enumerate((2, 3)):
            chi = ctx.chi0_q(iq)[..., 0]
            ref = ctx.epsinv_q()[..., 0]
            ctx.write_q()
            q = np.loadtxt(os.path.join(root, "dir-eps", "q%03d" % iq, "dat.sq"))
            LG = synth.sphere(bvec, kw["ecut_for_eps"], q)
            ql = np.linalg.norm((LG + q[None, :]) @ bvec, axis=1)
            eps = _eps_from_chi(chi, ql)
            ng, nmat = eps.shape[0], eps.shape[2]
            a = _to_device(eps, torch)
            if call == 0:           # out of place: the input stays as it was
                out = torch.empty_like(a)
                keep = a.clone()
                rc = L.rp_zinv_batched_noalloc(a.data_ptr(), out.data_ptr(), ng, nmat, stream.cuda_stream)
                assert rc == 0, L.rp_last_error(None)
                assert torch.equal(a, keep)
            else:                   # in place
                out = a
                rc = L.rp_zinv_batched_noalloc(a.data_ptr(), a.data_ptr(), ng, nmat, stream.cuda_stream)
                assert rc == 0, L.rp_last_error(None)
            got = _from_device(out, ng, nmat)
            err = normwise_err(got, ref)
            assert err < 1e-10, f"q{iq}: noalloc inverse differs from rp_epsinv_q by {err:.3e}"
            for e in range(nmat):
                np.testing.assert_allclose(got[:, :, e] @ eps[:, :, e], np.eye(ng), atol=1e-10)
