"""A q point split into several band-pair batches (pair_batch) gives the same
chi0 and eps^-1 as one batch: batches take whole virtual-band groups, or split
a group that is larger than the batch (pairs per virtual band = 4 here)."""
from __future__ import annotations

import pytest

from respackdev_gb300 import chiqw as rp
from tests.helpers import EM_TEST, normwise_err, run_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [(rp.PREC_FP64, 1e-12), (rp.PREC_FP16X3, 1e-7)])
def test_pair_batches_agree(case_dir, fresh_copy, prec, tol):
    kw = run_params("tiny")
    root = fresh_copy(case_dir("tiny"))
    res = {}
    for pb in (0, 5, 3):   # one batch; whole groups of 4; groups split 3 + 1
        with rp.Context(root, rp.default_params(precision=prec, pair_batch=pb, **kw), EM_TEST) as ctx:
            res[pb] = [(ctx.chi0_q(iq), ctx.epsinv_q()) for iq in (1, 2)]
    for pb in (5, 3):
        for (chi, eps), (chi0, eps0) in zip(res[pb], res[0]):
            assert normwise_err(chi, chi0) < tol
            assert normwise_err(eps, eps0) < tol


@pytest.mark.parametrize("prec,tol", [(rp.PREC_FP64, 1e-12), (rp.PREC_FP16X3, 1e-6)])
def test_real_space_window_gives_the_same_chi0(case_dir, fresh_copy, prec, tol):
    """With ur_window the context keeps only the occupied bands' real-space
    functions resident and transforms each pair batch's virtual bands into a
    window of slots (here 3, so a q takes several batches); chi0 and eps^-1
    equal those of the context that holds every band, up to the order of the
    pair sums (FP64) and, on the split path, the batch-wise row scales of the
    operand planes (within the path's 1e-6)."""
    kw = run_params("tiny_metal")
    root = fresh_copy(case_dir("tiny_metal"))
    out = {}
    for win in (0, 3):
        with rp.Context(root, rp.default_params(precision=prec, ur_window=win, **kw), EM_TEST) as ctx:
            out[win] = [(ctx.chi0_q(iq), ctx.epsinv_q()) for iq in (1, 2, 5)]
    for (c0, e0), (c1, e1) in zip(out[0], out[3]):
        assert normwise_err(c1, c0) < tol
        assert normwise_err(e1, e0) < tol
