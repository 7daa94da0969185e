"""The tensor-core Gram kernel on CTA pairs (tc_pair=2: tcgen05.mma.cta_group::2,
256 x 256 blocks of 2 x 2 tiles, each CTA one row tile of the weighted operand
and one column tile of B) against single CTAs (tc_pair=1) on the same inputs:
every precision, the K-split path, a ragged group, the multi-tile headline
geometry, and the launch tuner's choice (tc_pair=0).

The same products into the same FP32 accumulators over the same sub-chunks:
chi equal up to the order of the float-pair sums."""
import numpy as np
import pytest

from respackdev_gb300 import chiqw as rp
from tests.helpers import EM_TEST, normwise_err

pytestmark = pytest.mark.gpu

KW = dict(green_func_delt=0.2721, ecut_for_eps=3.0, flg_crpa=1)


def _chi(root, qs, **kw):
    with rp.Context(root, rp.default_params(**dict(KW, **kw)), EM_TEST) as ctx:
        return [ctx.chi0_q(iq) for iq in qs]


@pytest.mark.parametrize("prec", [rp.PREC_FP16X3, rp.PREC_BF16X3, rp.PREC_FP16X2])
def test_pair_matches_single(case_dir, fresh_copy, prec):
    root = fresh_copy(case_dir("fcc_4k_40b"))
    one = _chi(root, (1, 2), precision=prec, tc_pair=1, tc_split=1)
    two = _chi(root, (1, 2), precision=prec, tc_pair=2, tc_split=1)
    for a, b in zip(two, one):
        err = normwise_err(a, b)
        print(f"prec={prec}: CTA pair vs single {err:.3e}")
        assert err <= 1e-8


def test_pair_with_k_splits(case_dir, fresh_copy):
    root = fresh_copy(case_dir("fcc_4k_40b"))
    ref = _chi(root, (2, 3), precision=rp.PREC_FP16X3, tc_pair=1, tc_split=1)
    for split in (2, 5):
        got = _chi(root, (2, 3), precision=rp.PREC_FP16X3, tc_pair=2, tc_split=split)
        for a, b in zip(got, ref):
            # another K partition moves the float-pair sums by ~1e-9 of chi
            assert normwise_err(a, b) <= 1e-8, split


def test_pair_ragged_group(case_dir, fresh_copy):
    roots = [fresh_copy(case_dir(n)) for n in ("fcc_4k_40b", "tiny")]
    probs_of = lambda ctxs: [(ctxs[0], 1), (ctxs[1], 2), (ctxs[0], 3), (ctxs[1], 1)]
    out = {}
    for pair in (1, 2):
        ctxs = [rp.Context(r, rp.default_params(precision=rp.PREC_FP16X3, tc_pair=pair, tc_split=1, **KW), EM_TEST)
                for r in roots]
        try:
            out[pair], _ = rp.chi0_batch(probs_of(ctxs), graph=True)
        finally:
            for c in ctxs:
                c.close()
    for a, b in zip(out[2], out[1]):
        assert normwise_err(a, b) <= 1e-8


def test_pair_headline_geometry(tmp_path):
    """NG about 600 (10 x 10 tiles): 15 blocks of 2 x 2 tiles per channel, the
    below-diagonal tiles of the diagonal blocks computed and never read."""
    from respackdev_gb300 import synth
    root = str(tmp_path / "h")
    synth.make_case(root, synth.CASES["headline_small"])
    kw = dict(precision=rp.PREC_FP16X3, fft_box=(36, 36, 36), max_pairs=32, ecut_for_eps=11.0,
              green_func_delt=0.2721, flg_crpa=1, tc_split=1)
    res = {}
    for pair in (1, 2, 0):
        with rp.Context(root, rp.default_params(tc_pair=pair, **kw), EM_TEST) as ctx:
            res[pair] = ctx.chi0_q(2)
    assert res[1].shape[0] > 512
    for pair in (2, 0):
        err = normwise_err(res[pair], res[1])
        print(f"headline geometry: tc_pair={pair} vs single {err:.3e}")
        assert err <= 1e-8
    assert np.isfinite(res[2]).all()
