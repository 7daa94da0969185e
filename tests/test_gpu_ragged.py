"""Ragged batches (rp_chi0_batch): cells of different lattices, k meshes, band
counts, G spheres and frequency grids whose chi0 problems share one
tensor-core launch inside one CUDA graph, checked against the same problems
one q at a time (rp_chi0_q) and against the oracle; and the K-split tuner's
splits against the unsplit contraction."""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from respackdev_gb300 import chiqw as rp
from respackdev_gb300 import synth
from tests.helpers import AU, EM_TEST, normwise_err

pytestmark = pytest.mark.gpu

# three cells, each with its own lattice, mesh, bands, cutoffs and frequency grid
CELLS = {
    "fcc": (synth.SynthSpec(lattice="fcc", a=10.26, nk=(2, 2, 2), nbands=14, nocc=4, ecut_psi=8.0, seed=31,
                            wan_lo=5, wan_hi=7), 3.0, EM_TEST),
    "bcc": (synth.SynthSpec(lattice="bcc", a=8.5, nk=(3, 3, 3), nbands=12, nocc=3, ecut_psi=7.0, seed=32,
                            wan_lo=4, wan_hi=6), 4.0, EM_TEST[:3]),
    "sc": (synth.SynthSpec(lattice="sc", a=7.0, nk=(2, 2, 2), nbands=16, nocc=5, ecut_psi=9.0, seed=33, metal=True,
                           wan_lo=6, wan_hi=8), 5.0,
           np.concatenate([EM_TEST, np.array([2.0j, 6.0j, 3.0]) / AU])),
}
PROBLEMS = [("fcc", 1), ("bcc", 3), ("sc", 2), ("fcc", 2), ("bcc", 1), ("sc", 1), ("fcc", 5), ("bcc", 14)]


@pytest.fixture(scope="module")
def cells(tmp_path_factory):
    base = tmp_path_factory.mktemp("ragged")
    out = {}
    for name, (spec, ecut, em) in CELLS.items():
        d = os.path.join(str(base), name)
        os.makedirs(d)
        synth.make_case(d, spec)
        out[name] = (d, ecut, em)
    return out


def _contexts(cells, prec, **extra):
    return {name: rp.Context(d, rp.default_params(precision=prec, green_func_delt=0.2721, ecut_for_eps=ecut,
                                                   **extra), em)
            for name, (d, ecut, em) in cells.items()}


def _close(ctxs):
    for c in ctxs.values():
        c.close()


@pytest.mark.parametrize("prec", [rp.PREC_FP16X3, rp.PREC_BF16X3])
def test_ragged_batch_matches_single_q(cells, prec):
    """One grouped launch (with and without the CUDA graph) gives every problem
    the chi0 that rp_chi0_q gives it alone: the same operands, splits and sums."""
    ctxs = _contexts(cells, prec)
    try:
        probs = [(ctxs[n], iq) for n, iq in PROBLEMS]
        single = [c.chi0_q(iq) for c, iq in probs]
        launches0 = ctxs["fcc"].kernel_launches()
        batched, sec = rp.chi0_batch(probs, graph=True)
        assert ctxs["fcc"].kernel_launches() > launches0
        plain, _ = rp.chi0_batch(probs, graph=False)
        shapes = set()
        for (n, iq), a, g, p in zip(PROBLEMS, single, batched, plain):
            assert g.shape == a.shape and p.shape == a.shape, (n, iq)
            shapes.add(a.shape)
            assert normwise_err(g, a) <= 1e-13, (n, iq, normwise_err(g, a))
            assert normwise_err(p, a) <= 1e-13, (n, iq)
        assert len(shapes) >= 4  # the batch really is ragged
        assert sec[1] > 0
    finally:
        _close(ctxs)


def test_ragged_batch_against_oracle(cells, tmp_path):
    """Problems of all three cells from one batch against the FP64 oracle (1e-6)."""
    import shutil
    roots = {}
    for name in ("fcc", "bcc", "sc"):
        d, ecut, em = cells[name]
        r = os.path.join(str(tmp_path), name)
        for sub in ("dir-wfn", "dir-wan"):
            shutil.copytree(os.path.join(d, sub), os.path.join(r, sub))
        qs = [iq for n, iq in PROBLEMS if n == name]
        p = orc.make_params(em=em, dump_chi=1, nthreads=8, green_func_delt=0.2721, ecut_for_eps=ecut, calc_num_k=qs)
        orc.calc_chiqw(r, p)
        roots[name] = (r, ecut, em)
    ctxs = {n: rp.Context(r, rp.default_params(precision=rp.PREC_FP16X3, green_func_delt=0.2721, ecut_for_eps=ecut), em)
            for n, (r, ecut, em) in roots.items()}
    try:
        probs = [(n, iq) for n, iq in PROBLEMS if n in roots]
        res, _ = rp.chi0_batch([(ctxs[n], iq) for n, iq in probs])
        worst = 0.0
        for (n, iq), chi in zip(probs, res):
            ref = orc.read_chi_dump(os.path.join(roots[n][0], "dir-eps", "q%03d" % iq, "dat.chi0"))
            worst = max(worst, normwise_err(chi, ref))
        print(f"ragged batch vs oracle: chi rel err {worst:.3e}")
        assert worst < 1e-6
    finally:
        _close(ctxs)


def test_k_splits_agree_and_tuner_caches(case_dir, fresh_copy):
    """A small q point (few tiles) with 1, 2 and 8 K splits and with the tuner's
    choice: the same chi0 up to the rounding of the float-pair sums, whose low
    word carries the correction products in FP32 (about 2^-31 of chi per
    sub-chunk, so another K partition moves chi by ~1e-9); the tuner measures
    the shape once."""
    root = fresh_copy(case_dir("fcc_4k_40b"))
    kw = dict(green_func_delt=0.2721, ecut_for_eps=3.0, flg_crpa=1, precision=rp.PREC_FP16X3)
    em = EM_TEST
    res = {}
    for split in (1, 2, 8):
        with rp.Context(root, rp.default_params(tc_split=split, **kw), em) as ctx:
            res[split] = [ctx.chi0_q(iq) for iq in (2, 3)]
    rp.reset_tuner()
    assert rp.tuned_shapes() == 0
    with rp.Context(root, rp.default_params(tc_split=0, **kw), em) as ctx:
        res[0] = [ctx.chi0_q(iq) for iq in (2, 3)]
        assert rp.tuned_shapes() >= 1
    for split in (2, 8, 0):
        for a, b in zip(res[split], res[1]):
            assert normwise_err(a, b) <= 1e-8, (split, normwise_err(a, b))
