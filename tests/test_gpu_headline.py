"""Parity at the geometry of the 8x8x8-k / 200-band workload.

The workload's cell, cutoffs, FFT box and frequency grid (fcc a = 15.84 bohr,
20 Ry, 36^3 box, dielectric cutoff 11 Ry: NG about 600, so the tensor-core
Gram kernel runs 5 x 5 upper tiles and the pair densities take the 36^3 slab
instance) on a 4x4x4 mesh, with the first 32 band pairs so the oracle finishes
in seconds.  chi0 and eps^-1 of Gamma (three directions) and of two q != 0
points, FP64 and the FP16x3, BF16x3 and FP16x2 splits, against the oracle:
normwise relative error per frequency below 1e-6 (FP16x2: 2e-5).  The
mixed-precision inverse of the split path is also compared with the FP64
inverse of the same chi.
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from respackdev_gb300 import chiqw as rp
from respackdev_gb300 import synth
from tests.helpers import normwise_err, read_eps_record

pytestmark = pytest.mark.gpu

AU = 27.21151
QS = [1, 2, 7]
NPAIR = 32
BOX = (36, 36, 36)
KW = dict(ecut_for_eps=11.0, green_func_delt=0.2721, flg_crpa=1)


def _frequencies():
    """10 real 0-30 eV and 10 imaginary on a Gauss-Legendre grid over 0-30 eV (Hartree)."""
    x, _ = np.polynomial.legendre.leggauss(10)
    return np.concatenate([np.linspace(0.0, 30.0, 10), 1j * 15.0 * (x + 1.0)]) / AU


@pytest.fixture(scope="module")
def headline(tmp_path_factory):
    from respackdev_gb300 import build
    build.build()
    rp.load()
    root = str(tmp_path_factory.mktemp("headline_small"))
    synth.make_case(root, synth.CASES["headline_small"])
    em = _frequencies()
    orc.calc_chiqw(root, orc.make_params(em=em, dump_chi=1, nthreads=os.cpu_count() or 8, max_pairs=NPAIR,
                                         calc_num_k=QS, fft_box=BOX, **KW))
    ref = {}
    for iq in QS:
        qd = os.path.join(root, "dir-eps", "q%03d" % iq)
        chi = orc.read_chi_dump(os.path.join(qd, "dat.chi0"))
        ng, nen, ndir = chi.shape[0], chi.shape[2], chi.shape[3]
        eps = np.stack([read_eps_record(os.path.join(qd, "dat.epsqw.%03d" % (600 + ix)), ng, nen)
                        for ix in range(ndir)], axis=-1)
        ref[iq] = (chi, eps)
    return root, em, ref


# chi tolerance per precision: 1e-6 for FP64, FP16x3 and BF16x3 (the three-plane
# splits), FP16x2 (two planes, about 22 bits) its documented 2e-5
TOL = {rp.PREC_FP64: 1e-6, rp.PREC_FP16X3: 1e-6, rp.PREC_BF16X3: 1e-6, rp.PREC_FP16X2: 2e-5}


@pytest.mark.parametrize("prec", [rp.PREC_FP64, rp.PREC_FP16X3, rp.PREC_BF16X3, rp.PREC_FP16X2])
def test_headline_geometry_matches_oracle(headline, prec):
    root, em, ref = headline
    params = rp.default_params(precision=prec, fft_box=BOX, max_pairs=NPAIR, **KW)
    worst_chi = worst_eps = 0.0
    with rp.Context(root, params, em) as ctx:
        for iq in QS:
            chi = ctx.chi0_q(iq)
            eps = ctx.epsinv_q()
            rchi, reps = ref[iq]
            assert chi.shape == rchi.shape
            # the multi-tile Gram path: more than four 128-row tiles
            assert chi.shape[0] > 512, chi.shape
            assert not ctx.eps_fallback()
            worst_chi = max(worst_chi, normwise_err(chi, rchi))
            worst_eps = max(worst_eps, normwise_err(eps, reps))
    print(f"headline geometry prec={prec}: chi rel err {worst_chi:.3e}  epsinv rel err {worst_eps:.3e}")
    assert worst_chi < TOL[prec]
    assert worst_eps < TOL[prec]


def test_mixed_inverse_matches_fp64_inverse(headline):
    """The split path's eps^-1 (FP32 Gauss-Jordan + one float-pair Newton step)
    against the FP64 Gauss-Jordan of the same chi (eps_fp64=1)."""
    root, em, _ = headline
    base = dict(precision=rp.PREC_FP16X3, fft_box=BOX, max_pairs=NPAIR, **KW)
    worst = 0.0
    with rp.Context(root, rp.default_params(**base), em) as mixed, \
            rp.Context(root, rp.default_params(eps_fp64=1, **base), em) as full:
        for iq in QS:
            c1 = mixed.chi0_q(iq)
            c2 = full.chi0_q(iq)
            # same inputs, same kernels: chi equal up to the order of floating-point
            # sums, so the difference below is the inversion's
            assert normwise_err(c1, c2) < 1e-12
            e1 = mixed.epsinv_q()
            e2 = full.epsinv_q()
            worst = max(worst, normwise_err(e1, e2))
    print(f"mixed-precision vs FP64 inverse of the same chi: {worst:.3e}")
    # one Newton step leaves about |I - eps X0|^2 of the FP32 inverse X0
    assert worst < 1e-7
