"""The large end-to-end workload's geometry on a small mesh: fcc a = 15.84
bohr, 31.7 Ry (about 2980 plane waves, a 23^3 plane-wave cube in the real-space
transform), 48^3 box, dielectric cutoff 25.8 Ry (about 2180 G: 18 x 18 Gram
tiles), 40 bands on a 2x2x2 mesh given as 3 irreducible points of the cubic
group.  The virtual bands' real-space functions go through a window of two
slots per pair batch, as the 1000-band workload needs.  chi0 and eps^-1 of
Gamma and of a q != 0 point against the oracle (first 16 band pairs: within
1e-6 up to 20 eV, within the closed forms' conditioning at 30i eV), and a
dat.epsqw.600 record above 2 GiB written in gfortran's subrecords."""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from respackdev_gb300 import chiqw as rp
from respackdev_gb300 import synth
from tests.helpers import CLOSED_FORM_TOL, freq_errs, normwise_err, read_eps_record

pytestmark = pytest.mark.gpu

AU = 27.21151
BOX = (48, 48, 48)
KW = dict(ecut_for_eps=25.8, green_func_delt=0.2721, flg_crpa=1)
NPAIR = 16
QS = [1, 2]


def _em(n):
    """n/2 real frequencies over 0-30 eV and n/2 imaginary ones (Hartree)."""
    h = n // 2
    return np.concatenate([np.linspace(0.0, 30.0, n - h), 1j * np.linspace(30.0 / h, 30.0, h)]) / AU


@pytest.fixture(scope="module")
def large_small(tmp_path_factory):
    from respackdev_gb300 import build
    build.build()
    rp.load()
    root = str(tmp_path_factory.mktemp("large_small"))
    synth.make_case(root, synth.CASES["large_small"])
    return root


def test_large_geometry_matches_oracle(large_small):
    root = large_small
    em = _em(6)
    orc.calc_chiqw(root, orc.make_params(em=em, dump_chi=1, nthreads=os.cpu_count() or 8, max_pairs=NPAIR,
                                         calc_num_k=QS, fft_box=BOX, **KW))
    for prec in (rp.PREC_FP64, rp.PREC_FP16X3):
        params = rp.default_params(precision=prec, fft_box=BOX, max_pairs=NPAIR, ur_window=2, **KW)
        chi_err = np.zeros(len(em))
        eps_err = np.zeros(len(em))
        with rp.Context(root, params, em) as ctx:
            for iq in QS:
                chi = ctx.chi0_q(iq)
                eps = ctx.epsinv_q()
                qd = os.path.join(root, "dir-eps", "q%03d" % iq)
                ref = orc.read_chi_dump(os.path.join(qd, "dat.chi0"))
                assert chi.shape == ref.shape and chi.shape[0] > 2048, chi.shape
                chi_err = np.maximum(chi_err, freq_errs(chi, ref))
                er = np.stack([read_eps_record(os.path.join(qd, "dat.epsqw.%03d" % (600 + ix)), chi.shape[0], len(em))
                               for ix in range(chi.shape[3])], axis=-1)
                eps_err = np.maximum(eps_err, freq_errs(eps, er))
        print(f"large geometry prec={prec}: chi rel err per frequency {np.array2string(chi_err, precision=2)}  "
              f"epsinv {np.array2string(eps_err, precision=2)}")
        low = np.abs(em) * AU <= 20.0 + 1e-9
        assert chi_err[low].max() < 1e-6 and eps_err[low].max() < 1e-6
        assert chi_err.max() < CLOSED_FORM_TOL and eps_err.max() < CLOSED_FORM_TOL


def test_epsinv_record_above_2gib(large_small, tmp_path):
    """30 frequencies at NG about 2180: one dat.epsqw.600 record of 2.27e9
    bytes, above gfortran's 2^31 - 9 byte limit of one subrecord, so rp_write_q
    writes it in subrecords (chiqw.F:1531-1538 writes it as one record); the
    record reads back to the eps^-1 the context returned."""
    import shutil
    root = str(tmp_path / "run")
    shutil.copytree(os.path.join(large_small, "dir-wfn"), os.path.join(root, "dir-wfn"))
    shutil.copytree(os.path.join(large_small, "dir-wan"), os.path.join(root, "dir-wan"))
    em = _em(30)
    params = rp.default_params(precision=rp.PREC_FP16X3, fft_box=BOX, max_pairs=NPAIR, **KW)
    with rp.Context(root, params, em) as ctx:
        ctx.chi0_q(2, fetch=False)
        eps = ctx.epsinv_q()
        ctx.write_q()
    ng = eps.shape[0]
    path = os.path.join(root, "dir-eps", "q002", "dat.epsqw.600")
    nbytes = ng * ng * len(em) * 16
    assert nbytes > 2147483639
    with open(path, "rb") as f:
        head = np.frombuffer(f.read(4), dtype="<i4")[0]
    assert head < 0                      # a continued subrecord
    back = read_eps_record(path, ng, len(em))
    assert np.array_equal(back, eps[..., 0])
    assert os.path.getsize(path) == nbytes + 8 * ((nbytes + 2147483638) // 2147483639)
