"""The GB300 library against the CPU oracle (FP64 path), through the C ABI."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as orc
from respackdev_gb300 import chiqw as rp
from respackdev_gb300 import synth
from tests.helpers import (CLOSED_FORM_TOL, EM_TEST, case_name, freq_errs, namelist_text, normwise_err,
                           read_eps_record, run_params)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from respackdev_gb300 import build
    build.build()
    rp.load()


def _oracle_run(root, kw, qidx=None, **extra):
    p = orc.make_params(em=EM_TEST, dump_chi=1, nthreads=8, **kw, **extra,
                        **({"calc_num_k": qidx} if qidx else {}))
    return orc.calc_chiqw(root, p)


@pytest.mark.parametrize("case", ["tiny", "tiny_metal", "tiny_metal_crpa", "tiny_odd", "tiny_sym", "tiny_glide"])
def test_chi0_fp64_matches_oracle_all_q(case_dir, fresh_copy, case):
    """Every q point of the case: chi0 within 1e-6 (normwise per frequency),
    eps^-1 within 1e-6 of the oracle's."""
    kw = run_params(case)
    ref_root = fresh_copy(case_dir(case_name(case)))
    _oracle_run(ref_root, kw)
    params = rp.default_params(**kw)
    with rp.Context(ref_root, params, EM_TEST) as ctx:
        nq = ctx.L.rp_num_qirr(ctx._h)
        worst_chi = worst_eps = 0.0
        for iq in range(1, nq + 1):
            chi = ctx.chi0_q(iq)
            ref = orc.read_chi_dump(os.path.join(ref_root, "dir-eps", "q%03d" % iq, "dat.chi0"))
            assert chi.shape == ref.shape, (iq, chi.shape, ref.shape)
            worst_chi = max(worst_chi, normwise_err(chi, ref))
            eps = ctx.epsinv_q()
            ng, nen, ndir = eps.shape[0], eps.shape[2], eps.shape[3]
            for ix in range(ndir):
                er = read_eps_record(os.path.join(ref_root, "dir-eps", "q%03d" % iq, "dat.epsqw.%03d" % (600 + ix)),
                                     ng, nen)
                worst_eps = max(worst_eps, normwise_err(eps[..., ix], er))
        assert ctx.kernel_launches() > 0
    print(f"{case}: chi rel err {worst_chi:.3e}  epsinv rel err {worst_eps:.3e}")
    assert worst_chi < 1e-6
    assert worst_eps < 1e-6


def test_calc_chiqw_executable_writes_dir_eps(case_dir, fresh_copy, tmp_path):
    """rp_calc_chiqw < namelist writes the reference's dir-eps layout; a second
    run resumes (skips every q holding dat.log.400)."""
    from respackdev_gb300 import build
    kw = run_params("tiny")
    ref_root = fresh_copy(case_dir("tiny"))
    _oracle_run(ref_root, kw)
    run = str(tmp_path / "run")
    shutil.copytree(os.path.join(case_dir("tiny"), "dir-wfn"), os.path.join(run, "dir-wfn"))
    text = namelist_text(kw, EM_TEST)
    r = subprocess.run([build.EXE], input=text, text=True, cwd=run, capture_output=True)
    assert r.returncode == 0, r.stderr
    for iq in range(1, 9):
        qd = os.path.join(run, "dir-eps", "q%03d" % iq)
        rd = os.path.join(ref_root, "dir-eps", "q%03d" % iq)
        assert sorted(os.listdir(qd)) == sorted(x for x in os.listdir(rd) if x != "dat.chi0")
        np.testing.assert_allclose(np.loadtxt(os.path.join(qd, "dat.sq")), np.loadtxt(os.path.join(rd, "dat.sq")))
        a = synth.read_unformatted_records(os.path.join(qd, "dat.epsqw.600"))[0]
        b = synth.read_unformatted_records(os.path.join(rd, "dat.epsqw.600"))[0]
        assert len(a) == len(b)
        a = np.frombuffer(a, dtype=np.complex128); b = np.frombuffer(b, dtype=np.complex128)
        assert np.abs(a - b).max() / np.abs(b).max() < 1e-6
        ta = np.loadtxt(os.path.join(qd, "dat.epsqw.600001"))
        tb = np.loadtxt(os.path.join(rd, "dat.epsqw.600001"))
        np.testing.assert_allclose(ta, tb, atol=2e-9)
    wg = np.loadtxt(os.path.join(run, "dir-eps", "dat.wgrid"), skiprows=1)
    np.testing.assert_allclose(wg[:, 0] + 1j * wg[:, 1], EM_TEST, atol=1e-10)
    # resume: nothing left to do, files untouched
    mt = os.path.getmtime(os.path.join(run, "dir-eps", "q003", "dat.epsqw.600"))
    os.remove(os.path.join(run, "dir-eps", "q005", "dat.log.400"))
    r = subprocess.run([build.EXE], input=text, text=True, cwd=run, capture_output=True)
    assert r.returncode == 0, r.stderr
    assert os.path.getmtime(os.path.join(run, "dir-eps", "q003", "dat.epsqw.600")) == mt
    assert os.path.exists(os.path.join(run, "dir-eps", "q005", "dat.log.400"))


def test_bad_input_reports_error(case_dir, fresh_copy):
    root = fresh_copy(case_dir("tiny"))
    with pytest.raises(RuntimeError, match="outside dat.sample-k"):
        with rp.Context(root, rp.default_params(**run_params("tiny")), EM_TEST) as ctx:
            ctx.chi0_q(99)
    with pytest.raises(RuntimeError, match="cannot open"):
        rp.Context(root + "/nonexistent", rp.default_params(), EM_TEST)


@pytest.mark.parametrize("case,qs", [("tiny", [1, 2, 5]), ("tiny_metal", [1, 3]), ("fcc_4k_40b", [1, 2, 7]),
                                     ("tiny_glide", [1, 4, 8])])
@pytest.mark.parametrize("pair64", [0, 1])
@pytest.mark.parametrize("prec", [rp.PREC_FP16X3, rp.PREC_BF16X3, rp.PREC_FP16X2])
def test_chi0_tensor_core_matches_oracle(case_dir, fresh_copy, case, qs, prec, pair64):
    """Split-precision tcgen05 contraction: chi0 and eps^-1 within 1e-6 (normwise
    per frequency) of the FP64 oracle for the three-term FP16 split, with FP32
    or FP64 pair densities; eps^-1 from the mixed-precision inverse."""
    if pair64 and prec != rp.PREC_FP16X3:
        pytest.skip("FP64 pair densities are checked with one split")
    kw = run_params(case)
    ref_root = fresh_copy(case_dir(case_name(case)))
    _oracle_run(ref_root, kw, qidx=qs)
    with rp.Context(ref_root, rp.default_params(precision=prec, pair_fp64=pair64, **kw), EM_TEST) as ctx:
        worst = worst_eps = 0.0
        for iq in qs:
            chi = ctx.chi0_q(iq)
            ref = orc.read_chi_dump(os.path.join(ref_root, "dir-eps", "q%03d" % iq, "dat.chi0"))
            worst = max(worst, normwise_err(chi, ref))
            eps = ctx.epsinv_q()
            # the split precisions invert with the FP32 Gauss-Jordan plus one float-pair
            # Newton step; these well-conditioned cases never need the FP64 fallback
            assert not ctx.eps_fallback(), f"q{iq}: mixed-precision inverse fell back to FP64"
            ng, nen = eps.shape[0], eps.shape[2]
            er = read_eps_record(os.path.join(ref_root, "dir-eps", "q%03d" % iq, "dat.epsqw.600"), ng, nen)
            worst_eps = max(worst_eps, normwise_err(eps[..., 0], er))
    print(f"{case} prec={prec} pair64={pair64}: chi rel err {worst:.3e} epsinv {worst_eps:.3e}")
    # the 1e-6 target holds for the three-term FP16 split; the BF16 split keeps
    # 23 bits, held to 1e-5, and the two-term FP16 split 22, held to 2e-5
    bound = {rp.PREC_FP16X3: 1e-6, rp.PREC_BF16X3: 1e-5}.get(prec, 2e-5)
    assert worst < bound
    assert worst_eps < bound


def test_gen_grid_matches_oracle(case_dir, fresh_copy, tmp_path):
    """Without an explicit grid both take gen_grid (gen_grid.f90:1-39, called
    at chiqw.F:1184-1192): the same dat.wgrid, and chi0 on that grid within
    1e-6 up to 2 Ha; the two highest frequencies (2.8 and 3.9 Ha, far above the
    tetrahedra's spread) within the closed forms' own conditioning."""
    from respackdev_gb300 import build
    kw = run_params("tiny")
    ref_root = fresh_copy(case_dir("tiny"))
    orc.calc_chiqw(ref_root, orc.make_params(dump_chi=1, nthreads=8, calc_num_k=[2], num_freq_grid=20, **kw))
    run = str(tmp_path / "run")
    shutil.copytree(os.path.join(case_dir("tiny"), "dir-wfn"), os.path.join(run, "dir-wfn"))
    # &param_chiqw, then the q list (m_rdinput.f90:97-103), then &param_gpu
    text = namelist_text(dict(kw, num_freq_grid=20, flg_calc_type=2, n_calc_q=1)) + " 2\n&param_gpu dump_chi=1 /\n"
    r = subprocess.run([build.EXE], input=text, text=True, cwd=run, capture_output=True)
    assert r.returncode == 0, r.stderr
    w1 = open(os.path.join(run, "dir-eps", "dat.wgrid")).read()
    w2 = open(os.path.join(ref_root, "dir-eps", "dat.wgrid")).read()
    assert w1 == w2
    g1 = np.loadtxt(os.path.join(run, "dir-eps", "dat.wgrid"), skiprows=1)
    assert g1.shape == (20, 2) and np.all(np.diff(g1[:, 0]) > 0)
    chi = orc.read_chi_dump(os.path.join(run, "dir-eps", "q002", "dat.chi0"))
    ref = orc.read_chi_dump(os.path.join(ref_root, "dir-eps", "q002", "dat.chi0"))
    assert chi.shape == ref.shape and chi.shape[2] == 20
    err = freq_errs(chi, ref)
    low = g1[:, 0] < 2.0
    assert low.sum() == 18
    assert err[low].max() < 1e-6, err
    assert err.max() < CLOSED_FORM_TOL, err
