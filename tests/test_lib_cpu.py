"""Host-side checks of the library that need no GPU: it builds for sm_103a,
loads, exports every symbol the C header declares, and its namelist parser
follows &param_chiqw (src/chiqw/m_rdinput.f90)."""
import os
import re

import numpy as np
import pytest

from respackdev_gb300 import build
from respackdev_gb300 import chiqw as rp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "respack_gb300.h")).read()
    names = set(re.findall(r"\b(rp_[a-z0-9_]+)\s*\(", hdr))
    assert {"rp_ctx_create", "rp_chi0_q", "rp_epsinv_q", "rp_calc_chiqw", "rp_last_error"} <= names
    L = rp.load()
    for n in sorted(names):
        assert hasattr(L, n), n


def test_defaults_follow_m_rdinput():
    p = rp.default_params()
    assert p.num_freq_grid == 70 and abs(p.green_func_delt - 0.1) < 1e-15
    assert abs(p.max_excitation_energy - 200.0) < 1e-12 and p.file_num_eps_base_start == 600000
    assert p.file_num_log_start == 400 and p.file_num_eps_start == 600 and p.flg_calc_type == 0


def test_namelist_parser():
    text = """ &PARAM_CHIQW
  N_CALC_BAND= 40 ,   ! comment
  Ecut_for_eps = 3.0D0, SHIFT_EF=0.0d0
  Green_func_delt=0.1d0,MAX_EXCITATION_ENERGY=50.0
  flg_cRPA=1 , flg_calc_type=2, n_calc_q = 3,
  MPI_num_qcomm=2
 /
 1 2
 5
 &param_gpu precision='bf16x3', fft_box = 24, 24, 24, freq_re_ev=0.0,2.0 freq_im_ev=0.0,0.5,
  tc_split=4, pair_batch=100, write_eps_f32=1, tc_pair=2, tetra_fp64=1, ur_window=3, eps_fp64=1,
  tail_model='net.bin' /
"""
    p, q, em = rp.parse_namelist(text)
    assert p.tc_split == 4 and p.pair_batch == 100 and p.write_eps_f32 == 1
    assert p.tc_pair == 2 and p.tetra_fp64 == 1 and p.ur_window == 3 and p.eps_fp64 == 1
    assert p.tail_model == b"net.bin"
    assert p.n_calc_band == 40 and p.flg_crpa == 1 and p.flg_calc_type == 2 and p.mpi_num_qcomm == 2
    assert abs(p.ecut_for_eps - 3.0) < 1e-15 and abs(p.max_excitation_energy - 50.0) < 1e-15
    assert q == [1, 2, 5]
    assert p.precision == rp.PREC_BF16X3 and list(p.fft_box) == [24, 24, 24]
    np.testing.assert_allclose(em, np.array([0.0, 2.0 + 0.5j]) / 27.21151)


@pytest.mark.parametrize("bad,msg", [
    ("&param_chiqw foo=1 /", "unknown name"),
    ("&param_chiqw flg_calc_type=2 /", "n_calc_q should not be zero"),
    ("&other x=1 /", "not found"),
    ("&param_chiqw n_calc_q=3 /\n 1 2\n", "shorter than n_calc_q"),
])
def test_namelist_errors(bad, msg):
    with pytest.raises(ValueError, match=msg):
        rp.parse_namelist(bad)
