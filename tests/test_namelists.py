"""The reference's own sample namelists (tests/golden/namelists/, copied by
make_namelist_fixtures.py) through the library's parsers.

Every sample but TiO2 holds &param_chiqw and &param_calc_int among the groups
of RESPACK's other programs (wannier, interpolation, visualization); the
parsers must read the two groups and skip the rest, as the reference's
`read(5, nml=...)` does (src/chiqw/m_rdinput.f90:76,
src/calc_int/m_rdinput.f90:33).  TiO2 has neither group, so the reference's
namelist read fails on it, and so must ours.
"""
import glob
import os

import pytest

from respackdev_gb300 import build
from respackdev_gb300 import calc_int as ci
from respackdev_gb300 import chiqw as rp

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "namelists")
FILES = sorted(glob.glob(os.path.join(HERE, "*.in")))

# values the samples set (everything else keeps the m_rdinput defaults)
CHIQW = {
    "La2CuO4": dict(ecut_for_eps=3.0, flg_crpa=1),
    "SrVO3": dict(ecut_for_eps=5.0, flg_crpa=1),
}
CALC_INT = {
    "La2CuO4": dict(ix_intj_min=-1, ix_intj_max=1, iy_intj_min=-1, iy_intj_max=1, iz_intj_min=-1, iz_intj_max=1),
}


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def test_all_nine_samples_present():
    assert len(FILES) == 9, FILES


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
def test_sample_namelist(path):
    text = open(path).read()
    material = os.path.basename(path).split("_", 1)[1][:-3]
    if material == "TiO2":
        with pytest.raises(ValueError, match="not found"):
            rp.parse_namelist(text)
        with pytest.raises(ValueError, match="not found"):
            ci.parse_namelist(text)
        return
    p, q, em = rp.parse_namelist(text)
    d = rp.default_params()
    want = CHIQW.get(material, {})
    for name, _ in rp.Params._fields_:
        got, ref = getattr(p, name), getattr(d, name)
        if name in want:
            assert got == pytest.approx(want[name]), name
        elif name != "fft_box":
            assert got == ref, name
    assert q == [] and em is None
    pi = ci.parse_namelist(text)
    di = ci.default_params()
    want = CALC_INT.get(material, {})
    for name, _ in ci.IntParams._fields_:
        if name == "fft_box":
            continue
        got, ref = getattr(pi, name), getattr(di, name)
        assert got == pytest.approx(want.get(name, ref)), name
