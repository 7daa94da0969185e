import os
import shutil
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def case_dir(tmp_path_factory):
    """Return a function name -> directory holding that synthetic case's dir-wfn/dir-wan."""
    from respackdev_gb300 import synth

    base = tmp_path_factory.mktemp("cases")
    made = {}

    def get(name: str) -> str:
        if name not in made:
            d = os.path.join(str(base), name)
            os.makedirs(d, exist_ok=True)
            synth.make_case(d, synth.CASES[name])
            made[name] = d
        return made[name]

    return get


@pytest.fixture
def fresh_copy(tmp_path):
    """Copy a case directory's inputs (dir-wfn, dir-wan) into a fresh run directory."""

    def copy(src: str) -> str:
        dst = os.path.join(str(tmp_path), os.path.basename(src))
        os.makedirs(dst, exist_ok=True)
        for sub in ("dir-wfn", "dir-wan"):
            if os.path.isdir(os.path.join(src, sub)):
                shutil.copytree(os.path.join(src, sub), os.path.join(dst, sub))
        return dst

    return copy


@pytest.fixture(scope="session")
def int_case(tmp_path_factory):
    """Return a function name -> directory holding a Wannier case with dir-eps
    made by the oracle's chiqw (all q points, the frequencies of EM_INT)."""
    from oracle import oracle as orc
    from respackdev_gb300 import synth
    from tests.helpers import EM_INT

    base = tmp_path_factory.mktemp("int_cases")
    made = {}

    def get(name: str) -> str:
        if name not in made:
            d = os.path.join(str(base), name)
            os.makedirs(d, exist_ok=True)
            synth.make_case(d, synth.CASES[name])
            orc.calc_chiqw(d, orc.make_params(em=EM_INT, green_func_delt=0.2721, ecut_for_eps=3.0, nthreads=4))
            made[name] = d
        return made[name]

    return get


@pytest.fixture
def int_copy(tmp_path):
    """Copy a calc_int case (dir-wfn, dir-wan, dir-eps) into a fresh directory."""

    def copy(src: str) -> str:
        dst = os.path.join(str(tmp_path), os.path.basename(src))
        os.makedirs(dst, exist_ok=True)
        for sub in ("dir-wfn", "dir-wan", "dir-eps"):
            shutil.copytree(os.path.join(src, sub), os.path.join(dst, sub))
        return dst

    return copy
