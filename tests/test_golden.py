"""The committed golden fixtures (tests/golden/, made by make_golden.py from the
oracle) against the synthetic generator, the oracle and the GPU library."""
from __future__ import annotations

import os

import numpy as np
import pytest

from respackdev_gb300 import chiqw as rp
from tests.golden import make_golden as mg
from tests.helpers import normwise_err


def _load(case):
    d = np.load(mg.golden_path(case))
    return {k: d[k] for k in d.files}


@pytest.mark.parametrize("case", list(mg.GOLDEN))
def test_generator_reproduces_golden_inputs(case, case_dir):
    g = _load(case)
    assert mg.input_digest(case_dir(case)) == str(g["digest"])


@pytest.mark.parametrize("case", list(mg.GOLDEN))
def test_oracle_reproduces_golden(case, case_dir, fresh_copy):
    g = _load(case)
    got = mg.compute(case, fresh_copy(case_dir(case)))
    for iq in g["qs"]:
        for name in ("chi0", "epsinv"):
            key = f"{name}_q{iq}"
            assert got[key].shape == g[key].shape
            err = normwise_err(got[key], g[key])
            assert err < 1e-12, f"{case} {key}: oracle drifted from the golden fixture by {err:.3e}"


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [rp.PREC_FP64, rp.PREC_FP16X3])
@pytest.mark.parametrize("case", list(mg.GOLDEN))
def test_gpu_matches_golden(case, prec, case_dir, fresh_copy):
    g = _load(case)
    kw, qs = mg.GOLDEN[case]
    root = fresh_copy(case_dir(case))
    with rp.Context(root, rp.default_params(precision=prec, **kw), g["em"]) as ctx:
        for iq in qs:
            chi = ctx.chi0_q(iq)
            eps = ctx.epsinv_q()
            for name, got in (("chi0", chi), ("epsinv", eps)):
                ref = g[f"{name}_q{iq}"]
                assert got.shape == ref.shape
                err = normwise_err(got, ref)
                # parity bound of the chiqw path: chi relative error <= 1e-6
                assert err < 1e-6, f"{case} q{iq} {name} (precision {prec}): {err:.3e}"
