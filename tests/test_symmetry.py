"""Symmetry-reduced inputs: an irreducible dat.sample-k with the 48 cubic
operations in dat.symmetry (and, for tiny_glide, the diamond structure's
fractional translation, nnp = 4), against the identity-only input that lists
the same wave functions on the whole mesh (synth.full_mesh_equivalent).

The reference unfolds the irreducible points (chiqw.F:437-480: rotations,
time reversal, the RW wraps of kcheck / kcheck_trs) and rotates their
coefficients with make_C0 (chiqw_sub.F:264-322: R^-1 (G + RW), the phase
exp(-2 pi i G.pg/nnp), conjugation for time reversal).  Both inputs describe
the same full-mesh wave functions, so chi0 and eps^-1 of every irreducible q
must agree.  Here the oracle runs both; the GPU tests run the library on the
symmetry-reduced input against the oracle."""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from respackdev_gb300 import synth
from tests.helpers import EM_TEST, normwise_err, read_eps_record, run_params


@pytest.fixture(scope="module")
def sym_pair(tmp_path_factory):
    made = {}

    def get(name):
        if name not in made:
            base = tmp_path_factory.mktemp(name)
            red, full = str(base / "reduced"), str(base / "full")
            os.makedirs(red)
            os.makedirs(full)
            d = synth.make_case(red, synth.CASES[name])
            f = synth.make_full_mesh_case(full, synth.CASES[name])
            made[name] = (red, full, d, f)
        return made[name]

    return get


def test_irreducible_mesh_and_unfold():
    """8 irreducible points of the fcc 4x4x4 mesh under O_h and time reversal;
    the unfold covers the mesh once; the unfolded bands stay orthonormal."""
    for name in ("tiny_sym", "tiny_glide"):
        d = synth.generate(synth.CASES[name])
        assert d.kpts.shape[0] == 8 and len(d.rg) == 48
        f = synth.full_mesh_equivalent(d)
        assert f.kpts.shape[0] == 64
        mesh = synth.gamma_mesh((4, 4, 4))
        for k in mesh:
            assert sum(np.all(np.abs(f.kpts - k) < 1e-6, axis=1)) == 1
        for c in f.coeffs:
            np.testing.assert_allclose(c.conj().T @ c, np.eye(c.shape[1]), atol=1e-12)
    assert synth.generate(synth.CASES["tiny_glide"]).nnp == 4


@pytest.mark.parametrize("name", ["tiny_sym", "tiny_glide"])
def test_oracle_symmetry_reduced_equals_full_mesh(name, sym_pair):
    red, full, d, f = sym_pair(name)
    kw = run_params(name)
    nq = d.kpts.shape[0]
    # the irreducible q points inside the full list
    qfull = []
    for k in d.kpts:
        hit = np.where(np.all(np.abs(f.kpts - k) < 1e-6, axis=1))[0]
        assert hit.size == 1
        qfull.append(int(hit[0]) + 1)
    orc.calc_chiqw(red, orc.make_params(em=EM_TEST, dump_chi=1, nthreads=8, **kw))
    orc.calc_chiqw(full, orc.make_params(em=EM_TEST, dump_chi=1, nthreads=8, calc_num_k=qfull, **kw))
    worst = 0.0
    for iq in range(1, nq + 1):
        a = orc.read_chi_dump(os.path.join(red, "dir-eps", "q%03d" % iq, "dat.chi0"))
        b = orc.read_chi_dump(os.path.join(full, "dir-eps", "q%03d" % qfull[iq - 1], "dat.chi0"))
        assert a.shape == b.shape
        assert np.abs(b).max() > 0
        worst = max(worst, normwise_err(a, b))
        ng, nen = a.shape[0], a.shape[2]
        for ix in range(a.shape[3]):
            ea = read_eps_record(os.path.join(red, "dir-eps", "q%03d" % iq, "dat.epsqw.%03d" % (600 + ix)), ng, nen)
            eb = read_eps_record(os.path.join(full, "dir-eps", "q%03d" % qfull[iq - 1], "dat.epsqw.%03d" % (600 + ix)),
                                 ng, nen)
            worst = max(worst, normwise_err(ea, eb))
    print(f"{name}: symmetry-reduced vs full mesh {worst:.3e}")
    assert worst < 1e-11
