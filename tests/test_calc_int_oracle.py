"""The calc_int restatement (oracle) on its own: properties the V, W, X, J of
calc_w3d / calc_j3d must have whatever the implementation, and the files it
writes.  No GPU."""
from __future__ import annotations

import os

import numpy as np
import pytest

from oracle import oracle as orc
from respackdev_gb300 import calc_int as ci
from respackdev_gb300 import synth
from tests.helpers import AU, read_int_matrix


def _run(root, **kw):
    kw.setdefault("nthreads", 4)
    return orc.calc_int(root, orc.make_int_params(**kw))


def _minus_R(a):
    """a[i, j, R] -> a[i, j, -R] on the symmetric -Na..Na box."""
    return a[:, :, ::-1, ::-1, ::-1]


@pytest.mark.parametrize("case", ["tiny_wan", "odd_wan"])
def test_hermitian_and_consistent(case, int_case, int_copy):
    root = int_copy(int_case(case))
    dims, o = _run(root, ix_min=-1, ix_max=1, write_files=0)
    V, W, X, J = o["V"], o["W"], o["X"], o["J"]
    na = tuple(dims.na)
    # V_ij(R) = conj(V_ji(-R)) (the bare interaction is Hermitian)
    np.testing.assert_allclose(V, np.conj(_minus_R(V).transpose(1, 0, 2, 3, 4)), atol=1e-12 * np.abs(V).max())
    # (W is not: the broadening i delta of chiqw makes even the static eps^-1 complex)
    # X_ii(R=0) = V_ii(R=0) and J_ii(R=0) = W_ii(R=0): rho_ii at R = 0 is the rho_i of calc_w3d
    c = tuple(na)
    np.testing.assert_allclose(np.diag(X[:, :, c[0], c[1], c[2]]), np.diag(V[:, :, c[0], c[1], c[2]]), rtol=1e-12)
    for e in range(W.shape[-1]):
        np.testing.assert_allclose(np.diag(J[:, :, c[0], c[1], c[2], e]), np.diag(W[:, :, c[0], c[1], c[2], e]),
                                   rtol=1e-12)
    # X and J are zero outside the requested range, non-zero inside
    assert np.all(X[:, :, :, na[1] + 1:, :] == 0) if na[1] > 0 else True
    assert np.abs(X[:, :, :, c[1], c[2]]).min() >= 0
    # on-site bare repulsion of the Gaussian orbitals is positive and larger than the screened one
    d = np.real(np.diag(V[:, :, c[0], c[1], c[2]]))
    assert np.all(d > 0)
    assert np.all(np.real(np.diag(W[:, :, c[0], c[1], c[2], 0])) < d)


def test_identity_screening_gives_bare(int_case, int_copy):
    """With eps^-1 = 1 in every dat.epsqw file, W equals V and J equals X."""
    root = int_copy(int_case("tiny_wan"))
    d = synth.generate(synth.CASES["tiny_wan"])
    eps = os.path.join(root, "dir-eps")
    for q in sorted(os.listdir(eps)):
        qd = os.path.join(eps, q)
        if not os.path.isdir(qd):
            continue
        for name in os.listdir(qd):
            if not name.startswith("dat.epsqw.") or len(name) != len("dat.epsqw.600"):
                continue
            rec = synth.read_unformatted_records(os.path.join(qd, name))[0]
            n = len(rec) // 16
            ne = 3
            ng = int(round((n // ne) ** 0.5))
            a = np.zeros((ne, ng, ng), dtype=np.complex128)
            a[:, np.arange(ng), np.arange(ng)] = 1.0
            with open(os.path.join(qd, name), "wb") as f:
                synth.write_unformatted_record(f, a.tobytes())
    del d
    dims, o = _run(root, ix_min=-1, ix_max=1, write_files=0)
    for e in range(dims.ne):
        np.testing.assert_allclose(o["W"][..., e], o["V"], rtol=0, atol=1e-12 * np.abs(o["V"]).max())
        np.testing.assert_allclose(o["J"][..., e], o["X"], rtol=0, atol=1e-12 * np.abs(o["X"]).max())


def test_files_match_arrays(int_case, int_copy):
    root = int_copy(int_case("tiny_wan"))
    dims, o = _run(root, ix_min=0, ix_max=1, calc_ifreq=2)
    nwf, na = dims.nwf, tuple(dims.na)
    Vf = read_int_matrix(os.path.join(root, "dir-intW", "dat.Vmat"), nwf)
    Wf = read_int_matrix(os.path.join(root, "dir-intW", "dat.Wmat"), nwf)
    Xf = read_int_matrix(os.path.join(root, "dir-intJ", "dat.Xmat"), nwf)
    Jf = read_int_matrix(os.path.join(root, "dir-intJ", "dat.Jmat"), nwf)
    assert len(Vf) == (2 * na[0] + 1) * (2 * na[1] + 1) * (2 * na[2] + 1)
    assert sorted(Xf) == [(a, 0, 0) for a in (0, 1)]
    for R, M in Vf.items():
        idx = tuple(r + n for r, n in zip(R, na))
        np.testing.assert_allclose(M, o["V"][(slice(None), slice(None)) + idx] * AU, atol=2e-10)
        np.testing.assert_allclose(Wf[R], o["W"][(slice(None), slice(None)) + idx + (1,)] * AU, atol=2e-10)
    for R, M in Xf.items():
        idx = tuple(r + n for r, n in zip(R, na))
        np.testing.assert_allclose(M, o["X"][(slice(None), slice(None)) + idx] * AU, atol=2e-10)
        np.testing.assert_allclose(Jf[R], o["J"][(slice(None), slice(None)) + idx + (1,)] * AU, atol=2e-10)
    # UvsE / JvsE: the R = 0 element against frequency
    u = np.loadtxt(os.path.join(root, "dir-intW", "dat.UvsE.001-002"))
    c = tuple(na)
    np.testing.assert_allclose(u[:, 2] + 1j * u[:, 3], o["W"][0, 1, c[0], c[1], c[2], :] * AU, atol=1e-5)
    # mvmc: the on-site W of every site
    lines = open(os.path.join(root, "dir-mvmc", "zCoulombIntra.def")).read().splitlines()
    assert int(lines[1].split()[1]) == nwf * 8
    vals = np.array([float(x.split()[1]) for x in lines[5:]])
    np.testing.assert_allclose(vals[:nwf], np.real(np.diag(o["W"][:, :, c[0], c[1], c[2], 1])) * AU, atol=1e-9)
    for name in ("zCoulombInter.def", "zHund.def", "zExchange.def", "zPairHop.def"):
        assert os.path.getsize(os.path.join(root, "dir-mvmc", name)) > 0


def test_calc_int_namelist_parser():
    p = ci.parse_namelist("&param_calc_int\n CALC_IFREQ=3, IX_INTJ_MIN=-1, ix_intJ_max=2\n"
                          " wcut_mvmc=1.5 /\n&param_gpu\n fft_box=8 8 8, read_eps_f32=0 /\n")
    assert (p.calc_ifreq, p.ix_intj_min, p.ix_intj_max, p.iy_intj_min) == (3, -1, 2, 0)
    assert p.read_eps_f32 == 0 and ci.default_params().read_eps_f32 == 1
    assert p.wcut_mvmc == 1.5 and p.jcut_mvmc == 0.3 and list(p.fft_box) == [8, 8, 8]
    with pytest.raises(ValueError):
        ci.parse_namelist("&param_calc_int\n bogus=1 /\n")
    with pytest.raises(ValueError):
        ci.parse_namelist("&param_chiqw\n Ecut_for_eps=3 /\n")
