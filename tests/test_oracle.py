"""The CPU oracle checked on its own: numpy, quadrature and a plane-wave brute force.

The reference ships no tests or golden outputs for this path (parity is
unpinned by the reference), so the oracle is pinned here against independent
computations of the same quantities."""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from respackdev_gb300 import synth
from tests import brute

AU = 27.21151


def test_fft_matches_numpy():
    rng = np.random.default_rng(0)
    for shape in [(8, 8, 8), (10, 6, 5), (12, 9, 15), (7, 4, 3)]:
        a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        np.testing.assert_allclose(orc.fft3(a, True), np.fft.fftn(a) / a.size, atol=1e-14)
        np.testing.assert_allclose(orc.fft3(a, False), np.fft.ifftn(a) * a.size, atol=1e-12)


def test_zinv_matches_numpy():
    rng = np.random.default_rng(1)
    for n in (1, 5, 31):
        m = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + 3 * np.eye(n)
        np.testing.assert_allclose(orc.zinv(m), np.linalg.inv(m), atol=1e-12)


def test_algn235_and_gen_grid():
    L = orc.lib()
    assert [L.orc_algn235(n) for n in (1, 7, 11, 13, 14, 17, 49)] == [1, 8, 12, 15, 15, 18, 50]
    em = orc.gen_grid(70, 1.5)
    assert em[0] == 0 and np.all(np.diff(em.real) > 0)
    # first step is 0.05 eV (gen_grid.f90: dlt = 0.05/au)
    assert abs(em[1].real - 0.05 / AU) < 1e-6
    # the log part ends at E (the last point of the 90% part is E)
    assert abs(em[62].real - 1.5) < 1e-6


def _stroud(n=48):
    """Conical-product Gauss rule on the unit simplex: points (x,y,z), weights."""
    x, w = np.polynomial.legendre.leggauss(n)
    u = 0.5 * (x + 1); wu = 0.5 * w
    U, V, W = np.meshgrid(u, u, u, indexing="ij")
    WU, WV, WW = np.meshgrid(wu, wu, wu, indexing="ij")
    X = U
    Y = V * (1 - U)
    Z = W * (1 - U) * (1 - V)
    J = (1 - U) ** 2 * (1 - V)
    return X.ravel(), Y.ravel(), Z.ravel(), (WU * WV * WW * J).ravel()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_tetra_uncut_matches_quadrature(seed):
    """One tetrahedron with every vertex occupied-to-empty: vertex weights are
    dsgn * int_simplex lambda_v / (dsgn*g(lambda) + w), g = -(e2-e1) + i delt."""
    rng = np.random.default_rng(seed)
    ee1 = -0.3 - 0.05 * rng.random(4)
    ee2 = 0.4 + 0.2 * rng.random(4)
    delt = 0.01
    em = np.array([0.0, 0.3, 0.9, 1.7 + 0.2j])
    X, Y, Z, W = _stroud()
    lam = np.stack([1 - X - Y - Z, X, Y, Z])
    for dsgn in (1.0, -1.0):
        out = np.zeros((4, em.size), dtype=np.complex128)
        rc = orc.lib().orc_tt_one(0.001, 0.001, ee1.ctypes.data, ee2.ctypes.data, 0.0, 0.0, delt, dsgn, em.size,
                                  em.ctypes.data, out.ctypes.data)
        assert rc == 0
        g0 = -(ee2 - ee1) + 1j * delt
        gl = np.einsum("a,ap->p", g0, lam)
        # the closed forms cancel like 1/(g_a-g_b)^3 when two vertices come close
        # (here as close as 0.2% apart, just outside the 0.1% degeneracy
        # threshold); the vertex sum does not suffer from it
        for ie, w in enumerate(em):
            f = 1.0 / (dsgn * gl + w)
            ref = dsgn * np.einsum("ap,p,p->a", lam, f, W)
            np.testing.assert_allclose(out[:, ie], ref, rtol=2e-6, atol=1e-9)
            np.testing.assert_allclose(out[:, ie].sum(), ref.sum(), rtol=1e-9)


def test_tetra_degenerate_cases_continuous():
    """Near-degenerate vertex energies take the closed forms of calc()'s special
    cases; they must agree with the quadrature too."""
    em = np.array([0.2, 0.35], dtype=np.complex128)  # off resonance: Gauss quadrature cannot resolve a near-pole
    X, Y, Z, W = _stroud()
    lam = np.stack([1 - X - Y - Z, X, Y, Z])
    for ee2 in ([0.5, 0.5, 0.7, 0.9], [0.5, 0.5, 0.5, 0.9], [0.5, 0.5, 0.8, 0.8], [0.6, 0.6, 0.6, 0.6]):
        ee1 = np.full(4, -0.2)
        ee2 = np.array(ee2, dtype=float)
        out = np.zeros((4, em.size), dtype=np.complex128)
        assert orc.lib().orc_tt_one(0.001, 0.001, ee1.ctypes.data, ee2.ctypes.data, 0.0, 0.0, 0.01, 1.0, em.size,
                                    em.ctypes.data, out.ctypes.data) == 0
        g0 = -(ee2 - ee1) + 0.01j
        gl = np.einsum("a,ap->p", g0, lam)
        for ie, w in enumerate(em):
            ref = np.einsum("ap,p,p->a", lam, 1.0 / (gl + w), W)
            # the degenerate forms average the equal vertices' energies
            np.testing.assert_allclose(out[:, ie].sum(), ref.sum(), rtol=1e-9)


def test_tetra_fermi_cut_matches_monte_carlo():
    """Tetrahedra cut by the Fermi level: only the part with e2 > E_F and e1 < E_F counts."""
    rng = np.random.default_rng(5)
    ee1 = np.array([-0.2, 0.1, -0.05, 0.15])
    ee2 = np.array([0.3, -0.1, 0.2, 0.05])
    em = np.array([0.05, 0.7], dtype=np.complex128)
    out = np.zeros((4, em.size), dtype=np.complex128)
    assert orc.lib().orc_tt_one(0.001, 0.001, ee1.ctypes.data, ee2.ctypes.data, 0.0, 0.0, 0.02, 1.0, em.size,
                                em.ctypes.data, out.ctypes.data) == 0
    n = 4_000_000
    p = rng.dirichlet(np.ones(4), size=n).T  # uniform on the simplex
    e1 = ee1 @ p; e2 = ee2 @ p
    occ = (e2 > 0.0) & (e1 < 0.0)
    g = -(e2 - e1) + 0.02j
    vol = 1.0 / 6.0
    for ie, w in enumerate(em):
        ref = vol * np.mean(p * (occ / (g + w))[None, :], axis=1)
        np.testing.assert_allclose(out[:, ie], ref, rtol=0, atol=3e-3 * np.abs(ref).max())


def test_mkidx_tiles_the_cell():
    d = synth.generate(synth.CASES["tiny"])
    imt = orc.mkidx((3, 3, 3), d.bvec).reshape(-1, 4)
    assert imt.shape == (6 * 27, 4) and imt.min() == 1 and imt.max() == 27
    assert all(len(set(t)) == 4 for t in imt)
    # every mesh point is a vertex of 24 tetrahedra
    assert np.all(np.bincount(imt.ravel())[1:] == 24)


def _tetra_fn(nk, imt, f, delt, em):
    def t(e1, e2, dsgn):
        return orc.ttrhdrn_chi0(0.001, 0.001, nk, imt, e1, e2, f, f, delt, dsgn, em)
    return t


@pytest.mark.parametrize("qidx", [2, 5])
def test_chi0_matches_planewave_bruteforce(case_dir, fresh_copy, qidx):
    spec = synth.CASES["tiny"]
    root = fresh_copy(case_dir("tiny"))
    d = synth.generate(spec)
    em = np.array([0.0, 0.15, 0.3 + 0.05j])
    box = (18, 18, 18)  # alias-free for this basis
    p = orc.make_params(green_func_delt=0.2721, ecut_for_eps=3.0, em=em, dump_chi=1, nthreads=2,
                        fft_box=box, calc_num_k=[qidx])
    orc.calc_chiqw(root, p)
    chi = orc.read_chi_dump(os.path.join(root, "dir-eps", "q%03d" % qidx, "dat.chi0"))[..., 0]
    q = d.kpts[qidx - 1]
    imt = orc.mkidx(spec.nk, d.bvec)
    ref, LG = brute.chi0_brute(d, q, 3.0, em, 0.2721, 0.001, 0.001, spec.nbands,
                               (list(range(spec.nocc)), list(range(spec.nocc, spec.nbands))),
                               imt1=imt, nk=spec.nk, tetra=_tetra_fn(spec.nk, imt, d.efermi, 0.2721 / AU, em))
    assert chi.shape == ref.shape
    err = np.abs(chi - ref).max() / np.abs(ref).max()
    assert err < 1e-6, err


@pytest.mark.parametrize("lattice,a,nk,ecut_psi", [("bcc", 8.5, (2, 2, 2), 7.0), ("sc", 7.0, (2, 2, 2), 7.0)])
def test_chi0_bruteforce_other_lattices(tmp_path, lattice, a, nk, ecut_psi):
    """The same plane-wave check on a body-centred and a simple cubic cell,
    with an alias-free box from the cell's own plane-wave extent."""
    spec = synth.SynthSpec(lattice=lattice, a=a, nk=nk, nbands=10, nocc=4, ecut_psi=ecut_psi, seed=41,
                           wan_lo=5, wan_hi=7)
    root = str(tmp_path)
    d = synth.make_case(root, spec)
    ext = np.max([np.abs(g).max(0) for g in d.kg], axis=0)
    box = tuple(int(4 * r + 2) for r in ext)
    em = np.array([0.0, 0.2, 0.1 + 0.05j])
    qidx = 2
    p = orc.make_params(green_func_delt=0.2721, ecut_for_eps=2.5, em=em, dump_chi=1, nthreads=2, fft_box=box,
                        calc_num_k=[qidx])
    orc.calc_chiqw(root, p)
    chi = orc.read_chi_dump(os.path.join(root, "dir-eps", "q%03d" % qidx, "dat.chi0"))[..., 0]
    imt = orc.mkidx(spec.nk, d.bvec)
    ref, LG = brute.chi0_brute(d, d.kpts[qidx - 1], 2.5, em, 0.2721, 0.001, 0.001, spec.nbands,
                               (list(range(spec.nocc)), list(range(spec.nocc, spec.nbands))),
                               imt1=imt, nk=spec.nk, tetra=_tetra_fn(spec.nk, imt, d.efermi, 0.2721 / AU, em))
    assert chi.shape == ref.shape and chi.shape[0] > 5
    err = np.abs(chi - ref).max() / np.abs(ref).max()
    assert err < 1e-6, err


def test_eps_files_invert_chi(case_dir, fresh_copy):
    """dat.epsqw.600 holds (1 - v chi_total)^-1 of the dumped chi (q != 0) and
    the diagonal text file matches it."""
    spec = synth.CASES["tiny"]
    root = fresh_copy(case_dir("tiny"))
    d = synth.generate(spec)
    em = np.array([0.0, 0.2])
    p = orc.make_params(green_func_delt=0.2721, ecut_for_eps=3.0, em=em, dump_chi=1, nthreads=2, calc_num_k=[3])
    orc.calc_chiqw(root, p)
    qd = os.path.join(root, "dir-eps", "q003")
    chi = orc.read_chi_dump(os.path.join(qd, "dat.chi0"))[..., 0]
    rec = synth.read_unformatted_records(os.path.join(qd, "dat.epsqw.600"))
    assert len(rec) == 1
    ng = chi.shape[0]
    epsinv = np.frombuffer(rec[0], dtype=np.complex128).reshape((2, ng, ng)).transpose(2, 1, 0)
    q = np.loadtxt(os.path.join(qd, "dat.sq"))
    LG = synth.sphere(d.bvec, 3.0, q)
    ql = np.linalg.norm((LG + q[None, :]) @ d.bvec, axis=1)
    for ie in range(2):
        eps = np.eye(ng) - 2.0 * chi[:, :, ie] * 4 * np.pi / np.outer(ql, ql)
        np.testing.assert_allclose(epsinv[:, :, ie] @ eps, np.eye(ng), atol=1e-10)
        diag = np.loadtxt(os.path.join(qd, "dat.epsqw.%06d" % (600001 + ie)))
        np.testing.assert_allclose(diag[:, 0], ql, atol=1e-9)
        np.testing.assert_allclose(diag[:, 1] + 1j * diag[:, 2], np.diag(epsinv[:, :, ie]), atol=2e-10)


def test_resume_skips_finished_q(case_dir, fresh_copy):
    """flg_calc_type=0 skips every dir-eps/qNNN that already holds dat.log.400
    (chiqw.F:593-608): a second run computes nothing."""
    root = fresh_copy(case_dir("tiny"))
    em = np.array([0.0, 0.2])
    p = orc.make_params(green_func_delt=0.2721, ecut_for_eps=3.0, em=em, nthreads=2)
    r1 = orc.calc_chiqw(root, p)
    assert r1.nq_done == 8
    os.remove(os.path.join(root, "dir-eps", "q004", "dat.log.400"))
    r2 = orc.calc_chiqw(root, p)
    assert r2.nq_done == 1
