"""Host side of the band-tail correction (respackdev_gb300/tail.py): shells,
features, targets and the correction, on seeded arrays (no GPU)."""
import numpy as np

from respackdev_gb300 import tail


def _chi(rng, ng, nen):
    a = rng.standard_normal((ng, ng, nen)) + 1j * rng.standard_normal((ng, ng, nen))
    return a + a.transpose(1, 0, 2).conj()


def test_shells_are_equal_count_quantiles_and_skip_the_head():
    rng = np.random.default_rng(1)
    ql = np.concatenate([[0.0], rng.uniform(0.1, 3.0, 40)])
    sh = tail.shells(ql, 4)
    assert sh[0] == -1 and set(sh[1:]) == {0, 1, 2, 3}
    counts = np.bincount(sh[1:], minlength=4)
    assert counts.max() - counts.min() <= 1
    # shells follow |q+G|: every G of shell s is shorter than every G of shell s+1
    for s in range(3):
        assert ql[sh == s].max() <= ql[sh == s + 1].min()


def test_targets_applied_exactly_give_the_full_shell_means():
    """Feeding the targets back as the prediction moves each shell's mean of
    v chi on the diagonal to the full sum's; off-diagonal elements and the
    head are left alone."""
    rng = np.random.default_rng(2)
    ng, nen, nshell = 30, 3, 4
    ql = np.concatenate([[0.0], rng.uniform(0.2, 2.5, ng - 1)])
    chi_t, chi_f = _chi(rng, ng, nen), _chi(rng, ng, nen)
    T = tail.targets(chi_t, chi_f, ql, nshell)
    assert T.shape == (nen * nshell, tail.NOUT)
    out = tail.apply(chi_t, T, ql, nshell)
    sh = tail.shells(ql, nshell)
    v = np.where(ql > 0, 4 * np.pi / np.where(ql > 0, ql, 1) ** 2, 0)
    d_out = np.einsum("ggw->gw", out) * v[:, None]
    d_full = np.einsum("ggw->gw", chi_f) * v[:, None]
    for s in range(nshell):
        m = sh == s
        np.testing.assert_allclose(d_out[m].mean(0), d_full[m].mean(0), rtol=1e-12, atol=1e-12)
    off = ~np.eye(ng, dtype=bool)
    assert np.array_equal(out[off], chi_t[off])
    assert np.array_equal(out[0, 0], chi_t[0, 0])


def test_features_layout():
    rng = np.random.default_rng(3)
    ng, nen, nshell = 25, 4, 4
    ql = rng.uniform(0.2, 2.5, ng)
    em = np.array([0.0, 0.1, 0.05j, 0.2j])
    stats = tail.band_stats(rng.uniform(-0.5, 1.0, (20, 8)), 0.0, 12)
    X, sh = tail.features(_chi(rng, ng, nen), ql, em, stats, nshell)
    assert X.shape == (nen * nshell, tail.NFEAT) and np.all(np.isfinite(X))
    Xr = X.reshape(nen, nshell, tail.NFEAT)
    np.testing.assert_allclose(Xr[:, :, 3], np.repeat(em.real[:, None], nshell, 1))
    np.testing.assert_allclose(Xr[:, :, 4], np.repeat(em.imag[:, None], nshell, 1))
    np.testing.assert_allclose(Xr[0, :, 8], (np.arange(nshell) + 0.5) / nshell)
    assert np.all(np.diff(Xr[0, :, 0]) > 0)   # shell mean |q+G| grows with the shell
    e_lo, e_mean, ratio = stats
    assert e_lo <= e_mean and abs(ratio - 8 / 12) < 1e-15
    assert tail.band_stats(np.zeros((5, 2)), 0.0, 5) == (0.0, 0.0, 0.0)
