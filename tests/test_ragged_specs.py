"""The ragged workload's seeded cells stay inside the ranges they are drawn
from (fcc/bcc/sc, a 8-14 bohr, k 3^3-6^3, 60-300 bands, 40-400 G, 4-16
frequencies), and every cell can hold its bands and its dielectric sphere."""
import numpy as np

import bench
from respackdev_gb300 import synth

VOL = {"fcc": 0.25, "bcc": 0.5, "sc": 1.0}


def _count(vol, ecut):
    return vol * ecut ** 1.5 / (6 * np.pi ** 2)


def test_ragged_cells_in_range_and_seeded():
    cells = bench.ragged_specs()
    assert len(cells) == bench.RAGGED_CELLS == 12
    assert {c[0].lattice for c in cells} == {"fcc", "bcc", "sc"}
    for spec, ecut_eps, em in cells:
        assert 8.0 <= spec.a <= 14.0
        assert spec.nk[0] == spec.nk[1] == spec.nk[2] and 3 <= spec.nk[0] <= 6
        assert 60 <= spec.nbands <= 300 and spec.nocc == 8
        vol = VOL[spec.lattice] * spec.a ** 3
        assert _count(vol, spec.ecut_psi) >= 1.3 * spec.nbands   # enough plane waves for the bands
        assert 40 <= round(_count(vol, ecut_eps)) <= 400           # target dielectric sphere
        assert spec.ecut_psi >= 1.5 * ecut_eps - 1e-9
        assert 4 <= len(em) <= 16
        assert np.all(np.abs(em.real) <= 30.0 / bench.AU + 1e-12) and np.all(em.imag >= 0)
    # seeded: the same draw twice, another seed another draw
    again = bench.ragged_specs()
    assert all(a[0] == b[0] and a[1] == b[1] and np.array_equal(a[2], b[2]) for a, b in zip(cells, again))
    other = bench.ragged_specs(seed=8)
    assert any(a[0] != b[0] for a, b in zip(cells, other))


def test_smallest_ragged_cell_generates():
    """The smallest cell of the draw is written as a dir-wfn whose per-k plane
    wave lists hold more coefficients than bands (orthonormal bands exist)."""
    cells = bench.ragged_specs()
    spec = min((c[0] for c in cells), key=lambda s: s.nk[0] ** 3 * s.nbands)
    d = synth.generate(spec)
    assert d.kpts.shape[0] == spec.nk[0] ** 3
    for c in d.coeffs:
        assert c.shape[0] >= spec.nbands
        g = c.conj().T @ c
        assert np.allclose(g, np.eye(spec.nbands), atol=1e-10)
