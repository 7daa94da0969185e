"""The band-tail network on larger cells than test_gpu_tail.py: 16 seeded fcc
cells on a 4x4x4 mesh with NFULL bands, chi0 truncated at NTRUNC bands, six
q points each; the network trains on 12 cells and is measured on the other 4
against the full band sum, for chi0 and for eps^-1 (the corrected chi0 through
rp_epsinv_chi_q).  With NFULL = 800 and 24 cells (18 / 6) the same code is the
800-band measurement of the design notes."""
from __future__ import annotations

import os
import shutil
import tempfile

import numpy as np
import pytest

from respackdev_gb300 import chiqw as rp
from respackdev_gb300 import synth
from respackdev_gb300 import tail

pytestmark = pytest.mark.gpu

NTRUNC, NFULL, NSHELL, ECUT = 100, 400, 8, 6.0
NCELL, NTRAIN = 16, 12
QS = [2, 3, 5, 9, 17, 22]
EM = np.array([0.0, 2.0, 6.0, 0.5j, 3.0j]) / synth.AU_EV


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_tail_correction_on_larger_cells():
    kw = dict(green_func_delt=0.2721, ecut_for_eps=ECUT, precision=rp.PREC_FP16X3)
    # plane waves: at 30 Ry every k of the mesh has at least 725 (> NFULL)
    ecut_psi = 30.0 if NFULL <= 700 else 40.0
    cells = []
    for c in range(NCELL):
        spec = synth.SynthSpec(lattice="fcc", a=10.26, nk=(4, 4, 4), nbands=NFULL, nocc=8, ecut_psi=ecut_psi,
                               seed=500 + c, wan_lo=9, wan_hi=11)
        root = tempfile.mkdtemp(prefix="rp_tail_scale_")
        try:
            d = synth.make_case(root, spec)
            stats = tail.band_stats(d.energies, d.efermi, NTRUNC)
            out = []
            with rp.Context(root, rp.default_params(n_calc_band=NTRUNC, **kw), EM) as ct, \
                    rp.Context(root, rp.default_params(n_calc_band=NFULL, **kw), EM) as cf:
                for iq in QS:
                    chi_t = ct.chi0_q(iq)
                    eps_t = ct.epsinv_q()
                    chi_f = cf.chi0_q(iq)
                    eps_f = cf.epsinv_q()
                    ct.write_q()
                    q = np.loadtxt(os.path.join(root, "dir-eps", "q%03d" % iq, "dat.sq"))
                    LG = synth.sphere(d.bvec, ECUT, q)
                    ql = np.linalg.norm((LG + q[None, :]) @ d.bvec, axis=1)
                    assert len(ql) == chi_t.shape[0]
                    out.append((iq, chi_t[..., 0], chi_f[..., 0], ql, eps_t, eps_f))
            cells.append((root, stats, out))
        finally:
            if c < NTRAIN:  # the training cells' inputs are not needed again
                shutil.rmtree(root, ignore_errors=True)
    X, T = [], []
    for _, stats, qs in cells[:NTRAIN]:
        for _, chi_t, chi_f, ql, _, _ in qs:
            X.append(tail.features(chi_t, ql, EM, stats, NSHELL)[0])
            T.append(tail.targets(chi_t, chi_f, ql, NSHELL))
    X, T = np.concatenate(X), np.concatenate(T)
    et, ec, eet, eec = [], [], [], []
    try:
        with tail.TailMLP(seed=3) as m:
            m.train(X, T, steps=4000, batch=256, lr=1e-3)
            for root, stats, qs in cells[NTRAIN:]:
                with rp.Context(root, rp.default_params(n_calc_band=NTRUNC, **kw), EM) as ct:
                    for iq, chi_t, chi_f, ql, eps_t, eps_f in qs:
                        pred = m.forward(tail.features(chi_t, ql, EM, stats, NSHELL)[0])
                        chi_c = tail.apply(chi_t, pred, ql, NSHELL)
                        et.append(_rel(chi_t, chi_f))
                        ec.append(_rel(chi_c, chi_f))
                        ct.chi0_q(iq)
                        eps_c = ct.epsinv_chi_q(chi_c[..., None])
                        eet.append(_rel(eps_t, eps_f))
                        eec.append(_rel(eps_c, eps_f))
    finally:
        for root, _, _ in cells[NTRAIN:]:
            shutil.rmtree(root, ignore_errors=True)
    cg, eg = np.mean(et) / np.mean(ec), np.mean(eet) / np.mean(eec)
    print(f"{NCELL} cells, {NFULL} bands truncated at {NTRUNC}, {len(X)} samples: held-out chi error "
          f"{np.mean(et):.3e} -> {np.mean(ec):.3e} ({cg:.1f}x), eps^-1 {np.mean(eet):.3e} -> {np.mean(eec):.3e} "
          f"({eg:.1f}x)")
    assert cg > 1.3 and eg > 1.5
