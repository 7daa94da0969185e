"""The band-tail MLP on the GPU (rp_mlp_* of the C ABI): forward pass, loss
and gradients against the numpy restatement (oracle/mlp_ref.py), training,
and the held-out gain of the tail-corrected chi0 over the truncated band sum,
with the full band sum as the measure of the error."""
from __future__ import annotations

import dataclasses
import os
import tempfile

import numpy as np
import pytest

from oracle import mlp_ref
from respackdev_gb300 import chiqw as rp
from respackdev_gb300 import synth
from respackdev_gb300 import tail

pytestmark = pytest.mark.gpu


def _rand_params(m: tail.TailMLP, rng, scale=0.3):
    return (rng.standard_normal(m.nparams) * scale).astype(np.float32)


def test_forward_and_gradients_match_oracle():
    rng = np.random.default_rng(11)
    nin, nhid, nout, n = 9, 128, 2, 300
    with tail.TailMLP(nin, nout, nhid, seed=5) as m:
        p = _rand_params(m, rng, 0.15)
        m.set_params(p)
        assert np.array_equal(m.params(), p)
        x = rng.standard_normal((n, nin)).astype(np.float32)
        t = rng.standard_normal((n, nout)).astype(np.float32)
        y = m.forward(x)
        yr, _ = mlp_ref.forward(p, x, nin, nhid, nout)
        assert np.abs(y - yr).max() <= 1e-4 * np.abs(yr).max()
        loss, g = m.gradients(x, t)
        lr_, gr = mlp_ref.loss_and_grad(p, x, t, nin, nhid, nout)
        assert abs(loss - lr_) <= 1e-5 * lr_
        # every parameter block, relative to its own largest gradient
        sizes = [nhid * nin, nhid, nhid * nhid, nhid, nout * nhid, nout]
        o = 0
        for sz in sizes:
            blk, ref = g[o:o + sz], gr[o:o + sz]
            assert np.abs(blk - ref).max() <= 1e-4 * np.abs(ref).max() + 1e-12, (o, sz)
            o += sz


def test_training_fits_a_smooth_map():
    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, size=(2048, 4)).astype(np.float32)
    t = np.stack([np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2], np.cos(x[:, 3]) - 0.5 * x[:, 0] ** 2], 1).astype(np.float32)
    with tail.TailMLP(4, 2, 128, seed=1) as m:
        l0, _ = m.gradients(x, t)
        losses = m.train(x, t, steps=1500, batch=256, lr=2e-3)
        l1, _ = m.gradients(x, t)
    assert np.all(np.isfinite(losses))
    assert l1 < l0 / 20, (l0, l1)


# --- band-tail correction on synthetic cells ---------------------------------

EM = np.array([0.0, 2.0, 6.0, 0.5j, 3.0j]) / synth.AU_EV
NTRUNC, NFULL, NSHELL = 12, 36, 8
QS = list(range(2, 9))        # the q != 0 points of the 2x2x2 mesh


def _cell(seed: int):
    spec = dataclasses.replace(synth.CASES["tiny"], nbands=NFULL, seed=seed)
    root = tempfile.mkdtemp(prefix="rp_tail_")
    d = synth.make_case(root, spec)
    stats = tail.band_stats(d.energies, d.efermi, NTRUNC)
    kw = dict(green_func_delt=0.2721, ecut_for_eps=3.0, precision=rp.PREC_FP64)
    out = []
    with rp.Context(root, rp.default_params(n_calc_band=NTRUNC, **kw), EM) as ct, \
            rp.Context(root, rp.default_params(n_calc_band=NFULL, **kw), EM) as cf:
        for iq in QS:
            chi_t = ct.chi0_q(iq)[..., 0]
            chi_f = cf.chi0_q(iq)[..., 0]
            # |q+G| in the library's G order, from the q it writes to dat.sq
            ct.epsinv_q(fetch=False)
            ct.write_q()
            q = np.loadtxt(os.path.join(root, "dir-eps", "q%03d" % iq, "dat.sq"))
            LG = synth.sphere(d.bvec, 3.0, q)
            ql = np.linalg.norm((LG + q[None, :]) @ d.bvec, axis=1)
            assert chi_t.shape[0] == len(LG)
            out.append((chi_t, chi_f, ql))
    return stats, out


@pytest.fixture(scope="module")
def cells():
    return [_cell(100 + s) for s in range(8)]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_tail_correction_beats_truncation(cells):
    train, held = cells[:6], cells[6:]
    X, T = [], []
    for stats, qs in train:
        for chi_t, chi_f, ql in qs:
            X.append(tail.features(chi_t, ql, EM, stats, NSHELL)[0])
            T.append(tail.targets(chi_t, chi_f, ql, NSHELL))
    X, T = np.concatenate(X), np.concatenate(T)
    with tail.TailMLP(seed=3) as m:
        m.train(X, T, steps=3000, batch=128, lr=1e-3)
        e_trunc, e_corr = [], []
        for stats, qs in held:
            for chi_t, chi_f, ql in qs:
                pred = m.forward(tail.features(chi_t, ql, EM, stats, NSHELL)[0])
                chi_c = tail.apply(chi_t, pred, ql, NSHELL)
                e_trunc.append(_rel(chi_t, chi_f))
                e_corr.append(_rel(chi_c, chi_f))
    et, ec = float(np.mean(e_trunc)), float(np.mean(e_corr))
    print(f"held-out chi error: truncated {et:.3e}, tail-corrected {ec:.3e} ({et / ec:.1f}x smaller)")
    assert ec < 0.5 * et


def test_tail_correction_in_the_product_path(cells, tmp_path):
    """The trained network saved as a tail_model file and attached to a
    context truncated at N_CALC_BAND: rp_chi0_q adds the correction on the
    device (the same chi0 as tail.apply on the host, to FP32 feature rounding),
    and eps^-1 from the corrected chi0 is closer to the full-band eps^-1 than
    eps^-1 of the truncated sum.  rp_epsinv_chi_q inverts a caller chi0: given
    the host-corrected chi0 it returns the same eps^-1."""
    train = cells[:6]
    X, T = [], []
    for stats, qs in train:
        for chi_t, chi_f, ql in qs:
            X.append(tail.features(chi_t, ql, EM, stats, NSHELL)[0])
            T.append(tail.targets(chi_t, chi_f, ql, NSHELL))
    X, T = np.concatenate(X), np.concatenate(T)
    model = str(tmp_path / "dat.tail")
    kw = dict(green_func_delt=0.2721, ecut_for_eps=3.0, precision=rp.PREC_FP64)
    e_trunc, e_corr = [], []
    with tail.TailMLP(seed=3) as m:
        m.train(X, T, steps=3000, batch=128, lr=1e-3)
        m.save(model, NSHELL)
        for seed in (106, 107):       # the held-out cells
            spec = dataclasses.replace(synth.CASES["tiny"], nbands=NFULL, seed=seed)
            root = tempfile.mkdtemp(prefix="rp_tailp_")
            d = synth.make_case(root, spec)
            stats = tail.band_stats(d.energies, d.efermi, NTRUNC)
            with rp.Context(root, rp.default_params(n_calc_band=NTRUNC, tail_model=model, **kw), EM) as cc, \
                    rp.Context(root, rp.default_params(n_calc_band=NTRUNC, **kw), EM) as ct, \
                    rp.Context(root, rp.default_params(n_calc_band=NFULL, **kw), EM) as cf:
                for iq in QS:
                    chi_c = cc.chi0_q(iq)
                    assert cc.tail_applied() and not ct.tail_applied()
                    eps_c = cc.epsinv_q()
                    chi_t = ct.chi0_q(iq)
                    eps_t = ct.epsinv_q()
                    cf.chi0_q(iq)
                    eps_f = cf.epsinv_q()
                    # |q+G| in the library's G order, from the q it writes to dat.sq
                    ct.write_q()
                    q = np.loadtxt(os.path.join(root, "dir-eps", "q%03d" % iq, "dat.sq"))
                    LG = synth.sphere(d.bvec, 3.0, q)
                    ql = np.linalg.norm((LG + q[None, :]) @ d.bvec, axis=1)
                    assert len(ql) == chi_t.shape[0]
                    pred = m.forward(tail.features(chi_t[..., 0], ql, EM, stats, NSHELL)[0])
                    chi_h = tail.apply(chi_t[..., 0], pred, ql, NSHELL)
                    assert _rel(chi_c[..., 0], chi_h) < 1e-5
                    # the host-corrected chi0 through rp_epsinv_chi_q gives the same eps^-1
                    eps_h = ct.epsinv_chi_q(chi_h)
                    assert _rel(eps_h, eps_c) < 1e-5
                    e_trunc.append(_rel(eps_t, eps_f))
                    e_corr.append(_rel(eps_c, eps_f))
    et, ec = float(np.mean(e_trunc)), float(np.mean(e_corr))
    print(f"held-out eps^-1 error: truncated {et:.3e}, tail-corrected (device) {ec:.3e} ({et / ec:.1f}x smaller)")
    assert ec < et
