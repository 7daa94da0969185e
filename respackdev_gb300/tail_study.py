"""Train and measure the band-tail network on seeded synthetic cells.

    python -m respackdev_gb300.tail_study --cells 64 --nk 6 --nfull 800 --ntrunc 100

Each cell (fcc, a = 10.26 bohr, a Gamma-centred nk^3 mesh, nfull bands of
seeded coefficients) is generated by `synth` in a spawn pool that runs ahead of
the GPU; chi0 is taken with the band sum truncated at ntrunc and in full
(FP16x3) at six q points, and the cell's inputs are deleted.  The network
trains on the first cells and is measured on the rest: the relative chi0 error
of the truncated and of the corrected sum against the full one, and the same
for eps^-1 (eps = 1 - 2 v chi, v = 4 pi / (|q+G| |q+G'|), q != 0, the
corrected one inverted on the host)."""
from __future__ import annotations

import argparse
import multiprocessing as mp
import os
import shutil
import tempfile
import time

import numpy as np

from . import synth

NSHELL, ECUT_EPS = 8, 6.0


def _gen(args):
    seed, nk, nfull = args
    # plane waves at every k of the mesh: at least 725 at 30 Ry, 1139 at 40 Ry
    ecut_psi = 30.0 if nfull <= 700 else 40.0
    spec = synth.SynthSpec(lattice="fcc", a=10.26, nk=(nk, nk, nk), nbands=nfull, nocc=8, ecut_psi=ecut_psi,
                           seed=seed, wan_lo=9, wan_hi=11)
    root = tempfile.mkdtemp(prefix="rp_tail_study_")
    d = synth.make_case(root, spec)
    return root, d.energies, d.efermi, d.bvec


def run(cells: int, nk: int, nfull: int, ntrunc: int, held: int, workers: int, steps: int) -> dict:
    from . import chiqw as rp
    from . import tail
    nq = nk ** 3
    qs = [q for q in (2, 5, 9, 17, 40, 80) if q <= nq]
    qs += [q for q in range(3, nq + 1) if q not in qs][:6 - len(qs)]
    t0 = time.time()
    pool = mp.get_context("spawn").Pool(workers)
    gen = pool.imap(_gen, [(700 + c, nk, nfull) for c in range(cells)])
    em = np.array([0.0, 2.0, 6.0, 0.5j, 3.0j]) / synth.AU_EV
    kw = dict(green_func_delt=0.2721, ecut_for_eps=ECUT_EPS, precision=rp.PREC_FP16X3)
    data = []
    for root, energies, efermi, bvec in gen:
        try:
            stats = tail.band_stats(energies, efermi, ntrunc)
            out = []
            with rp.Context(root, rp.default_params(n_calc_band=ntrunc, **kw), em) as ct, \
                    rp.Context(root, rp.default_params(n_calc_band=nfull, **kw), em) as cf:
                for iq in qs:
                    chi_t = ct.chi0_q(iq)
                    eps_t = ct.epsinv_q()
                    chi_f = cf.chi0_q(iq)
                    eps_f = cf.epsinv_q()
                    ct.write_q()
                    q = np.loadtxt(os.path.join(root, "dir-eps", "q%03d" % iq, "dat.sq"))
                    lg = synth.sphere(bvec, ECUT_EPS, q)
                    ql = np.linalg.norm((lg + q[None, :]) @ bvec, axis=1)
                    out.append((chi_t[..., 0], chi_f[..., 0], ql, eps_t[..., 0], eps_f[..., 0]))
            data.append((stats, out))
        finally:
            shutil.rmtree(root, ignore_errors=True)
    pool.close()
    pool.join()
    ntrain = cells - held
    X, T = [], []
    for stats, qv in data[:ntrain]:
        for chi_t, chi_f, ql, _, _ in qv:
            X.append(tail.features(chi_t, ql, em, stats, NSHELL)[0])
            T.append(tail.targets(chi_t, chi_f, ql, NSHELL))
    X, T = np.concatenate(X), np.concatenate(T)

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    et, ec, eet, eec = [], [], [], []
    with tail.TailMLP(seed=3) as m:
        m.train(X, T, steps=steps, batch=256, lr=1e-3)
        for stats, qv in data[ntrain:]:
            for chi_t, chi_f, ql, eps_t, eps_f in qv:
                pred = m.forward(tail.features(chi_t, ql, em, stats, NSHELL)[0])
                chi_c = tail.apply(chi_t, pred, ql, NSHELL)
                v = 4.0 * np.pi / np.outer(ql, ql)
                eps_c = np.stack([np.linalg.inv(np.eye(len(ql)) - 2.0 * chi_c[:, :, e] * v)
                                  for e in range(chi_c.shape[2])], axis=2)
                et.append(rel(chi_t, chi_f))
                ec.append(rel(chi_c, chi_f))
                eet.append(rel(eps_t, eps_f))
                eec.append(rel(eps_c, eps_f))
    return {"cells": cells, "nk": nk, "nfull": nfull, "ntrunc": ntrunc, "held_out": held, "samples": len(X),
            "chi_err_truncated": float(np.mean(et)), "chi_err_corrected": float(np.mean(ec)),
            "epsinv_err_truncated": float(np.mean(eet)), "epsinv_err_corrected": float(np.mean(eec)),
            "seconds": time.time() - t0}


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--cells", type=int, default=64)
    ap.add_argument("--nk", type=int, default=6)
    ap.add_argument("--nfull", type=int, default=800)
    ap.add_argument("--ntrunc", type=int, default=100)
    ap.add_argument("--held", type=int, default=16)
    ap.add_argument("--workers", type=int, default=8, help="input-generation processes")
    ap.add_argument("--steps", type=int, default=6000, help="training steps")
    a = ap.parse_args()
    r = run(a.cells, a.nk, a.nfull, a.ntrunc, a.held, a.workers, a.steps)
    print(r)


if __name__ == "__main__":
    main()
