"""Independent plane-wave brute force of chi0(q, w) for small synthetic cases.

Test helper.  It shares no code with the C oracle except the tetrahedron
weights (which tests/test_oracle.py checks against quadrature on their own):
the Brillouin-zone unfolding, the plane-wave lists and the pair densities are
recomputed here from the synthetic data.  The pair density is the G-space
convolution

    rho_ij(k, G) = sum_G2 conj(c_{i,k+q}(G2 + G + s)) c_{j,k}(G2),

which equals the reference's FFT route (src/chiqw/chiqw_sub.F:97-205) when the
FFT box is large enough not to alias; tests pass such a box to the oracle.
"""
from __future__ import annotations

import numpy as np

from respackdev_gb300 import synth

AU = 27.21151


def _kcheck(k, trs):
    k = np.array(k, dtype=float)
    RW = np.zeros(3, dtype=int)
    d = 1e-6 if not trs else -1e-6
    for i in range(3):
        if not trs:
            if k[i] > 1.5 + d: k[i] -= 2; RW[i] = -2
            if k[i] > 0.5 + d: k[i] -= 1; RW[i] = -1
            if k[i] <= -1.5 + d: k[i] += 2; RW[i] = 2
            if k[i] <= -0.5 + d: k[i] += 1; RW[i] = 1
        else:
            if k[i] >= 1.5 + d: k[i] -= 2; RW[i] = -2
            if k[i] >= 0.5 + d: k[i] -= 1; RW[i] = -1
            if k[i] < -1.5 + d: k[i] += 2; RW[i] = 2
            if k[i] < -0.5 + d: k[i] += 1; RW[i] = 1
    return k, RW


def unfold(kirr):
    """Identity symmetry + time reversal, in the reference's order (chiqw.F:437-480)."""
    SK0, src = [], []
    for ik, k in enumerate(kirr):
        for trs in (False, True):
            kt, RW = _kcheck(k, trs)
            kk = -kt if trs else kt
            if any(np.all(np.abs(np.array(s) - kk) < 1e-4) for s in SK0):
                continue
            SK0.append(kk)
            src.append((ik, -1 if trs else 1, RW))
    return np.array(SK0), src


def full_coeffs(d: synth.SynthData, SK0, src, nband):
    """Per full k: dict G(tuple) -> coefficient vector over bands."""
    out = []
    for jk, (ik, t, RW) in enumerate(src):
        G = d.kg[ik]
        C = d.coeffs[ik][:, :nband]
        m = {}
        for g, c in zip(G, C):
            if t == 1:
                gg = tuple(int(x) for x in (g - RW))
                m[gg] = c
            else:
                # C0(G) = conj(C_irr(-G + RW))  ->  G = -(g - RW)
                gg = tuple(int(x) for x in (-(g - RW)))
                m[gg] = np.conj(c)
        out.append(m)
    return out


def chi0_brute(d: synth.SynthData, q_frac, ecut_eps, em, delt_ev, dmna, dmnr, nband, nocc_bands,
               prob=None, imt1=None, nk=None, tetra=None):
    """chi0(G, G', w) (after /VOLUME, before the spin factor) for one q != 0.

    ``nocc_bands``: (occupied absolute band list, virtual absolute band list),
    0-based, in the reference's pair order (occupied outer, virtual inner).
    ``tetra(e1_mesh, e2_mesh, dsgn)`` returns xo(k_mesh, w)."""
    SK0, src = unfold(d.kpts)
    NTK = SK0.shape[0]
    coeffs = full_coeffs(d, SK0, src, nband)
    LG = synth.sphere(d.bvec, ecut_eps, np.asarray(q_frac))
    NG = LG.shape[0]
    delt = delt_ev / AU
    occ, vir = nocc_bands
    # k+q on the mesh and the folding shift
    kpq, shifts = [], []
    for ik in range(NTK):
        s = SK0[ik] + q_frac
        sh = np.zeros(3, dtype=int)
        for i in range(3):
            if s[i] > 1.5 + 1e-6: s[i] -= 2; sh[i] = 2
            if s[i] > 0.5 + 1e-6: s[i] -= 1; sh[i] = 1
            if s[i] <= -1.5 + 1e-6: s[i] += 2; sh[i] = -2
            if s[i] <= -0.5 + 1e-6: s[i] += 1; sh[i] = -1
        j = [jk for jk in range(NTK) if np.all(np.abs(SK0[jk] - s) < 1e-6)]
        kpq.append(j[-1])
        shifts.append(sh)
    # mesh index of each k (make_index_kpt)
    nkb = np.array(nk)
    idx = np.zeros(NTK, dtype=int)
    for ik in range(NTK):
        if NTK % 2:
            ix = np.rint(SK0[ik] * nkb + (nkb - 1) / 2.0).astype(int)
        else:
            ix = np.rint(SK0[ik] * nkb + nkb / 2.0).astype(int) - 1
        idx[ik] = ix[0] + nkb[0] * (ix[1] + nkb[1] * ix[2])
    chi = np.zeros((NG, NG, len(em)), dtype=np.complex128)
    E = d.energies  # (band, k_irr)
    for jb in occ:
        for ib in vir:
            rho = np.zeros((NTK, NG), dtype=np.complex128)
            for ik in range(NTK):
                ck, ckq = coeffs[ik], coeffs[kpq[ik]]
                for g, G in enumerate(LG):
                    acc = 0j
                    for G2, c in ck.items():
                        key = (G2[0] + G[0] + shifts[ik][0], G2[1] + G[1] + shifts[ik][1], G2[2] + G[2] + shifts[ik][2])
                        cq = ckq.get(key)
                        if cq is not None:
                            acc += np.conj(cq[ib]) * c[jb]
                    rho[ik, g] = acc
            e1 = np.array([np.float32(E[jb, src[ik][0]]) for ik in range(NTK)], dtype=np.float64)
            e2 = np.array([np.float32(E[ib, src[kpq[ik]][0]]) for ik in range(NTK)], dtype=np.float64)
            e1m = np.zeros(NTK); e2m = np.zeros(NTK)
            e1m[idx] = e1; e2m[idx] = e2
            xo = tetra(e1m, e2m, 1.0) + tetra(e1m, e2m, -1.0)
            w = xo[idx, :]  # (k, w)
            pp = np.ones(NTK, dtype=np.complex128)
            if prob is not None:
                pp = np.array([1.0 - prob[jb, ik] * prob[ib, kpq[ik]] for ik in range(NTK)])
            wk = w * (pp / NTK)[:, None]
            chi += np.einsum("kw,kg,kh->ghw", wk, np.conj(rho), rho)
    return chi / d.volume, LG
