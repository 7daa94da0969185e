"""Seeded synthetic band-structure inputs in RESPACK's file formats.

The reference ships no ``dir-wfn`` (it needs Quantum ESPRESSO / xTAPP runs), so
every workload of this package is generated here from a seed and written in the
exact formats the reference reads:

* ``dir-wfn/dat.{bandcalc,lattice,symmetry,sample-k,nkm,eigenvalue,kg}`` as
  list-directed text and ``dir-wfn/dat.wfn`` as a Fortran unformatted
  sequential file (one ``ncomp`` record, then one record of ``NGI(k)``
  complex(8) coefficients per (k, band)).  Writers follow
  ``util/qe2respack/qe2respack.f90:118-272``; readers are
  ``src/chiqw/chiqw.F:87-329`` and ``:1106-1158``.
* ``dir-wan/dat.ns-nb``, ``dat.umat`` (list-directed complex ``(re,im)``),
  ``dat.wan`` (unformatted: ``NWF`` then one record of ``NG0(k) x NWF``
  complex(8) per full-mesh k) and ``dat.wan-center``; writers follow
  ``src/wannier/wannier.F:567-572, 2127-2215``.

Units follow the reference: lengths in bohr, band energies and the Fermi
level in Hartree, the wave-function cutoff in Rydberg (|k+G|^2 in bohr^-2).
By default the symmetry file lists the identity only and the sample-k list
holds the whole Gamma-centred mesh, so the reference's unfolding (time
reversal included, ``chiqw.F:437-480``) reproduces the mesh.  With
``sym="oh"`` / ``"oh_glide"`` it lists the 48 cubic operations (with the
diamond structure's fractional translation on half of them) and only the
irreducible points, as a DFT converter writes them; ``full_mesh_equivalent``
gives the identity-only input with the same unfolded wave functions.
"""
from __future__ import annotations

import dataclasses
import os
import struct
from typing import List, Optional, Sequence

import numpy as np

AU_EV = 27.21151  # Hartree in eV, as src/chiqw/config.h:19
TPI = 2.0 * np.pi


@dataclasses.dataclass
class SynthSpec:
    """What to generate.  Energies are in eV here and written in Hartree."""

    lattice: str = "fcc"          # fcc | bcc | sc
    a: float = 10.26              # conventional lattice constant (bohr)
    nk: Sequence[int] = (4, 4, 4)  # Gamma-centred Monkhorst-Pack mesh
    nbands: int = 40
    nocc: int = 8
    ecut_psi: float = 16.0        # Ry
    gap_ev: float = 1.0
    top_ev: float = 40.0
    occ_width_ev: float = 10.0    # spread of the occupied manifold
    disp_ev: float = 0.6          # band dispersion amplitude
    metal: bool = False           # Fermi level inside the lowest empty bands
    seed: int = 1234
    shuffle_g: bool = True        # write each PW list in a seeded order
    # band-cRPA target window (1-based, inclusive) written to dir-wan
    wan_lo: int = 9
    wan_hi: int = 11
    wan_mode: str = "identity"    # identity | random  (dat.umat)
    nwf: int = 0                  # Wannier orbitals for calc_int (0 = none)
    wan_sigma: float = 1.2        # Gaussian width of the synthetic orbitals (bohr)
    # symmetry written to dat.symmetry: "identity" (the whole mesh in
    # dat.sample-k), "oh" (the 48 point operations of the cubic lattice, an
    # irreducible dat.sample-k) or "oh_glide" (as "oh", with the fractional
    # translation (1/4, 1/4, 1/4) of the diamond structure on the 24
    # operations outside T_d: nnp = 4)
    sym: str = "identity"


# ----------------------------------------------------------------------------
# lattice and mesh
# ----------------------------------------------------------------------------
def lattice_vectors(kind: str, a: float) -> np.ndarray:
    h = 0.5 * a
    if kind == "fcc":
        return np.array([[0, h, h], [h, 0, h], [h, h, 0]], dtype=np.float64)
    if kind == "bcc":
        return np.array([[-h, h, h], [h, -h, h], [h, h, -h]], dtype=np.float64)
    if kind == "sc":
        return np.eye(3) * a
    raise ValueError(f"unknown lattice {kind!r}")


def reciprocal(avec: np.ndarray):
    a1, a2, a3 = avec
    vol = float(np.dot(a1, np.cross(a2, a3)))
    b1 = np.cross(a2, a3) * TPI / vol
    b2 = np.cross(a3, a1) * TPI / vol
    b3 = np.cross(a1, a2) * TPI / vol
    return np.array([b1, b2, b3]), vol


def fold_half(x: float) -> float:
    """Map a fractional coordinate into (-1/2, 1/2]."""
    y = x - np.floor(x + 0.5)
    if y <= -0.5 + 1e-12:
        y += 1.0
    return float(y)


def gamma_mesh(nk: Sequence[int]) -> np.ndarray:
    n1, n2, n3 = nk
    pts = []
    for i3 in range(n3):
        for i2 in range(n2):
            for i1 in range(n1):
                pts.append([fold_half(i1 / n1), fold_half(i2 / n2), fold_half(i3 / n3)])
    return np.array(pts, dtype=np.float64)


def sphere(bvec: np.ndarray, ecut: float, k: np.ndarray) -> np.ndarray:
    """Integer G with |k+G|^2 <= ecut, in the triple-loop order of the
    reference's ``make_KG0`` (``chiqw_sub.F:785-801``: first index outermost)."""
    # n_i = (k+G).a_i/(2 pi) - k_i and |(k+G).a_i| <= sqrt(ecut)|a_i|
    avec = TPI * np.linalg.inv(bvec).T
    alen = np.linalg.norm(avec, axis=1)
    nmax = (np.sqrt(ecut) * alen / TPI + np.abs(k) + 2).astype(int)
    r = [np.arange(-nmax[i], nmax[i] + 1) for i in range(3)]
    g1, g2, g3 = np.meshgrid(r[0], r[1], r[2], indexing="ij")
    G = np.stack([g1.ravel(), g2.ravel(), g3.ravel()], axis=1)
    kg = (G + k[None, :]) @ bvec
    sel = np.einsum("ij,ij->i", kg, kg) <= ecut
    return G[sel].astype(np.int64)


# ----------------------------------------------------------------------------
# band energies (eV) and coefficients
# ----------------------------------------------------------------------------
def band_energies(spec: SynthSpec, kpts: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    """(nbands, nk) energies in eV with E_F = 0.

    The occupied manifold is a seeded 8-orbital-style tight-binding model
    (cosine dispersion on the three reciprocal axes), the empty bands are
    spread uniformly up to ``top_ev`` with their own dispersion.  A gap of
    ``gap_ev`` separates them unless ``metal`` is set, in which case the Fermi
    level cuts through the lowest empty bands."""
    nb, nocc = spec.nbands, spec.nocc
    nk = kpts.shape[0]
    cosk = np.cos(TPI * kpts)            # (nk, 3)
    cos2 = np.cos(TPI * (kpts[:, [0]] + kpts[:, [1]] - kpts[:, [2]]))[:, 0]
    E = np.zeros((nb, nk))
    for n in range(nocc):
        c = -spec.occ_width_ev + (spec.occ_width_ev - 1.0) * (n / max(nocc - 1, 1))
        t = rng.uniform(0.2, 1.0, size=3) * spec.disp_ev / 3.0
        t2 = rng.uniform(-0.3, 0.3) * spec.disp_ev / 3.0
        E[n] = c + cosk @ t + t2 * cos2
    nun = nb - nocc
    for m in range(nun):
        frac = m / max(nun - 1, 1)
        c = frac * spec.top_ev
        t = rng.uniform(0.2, 1.0, size=3) * spec.disp_ev
        t2 = rng.uniform(-0.3, 0.3) * spec.disp_ev
        E[nocc + m] = c + cosk @ t + t2 * cos2
    vbm = E[:nocc].max()
    E[:nocc] += -0.5 * spec.gap_ev - vbm
    cbm = E[nocc:].min()
    E[nocc:] += 0.5 * spec.gap_ev - cbm
    if spec.metal:
        # put E_F inside the first empty band: mid-way between its min and max
        lo, hi = E[nocc].min(), E[nocc].max()
        shift = 0.5 * (lo + hi)
        E -= shift
    return E


def orthonormal_coeffs(npw: int, nb: int, rng: np.random.Generator) -> np.ndarray:
    """Gram-Schmidt (QR) orthonormalised complex Gaussian columns (npw, nb)."""
    z = rng.standard_normal((npw, nb)) + 1j * rng.standard_normal((npw, nb))
    q, r = np.linalg.qr(z)
    # fix the phase convention so the result is independent of the LAPACK sign choice
    d = np.diag(r)
    q = q * (d / np.abs(d))[None, :]
    return np.ascontiguousarray(q)


# ----------------------------------------------------------------------------
# Fortran file helpers
# ----------------------------------------------------------------------------
def fmt_real(x: float) -> str:
    return f"{x: .16E}"


def write_unformatted_record(f, payload: bytes):
    """One Fortran sequential unformatted record (4-byte markers, gfortran)."""
    n = len(payload)
    if n > 2147483639:
        raise ValueError("records above 2 GiB are written by the C writer")
    f.write(struct.pack("<i", n))
    f.write(payload)
    f.write(struct.pack("<i", n))


def read_unformatted_records(path: str) -> List[bytes]:
    out = []
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        (n,) = struct.unpack_from("<i", data, pos)
        cont = n < 0
        n = abs(n)
        chunk = data[pos + 4: pos + 4 + n]
        pos += 8 + n
        while cont:
            (m,) = struct.unpack_from("<i", data, pos)
            cont = m < 0
            m = abs(m)
            chunk += data[pos + 4: pos + 4 + m]
            pos += 8 + m
        out.append(chunk)
    return out


# ----------------------------------------------------------------------------
# main generator
# ----------------------------------------------------------------------------
@dataclasses.dataclass
class SynthData:
    avec: np.ndarray
    bvec: np.ndarray
    volume: float
    kpts: np.ndarray           # (nk, 3) fractional (the irreducible list with symmetry)
    kg: List[np.ndarray]       # per k: (npw_k, 3) int
    coeffs: List[np.ndarray]   # per k: (npw_k, nbands) complex
    energies: np.ndarray       # (nbands, nk) Hartree
    efermi: float              # Hartree
    ecut_psi: float            # Ry
    # dat.symmetry: rotations on fractional reciprocal coordinates (k' = rg k,
    # identity first), fractional translations pg / nnp
    rg: List[np.ndarray] = dataclasses.field(default_factory=lambda: [np.eye(3, dtype=np.int64)])
    pg: List[np.ndarray] = dataclasses.field(default_factory=lambda: [np.zeros(3, dtype=np.int64)])
    nnp: int = 1


def cubic_point_group(bvec: np.ndarray, glide: bool = False):
    """The 48 operations of O_h on fractional reciprocal coordinates (the
    reference's SK0 = rg SKI, chiqw.F:437-480), identity first: for each signed
    permutation R (Cartesian) rg = B^-T R B^T, an integer matrix for the fcc,
    bcc and simple-cubic lattices.  With glide, the operations outside T_d
    (sign product -1) carry the translation (1/4, 1/4, 1/4) of the primitive
    vectors (pg = (1, 1, 1), nnp = 4)."""
    import itertools
    BT = bvec.T
    BTinv = np.linalg.inv(BT)
    ops = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1, -1), repeat=3):
            R = np.zeros((3, 3))
            for i in range(3):
                R[i, perm[i]] = signs[i]
            rg = BTinv @ R @ BT
            rgi = np.rint(rg).astype(np.int64)
            if not np.allclose(rg, rgi, atol=1e-9):
                raise ValueError("the lattice does not have the cubic point group")
            tau = np.ones(3, dtype=np.int64) if (glide and signs[0] * signs[1] * signs[2] < 0) else np.zeros(3, np.int64)
            ident = perm == (0, 1, 2) and signs == (1, 1, 1)
            ops.append((0 if ident else 1, rgi, tau))
    ops.sort(key=lambda o: o[0])
    return [o[1] for o in ops], [o[2] for o in ops], (4 if glide else 1)


def _kkey(k: np.ndarray):
    """Hash key of a mesh point: the reference compares k points to 1e-4
    (chiqw.F:452-455); mesh coordinates are far apart on that scale."""
    return tuple(int(x) for x in np.rint(np.asarray(k) * 1.0e4))


def unfold_plan(kirr: np.ndarray, rg: List[np.ndarray]):
    """The full mesh the reference builds from an irreducible list
    (chiqw.F:437-480): per irreducible k and operation the image R k folded by
    kcheck, then its time-reversed image folded by kcheck_trs, each kept when
    new.  Returns [(SK0, numirr, numrot, trs, RW)] in that order (0-based)."""
    out, seen = [], set()
    for ik in range(kirr.shape[0]):
        for iop, R in enumerate(rg):
            kt, RW = _kcheck(R @ kirr[ik], False)
            if _kkey(kt) not in seen:
                seen.add(_kkey(kt))
                out.append((kt, ik, iop, 1, RW))
            kt, RW = _kcheck(R @ kirr[ik], True)
            if _kkey(-kt) not in seen:
                seen.add(_kkey(-kt))
                out.append((-kt, ik, iop, -1, RW))
    return out


def irreducible_mesh(nk: Sequence[int], rg: List[np.ndarray]) -> np.ndarray:
    """Irreducible points of the Gamma-centred mesh under rg and time reversal,
    the first of each star in mesh order, such that unfold_plan covers the mesh."""
    mesh = gamma_mesh(nk)
    kept: List[np.ndarray] = []
    covered = set()
    for k in mesh:
        if _kkey(k) in covered:
            continue
        kept.append(k)
        for R in rg:
            covered.add(_kkey(_kcheck(R @ k, False)[0]))
            covered.add(_kkey(-_kcheck(R @ k, True)[0]))
    if len(unfold_plan(np.array(kept), rg)) != mesh.shape[0]:
        raise ValueError("the operations do not map the mesh onto itself")
    return np.array(kept)


def _check_cutoff(bvec: np.ndarray, ecut: float, kpts: np.ndarray):
    """No |k+G|^2 within 1e-9 (relative) of the cutoff, so that every reader's
    sphere (numpy here, C in the library and the oracle) holds the same G."""
    for k in kpts:
        avec = TPI * np.linalg.inv(bvec).T
        nmax = (np.sqrt(ecut) * np.linalg.norm(avec, axis=1) / TPI + np.abs(k) + 2).astype(int)
        r = [np.arange(-nmax[i], nmax[i] + 1) for i in range(3)]
        g = np.stack(np.meshgrid(*r, indexing="ij"), axis=-1).reshape(-1, 3)
        kg = (g + k[None, :]) @ bvec
        e = np.einsum("ij,ij->i", kg, kg)
        if np.any(np.abs(e - ecut) < 1e-9 * ecut):
            raise ValueError(f"a plane wave lies on the cutoff sphere at k = {k}")


def generate(spec: SynthSpec) -> SynthData:
    rng = np.random.default_rng(spec.seed)
    avec = lattice_vectors(spec.lattice, spec.a)
    bvec, vol = reciprocal(avec)
    rg, pg, nnp = [np.eye(3, dtype=np.int64)], [np.zeros(3, dtype=np.int64)], 1
    if spec.sym == "identity":
        kpts = gamma_mesh(spec.nk)
    elif spec.sym in ("oh", "oh_glide"):
        rg, pg, nnp = cubic_point_group(bvec, glide=spec.sym == "oh_glide")
        kpts = irreducible_mesh(spec.nk, rg)
        _check_cutoff(bvec, spec.ecut_psi, gamma_mesh(spec.nk))
    else:
        raise ValueError(f"unknown symmetry {spec.sym!r}")
    Eev = band_energies(spec, kpts, rng)
    kg, coeffs = [], []
    for ik in range(kpts.shape[0]):
        G = sphere(bvec, spec.ecut_psi, kpts[ik])
        if spec.shuffle_g:
            G = G[rng.permutation(G.shape[0])]
        kg.append(G)
        coeffs.append(orthonormal_coeffs(G.shape[0], spec.nbands, rng))
    return SynthData(avec=avec, bvec=bvec, volume=vol, kpts=kpts, kg=kg, coeffs=coeffs,
                     energies=Eev / AU_EV, efermi=0.0, ecut_psi=spec.ecut_psi, rg=rg, pg=pg, nnp=nnp)


def full_mesh_equivalent(d: SynthData) -> SynthData:
    """The same wave functions as an identity-only input: the full mesh in the
    order of the reference's unfold of d (chiqw.F:437-480), each point with its
    make_KG0 plane waves and the coefficients make_C0 gives it
    (chiqw_sub.F:264-322: C(G) = C_irr(R^-1 (G + RW)) exp(-2 pi i G.pg/nnp),
    with G negated and the result conjugated for a time-reversed image), and
    the energies of its irreducible point.  Reading this input unfolds to the
    same full mesh and the same coefficients, so every chi0 and eps^-1 must
    agree with d's up to rounding: each time-reversed image follows its
    partner in the list, and the identity-only unfold rebuilds it from that
    partner by conjugation, as d's unfold does."""
    plan = unfold_plan(d.kpts, d.rg)
    kpts, kg, coeffs, E = [], [], [], []
    for sk0, ik, iop, trs, RW in plan:
        G = sphere(d.bvec, d.ecut_psi, sk0)
        rinv = np.rint(np.linalg.inv(d.rg[iop])).astype(np.int64)
        pack = {tuple(int(x) for x in g): i for i, g in enumerate(d.kg[ik])}
        src = G if trs == 1 else -G
        idx = [pack[tuple(int(x) for x in rinv @ (g + RW))] for g in src]
        pf = np.exp(-1j * TPI * (src @ d.pg[iop]) / d.nnp)
        C = d.coeffs[ik][idx, :] * pf[:, None]
        if trs == -1:
            C = np.conj(C)
        kpts.append(sk0)
        kg.append(G)
        coeffs.append(np.ascontiguousarray(C))
        E.append(d.energies[:, ik])
    return SynthData(avec=d.avec, bvec=d.bvec, volume=d.volume, kpts=np.array(kpts), kg=kg, coeffs=coeffs,
                     energies=np.stack(E, axis=1), efermi=d.efermi, ecut_psi=d.ecut_psi)


def write_dir_wfn(root: str, d: SynthData, ncomp: int = 1):
    w = os.path.join(root, "dir-wfn")
    os.makedirs(w, exist_ok=True)
    nk = d.kpts.shape[0]
    nb = d.energies.shape[0]
    with open(os.path.join(w, "dat.bandcalc"), "w") as f:
        f.write(fmt_real(d.ecut_psi) + "\n")
        f.write(fmt_real(d.efermi) + "\n")
        f.write(fmt_real(0.0) + "\n")
    with open(os.path.join(w, "dat.lattice"), "w") as f:
        for v in d.avec:
            f.write(" ".join(fmt_real(x) for x in v) + "\n")
    with open(os.path.join(w, "dat.symmetry"), "w") as f:
        f.write("%5d\n%5d\n" % (len(d.rg), d.nnp))
        for R, t in zip(d.rg, d.pg):
            # ((rg(i,j), i=1,3), j=1,3): column by column (chiqw.F:196)
            f.write("".join("%3d" % int(R[i, j]) for j in range(3) for i in range(3)) + "\n")
            f.write("%3d%3d%3d\n" % tuple(int(x) for x in t))
    with open(os.path.join(w, "dat.sample-k"), "w") as f:
        f.write("%12d\n" % nk)
        for k in d.kpts:
            f.write(" ".join(fmt_real(x) for x in k) + "\n")
    with open(os.path.join(w, "dat.nkm"), "w") as f:
        for G in d.kg:
            f.write("%12d\n" % G.shape[0])
    with open(os.path.join(w, "dat.kg"), "w") as f:
        for G in d.kg:
            f.write("%12d\n" % G.shape[0])
            for g in G:
                f.write("%12d%12d%12d\n" % tuple(int(x) for x in g))
    with open(os.path.join(w, "dat.eigenvalue"), "w") as f:
        f.write("%12d\n" % nb)
        for ik in range(nk):
            for ib in range(nb):
                f.write(fmt_real(d.energies[ib, ik]) + "\n")
    with open(os.path.join(w, "dat.wfn"), "wb") as f:
        write_unformatted_record(f, struct.pack("<i", ncomp))
        for ik in range(nk):
            c = d.coeffs[ik]
            for ib in range(nb):
                write_unformatted_record(f, np.ascontiguousarray(c[:, ib]).astype("<c16").tobytes())


def _kcheck(k: np.ndarray, trs: bool):
    """kcheck / kcheck_trs (chiqw_sub.F:668-771): fold a rotated k into the
    first zone; returns the folded k and the integer shift RW."""
    k = k.copy()
    RW = np.zeros(3, dtype=np.int64)
    for i in range(3):
        if not trs:
            d = 1.0e-6
            if k[i] > 1.5 + d: k[i] -= 2.0; RW[i] = -2
            if k[i] > 0.5 + d: k[i] -= 1.0; RW[i] = -1
            if k[i] <= -1.5 + d: k[i] += 2.0; RW[i] = 2
            if k[i] <= -0.5 + d: k[i] += 1.0; RW[i] = 1
        else:
            d = -1.0e-6
            if k[i] >= 1.5 + d: k[i] -= 2.0; RW[i] = -2
            if k[i] >= 0.5 + d: k[i] -= 1.0; RW[i] = -1
            if k[i] < -1.5 + d: k[i] += 2.0; RW[i] = 2
            if k[i] < -0.5 + d: k[i] += 1.0; RW[i] = 1
    return k, RW


def unfold_full_mesh(d: SynthData):
    """Full k mesh in the reference's order (chiqw.F:437-480, calc_intW.F:210-272:
    per irreducible k the symmetry image, then its time-reversed image, each kept
    when new) with its plane-wave lists (make_KG0 at R k + RW, negated for the
    time-reversed images).  The synthetic inputs carry only the identity, so
    R = 1.  Returns (SK0 (ntk, 3), list of (ng, 3) int arrays)."""
    ecut = 0.0
    for ik in range(d.kpts.shape[0]):
        kG = (d.kg[ik] + d.kpts[ik][None, :]) @ d.bvec
        ecut = max(ecut, float(np.einsum("ij,ij->i", kG, kG).max()))
    ecut += 1.0e-8
    sk0, kgs = [], []
    for ik in range(d.kpts.shape[0]):
        for trs in (False, True):
            kt, RW = _kcheck(d.kpts[ik].astype(np.float64), trs)
            cand = -kt if trs else kt
            if any(np.all(np.abs(x - cand) < 1.0e-4) for x in sk0):
                continue
            G = sphere(d.bvec, ecut, d.kpts[ik] + RW)
            sk0.append(cand)
            kgs.append(-G if trs else G)
    return np.array(sk0), kgs


def write_dir_wan(root: str, spec: SynthSpec, d: SynthData, full_kg: Optional[List[np.ndarray]] = None,
                  full_k: Optional[np.ndarray] = None):
    """Band-cRPA target window (dat.ns-nb, dat.umat) and, when ``spec.nwf`` is
    set, synthetic Gaussian Wannier orbitals (dat.wan, dat.wan-center) on the
    full-mesh plane-wave lists ``full_kg`` (the lists the reference rebuilds
    with ``make_KG0``)."""
    w = os.path.join(root, "dir-wan")
    os.makedirs(w, exist_ok=True)
    rng = np.random.default_rng(spec.seed + 7)
    # dat.ns-nb and dat.umat hold every point of the full mesh (chiqw.F:873-894)
    nk = int(np.prod(spec.nk))
    nwin = spec.wan_hi - spec.wan_lo + 1
    with open(os.path.join(w, "dat.ns-nb"), "w") as f:
        for _ in range(nk):
            f.write("%12d%12d\n" % (spec.wan_lo - 1, nwin))
    with open(os.path.join(w, "dat.umat"), "w") as f:
        f.write("%12d\n" % nwin)
        for _ in range(nk):
            if spec.wan_mode == "identity":
                U = np.eye(nwin, dtype=np.complex128)
            else:
                z = rng.standard_normal((nwin, nwin)) + 1j * rng.standard_normal((nwin, nwin))
                q, _ = np.linalg.qr(z)
                U = q * rng.uniform(0.6, 1.0, size=(nwin, 1))  # partial weight
            for ib in range(nwin):
                f.write(" ".join("(%s,%s)" % (fmt_real(U[ib, jw].real).strip(), fmt_real(U[ib, jw].imag).strip())
                                 for jw in range(nwin)) + "\n")
    if spec.nwf > 0:
        if len(d.rg) > 1:
            raise ValueError("synthetic Wannier orbitals are written for identity-only inputs")
        if full_kg is None or full_k is None:
            full_k, full_kg = unfold_full_mesh(d)
        centers = rng.uniform(0.0, 1.0, size=(spec.nwf, 3)) @ d.avec
        with open(os.path.join(w, "dat.wan-center"), "w") as f:
            f.write("#Wannier center\n#1:x, 2:y, 3:z (in xyz coord)\n")
            for c in centers:
                f.write("".join("%20.10f" % x for x in c) + "\n")
        with open(os.path.join(w, "dat.wan"), "wb") as f:
            write_unformatted_record(f, struct.pack("<i", spec.nwf))
            for ik in range(full_k.shape[0]):
                G = full_kg[ik]
                kG = (G + full_k[ik][None, :]) @ d.bvec
                k2 = np.einsum("ij,ij->i", kG, kG)
                cols = []
                for iw in range(spec.nwf):
                    sig = spec.wan_sigma * (1.0 + 0.15 * iw)
                    c = np.exp(-0.5 * sig * sig * k2) * np.exp(-1j * (kG @ centers[iw]))
                    c /= np.linalg.norm(c)
                    cols.append(c)
                C = np.stack(cols, axis=1)  # (NG0, NWF), column-major record
                write_unformatted_record(f, np.asfortranarray(C).T.ravel().astype("<c16").tobytes())


def make_case(root: str, spec: SynthSpec, with_wan: bool = True) -> SynthData:
    d = generate(spec)
    write_dir_wfn(root, d)
    if with_wan:
        write_dir_wan(root, spec, d)
    return d


def make_full_mesh_case(root: str, spec: SynthSpec) -> SynthData:
    """The identity-only input equivalent to the symmetry-reduced case of spec
    (full_mesh_equivalent), with the same dir-wan."""
    d = full_mesh_equivalent(generate(spec))
    write_dir_wfn(root, d)
    write_dir_wan(root, spec, d)
    return d


# Named synthetic cases used by the tests, the smoke check and the bench.
CASES = {
    # two-by-two-by-two mesh, small basis: the quick parity case
    "tiny": SynthSpec(nk=(2, 2, 2), nbands=12, nocc=4, ecut_psi=8.0, seed=11,
                      wan_lo=5, wan_hi=7),
    "tiny_metal": SynthSpec(nk=(2, 2, 2), nbands=12, nocc=4, ecut_psi=8.0, seed=12,
                            metal=True, wan_lo=5, wan_hi=7, wan_mode="random"),
    # odd mesh exercises the odd branch of make_index_kpt
    "tiny_odd": SynthSpec(nk=(3, 3, 3), nbands=10, nocc=4, ecut_psi=6.0, seed=13,
                          wan_lo=5, wan_hi=6),
    # Wannier orbitals for calc_int (V, W, X, J) on the tiny and odd meshes
    "tiny_wan": SynthSpec(nk=(2, 2, 2), nbands=12, nocc=4, ecut_psi=8.0, seed=21,
                          wan_lo=5, wan_hi=7, nwf=3, wan_sigma=1.2),
    "odd_wan": SynthSpec(nk=(3, 3, 3), nbands=10, nocc=4, ecut_psi=6.0, seed=23,
                         wan_lo=5, wan_hi=6, nwf=2, wan_sigma=1.0),
    # five Gaussian Wannier orbitals on a 3x3x3 mesh with 24 bands (static U/J)
    "wan5": SynthSpec(nk=(3, 3, 3), nbands=24, nocc=4, ecut_psi=8.0, seed=25,
                      wan_lo=5, wan_hi=9, nwf=5, wan_sigma=1.1),
    # fcc a=10.26, 4x4x4 k, 40 bands, 16 Ry, E_F mid-gap, target bands 9-11
    "fcc_4k_40b": SynthSpec(nk=(4, 4, 4), nbands=40, nocc=8, ecut_psi=16.0, seed=1234),
    # the cubic point group on an fcc 4x4x4 mesh: 8 irreducible points unfold
    # to 64 (rotations, time reversal, zone-boundary wraps)
    "tiny_sym": SynthSpec(nk=(4, 4, 4), nbands=10, nocc=4, ecut_psi=6.3, seed=31, wan_lo=5, wan_hi=6,
                          shuffle_g=True, sym="oh"),
    # the same with the diamond structure's fractional translation (nnp = 4)
    # on half the operations, and a metal with a random cRPA projection
    "tiny_glide": SynthSpec(nk=(4, 4, 4), nbands=10, nocc=4, ecut_psi=6.3, seed=32, wan_lo=5, wan_hi=6,
                            shuffle_g=True, sym="oh_glide", metal=True, wan_mode="random"),
    # the 8x8x8-k / 200-band workload's cell, cutoffs and FFT box (fcc a=15.84,
    # 20 Ry, 36^3 box, about 600 G at 11 Ry) on a 4x4x4 mesh with 100 bands
    "headline_small": SynthSpec(lattice="fcc", a=15.84, nk=(4, 4, 4), nbands=100, nocc=8, ecut_psi=20.0,
                                seed=2024, wan_lo=9, wan_hi=11, shuffle_g=False),
    # the 8x8x8-k / 200-band workload itself
    "headline": SynthSpec(lattice="fcc", a=15.84, nk=(8, 8, 8), nbands=200, nocc=8, ecut_psi=20.0,
                          seed=2024, wan_lo=9, wan_hi=11, shuffle_g=False),
    # the large end-to-end workload: 10x10x10 k (47 irreducible points under the
    # cubic group), 1000 bands, 31.7 Ry (about 2980 plane waves; 48^3 box),
    # dielectric cutoff 25.8 Ry (about 2180 G)
    "large": SynthSpec(lattice="fcc", a=15.84, nk=(10, 10, 10), nbands=1000, nocc=8, ecut_psi=31.7,
                       seed=2025, wan_lo=9, wan_hi=11, shuffle_g=False, sym="oh"),
    # its cell, cutoffs and box on a 2x2x2 mesh with 40 bands (parity case)
    "large_small": SynthSpec(lattice="fcc", a=15.84, nk=(2, 2, 2), nbands=40, nocc=8, ecut_psi=31.7,
                             seed=2026, wan_lo=9, wan_hi=11, shuffle_g=False, sym="oh"),
}
