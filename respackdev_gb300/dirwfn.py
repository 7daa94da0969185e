"""dir-wfn front end: RESPACK's symmetry file from a plane-wave code's
symmetry operations, and a validator of a dir-wfn directory.

`util/qe2respack/qe2respack.f90` converts Quantum ESPRESSO output to dir-wfn:
the text and unformatted files at :118-200, the symmetry file in
`convert_sym` at :204-272.  `symmetry_text` restates that conversion:
  - nnp is the smallest n in 1..1000 for which every fractional translation
    times n is an integer within 1e-7 (:236-252);
  - tau = -nint(n * ftau) (:245-249);
  - each rotation (QE's 9 integers, column by column) is inverted, checked to
    be integral and written column by column as 9I3, then tau as 3I3
    (:254-269).
`validate` checks a dir-wfn directory against the layout the chiqw readers
use (`src/chiqw/chiqw.F:87-329` for the text files, :1106-1158 for dat.wfn):
  - every file is there;
  - the k count of dat.sample-k, dat.nkm, dat.kg, dat.eigenvalue and dat.wfn
    agree, and each k's plane-wave count agrees between dat.nkm, dat.kg and
    its dat.wfn records;
  - the plane waves of each k are inside the cutoff sphere |k+G|^2 <= Ecut
    (bohr^-2, Ecut in Ry as dat.bandcalc holds it) and have no repeats;
  - the bands of each k are orthonormal (optionally on a sample of k);
  - the eigenvalues of each k ascend;
  - every symmetry rotation is integral, of determinant +-1, and keeps the
    lattice's metric.
It returns the problems found; an empty list means the directory is usable.
Usage: python -m respackdev_gb300.dirwfn <run directory>
"""
from __future__ import annotations

import os
import struct
import sys
from typing import List, Optional, Sequence

import numpy as np

FILES = ("dat.bandcalc", "dat.lattice", "dat.symmetry", "dat.sample-k", "dat.nkm", "dat.kg", "dat.eigenvalue",
         "dat.wfn")


def _nint(x):
    """Fortran NINT / IDNINT: nearest integer, halves away from zero."""
    x = np.asarray(x, dtype=np.float64)
    return (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64)


def symmetry_text(rotations: Sequence[Sequence[int]], ftau: Sequence[Sequence[float]], max_nnp: int = 1000) -> str:
    """dat.symmetry for QE's symmetry operations: rotations as QE's 9-integer
    ROTATION data (column by column), ftau its FRACTIONAL_TRANSLATION (crystal
    units).  Raises ValueError where qe2respack would write nothing (no
    common denominator up to max_nnp) or stop (a non-integral inverse)."""
    rot = np.asarray(rotations, dtype=np.int64).reshape(-1, 9)
    ft = np.asarray(ftau, dtype=np.float64).reshape(-1, 3)
    if rot.shape[0] != ft.shape[0]:
        raise ValueError("one fractional translation per rotation")
    nnp = None
    for n in range(1, max_nnp + 1):
        if np.all(np.abs(ft * n - _nint(ft * n)) <= 1.0e-7):
            nnp = n
            break
    if nnp is None:
        raise ValueError(f"no common denominator of the fractional translations up to {max_nnp}")
    tau = -_nint(ft * nnp)
    lines = ["%5d" % rot.shape[0], "%5d" % nnp]
    for r, t in zip(rot, tau):
        mat = r.reshape(3, 3).T.astype(np.float64)   # mat(k, j) = rot(3 (j-1) + k)
        inv = np.linalg.inv(mat)
        if np.any(np.abs(inv - _nint(inv)) > 1.0e-10):
            raise ValueError("something wrong in symmetry matrix: its inverse is not integral")
        lines.append("".join("%3d" % v for v in _nint(inv).T.reshape(-1)))   # column by column
        lines.append("".join("%3d" % v for v in t))
    return "\n".join(lines) + "\n"


def _fixed_ints(line: str, width: int, n: int) -> List[int]:
    line = line.rstrip("\n")
    if len(line) >= width * n:
        return [int(line[i * width:(i + 1) * width]) for i in range(n)]
    return [int(x) for x in line.split()][:n]


def _reals(path: str) -> List[float]:
    out = []
    with open(path) as f:
        for tok in f.read().replace(",", " ").split():
            out.append(float(tok.replace("D", "E").replace("d", "e")))
    return out


def _records(path: str):
    """Unformatted sequential records (4-byte markers), as byte strings."""
    recs = []
    with open(path, "rb") as f:
        while True:
            head = f.read(4)
            if not head:
                break
            if len(head) < 4:
                raise ValueError("truncated record marker")
            (n,) = struct.unpack("<i", head)
            body = f.read(n)
            tail = f.read(4)
            if len(body) < n or len(tail) < 4 or struct.unpack("<i", tail)[0] != n:
                raise ValueError("truncated or inconsistent record")
            recs.append(body)
    return recs


def validate(root: str, check_orthonormal: bool = True, max_k_orthonormal: Optional[int] = None,
             tol: float = 1.0e-6) -> List[str]:
    """Problems of root/dir-wfn (an empty list: usable by the chiqw readers)."""
    w = os.path.join(root, "dir-wfn")
    probs: List[str] = []
    missing = [f for f in FILES if not os.path.exists(os.path.join(w, f))]
    if missing:
        return ["missing " + ", ".join(missing)]
    try:
        ecut, efermi = _reals(os.path.join(w, "dat.bandcalc"))[:2]
        avec = np.array(_reals(os.path.join(w, "dat.lattice"))[:9]).reshape(3, 3)
        sk = _reals(os.path.join(w, "dat.sample-k"))
        nk = int(sk[0])
        kpts = np.array(sk[1:1 + 3 * nk]).reshape(nk, 3)
        nkm = [int(x) for x in _reals(os.path.join(w, "dat.nkm"))]
        ev = _reals(os.path.join(w, "dat.eigenvalue"))
        nb = int(ev[0])
        ev = ev[1:]
    except (ValueError, IndexError) as e:
        return [f"unreadable text file: {e}"]
    if len(sk) - 1 != 3 * nk:
        probs.append(f"dat.sample-k: {nk} k points announced, {(len(sk) - 1) / 3:g} given")
    if len(nkm) != nk:
        probs.append(f"dat.nkm: {len(nkm)} counts for {nk} k points")
    if len(ev) != nk * nb:
        probs.append(f"dat.eigenvalue: {len(ev)} values for {nk} k x {nb} bands")
    # plane-wave lists
    kg: List[np.ndarray] = []
    with open(os.path.join(w, "dat.kg")) as f:
        toks = f.read().split()
    pos = 0
    try:
        for ik in range(nk):
            n = int(toks[pos]); pos += 1
            g = np.array([int(t) for t in toks[pos:pos + 3 * n]], dtype=np.int64)
            if g.size != 3 * n:
                raise IndexError
            kg.append(g.reshape(n, 3)); pos += 3 * n
    except (IndexError, ValueError):
        probs.append(f"dat.kg: ends inside k point {len(kg) + 1}")
    if pos != len(toks) and len(kg) == nk:
        probs.append("dat.kg: data after the last k point")
    bvec = 2.0 * np.pi * np.linalg.inv(avec).T   # rows b_i, a_i . b_j = 2 pi delta_ij
    for ik, g in enumerate(kg):
        if ik < len(nkm) and g.shape[0] != nkm[ik]:
            probs.append(f"k {ik + 1}: dat.kg holds {g.shape[0]} G, dat.nkm {nkm[ik]}")
        if len({tuple(x) for x in g}) != g.shape[0]:
            probs.append(f"k {ik + 1}: repeated G in dat.kg")
        q2 = np.sum(((g + kpts[ik][None, :]) @ bvec) ** 2, axis=1)
        if q2.size and q2.max() > ecut * (1 + 1e-8) + 1e-10:
            probs.append(f"k {ik + 1}: G outside the cutoff sphere (|k+G|^2 = {q2.max():.6g} > Ecut = {ecut:.6g})")
    # eigenvalues
    if len(ev) == nk * nb:
        e = np.array(ev).reshape(nk, nb)
        bad = [ik + 1 for ik in range(nk) if np.any(np.diff(e[ik]) < -1e-10)]
        if bad:
            probs.append(f"eigenvalues not ascending at k {bad[:5]}")
    # wave functions
    try:
        recs = _records(os.path.join(w, "dat.wfn"))
    except ValueError as e:
        probs.append(f"dat.wfn: {e}")
        recs = None
    if recs is not None:
        ncomp = struct.unpack("<i", recs[0][:4])[0] if recs and len(recs[0]) >= 4 else -1
        if ncomp != 1:
            probs.append(f"dat.wfn: ncomp = {ncomp} (the chiqw path reads one component)")
        if len(recs) != 1 + nk * nb:
            probs.append(f"dat.wfn: {len(recs) - 1} band records for {nk} k x {nb} bands")
        else:
            ks = range(nk) if max_k_orthonormal is None else \
                np.unique(np.linspace(0, nk - 1, min(nk, max_k_orthonormal)).astype(int))
            for ik in range(nk):
                npw = nkm[ik] if ik < len(nkm) else -1
                rs = recs[1 + ik * nb:1 + (ik + 1) * nb]
                if any(len(r) != 16 * npw for r in rs):
                    probs.append(f"k {ik + 1}: a dat.wfn record is not {npw} complex(8)")
                    continue
                if check_orthonormal and ik in ks:
                    c = np.frombuffer(b"".join(rs), dtype="<c16").reshape(nb, npw)
                    err = np.abs(c.conj() @ c.T - np.eye(nb)).max()
                    if err > tol:
                        probs.append(f"k {ik + 1}: bands not orthonormal (max |<i|j> - delta| = {err:.3g})")
    # symmetry
    try:
        with open(os.path.join(w, "dat.symmetry")) as f:
            lines = [ln for ln in f.read().splitlines() if ln.strip()]
        nsym, nnp = int(lines[0].split()[0]), int(lines[1].split()[0])
        if nnp < 1:
            probs.append(f"dat.symmetry: nnp = {nnp}")
        gmet = avec @ avec.T
        for i in range(nsym):
            r = np.array(_fixed_ints(lines[2 + 2 * i], 3, 9), dtype=np.int64).reshape(3, 3).T
            _fixed_ints(lines[3 + 2 * i], 3, 3)
            det = round(np.linalg.det(r))
            keeps = np.allclose(r.T @ gmet @ r, gmet, atol=1e-6 * np.abs(gmet).max()) or \
                np.allclose(r @ np.linalg.inv(gmet) @ r.T, np.linalg.inv(gmet), atol=1e-6 * np.abs(np.linalg.inv(gmet)).max())
            if abs(det) != 1 or not keeps:
                probs.append(f"dat.symmetry: operation {i + 1} is not a symmetry of the lattice")
        if len(lines) < 2 + 2 * nsym:
            probs.append(f"dat.symmetry: {nsym} operations announced, fewer given")
    except (ValueError, IndexError) as e:
        probs.append(f"dat.symmetry: unreadable ({e})")
    return probs


def main(argv: Sequence[str]) -> int:
    if len(argv) != 1:
        print("usage: python -m respackdev_gb300.dirwfn <run directory>", file=sys.stderr)
        return 2
    probs = validate(argv[0])
    for p in probs:
        print(p)
    if not probs:
        print("dir-wfn ok")
    return 1 if probs else 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
