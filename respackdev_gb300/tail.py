"""Band-tail correction of chi0 by a small network (no reference counterpart).

chi0 summed over the bands up to a truncation misses the contribution of the
bands above it.  Per q, frequency and |q+G| shell, a network predicts that
tail on the diagonal of chi0 from features of the truncated chi0 and of the
band energies; the full band sum generates the training targets and measures
the error (tests/test_gpu_tail.py).  The network's training and inference run in
the library (rp_mlp_* of include/respack_gb300.h, respackdev_gb300/csrc/rp_mlp.cu);
this module builds the features and targets and applies the correction.

Quantities are made dimensionless with the Coulomb factor v = 4 pi / |q+G|^2:
features carry v chi0 and energies in Hartree, and the targets are the shell
means of v (chi_full - chi_trunc) on the diagonal, times TSCALE.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence, Tuple

import numpy as np

from . import chiqw as rp

NFEAT = 9
NOUT = 2
TSCALE = 100.0


def _lib() -> C.CDLL:
    L = rp.load()
    if not getattr(L, "_mlp_ready", False):
        vp, fp = C.c_void_p, C.POINTER(C.c_float)
        L.rp_mlp_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.c_int]
        L.rp_mlp_create.restype = C.c_int
        L.rp_mlp_nparams.argtypes = [vp]
        L.rp_mlp_nparams.restype = C.c_int
        L.rp_mlp_get_params.argtypes = [vp, fp]
        L.rp_mlp_set_params.argtypes = [vp, fp]
        L.rp_mlp_forward.argtypes = [vp, fp, C.c_int, fp]
        L.rp_mlp_gradients.argtypes = [vp, fp, fp, C.c_int, fp, fp]
        L.rp_mlp_train.argtypes = [vp, fp, fp, C.c_int, C.c_int, C.c_int, C.c_float, fp]
        L.rp_mlp_last_error.argtypes = [vp]
        L.rp_mlp_last_error.restype = C.c_char_p
        L.rp_mlp_destroy.argtypes = [vp]
        L.rp_mlp_destroy.restype = None
        for f in ("rp_mlp_get_params", "rp_mlp_set_params", "rp_mlp_forward", "rp_mlp_gradients", "rp_mlp_train"):
            getattr(L, f).restype = C.c_int
        L._mlp_ready = True
    return L


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class TailMLP:
    """The library's MLP (nin -> nhid -> nhid -> nout) on one GPU."""

    def __init__(self, nin: int = NFEAT, nout: int = NOUT, nhid: int = 128, seed: int = 0, device: int = 0):
        self.L = _lib()
        self.nin, self.nout, self.nhid = nin, nout, nhid
        self._h = C.c_void_p()
        rc = self.L.rp_mlp_create(C.byref(self._h), nin, nhid, nout, seed, device)
        if rc != 0:
            raise RuntimeError(f"rp_mlp_create failed ({rc}): {self.L.rp_last_error(None).decode()}")

    def _check(self, rc: int):
        if rc != 0:
            raise RuntimeError(f"rp_mlp ({rc}): {self.L.rp_mlp_last_error(self._h).decode()}")

    @property
    def nparams(self) -> int:
        return int(self.L.rp_mlp_nparams(self._h))

    def params(self) -> np.ndarray:
        p = np.empty(self.nparams, dtype=np.float32)
        self._check(self.L.rp_mlp_get_params(self._h, _ptr(p)))
        return p

    def set_params(self, p) -> None:
        p = _f32(p)
        if p.size != self.nparams:
            raise ValueError(f"expected {self.nparams} parameters, got {p.size}")
        self._check(self.L.rp_mlp_set_params(self._h, _ptr(p)))

    def forward(self, x) -> np.ndarray:
        x = _f32(x)
        y = np.empty((x.shape[0], self.nout), dtype=np.float32)
        self._check(self.L.rp_mlp_forward(self._h, _ptr(x), x.shape[0], _ptr(y)))
        return y

    def gradients(self, x, t) -> Tuple[float, np.ndarray]:
        x, t = _f32(x), _f32(t)
        loss = np.zeros(1, dtype=np.float32)
        g = np.empty(self.nparams, dtype=np.float32)
        self._check(self.L.rp_mlp_gradients(self._h, _ptr(x), _ptr(t), x.shape[0], _ptr(loss), _ptr(g)))
        return float(loss[0]), g

    def train(self, x, t, steps: int, batch: int = 128, lr: float = 1e-3) -> np.ndarray:
        x, t = _f32(x), _f32(t)
        losses = np.empty(steps, dtype=np.float32)
        self._check(self.L.rp_mlp_train(self._h, _ptr(x), _ptr(t), x.shape[0], steps, batch, lr, _ptr(losses)))
        return losses

    def save(self, path: str, nshell: int, tscale: float = TSCALE) -> None:
        """Write the network for a context's &param_gpu tail_model: int32 magic
        "RPTL", version 1, nin, nhid, nout, nshell; float32 tscale and padding;
        the float32 parameters.  rp_chi0_q then applies the correction on the
        device, with the shells, features and scale of this module."""
        hdr = np.array([0x4C545052, 1, self.nin, self.nhid, self.nout, int(nshell)], dtype="<i4")
        with open(path, "wb") as f:
            f.write(hdr.tobytes())
            f.write(np.array([tscale, 0.0], dtype="<f4").tobytes())
            f.write(self.params().astype("<f4").tobytes())

    def close(self):
        if self._h:
            self.L.rp_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def shells(qglen: np.ndarray, nshell: int) -> np.ndarray:
    """Shell index (0..nshell-1, by equal-count |q+G| quantiles) of every G; -1
    for |q+G| = 0 (the head at Gamma, which is not corrected).  The G are
    ordered by |q+G| rounded to 2^-30, then by index, so that lengths equal by
    symmetry (which two codes compute to different last bits) tie the same way
    here and in the library (rp_ctx.cpp, tail_apply)."""
    ql = np.asarray(qglen, dtype=np.float64)
    idx = np.full(ql.shape, -1, dtype=np.int64)
    ok = ql > 0
    order = np.argsort(np.rint(ql[ok] * 2.0 ** 30), kind="stable")
    s = np.empty(order.size, dtype=np.int64)
    s[order] = np.minimum((np.arange(order.size) * nshell) // max(order.size, 1), nshell - 1)
    idx[ok] = s
    return idx


def band_stats(energies: np.ndarray, efermi: float, ntrunc: int) -> Tuple[float, float, float]:
    """(lowest excluded band energy, mean excluded band energy, both minus E_F, in
    Hartree; and the number of excluded over included bands) from energies
    (nbands, nk) of every band the full sum would use."""
    ex = np.asarray(energies)[ntrunc:] - efermi
    if ex.size == 0:
        return 0.0, 0.0, 0.0
    return float(ex.min()), float(ex.mean()), float(ex.shape[0]) / float(max(ntrunc, 1))


def features(chi_trunc: np.ndarray, qglen: np.ndarray, em: Sequence[complex], stats: Tuple[float, float, float],
             nshell: int) -> Tuple[np.ndarray, np.ndarray]:
    """Features (nen * nshell, NFEAT) of one q and the G -> shell map.
    chi_trunc: (ng, ng, nen) complex, the truncated-band chi0."""
    sh = shells(qglen, nshell)
    ql = np.asarray(qglen, dtype=np.float64)
    nen = chi_trunc.shape[2]
    v = np.where(ql > 0, 4.0 * np.pi / np.where(ql > 0, ql, 1.0) ** 2, 0.0)
    d = np.einsum("ggw->gw", chi_trunc) * v[:, None]          # v chi on the diagonal
    X = np.zeros((nen, nshell, NFEAT), dtype=np.float64)
    e_lo, e_mean, ratio = stats
    for s in range(nshell):
        m = sh == s
        if not m.any():
            continue
        dm = d[m].mean(0)
        X[:, s, 0] = ql[m].mean()
        X[:, s, 1] = dm.real
        X[:, s, 2] = dm.imag
        X[:, s, 8] = (s + 0.5) / nshell
    w = np.asarray(em)
    X[:, :, 3] = w.real[:, None]
    X[:, :, 4] = w.imag[:, None]
    X[:, :, 5] = e_lo
    X[:, :, 6] = e_mean
    X[:, :, 7] = ratio
    return X.reshape(nen * nshell, NFEAT), sh


def targets(chi_trunc: np.ndarray, chi_full: np.ndarray, qglen: np.ndarray, nshell: int) -> np.ndarray:
    """Shell means of v (chi_full - chi_trunc) on the diagonal, times TSCALE:
    (nen * nshell, 2) as (re, im)."""
    sh = shells(qglen, nshell)
    ql = np.asarray(qglen, dtype=np.float64)
    nen = chi_trunc.shape[2]
    v = np.where(ql > 0, 4.0 * np.pi / np.where(ql > 0, ql, 1.0) ** 2, 0.0)
    d = (np.einsum("ggw->gw", chi_full) - np.einsum("ggw->gw", chi_trunc)) * v[:, None]
    T = np.zeros((nen, nshell, NOUT), dtype=np.float64)
    for s in range(nshell):
        m = sh == s
        if m.any():
            dm = d[m].mean(0) * TSCALE
            T[:, s, 0] = dm.real
            T[:, s, 1] = dm.imag
    return T.reshape(nen * nshell, NOUT)


def apply(chi_trunc: np.ndarray, pred: np.ndarray, qglen: np.ndarray, nshell: int) -> np.ndarray:
    """chi_trunc plus the predicted tail on the diagonal (pred from the network,
    (nen * nshell, 2)); the G with |q+G| = 0 keeps its value."""
    sh = shells(qglen, nshell)
    ql = np.asarray(qglen, dtype=np.float64)
    nen = chi_trunc.shape[2]
    p = np.asarray(pred, dtype=np.float64).reshape(nen, nshell, NOUT) / TSCALE
    out = np.array(chi_trunc, copy=True)
    for g in np.nonzero(sh >= 0)[0]:
        corr = (p[:, sh[g], 0] + 1j * p[:, sh[g], 1]) * ql[g] ** 2 / (4.0 * np.pi)
        out[g, g, :] += corr
    return out
