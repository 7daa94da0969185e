"""ctypes mirror of the calc_int part of the C ABI (include/respack_gb300.h):
the Wannier-basis bare / screened Coulomb (calc_w3d: V, W) and exchange
(calc_j3d: X, J) integrals of RESPACK's src/calc_int."""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from .chiqw import load as _load_lib


class IntParams(C.Structure):
    _fields_ = [("calc_ifreq", C.c_int), ("ix_intj_min", C.c_int), ("ix_intj_max", C.c_int),
                ("iy_intj_min", C.c_int), ("iy_intj_max", C.c_int), ("iz_intj_min", C.c_int),
                ("iz_intj_max", C.c_int), ("wcut_mvmc", C.c_double), ("jcut_mvmc", C.c_double),
                ("fft_box", C.c_int * 3), ("device", C.c_int), ("write_files", C.c_int),
                ("read_eps_f32", C.c_int)]


_bound = False


def load() -> C.CDLL:
    global _bound
    L = _load_lib()
    if not _bound:
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.rp_int_default_params.argtypes = [C.POINTER(IntParams)]
        L.rp_int_parse_namelist.argtypes = [C.c_char_p, C.POINTER(IntParams)]
        L.rp_int_parse_namelist.restype = C.c_int
        L.rp_int_create.argtypes = [C.POINTER(vp), C.c_char_p, C.POINTER(IntParams)]
        L.rp_int_create.restype = C.c_int
        L.rp_int_dims.argtypes = [vp, ip, ip, ip, ip]
        L.rp_int_dims.restype = C.c_int
        L.rp_int_w3d.argtypes = [vp, vp, vp]
        L.rp_int_w3d.restype = C.c_int
        L.rp_int_j3d.argtypes = [vp, vp, vp]
        L.rp_int_j3d.restype = C.c_int
        L.rp_int_stage_times.argtypes = [vp, dp]
        L.rp_int_stage_times.restype = C.c_int
        L.rp_int_last_error.argtypes = [vp]
        L.rp_int_last_error.restype = C.c_char_p
        L.rp_int_destroy.argtypes = [vp]
        L.rp_calc_w3d.argtypes = [C.c_char_p, C.c_char_p]
        L.rp_calc_w3d.restype = C.c_int
        L.rp_calc_j3d.argtypes = [C.c_char_p, C.c_char_p]
        L.rp_calc_j3d.restype = C.c_int
        _bound = True
    return L


def default_params(**kw) -> IntParams:
    p = IntParams()
    load().rp_int_default_params(C.byref(p))
    box = kw.pop("fft_box", None)
    for k, v in kw.items():
        setattr(p, k, v)
    if box is not None:
        p.fft_box[0], p.fft_box[1], p.fft_box[2] = box
    return p


def parse_namelist(text: str, params: Optional[IntParams] = None) -> IntParams:
    p = params or default_params()
    L = load()
    if L.rp_int_parse_namelist(text.encode(), C.byref(p)):
        raise ValueError(L.rp_int_last_error(None).decode())
    return p


class IntContext:
    """One run directory (dir-wfn, dir-wan, dir-eps) on the device."""

    def __init__(self, root: str, params: Optional[IntParams] = None):
        self.L = load()
        self.root = root
        self.params = params or default_params()
        self._h = C.c_void_p()
        if self.L.rp_int_create(C.byref(self._h), root.encode(), C.byref(self.params)):
            raise RuntimeError("rp_int_create failed: " + self.L.rp_int_last_error(None).decode())
        nwf, ne, ntq = C.c_int(), C.c_int(), C.c_int()
        na = (C.c_int * 3)()
        self.L.rp_int_dims(self._h, C.byref(nwf), C.byref(ne), C.byref(ntq), na)
        self.nwf, self.ne, self.ntq, self.na = nwf.value, ne.value, ntq.value, tuple(na)

    def _shape(self):
        return (self.nwf, self.nwf) + tuple(2 * a + 1 for a in self.na)

    def _run(self, fn, with_ne: bool = True):
        a = np.zeros(self._shape(), dtype=np.complex128, order="F")
        b = np.zeros(self._shape() + (self.ne,), dtype=np.complex128, order="F")
        if fn(self._h, a.ctypes.data, b.ctypes.data):
            raise RuntimeError(self.L.rp_int_last_error(self._h).decode())
        return a, b

    def w3d(self):
        """(V, W): V[i, j, R1, R2, R3], W[..., e] in Hartree, R index = R + Na."""
        return self._run(self.L.rp_int_w3d)

    def j3d(self):
        """(X, J) on the same box, zero outside the IX/IY/IZ range."""
        return self._run(self.L.rp_int_j3d)

    def stage_times(self) -> np.ndarray:
        t = (C.c_double * 5)()
        self.L.rp_int_stage_times(self._h, t)
        return np.array(t[:])

    def close(self):
        if self._h:
            self.L.rp_int_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def calc_w3d(root: str, namelist_text: str) -> None:
    L = load()
    if L.rp_calc_w3d(root.encode(), namelist_text.encode()):
        raise RuntimeError(L.rp_int_last_error(None).decode())


def calc_j3d(root: str, namelist_text: str) -> None:
    L = load()
    if L.rp_calc_j3d(root.encode(), namelist_text.encode()):
        raise RuntimeError(L.rp_int_last_error(None).decode())
