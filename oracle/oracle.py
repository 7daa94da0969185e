"""ctypes binding of the CPU oracle (librp_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the respackdev_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "librp_oracle.so")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("rp_oracle.c", "rp_oracle_int.c", "rp_oracle.h")]
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(s) for s in srcs):
        subprocess.check_call(["make", "-s", "-C", HERE])
    return LIB


class Params(C.Structure):
    _fields_ = [
        ("n_calc_band", C.c_int), ("ecut_for_eps", C.c_double), ("shift_ef", C.c_double),
        ("max_excitation_energy", C.c_double), ("green_func_delt", C.c_double),
        ("ttrhdrn_dmna", C.c_double), ("ttrhdrn_dmnr", C.c_double), ("num_freq_grid", C.c_int),
        ("lower_bound_energy_window", C.c_double), ("upper_bound_energy_window", C.c_double),
        ("flg_crpa", C.c_int), ("flg_calc_type", C.c_int), ("file_num_log_start", C.c_int),
        ("file_num_eps_start", C.c_int), ("file_num_eps_base_start", C.c_int), ("n_calc_q", C.c_int),
        ("calc_num_k", C.POINTER(C.c_int)), ("nen_explicit", C.c_int), ("em_explicit", C.POINTER(C.c_double)),
        ("fft_box", C.c_int * 3), ("dump_chi", C.c_int), ("write_eps", C.c_int), ("nthreads", C.c_int),
        ("max_pairs", C.c_int), ("max_q", C.c_int), ("max_k", C.c_int),
    ]


class Report(C.Structure):
    _fields_ = [("nq_done", C.c_int), ("ntk", C.c_int), ("ng_last", C.c_int), ("npair_last", C.c_int),
                ("npair_full_last", C.c_int), ("nen", C.c_int), ("fft_box", C.c_int * 3),
                ("seconds_total", C.c_double), ("seconds_last_q", C.c_double), ("nk_used_last", C.c_int)]


class IntParams(C.Structure):
    _fields_ = [("calc_ifreq", C.c_int), ("ix_min", C.c_int), ("ix_max", C.c_int), ("iy_min", C.c_int),
                ("iy_max", C.c_int), ("iz_min", C.c_int), ("iz_max", C.c_int), ("wcut_mvmc", C.c_double),
                ("jcut_mvmc", C.c_double), ("fft_box", C.c_int * 3), ("nthreads", C.c_int),
                ("write_files", C.c_int), ("do_w", C.c_int), ("do_j", C.c_int)]


class IntDims(C.Structure):
    _fields_ = [("nwf", C.c_int), ("ne", C.c_int), ("ntq", C.c_int), ("na", C.c_int * 3), ("nkb", C.c_int * 3),
                ("box", C.c_int), ("fft_box", C.c_int * 3), ("seconds", C.c_double)]


_lib: Optional[C.CDLL] = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_default_params.argtypes = [C.POINTER(Params)]
        L.orc_calc_chiqw.argtypes = [C.c_char_p, C.POINTER(Params), C.POINTER(Report)]
        L.orc_calc_chiqw.restype = C.c_int
        L.orc_fft3.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int]
        L.orc_gen_grid.argtypes = [C.c_int, C.c_double, C.c_void_p]
        L.orc_algn235.argtypes = [C.c_int]
        L.orc_algn235.restype = C.c_int
        L.orc_zinv.argtypes = [C.c_int, C.c_void_p]
        L.orc_zinv.restype = C.c_int
        L.orc_ttrhdrn_mkidx.argtypes = [C.c_int] * 3 + [C.c_void_p] * 4
        L.orc_ttrhdrn_chi0.argtypes = [C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_ttrhdrn_chi0.restype = C.c_int
        L.orc_ttrhdrn_simple.argtypes = [C.c_double, C.c_double, C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 4
        L.orc_ttrhdrn_simple.restype = C.c_int
        L.orc_tt_one.argtypes = [C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                 C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_tt_one.restype = C.c_int
        L.orc_last_error.restype = C.c_char_p
        L.orc_int_default_params.argtypes = [C.POINTER(IntParams)]
        L.orc_calc_int.argtypes = [C.c_char_p, C.POINTER(IntParams), C.POINTER(IntDims)] + [C.c_void_p] * 4
        L.orc_calc_int.restype = C.c_int
        _lib = L
    return _lib


def make_params(**kw) -> Params:
    p = Params()
    lib().orc_default_params(C.byref(p))
    em = kw.pop("em", None)
    box = kw.pop("fft_box", None)
    qlist = kw.pop("calc_num_k", None)
    for k, v in kw.items():
        setattr(p, k, v)
    if em is not None:
        arr = np.ascontiguousarray(np.asarray(em, dtype=np.complex128))
        p._em = arr  # keep alive
        p.nen_explicit = arr.size
        p.em_explicit = arr.ctypes.data_as(C.POINTER(C.c_double))
    if box is not None:
        p.fft_box[0], p.fft_box[1], p.fft_box[2] = box
    if qlist is not None:
        arr = np.ascontiguousarray(np.asarray(qlist, dtype=np.int32))
        p._q = arr
        p.n_calc_q = arr.size
        p.calc_num_k = arr.ctypes.data_as(C.POINTER(C.c_int))
        if p.flg_calc_type == 0:
            p.flg_calc_type = 2
    return p


def calc_chiqw(root: str, params: Params) -> Report:
    rep = Report()
    rc = lib().orc_calc_chiqw(root.encode(), C.byref(params), C.byref(rep))
    if rc != 0:
        raise RuntimeError("oracle failed: " + lib().orc_last_error().decode())
    return rep


def read_chi_dump(path: str) -> np.ndarray:
    """dat.chi0 dump: int32 [NG, nen, ndir, npair] then complex128 (NG,NG,nen,ndir) column-major."""
    with open(path, "rb") as f:
        hdr = np.frombuffer(f.read(16), dtype=np.int32)
        ng, nen, ndir = int(hdr[0]), int(hdr[1]), int(hdr[2])
        data = np.frombuffer(f.read(), dtype=np.complex128)
    return data.reshape((ndir, nen, ng, ng)).transpose(3, 2, 1, 0)  # (ig, jg, ie, ix)


def fft3(a: np.ndarray, forward: bool) -> np.ndarray:
    """a indexed [x, y, z] (x fastest in memory via Fortran order)."""
    buf = np.asfortranarray(a.astype(np.complex128))
    n1, n2, n3 = buf.shape
    lib().orc_fft3(n1, n2, n3, buf.ctypes.data, 1 if forward else 0)
    return buf


def gen_grid(nt: int, e: float) -> np.ndarray:
    out = np.zeros(nt, dtype=np.complex128)
    lib().orc_gen_grid(nt, e, out.ctypes.data)
    return out


def zinv(a: np.ndarray) -> np.ndarray:
    buf = np.asfortranarray(a.astype(np.complex128))
    rc = lib().orc_zinv(buf.shape[0], buf.ctypes.data)
    if rc:
        raise np.linalg.LinAlgError("singular")
    return buf


def mkidx(nk: Sequence[int], bvec: np.ndarray) -> np.ndarray:
    n1, n2, n3 = nk
    out = np.zeros(4 * 6 * n1 * n2 * n3, dtype=np.int32)
    b = [np.ascontiguousarray(bvec[i], dtype=np.float64) for i in range(3)]
    lib().orc_ttrhdrn_mkidx(n1, n2, n3, b[0].ctypes.data, b[1].ctypes.data, b[2].ctypes.data, out.ctypes.data)
    return out


def ttrhdrn_chi0(dmna, dmnr, nk, imt1, e1, e2, f1, f2, delt, dsgn, em, xo=None):
    n1, n2, n3 = nk
    em = np.ascontiguousarray(em, dtype=np.complex128)
    e1 = np.ascontiguousarray(e1, dtype=np.float64)
    e2 = np.ascontiguousarray(e2, dtype=np.float64)
    if xo is None:
        xo = np.zeros((n1 * n2 * n3, em.size), dtype=np.complex128)
    rc = lib().orc_ttrhdrn_chi0(dmna, dmnr, n1, n2, n3, imt1.ctypes.data, e1.ctypes.data, e2.ctypes.data,
                                f1, f2, delt, dsgn, em.size, em.ctypes.data, xo.ctypes.data)
    if rc:
        raise RuntimeError(lib().orc_last_error().decode())
    return xo


def make_int_params(**kw) -> IntParams:
    p = IntParams()
    lib().orc_int_default_params(C.byref(p))
    box = kw.pop("fft_box", None)
    for k, v in kw.items():
        setattr(p, k, v)
    if box is not None:
        p.fft_box[0], p.fft_box[1], p.fft_box[2] = box
    return p


def calc_int(root: str, params: IntParams):
    """calc_w3d / calc_j3d restated: returns dims and V, W, X, J as complex arrays
    shaped (nwf, nwf, 2Na1+1, 2Na2+1, 2Na3+1[, ne]) in Fortran order."""
    dims = IntDims()
    p0 = IntParams.from_buffer_copy(params)
    p0.do_w = p0.do_j = p0.write_files = 0
    if lib().orc_calc_int(root.encode(), C.byref(p0), C.byref(dims), None, None, None, None):
        raise RuntimeError("oracle failed: " + lib().orc_last_error().decode())
    shape = (dims.nwf, dims.nwf, 2 * dims.na[0] + 1, 2 * dims.na[1] + 1, 2 * dims.na[2] + 1)
    out = {}
    bufs = []
    for name, extra in (("V", ()), ("W", (dims.ne,)), ("X", ()), ("J", (dims.ne,))):
        a = np.zeros(shape + extra, dtype=np.complex128, order="F")
        out[name] = a
        bufs.append(a.ctypes.data)
    if lib().orc_calc_int(root.encode(), C.byref(params), C.byref(dims), *bufs):
        raise RuntimeError("oracle failed: " + lib().orc_last_error().decode())
    return dims, out
