"""Python mirror of the C ABI in include/respack_gb300.h (ctypes).

Names and argument meanings follow the reference's calc_chiqw
(src/chiqw/chiqw.F): ``Context.chi0_q(iq)`` returns the array ``chiqw`` of
chiqw.F:1476 (``chiqwgm`` of :1989 at Gamma) for the iq-th entry of
dat.sample-k, ``Context.epsinv_q()`` the inverse dielectric matrix written to
dat.epsqw.600, ``calc_chiqw(root, namelist)`` the whole program.  Errors raise
``RuntimeError`` with the library's message; there is no CPU path: without the
built library or a CUDA device every call fails.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

PREC_FP64, PREC_FP16X2, PREC_BF16X3, PREC_FP16X3 = 0, 1, 2, 3


def library_path() -> str:
    return os.path.join(HERE, "lib", "librespack_gb300.so")


class Params(C.Structure):
    _fields_ = [
        ("n_calc_band", C.c_int), ("ecut_for_eps", C.c_double), ("shift_ef", C.c_double),
        ("max_excitation_energy", C.c_double), ("green_func_delt", C.c_double), ("ttrhdrn_dmna", C.c_double),
        ("ttrhdrn_dmnr", C.c_double), ("num_freq_grid", C.c_int), ("lower_bound_energy_window", C.c_double),
        ("upper_bound_energy_window", C.c_double), ("flg_crpa", C.c_int), ("flg_calc_type", C.c_int),
        ("file_num_log_start", C.c_int), ("file_num_eps_start", C.c_int), ("file_num_eps_base_start", C.c_int),
        ("n_calc_q", C.c_int), ("mpi_num_qcomm", C.c_int), ("precision", C.c_int), ("fft_box", C.c_int * 3),
        ("dump_chi", C.c_int), ("device", C.c_int), ("max_pairs", C.c_int), ("qshard_index", C.c_int),
        ("qshard_count", C.c_int), ("pair_fp64", C.c_int), ("tc_ksub", C.c_int),
        ("pair_batch", C.c_int), ("tc_split", C.c_int), ("tc_pair", C.c_int), ("write_eps_f32", C.c_int), ("eps_fp64", C.c_int),
        ("tetra_fp64", C.c_int), ("ur_window", C.c_int), ("tail_model", C.c_char * 256),
    ]


class Info(C.Structure):
    _fields_ = [("ntk", C.c_int), ("nk_irr", C.c_int), ("nkb", C.c_int * 3), ("ntg", C.c_int), ("ntb", C.c_int),
                ("ncb", C.c_int), ("nen", C.c_int), ("n_occ", C.c_int), ("n_vir", C.c_int), ("n_docc", C.c_int),
                ("n_pocc", C.c_int), ("n_uocc", C.c_int), ("fft_box", C.c_int * 3), ("volume", C.c_double),
                ("efermi", C.c_double), ("ecut_psi", C.c_double), ("ecut_eps", C.c_double),
                ("device_bytes", C.c_double)]


_lib: Optional[C.CDLL] = None


def load() -> C.CDLL:
    """Load the in-tree library (built by respackdev_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m respackdev_gb300.build`")
    L = C.CDLL(path)
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.rp_default_params.argtypes = [C.POINTER(Params)]
    L.rp_parse_namelist.argtypes = [C.c_char_p, C.POINTER(Params), ip, C.c_int, ip, dp, C.c_int, ip]
    L.rp_parse_namelist.restype = C.c_int
    L.rp_parse_error.restype = C.c_char_p
    L.rp_ctx_create.argtypes = [C.POINTER(vp), C.c_char_p, C.POINTER(Params), dp, C.c_int]
    L.rp_ctx_create.restype = C.c_int
    L.rp_ctx_info.argtypes = [vp, C.POINTER(Info)]
    L.rp_num_qirr.argtypes = [vp]
    L.rp_chi0_q.argtypes = [vp, C.c_int, vp, ip, ip]
    L.rp_chi0_q.restype = C.c_int
    L.rp_epsinv_q.argtypes = [vp, vp]
    L.rp_epsinv_q.restype = C.c_int
    L.rp_epsinv_chi_q.argtypes = [vp, vp, vp]
    L.rp_epsinv_chi_q.restype = C.c_int
    L.rp_tail_applied.argtypes = [vp]
    L.rp_tail_applied.restype = C.c_int
    L.rp_write_q.argtypes = [vp, C.c_char_p]
    L.rp_write_q.restype = C.c_int
    L.rp_calc_chiqw.argtypes = [C.c_char_p, C.c_char_p]
    L.rp_calc_chiqw.restype = C.c_int
    L.rp_stage_times.argtypes = [vp, dp]
    L.rp_q_dims.argtypes = [vp, C.c_int, ip, ip]
    L.rp_q_dims.restype = C.c_int
    L.rp_kernel_launches.argtypes = [vp]
    L.rp_kernel_launches.restype = C.c_longlong
    L.rp_transfer_bytes.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    L.rp_transfer_bytes.restype = C.c_int
    L.rp_eps_fallback.argtypes = [vp]
    L.rp_eps_fallback.restype = C.c_int
    L.rp_chi0_batch.argtypes = [C.POINTER(vp), ip, C.c_int, C.c_int, C.POINTER(vp), ip, ip, dp]
    L.rp_chi0_batch.restype = C.c_int
    L.rp_tuned_shapes.restype = C.c_int
    L.rp_reset_tuner.restype = None
    L.rp_zinv_batched_noalloc.argtypes = [vp, vp, C.c_int, C.c_int, vp]
    L.rp_zinv_batched_noalloc.restype = C.c_int
    L.rp_last_error.argtypes = [vp]
    L.rp_last_error.restype = C.c_char_p
    L.rp_ctx_destroy.argtypes = [vp]
    _lib = L
    return L


def default_params(**kw) -> Params:
    p = Params()
    load().rp_default_params(C.byref(p))
    for k, v in kw.items():
        if k == "fft_box":
            p.fft_box[0], p.fft_box[1], p.fft_box[2] = v
        elif k == "tail_model":
            p.tail_model = v.encode() if isinstance(v, str) else v
        else:
            setattr(p, k, v)
    return p


def parse_namelist(text: str):
    """(Params, q list, explicit frequencies in Hartree or None) of a namelist text."""
    L = load()
    p = Params()
    L.rp_default_params(C.byref(p))
    q = (C.c_int * 4096)()
    em = (C.c_double * 8192)()
    nq, ne = C.c_int(0), C.c_int(0)
    rc = L.rp_parse_namelist(text.encode(), C.byref(p), q, 4096, C.byref(nq), em, 4096, C.byref(ne))
    if rc:
        raise ValueError(L.rp_parse_error().decode())
    ems = None
    if ne.value:
        a = np.ctypeslib.as_array(em)[: 2 * ne.value]
        ems = a[0::2] + 1j * a[1::2]
    return p, list(q[: nq.value]), ems


class Context:
    """A device context of one run directory (dir-wfn, dir-wan)."""

    def __init__(self, root: str, params: Params, em: Optional[Sequence[complex]] = None):
        self.L = load()
        self.root = root
        self.params = params
        self._h = C.c_void_p()
        emarr = None
        n = 0
        if em is not None:
            emarr = np.ascontiguousarray(np.asarray(em, dtype=np.complex128))
            n = emarr.size
        ptr = emarr.ctypes.data_as(C.POINTER(C.c_double)) if emarr is not None else None
        rc = self.L.rp_ctx_create(C.byref(self._h), root.encode(), C.byref(params), ptr, n)
        if rc:
            raise RuntimeError(f"rp_ctx_create failed ({rc}): {self.L.rp_last_error(None).decode()}")
        self.ng = 0
        self.ndir = 1

    def _check(self, rc: int, what: str):
        if rc:
            raise RuntimeError(f"{what} failed ({rc}): {self.L.rp_last_error(self._h).decode()}")

    def info(self) -> Info:
        inf = Info()
        self.L.rp_ctx_info(self._h, C.byref(inf))
        return inf

    def q_dims(self, iq: int):
        ng, nd = C.c_int(0), C.c_int(0)
        self._check(self.L.rp_q_dims(self._h, iq, C.byref(ng), C.byref(nd)), "rp_q_dims")
        return ng.value, nd.value

    def chi0_q(self, iq: int, fetch: bool = True) -> Optional[np.ndarray]:
        """chi0 (after /VOLUME, before the spin factor) as (ng, ng, nen, ndir), column-major G order."""
        ng, nd = self.q_dims(iq)
        nen = self.info().nen
        out = np.empty(nd * nen * ng * ng, dtype=np.complex128) if fetch else None
        ngo, ndo = C.c_int(0), C.c_int(0)
        self._check(self.L.rp_chi0_q(self._h, iq, out.ctypes.data if fetch else None, C.byref(ngo), C.byref(ndo)),
                    "rp_chi0_q")
        self.ng, self.ndir = ngo.value, ndo.value
        if not fetch:
            return None
        return out.reshape(nd, nen, ng, ng).transpose(3, 2, 1, 0)

    def epsinv_q(self, fetch: bool = True) -> Optional[np.ndarray]:
        nen = self.info().nen
        if not fetch:
            self._check(self.L.rp_epsinv_q(self._h, None), "rp_epsinv_q")
            return None
        out = np.empty(self.ndir * nen * self.ng * self.ng, dtype=np.complex128)
        self._check(self.L.rp_epsinv_q(self._h, out.ctypes.data), "rp_epsinv_q")
        return out.reshape(self.ndir, nen, self.ng, self.ng).transpose(3, 2, 1, 0)

    def epsinv_chi_q(self, chi: np.ndarray, fetch: bool = True) -> Optional[np.ndarray]:
        """eps^-1 of the last chi0_q's q point from a caller chi0 shaped like chi0_q's."""
        nen = self.info().nen
        a = np.asarray(chi, dtype=np.complex128)
        if a.ndim == 3:
            a = a[..., None]
        if a.shape != (self.ng, self.ng, nen, self.ndir):
            raise ValueError(f"chi0 must be {(self.ng, self.ng, nen, self.ndir)}, got {a.shape}")
        buf = np.ascontiguousarray(a.transpose(3, 2, 1, 0))
        out = np.empty(self.ndir * nen * self.ng * self.ng, dtype=np.complex128) if fetch else None
        self._check(self.L.rp_epsinv_chi_q(self._h, buf.ctypes.data, out.ctypes.data if fetch else None),
                    "rp_epsinv_chi_q")
        if not fetch:
            return None
        return out.reshape(self.ndir, nen, self.ng, self.ng).transpose(3, 2, 1, 0)

    def tail_applied(self) -> bool:
        """True if the last chi0_q added the band-tail network's correction."""
        return bool(self.L.rp_tail_applied(self._h))

    def write_q(self, root: Optional[str] = None):
        self._check(self.L.rp_write_q(self._h, (root or self.root).encode()), "rp_write_q")

    def stage_times(self) -> np.ndarray:
        t = (C.c_double * 6)()
        self.L.rp_stage_times(self._h, t)
        return np.array(t[:])

    def tc_gram_seconds(self) -> float:
        """Device time of the tensor-core Gram kernel in the last chi0_q."""
        return float(self.stage_times()[5])

    def kernel_launches(self) -> int:
        return int(self.L.rp_kernel_launches(self._h))

    def eps_fallback(self) -> bool:
        """True if the last epsinv_q fell back from the mixed-precision to the FP64 inversion."""
        return bool(self.L.rp_eps_fallback(self._h))

    def transfer_bytes(self):
        """(host->device, device->host) bytes copied by this context's calls so far."""
        h, d = C.c_longlong(0), C.c_longlong(0)
        self.L.rp_transfer_bytes(self._h, C.byref(h), C.byref(d))
        return int(h.value), int(d.value)

    def close(self):
        if self._h:
            self.L.rp_ctx_destroy(self._h)
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


def calc_chiqw(root: str, namelist_text: str) -> None:
    """The whole calc_chiqw run in ``root`` (as ``calc_chiqw < input.in`` there)."""
    L = load()
    rc = L.rp_calc_chiqw(root.encode(), namelist_text.encode())
    if rc:
        raise RuntimeError(f"rp_calc_chiqw failed ({rc}): {L.rp_last_error(None).decode()}")


def plan_q(root: str, namelist_text: str) -> list:
    """1-based q points a calc_chiqw run with this namelist would compute in
    ``root`` (its &param_gpu q shard included).  Host only: needs no GPU."""
    L = load()
    L.rp_plan_q.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int)]
    L.rp_plan_q.restype = C.c_int
    cap = 4096
    buf = (C.c_int * cap)()
    n = C.c_int(0)
    rc = L.rp_plan_q(root.encode(), namelist_text.encode(), buf, cap, C.byref(n))
    if rc:
        raise RuntimeError(f"rp_plan_q failed ({rc}): {L.rp_last_error(None).decode()}")
    return list(buf[: min(n.value, cap)])


def chi0_batch(problems: Sequence, graph: bool = True, fetch: bool = True):
    """chi0 of a ragged batch: problems is a list of (Context, iq).  Every
    problem is prepared, then one tensor-core launch covers them all (inside a
    CUDA graph when graph is true).  Returns (list of chi0 arrays shaped like
    Context.chi0_q's, or None when fetch is false; seconds
    [preparation, graph device time, finishing])."""
    L = load()
    n = len(problems)
    if n == 0:
        return [], np.zeros(3)
    ctxs = (C.c_void_p * n)(*[c._h.value for c, _ in problems])
    iqs = (C.c_int * n)(*[int(iq) for _, iq in problems])
    outs, ptrs = [], (C.c_void_p * n)()
    if fetch:
        for i, (c, iq) in enumerate(problems):
            ng, nd = c.q_dims(iq)
            a = np.empty(nd * c.info().nen * ng * ng, dtype=np.complex128)
            outs.append(a)
            ptrs[i] = a.ctypes.data
    ngo, ndo = (C.c_int * n)(), (C.c_int * n)()
    sec = (C.c_double * 3)()
    rc = L.rp_chi0_batch(ctxs, iqs, n, 1 if graph else 0, ptrs if fetch else None, ngo, ndo, sec)
    if rc:
        raise RuntimeError(f"rp_chi0_batch failed ({rc}): {L.rp_last_error(problems[0][0]._h).decode()}")
    res = None
    if fetch:
        res = []
        for i, (c, _) in enumerate(problems):
            ng, nd, nen = ngo[i], ndo[i], c.info().nen
            res.append(outs[i].reshape(nd, nen, ng, ng).transpose(3, 2, 1, 0))
    return res, np.array(sec[:])


def tuned_shapes() -> int:
    """Shapes the tensor-core K-split tuner has measured in this process."""
    return int(load().rp_tuned_shapes())


def reset_tuner() -> None:
    load().rp_reset_tuner()
