"""calc_int on the GPU (rp_int_* of the C ABI) against the oracle: V, W of
calc_w3d and X, J of calc_j3d, the executables and their files."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as orc
from respackdev_gb300 import build as rp_build
from respackdev_gb300 import calc_int as ci
from tests.helpers import read_int_matrix

pytestmark = pytest.mark.gpu

# V, W, X, J relative to their largest element: the pair densities are rounded
# to single precision like the reference, everything after them is FP64
TOL = 1e-6


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("case,jr", [("tiny_wan", (0, 0)), ("tiny_wan", (-1, 1)), ("odd_wan", (-1, 1))])
def test_vwxj_match_oracle(case, jr, int_case, int_copy):
    src = int_case(case)
    root = int_copy(src)
    dims, ref = orc.calc_int(root, orc.make_int_params(nthreads=4, ix_min=jr[0], ix_max=jr[1], write_files=0))
    p = ci.default_params(ix_intj_min=jr[0], ix_intj_max=jr[1], write_files=0)
    with ci.IntContext(root, p) as c:
        assert (c.nwf, c.ne, c.na) == (dims.nwf, dims.ne, tuple(dims.na))
        V, W = c.w3d()
        X, J = c.j3d()
        t = c.stage_times()
    for name, got in (("V", V), ("W", W), ("X", X), ("J", J)):
        err = _rel(got, ref[name])
        assert err < TOL, f"{case} {name}: {err:.3e}"
    assert t[4] > 0


def test_executables_write_the_files(int_case, int_copy):
    rp_build.build()
    root = int_copy(int_case("tiny_wan"))
    nl = "&param_calc_int\n calc_ifreq=2, ix_intJ_min=0, ix_intJ_max=1, wcut_mvmc=0.5, jcut_mvmc=0.01 /\n"
    for prog in ("rp_calc_w3d", "rp_calc_j3d"):
        r = subprocess.run([os.path.join(rp_build.BINDIR, prog)], input=nl, text=True,
                           cwd=root, capture_output=True, timeout=600)
        assert r.returncode == 0, r.stderr
    dims, ref = orc.calc_int(root, orc.make_int_params(nthreads=4, ix_min=0, ix_max=1, calc_ifreq=2, write_files=0))
    na = tuple(dims.na)
    AU = 27.21151
    Vf = read_int_matrix(os.path.join(root, "dir-intW", "dat.Vmat"), dims.nwf)
    Jf = read_int_matrix(os.path.join(root, "dir-intJ", "dat.Jmat"), dims.nwf)
    scale = np.abs(ref["V"]).max() * AU
    for R, M in Vf.items():
        idx = tuple(r + n for r, n in zip(R, na))
        assert np.abs(M - ref["V"][(slice(None), slice(None)) + idx] * AU).max() < TOL * scale + 1e-9
    for R, M in Jf.items():
        idx = tuple(r + n for r, n in zip(R, na))
        assert np.abs(M - ref["J"][(slice(None), slice(None)) + idx + (1,)] * AU).max() < TOL * scale + 1e-9
    for f in ("zCoulombIntra.def", "zCoulombInter.def", "zHund.def", "zExchange.def", "zPairHop.def"):
        assert os.path.exists(os.path.join(root, "dir-mvmc", f))
    for f in ("dat.Wmat", "dat.VvsR.001", "dat.WvsR.003", "dat.UvsE.001-003"):
        assert os.path.exists(os.path.join(root, "dir-intW", f))


def test_bad_range_is_an_input_error(int_case, int_copy):
    root = int_copy(int_case("tiny_wan"))
    p = ci.default_params(ix_intj_min=-3, ix_intj_max=3, write_files=0)
    with ci.IntContext(root, p) as c:
        with pytest.raises(RuntimeError, match="intJ range"):
            c.j3d()


def test_complex4_eps_side_file_gives_the_same_w(int_case, int_copy):
    """dir-eps written by rp_calc_chiqw with write_eps_f32=1 carries
    dat.epsqw.c4 beside the FP64 records: complex(4) eps^-1 (Gamma: the mean
    of the three directions), what calc_int keeps of eps^-1 anyway.  W and J
    from the side files equal W and J from the FP64 records exactly, and the
    side file is half an FP64 record."""
    import shutil
    from respackdev_gb300 import chiqw as rp
    from tests.helpers import EM_INT, namelist_text
    root = int_copy(int_case("tiny_wan"))
    shutil.rmtree(os.path.join(root, "dir-eps"))
    rp.calc_chiqw(root, namelist_text(dict(green_func_delt=0.2721, ecut_for_eps=3.0), EM_INT,
                                      "precision='fp64', write_eps_f32=1"))
    qdirs = sorted(d for d in os.listdir(os.path.join(root, "dir-eps")) if d.startswith("q"))
    assert qdirs
    for q in qdirs:
        c4 = os.path.getsize(os.path.join(root, "dir-eps", q, "dat.epsqw.c4"))
        f8 = os.path.getsize(os.path.join(root, "dir-eps", q, "dat.epsqw.600"))
        assert c4 - 8 == (f8 - 8) // 2, (q, c4, f8)   # payload halves (4-byte record markers)
    out = {}
    for use in (0, 1):
        p = ci.default_params(ix_intj_min=0, ix_intj_max=1, write_files=0, read_eps_f32=use)
        with ci.IntContext(root, p) as c:
            out[use] = (c.w3d(), c.j3d())
    (V0, W0), (X0, J0) = out[0]
    (V1, W1), (X1, J1) = out[1]
    assert np.array_equal(V0, V1) and np.array_equal(X0, X1)
    assert np.array_equal(W0, W1) and np.array_equal(J0, J1)



def _def_entries(path):
    """Header lines, then (integer index tokens, value) of every data line of a z*.def file."""
    lines = open(path).read().splitlines()
    head, rows = lines[:5], []
    for ln in lines[5:]:
        tok = ln.split()
        if tok:
            rows.append((tuple(int(x) for x in tok[:-1]), float(tok[-1])))
    return head, rows


def test_mvmc_files_match_oracle_writer(int_case, int_copy, tmp_path):
    """dir-mvmc written by rp_calc_w3d + rp_calc_j3d against the oracle's
    restatement of wrt_mvmc (wrt_mvmc_w3d.f90:1-147, wrt_mvmc_j3d.f90): the
    same files, headers (counts and cuts) and site pairs, values within the
    calc_int tolerance."""
    import shutil
    rp_build.build()
    src = int_case("tiny_wan")
    gpu_root = int_copy(src)
    orc_root = str(tmp_path / "oracle_copy")
    for sub in ("dir-wfn", "dir-wan", "dir-eps"):
        shutil.copytree(os.path.join(src, sub), os.path.join(orc_root, sub))
    nl = "&param_calc_int\n calc_ifreq=2, ix_intJ_min=0, ix_intJ_max=1, wcut_mvmc=0.5, jcut_mvmc=0.01 /\n"
    for prog in ("rp_calc_w3d", "rp_calc_j3d"):
        r = subprocess.run([os.path.join(rp_build.BINDIR, prog)], input=nl, text=True,
                           cwd=gpu_root, capture_output=True, timeout=600)
        assert r.returncode == 0, r.stderr
    orc.calc_int(orc_root, orc.make_int_params(nthreads=4, ix_min=0, ix_max=1, calc_ifreq=2, wcut_mvmc=0.5,
                                               jcut_mvmc=0.01, write_files=1))
    names = sorted(os.listdir(os.path.join(orc_root, "dir-mvmc")))
    assert names == sorted(os.listdir(os.path.join(gpu_root, "dir-mvmc")))
    assert len(names) == 5
    for name in names:
        h1, r1 = _def_entries(os.path.join(gpu_root, "dir-mvmc", name))
        h2, r2 = _def_entries(os.path.join(orc_root, "dir-mvmc", name))
        assert h1 == h2, name
        assert [i for i, _ in r1] == [i for i, _ in r2], name
        v1 = np.array([v for _, v in r1])
        v2 = np.array([v for _, v in r2])
        assert r2, name
        assert np.abs(v1 - v2).max() <= TOL * np.abs(v2).max() + 1e-9, name


def test_static_uj_of_the_fast_path_within_5_mev(int_case, int_copy):
    """Five Gaussian Wannier orbitals: dir-eps from the split-precision chiqw
    (FP16x3 contraction, FP32-series tetrahedron weights, mixed-precision
    inverse) and the GPU calc_int, against the oracle's FP64 chiqw and calc_int.
    The static U (W at R = 0, w = 0) and J (J at R = 0, w = 0) agree within
    the 5 meV the fast path is held to (they agree far better)."""
    import shutil
    from respackdev_gb300 import chiqw as rp
    from tests.helpers import EM_INT, namelist_text
    src = int_case("wan5")
    AU = 27.21151
    dims, ref = orc.calc_int(src, orc.make_int_params(nthreads=8, ix_min=0, ix_max=1, write_files=0))
    root = int_copy(src)
    shutil.rmtree(os.path.join(root, "dir-eps"))
    rp.calc_chiqw(root, namelist_text(dict(green_func_delt=0.2721, ecut_for_eps=3.0), EM_INT, "precision='fp16x3'"))
    p = ci.default_params(ix_intj_min=0, ix_intj_max=1, write_files=0)
    with ci.IntContext(root, p) as c:
        assert c.nwf == 5
        V, W = c.w3d()
        X, J = c.j3d()
    c0 = tuple(dims.na)
    U_gpu, U_ref = W[:, :, c0[0], c0[1], c0[2], 0], ref["W"][:, :, c0[0], c0[1], c0[2], 0]
    J_gpu, J_ref = J[:, :, c0[0], c0[1], c0[2], 0], ref["J"][:, :, c0[0], c0[1], c0[2], 0]
    du = float(np.abs(U_gpu - U_ref).max()) * AU * 1e3
    dj = float(np.abs(J_gpu - J_ref).max()) * AU * 1e3
    print(f"static U/J, 5 orbitals: max |dU| {du:.3e} meV, max |dJ| {dj:.3e} meV "
          f"(U up to {np.abs(U_ref).max() * AU:.3f} eV)")
    assert du < 5.0 and dj < 5.0
    # the bare V does not depend on eps^-1: the GPU's equals the oracle's
    assert _rel(V, ref["V"]) < TOL
