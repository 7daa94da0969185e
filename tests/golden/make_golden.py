"""Generate the golden chi0 / eps^-1 fixtures of the parity tests.

The reference (Fortran + MPI + MKL) has no test vectors and cannot be built in
this image, so the fixtures are outputs of the C restatement of the reference
(oracle/) on seeded synthetic inputs.  They pin the oracle and the GPU library
against silent drift: the synthetic generator (checked through the SHA-256 of
the files it writes), the oracle (bitwise-close) and the library (within the
parity tolerance) must all keep reproducing them.

Usage:  python tests/golden/make_golden.py      (rewrites tests/golden/*.npz)
"""
from __future__ import annotations

import hashlib
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# case name -> (run parameters, q points)
GOLDEN = {
    "tiny": (dict(green_func_delt=0.2721, ecut_for_eps=3.0), [1, 2, 5]),
    "tiny_metal": (dict(green_func_delt=0.2721, ecut_for_eps=3.0, flg_crpa=1), [1, 3]),
}
AU = 27.21151
EM = np.concatenate([np.array([0.0, 1.5, 4.0, 10.0]) / AU, [0.5j / AU]]).astype(np.complex128)
INPUT_FILES = ["dir-wfn/dat.wfn", "dir-wfn/dat.eigenvalue", "dir-wfn/dat.kg", "dir-wfn/dat.sample-k",
               "dir-wfn/dat.lattice", "dir-wan/dat.umat"]


def input_digest(root: str) -> str:
    h = hashlib.sha256()
    for f in INPUT_FILES:
        p = os.path.join(root, f)
        if os.path.exists(p):
            with open(p, "rb") as fh:
                h.update(f.encode())
                h.update(fh.read())
    return h.hexdigest()


def golden_path(case: str) -> str:
    return os.path.join(HERE, f"chiqw_{case}.npz")


def compute(case: str, root: str) -> dict:
    """Run the oracle on a generated case; returns the arrays a fixture holds."""
    from oracle import oracle as orc
    from tests.helpers import read_eps_record

    kw, qs = GOLDEN[case]
    orc.calc_chiqw(root, orc.make_params(em=EM, dump_chi=1, nthreads=4, calc_num_k=qs, **kw))
    out = {"em": EM, "qs": np.array(qs), "digest": np.array(input_digest(root))}
    for iq in qs:
        qd = os.path.join(root, "dir-eps", "q%03d" % iq)
        chi = orc.read_chi_dump(os.path.join(qd, "dat.chi0"))
        ng, nen, ndir = chi.shape[0], chi.shape[2], chi.shape[3]
        eps = np.stack([read_eps_record(os.path.join(qd, "dat.epsqw.%d" % (600 + d)), ng, nen)
                        for d in range(ndir)], axis=-1)
        out[f"chi0_q{iq}"] = chi
        out[f"epsinv_q{iq}"] = eps
    return out


def main():
    from oracle import oracle as orc
    from respackdev_gb300 import synth

    orc.build()
    for case in GOLDEN:
        tmp = tempfile.mkdtemp(prefix="rp_golden_")
        try:
            synth.make_case(tmp, synth.CASES[case])
            arrs = compute(case, tmp)
            np.savez_compressed(golden_path(case), **arrs)
            print(case, os.path.getsize(golden_path(case)), "bytes")
        finally:
            shutil.rmtree(tmp, ignore_errors=True)


if __name__ == "__main__":
    main()
