"""Copy the reference's sample namelist files into tests/golden/namelists/.

RESPACK ships no tests or golden outputs for the chiqw / calc_int path; the
only fixtures it holds are the stdin namelists of its samples
(sample/<dft>/<material>/input.in), each with the &param_chiqw and
&param_calc_int groups its programs read (src/chiqw/m_rdinput.f90:41-76,
src/calc_int/m_rdinput.f90:15-33) among the groups of its other programs.
They are copied unchanged, one file per sample, named <dft>_<material>.in.

Run in a checkout that holds the RESPACK tree (the path is the first argument,
default /root/reference); the copies are committed, so the tests need no
reference tree.
"""
from __future__ import annotations

import glob
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "namelists")


def main(src: str) -> None:
    os.makedirs(OUT, exist_ok=True)
    files = sorted(glob.glob(os.path.join(src, "sample", "*", "*", "input.in")))
    if not files:
        raise SystemExit(f"no sample/*/*/input.in under {src}")
    for f in files:
        dft = os.path.basename(os.path.dirname(os.path.dirname(f)))
        mat = os.path.basename(os.path.dirname(f))
        name = ("qe" if dft == "quantum-espresso" else dft) + "_" + mat.split(".")[0] + ".in"
        shutil.copyfile(f, os.path.join(OUT, name))
        print(name)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
