"""dir-wfn front end (respackdev_gb300/dirwfn.py): qe2respack's symmetry
conversion on known operations, and the validator on generated directories
and on copies broken in one place each."""
import os
import shutil
import struct
import subprocess
import sys

import numpy as np
import pytest

from respackdev_gb300 import dirwfn, synth

IDENT = [1, 0, 0, 0, 1, 0, 0, 0, 1]


def test_symmetry_identity_matches_the_written_file(case_dir):
    """The identity alone is the dat.symmetry every generated case carries
    (and the chiqw reader accepts)."""
    txt = dirwfn.symmetry_text([IDENT], [[0.0, 0.0, 0.0]])
    with open(os.path.join(case_dir("tiny"), "dir-wfn", "dat.symmetry")) as f:
        assert f.read() == txt


def test_symmetry_translations_and_inverse():
    # a glide (mirror + half translation) and a 3-fold rotation with thirds:
    # the common denominator of 1/2 and 1/3 is 6
    mirror = [-1, 0, 0, 0, 1, 0, 0, 0, 1]
    c3 = [0, 1, 0, 0, 0, 1, 1, 0, 0]   # columns (0,1,0), (0,0,1), (1,0,0)
    txt = dirwfn.symmetry_text([IDENT, mirror, c3], [[0, 0, 0], [0.5, 0, 0], [1 / 3, 2 / 3, 0]])
    lines = txt.splitlines()
    assert lines[0] == "    3" and lines[1] == "    6"
    assert lines[2] == "  1  0  0  0  1  0  0  0  1" and lines[3] == "  0  0  0"
    assert lines[4] == " -1  0  0  0  1  0  0  0  1" and lines[5] == " -3  0  0"   # -nint(6 * 0.5)
    # the inverse of a permutation matrix is its transpose
    m = np.array(c3).reshape(3, 3).T
    inv = np.array([int(lines[6][3 * i:3 * i + 3]) for i in range(9)]).reshape(3, 3).T
    assert np.array_equal(inv, np.linalg.inv(m).round().astype(int)) and np.array_equal(inv, m.T)
    assert lines[7] == " -2 -4  0"
    # halves round away from zero like IDNINT
    assert dirwfn._nint([0.5, -0.5, 1.5, -2.5]).tolist() == [1, -1, 2, -3]


def test_symmetry_errors():
    with pytest.raises(ValueError, match="common denominator"):
        dirwfn.symmetry_text([IDENT], [[np.sqrt(2) / 10, 0, 0]])
    with pytest.raises(ValueError, match="not integral"):
        dirwfn.symmetry_text([[2, 0, 0, 0, 1, 0, 0, 0, 1]], [[0, 0, 0]])


@pytest.mark.parametrize("case", ["tiny", "tiny_odd", "tiny_metal"])
def test_generated_cases_validate(case_dir, case):
    assert dirwfn.validate(case_dir(case)) == []


def _copy(case_dir, tmp_path, case="tiny"):
    dst = os.path.join(str(tmp_path), case)
    shutil.copytree(os.path.join(case_dir(case), "dir-wfn"), os.path.join(dst, "dir-wfn"))
    return dst, os.path.join(dst, "dir-wfn")


def test_validator_finds_each_break(case_dir, tmp_path):
    root, w = _copy(case_dir, tmp_path)
    nkm = open(os.path.join(w, "dat.nkm")).read().split()
    # 1. a plane-wave count that disagrees with dat.kg and dat.wfn
    with open(os.path.join(w, "dat.nkm"), "w") as f:
        f.write("".join("%12d\n" % (int(x) + (1 if i == 2 else 0)) for i, x in enumerate(nkm)))
    p = dirwfn.validate(root)
    assert any("k 3: dat.kg holds" in x for x in p), p
    shutil.rmtree(root)

    # 2. a G far outside the cutoff sphere
    root, w = _copy(case_dir, tmp_path)
    lines = open(os.path.join(w, "dat.kg")).read().splitlines()
    lines[1] = "%12d%12d%12d" % (40, 0, 0)
    open(os.path.join(w, "dat.kg"), "w").write("\n".join(lines) + "\n")
    assert any("outside the cutoff sphere" in x for x in dirwfn.validate(root))
    shutil.rmtree(root)

    # 3. a band scaled by 1.1: not orthonormal
    root, w = _copy(case_dir, tmp_path)
    recs = dirwfn._records(os.path.join(w, "dat.wfn"))
    c = np.frombuffer(recs[3], dtype="<c16") * 1.1
    recs[3] = c.tobytes()
    with open(os.path.join(w, "dat.wfn"), "wb") as f:
        for r in recs:
            f.write(struct.pack("<i", len(r)) + r + struct.pack("<i", len(r)))
    assert any("not orthonormal" in x for x in dirwfn.validate(root))
    assert dirwfn.validate(root, check_orthonormal=False) == []
    shutil.rmtree(root)

    # 4. a truncated dat.wfn
    root, w = _copy(case_dir, tmp_path)
    path = os.path.join(w, "dat.wfn")
    data = open(path, "rb").read()
    open(path, "wb").write(data[:-100])
    assert any("dat.wfn" in x for x in dirwfn.validate(root))
    shutil.rmtree(root)

    # 5. eigenvalues out of order, and a missing file
    root, w = _copy(case_dir, tmp_path)
    ev = open(os.path.join(w, "dat.eigenvalue")).read().splitlines()
    ev[1], ev[2] = ev[2], ev[1]
    open(os.path.join(w, "dat.eigenvalue"), "w").write("\n".join(ev) + "\n")
    assert any("not ascending" in x for x in dirwfn.validate(root))
    os.remove(os.path.join(w, "dat.lattice"))
    assert dirwfn.validate(root) == ["missing dat.lattice"]
    shutil.rmtree(root)

    # 6. a rotation that is not a symmetry of the fcc lattice (a shear)
    root, w = _copy(case_dir, tmp_path)
    open(os.path.join(w, "dat.symmetry"), "w").write("    1\n    1\n  1  1  0  0  1  0  0  0  1\n  0  0  0\n")
    assert any("not a symmetry of the lattice" in x for x in dirwfn.validate(root))


def test_cli_exit_status(case_dir, tmp_path):
    env = dict(os.environ, PYTHONPATH=os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    r = subprocess.run([sys.executable, "-m", "respackdev_gb300.dirwfn", case_dir("tiny")], capture_output=True,
                       text=True, env=env)
    assert r.returncode == 0 and "dir-wfn ok" in r.stdout
    root, w = _copy(case_dir, tmp_path)
    os.remove(os.path.join(w, "dat.kg"))
    r = subprocess.run([sys.executable, "-m", "respackdev_gb300.dirwfn", root], capture_output=True, text=True,
                       env=env)
    assert r.returncode == 1 and "missing dat.kg" in r.stdout
