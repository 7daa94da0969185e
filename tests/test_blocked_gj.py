"""The blocked Gauss-Jordan update that gj_panel_kernel / gj_prows_kernel /
gj_trail_kernel implement, restated in numpy and checked against the
one-pivot-at-a-time elimination (partial pivoting on |re| + |im| among unused
rows, the unscrambled inverse as in gj_unscramble_kernel).

A panel of b columns runs its pivot steps alone; every other column x then
takes the b steps at once as x <- x - (E_P - Pan) x_P, i.e.
A[:, T] <- (A[:, T] with the pivot rows P zeroed) + Pan @ A_old[P, T],
because Gauss-Jordan leaves in panel column t the image of the unit vector of
pivot row P_t.  The GPU kernels are held to the FP64 oracle by the eps^-1
parity tests; this test pins the algebra they rely on."""
import numpy as np
import pytest


def _pivot(col, used):
    s = np.abs(col.real) + np.abs(col.imag)
    s[used] = -1.0
    return int(np.argmax(s))  # lowest row on ties, as the kernels


def _step(A, k, p):
    d = 1.0 / A[p, k]
    prow = A[p, :].copy()
    f = A[:, k] * d
    A -= np.outer(f, prow)
    A[:, k] = -f
    A[p, :] = prow * d
    A[p, k] = d


def gj_unblocked(A):
    A = A.copy()
    n = A.shape[0]
    used = np.zeros(n, bool)
    piv = []
    for k in range(n):
        p = _pivot(A[:, k], used)
        used[p] = True
        piv.append(p)
        _step(A, k, p)
    return A, piv


def gj_blocked(A, b):
    A = A.copy()
    n = A.shape[0]
    used = np.zeros(n, bool)
    piv = []
    for k0 in range(0, n, b):
        ks = list(range(k0, min(n, k0 + b)))
        pan = A[:, ks].copy()
        P = []
        for t, k in enumerate(ks):
            p = _pivot(pan[:, t], used)
            used[p] = True
            piv.append(p)
            P.append(p)
            _step(pan, t, p)
        T = [j for j in range(n) if j not in ks]
        a_old = A[np.ix_(P, T)].copy()          # gj_prows_kernel
        At = A[:, T]
        At[P, :] = 0.0                            # gj_trail_kernel
        A[:, T] = At + pan @ a_old
        A[:, ks] = pan
    return A, piv


def unscramble(A, piv):
    """inv(r, c) = A(piv[r], ipiv[c]) with ipiv[piv[k]] = k."""
    piv = np.asarray(piv)
    ipiv = np.empty_like(piv)
    ipiv[piv] = np.arange(len(piv))
    return A[piv][:, ipiv]


@pytest.mark.parametrize("n,b", [(70, 8), (61, 16), (33, 32), (40, 1), (17, 32)])
def test_blocked_matches_one_step_elimination(n, b):
    rng = np.random.default_rng(n * 100 + b)
    M = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    U, pu = gj_unblocked(M)
    B, pb = gj_blocked(M, b)
    assert pu == pb
    assert np.abs(U - B).max() <= 1e-12 * np.abs(U).max()
    X = unscramble(B, pb)
    assert np.abs(X @ M - np.eye(n)).max() < 1e-10


def test_blocked_pivots_rows_off_the_diagonal():
    """A matrix whose pivots are all off the diagonal (a scrambled, scaled
    permutation plus noise) takes the same pivots in both forms."""
    rng = np.random.default_rng(7)
    n = 24
    perm = rng.permutation(n)
    M = np.zeros((n, n), complex)
    M[perm, np.arange(n)] = 10.0 + rng.standard_normal(n)
    M += 0.1 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    U, pu = gj_unblocked(M)
    B, pb = gj_blocked(M, 5)
    assert pu == pb and pu != list(range(n))
    assert np.abs(unscramble(B, pb) - np.linalg.inv(M)).max() < 1e-12
