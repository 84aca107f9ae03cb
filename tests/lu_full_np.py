"""Vectorised restatement of mat_lu's full-pivoting elimination
(mat.h:4476-4574, scalar branch) for test sizes the scalar oracle cannot
reach in seconds.  Every operation rounds as the reference's does: the
multiplier is a_ik * (1 / a_kk), each product l * u is rounded before it is
subtracted, and the pivot is the first entry (row-major from (k, k)) of the
largest magnitude, NaN never winning.  Pinned against the scalar oracle by
tests/test_oracle.py."""
import numpy as np


def lu_full_np(A, eps):
    """Returns (packed LU, row pivots, column pivots, swaps): rowpiv[k] /
    colpiv[k] = the row / column swapped into position k at step k."""
    dt = A.dtype.type
    M = np.array(A, dtype=A.dtype, order="C", copy=True)
    n = M.shape[0]
    rowpiv = np.arange(n)
    colpiv = np.arange(n)
    swaps = 0
    for k in range(n - 1):
        akk = M[k, k]
        pr = pc = k
        if np.isnan(akk):
            mx = akk
        else:
            mag = np.abs(M[k:, k:])
            mag[np.isnan(mag)] = -1
            f = int(np.argmax(mag))
            i, j = divmod(f, n - k)
            mx = abs(akk)
            if mag[i, j] > mx:
                pr, pc, mx = k + i, k + j, mag[i, j]
        if mx < eps:
            continue
        if pr != k:
            M[[k, pr], :] = M[[pr, k], :]
            swaps += 1
        if pc != k:
            M[:, [k, pc]] = M[:, [pc, k]]
            swaps += 1
        rowpiv[k], colpiv[k] = pr, pc
        inv = dt(1) / M[k, k]
        M[k + 1:, k] = M[k + 1:, k] * inv
        M[k + 1:, k + 1:] -= np.multiply.outer(M[k + 1:, k], M[k, k + 1:])
    return M, rowpiv, colpiv, swaps


def perms(rowpiv, colpiv):
    """mat_lu's p and q from the recorded swaps (mat.h:4530-4545)."""
    n = len(rowpiv)
    p, q = np.arange(n), np.arange(n)
    for k in range(n - 1):
        p[[k, rowpiv[k]]] = p[[rowpiv[k], k]]
        q[[k, colpiv[k]]] = q[[colpiv[k], k]]
    return p, q
