"""The batched-solve workload (100,000 systems of orders U{4..128}, half
general U[-1,1] + n*I solved by LU, half SPD B^T B + n*I solved by Cholesky,
float32, one right-hand side each), packed as matgb_solve_batched_dev takes
it: matrices back to back (column-major, leading dimension = order) with
their offsets, right-hand sides likewise.  Shared by bench.py and the
schedule tuner."""
import numpy as np


def make(count=100000, seed=1005, dtype=np.float32):
    rs = np.random.default_rng(seed)
    ns = rs.integers(4, 129, count).astype(np.int32)
    kinds = (np.arange(count) % 2).astype(np.uint8)
    offA = np.zeros(count, np.int64)
    offA[1:] = np.cumsum(ns.astype(np.int64) ** 2)[:-1]
    offv = np.zeros(count, np.int64)
    offv[1:] = np.cumsum(ns.astype(np.int64))[:-1]
    totA = int(offA[-1] + ns[-1] ** 2)
    totv = int(offv[-1] + ns[-1])
    A = np.empty(totA, dtype)
    for n in range(4, 129):
        idx = np.nonzero(ns == n)[0]
        lu = idx[kinds[idx] == 0]
        sp = idx[kinds[idx] == 1]
        if len(lu):
            M = rs.uniform(-1, 1, (len(lu), n, n)).astype(dtype) + \
                n * np.eye(n, dtype=dtype)
            A[(offA[lu][:, None] + np.arange(n * n)).ravel()] = \
                M.transpose(0, 2, 1).reshape(len(lu), -1).ravel()
        if len(sp):
            Bm = rs.standard_normal((len(sp), n, n)).astype(dtype)
            M = np.matmul(Bm.transpose(0, 2, 1), Bm) + n * np.eye(n, dtype=dtype)
            A[(offA[sp][:, None] + np.arange(n * n)).ravel()] = \
                M.transpose(0, 2, 1).reshape(len(sp), -1).ravel()
    b = rs.standard_normal(totv).astype(dtype)
    return {"n": ns, "oA": offA, "ov": offv, "A": A, "b": b, "k": kinds}


def nbytes(w):
    """Algorithmic bytes of one pass: every matrix, right-hand side and
    solution once (4 (n^2 + 2n) per float system)."""
    return w["A"].nbytes + 2 * w["b"].nbytes
