"""The CPU baseline's restatement of the reference's NEON-path mat_solve
(oracle/neon_port.c) against the oracle (the reference's scalar path,
pinned to the reference): the same permutation and swap count on tie-free
inputs, packed factors and solutions within the parity suite's double
bound (1e-11 of max |ref|; the two differ only in summation order and FMA
contraction).  Here (x86) the port runs its portable packed loops; the
second test runs on the GPU host, an aarch64 Grace, where it takes the NEON
micro-kernel -- it is marked gpu only because that host runs the gpu
tests."""
import numpy as np
import pytest

from libmat_gb300 import rng
from oracle.loader import NeonPort, Oracle


def check(sizes):
    N, O = NeonPort(), Oracle("f64")
    for n in sizes:
        A = rng.normal(40 + n, (n, n), np.float64)
        b = rng.normal(41 + n, (n,), np.float64)
        M, p, s = N.plu(A)
        Mo, po, _, so = O.plu_inplace(A)
        assert np.array_equal(p, po) and s == so, n
        assert np.abs(M - Mo).max() / np.abs(Mo).max() <= 1e-11, n
        x, xo = N.solve(A, b), O.solve(A, b)
        assert np.abs(x - xo).max() / np.abs(xo).max() <= 1e-11, n
    return N.arch()


def test_neon_port_matches_oracle():
    check((1, 2, 7, 24, 25, 100, 257, 500))


@pytest.mark.gpu
def test_neon_port_matches_oracle_on_the_gpu_host():
    arch = check((1, 9, 24, 130, 333, 700))
    import platform
    if platform.machine() in ("aarch64", "arm64"):
        assert arch == "NEON"
