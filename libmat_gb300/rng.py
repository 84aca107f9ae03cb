"""Seeded synthetic inputs, identical on the host (numpy) and on the device
(matgb_fill_uniform_dev / matgb_fill_normal_dev in csrc/runtime.cu).

Element i (in column-major memory order) of a seeded fill uses
u_i = (splitmix64(seed * 0x100000001B3 + i) >> 11) * 2^-53 in [0, 1).
Uniform fills are bit-identical between host and device (integer hashing
plus exact double arithmetic, then one rounding to the element type).  Normal
fills use Box-Muller over pairs (2p, 2p+1); host and device libm may differ
in the last bit there.
"""
import numpy as np

_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_MUL = np.uint64(0x100000001B3)


def splitmix64(z):
    with np.errstate(over="ignore"):
        z = z + _GOLD
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def u01(seed, count, start=0):
    i = np.arange(start, start + count, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) * _MUL + i
    return (splitmix64(z) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def uniform(seed, shape, lo=-1.0, hi=1.0, dtype=np.float32):
    n = int(np.prod(shape))
    v = lo + (hi - lo) * u01(seed, n)
    return v.astype(dtype).reshape(shape, order="F")


def normal(seed, shape, dtype=np.float32):
    n = int(np.prod(shape))
    m = n + (n & 1)
    u = u01(seed, m)
    u1 = 1.0 - u[0::2]
    u2 = u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    t = 6.283185307179586 * u2
    out = np.empty(m)
    out[0::2] = r * np.cos(t)
    out[1::2] = r * np.sin(t)
    return out[:n].astype(dtype).reshape(shape, order="F")
