"""Seeded synthetic sources in the canonical host layout (V, 4, 3) complex128.

- ``z2_noise``: every component (+-1 +- i)/sqrt(2), the Z2 x Z2 noise of Chroma's zN_src
  (lib/meas/sources/zN_src.cc) with N = 4 restricted to those phases;
- ``gaussian``: independent standard normal real and imaginary parts;
- ``point``: delta(x, x0) delta(spin, s) delta(colour, c), the 12 sources of quarkProp4_a
  (lib/actions/ferm/qprop/quarkprop4_w.cc:70-117).
numpy's PCG64 generator keeps them identical across machines.
"""
import numpy as np


def volume(dims):
    return int(np.prod(dims))


def parity(dims):
    V = volume(dims)
    s = np.arange(V)
    x = s % dims[0]
    y = (s // dims[0]) % dims[1]
    z = (s // (dims[0] * dims[1])) % dims[2]
    t = s // (dims[0] * dims[1] * dims[2])
    return (x + y + z + t) % 2


def z2_noise(dims, seed, cb=None):
    rng = np.random.default_rng(seed)
    V = volume(dims)
    re = rng.integers(0, 2, size=(V, 4, 3)) * 2 - 1
    im = rng.integers(0, 2, size=(V, 4, 3)) * 2 - 1
    v = (re + 1j * im) / np.sqrt(2.0)
    if cb is not None:
        v[parity(dims) != cb] = 0
    return v.astype(np.complex128)


def gaussian(dims, seed, cb=None):
    rng = np.random.default_rng(seed)
    V = volume(dims)
    v = rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3))
    if cb is not None:
        v[parity(dims) != cb] = 0
    return v


def point(dims, spin, colour, x0=(0, 0, 0, 0)):
    V = volume(dims)
    v = np.zeros((V, 4, 3), dtype=np.complex128)
    s = x0[0] + dims[0] * (x0[1] + dims[1] * (x0[2] + dims[2] * x0[3]))
    v[s, spin, colour] = 1.0
    return v


def point_sources(dims, x0=(0, 0, 0, 0)):
    """The 12 spin-colour point sources, shape (12, V, 4, 3), index = colour * 4 + spin as in quarkProp4_a."""
    return np.stack([point(dims, s, c, x0) for c in range(3) for s in range(4)])
