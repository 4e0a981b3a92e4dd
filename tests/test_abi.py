"""CPU checks of the C-ABI library: it builds for sm_103a, loads, exports every entry point
include/gbclover.h declares, its host-side synthetic-field generator matches the oracle, and
without a GPU every device call fails with a status instead of falling back to the CPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from chroma_gb300 import gbclover as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from chroma_gb300 import build as B
    B.build()
    return G.load()


def header_entry_points():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"^\s*(?:int|void|const char\*)\s+(gbc_\w+)\s*\(", txt, re.M))
    return sorted(names)


def test_exports_every_declared_symbol(lib):
    names = header_entry_points()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n
    assert set(G.EXPORTS) <= set(names)


def test_strerror(lib):
    assert lib.gbc_strerror(0) == b"ok"
    assert lib.gbc_strerror(3) == b"solver did not converge"


@pytest.mark.parametrize("dims", [(3, 4, 4, 4), (4, 3, 4, 4), (4, 4, 5, 4), (4, 4, 4, 7), (4, 4, 4, 1)])
def test_create_rejects_odd_or_short_extent(lib, dims):
    # QDP++'s rb checkerboard needs every extent even: with an odd extent the wrap-around
    # neighbour has the site's own parity; the check runs before any CUDA call
    h = C.c_void_p()
    g = G.Geom((C.c_int * 4)(*dims), -1)
    a = G.Action(0.1, 1.0, 1.0, 0, 1.0, 1.0, 3, 0, 0.0)
    assert lib.gbc_create(C.byref(h), C.byref(g), C.byref(a), None) == 1
    assert not h.value


def test_create_rejects_bad_boundary(lib):
    h = C.c_void_p()
    a = G.Action(0.1, 1.0, 1.0, 0, 1.0, 1.0, 3, 0, 0.0)
    g = G.Geom((C.c_int * 4)(4, 4, 4, 4), 0)
    assert lib.gbc_create(C.byref(h), C.byref(g), C.byref(a), None) == 1


def test_synthetic_links_match_oracle(lib):
    from oracle import Oracle
    o = Oracle()
    dims = (4, 4, 4, 8)
    u = G.gauge_synthetic(dims, 0.3, 99, t_boundary=-1)
    ref = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 99), (1, 1, 1, -1))
    assert np.abs(u - ref).max() < 1e-14
    us = G.gauge_synthetic(dims, 0.2, 5, n_stout=4, rho=0.1, t_boundary=-1)
    ref = o.apply_bc(dims, o.stout(dims, o.gauge_hot(dims, 0.2, 5), 0.1, 4), (1, 1, 1, -1))
    assert np.abs(us - ref).max() < 1e-13
    u3 = G.gauge_synthetic(dims, 0.2, 5, n_stout=2, rho=0.1, smear_dirs=(1, 1, 1, 0), t_boundary=1)
    ref = o.stout(dims, o.gauge_hot(dims, 0.2, 5), 0.1, 2, smear_dirs=(1, 1, 1, 0))
    assert np.abs(u3 - ref).max() < 1e-13


def test_no_cpu_fallback_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(G.GBCError) as e:
        G.Context((4, 4, 4, 4), 0.1, 1.0)
    assert e.value.code == 2  # CUDA error, not a silent host path
