"""gbc_apply_meo_noalloc: the even-odd clover operator for callers that cannot allocate device
memory while they run (Chroma on QDP-JIT, whose pool allocator holds most of the GPU, or code that
must not let cudaMalloc/cudaFree synchronise the device).  The caller owns every buffer; the
library's only temporary is a static device array.

Checked through the C ABI against gbc_apply(GBC_OP_MEO, FP64) -- the ordinary entry point, whose
workspaces live in a context -- at the FP64 tolerance of the operator tests (1e-12 relative), on
two calls in a row with different inputs (the static scratch keeps the previous call's data, which
must not leak into the next result), for both signs, with and without a twisted-mass term.  Kept in a file of its own that pytest
collects last."""
import ctypes as C

import numpy as np
import pytest

from chroma_gb300 import gbclover as G
from chroma_gb300 import sources as S

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("twisted_m", [None, 0.05])
def test_noalloc_meo_matches_gbc_apply(twisted_m):
    """Plain clover and a twisted-mass term (+ isign i mu gamma_5, whose sign flips with isign)."""
    import torch
    dims = (8, 8, 8, 8)
    kappa, csw = 0.115, 1.0
    mass = 1 / (2 * kappa) - 4
    V = int(np.prod(dims))
    links = G.gauge_synthetic(dims, 0.3, 4242, t_boundary=-1)
    ctx = G.Context(dims, mass, csw, t_boundary=-1, max_rhs=2, twisted_m=twisted_m)
    try:
        ctx.load_gauge(links)
        clov, inv, _, _ = ctx.get_clover()
        lib = G.load()
        lib.gbc_apply_meo_noalloc.argtypes = [C.POINTER(G.Geom), C.POINTER(G.Action), C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        geom = G.Geom((C.c_int * 4)(*dims), -1)
        act = G.Action(mass, csw, csw, 0, 1.0, 1.0, 3, int(twisted_m is not None), float(twisted_m or 0.0))
        # caller-owned device buffers
        d_links = torch.from_numpy(links.view(np.float64).reshape(-1).copy()).cuda()
        d_clov = torch.from_numpy(clov.reshape(-1).copy()).cuda()
        d_inv = torch.from_numpy(inv.reshape(-1).copy()).cuda()
        par = S.parity(dims)
        for call, (seed, isign) in enumerate([(1, +1), (2, +1), (3, -1), (4, -1)]):
            x = S.gaussian(dims, seed).reshape(V, 12)
            d_in = torch.from_numpy(x.view(np.float64).reshape(-1).copy()).cuda()
            sentinel = 7.0
            d_out = torch.full((V * 24,), sentinel, dtype=torch.float64, device="cuda")
            rc = lib.gbc_apply_meo_noalloc(C.byref(geom), C.byref(act), d_links.data_ptr(), d_clov.data_ptr(),
                                           d_inv.data_ptr(), isign, d_out.data_ptr(), d_in.data_ptr(), None)
            assert rc == 0, (call, rc)
            torch.cuda.synchronize()
            got = d_out.cpu().numpy().view(np.complex128).reshape(V, 12)
            want = ctx.apply(G.OP_MEO, x, isign, 1, G.PREC_DOUBLE)[0]
            assert _rel(got[par == 1], want[par == 1]) < 1e-12, call
            # even sites of the output are left as the caller had them
            assert np.all(got[par == 0] == complex(sentinel, sentinel))
    finally:
        ctx.close()


def test_noalloc_rejects_lattice_beyond_scratch():
    lib = G.load()
    lib.gbc_apply_meo_noalloc.argtypes = [C.POINTER(G.Geom), C.POINTER(G.Action), C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    dims = (16, 16, 16, 64)  # 131072 sites per checkerboard > GBC_NOALLOC_MAX_VH = 65536
    geom = G.Geom((C.c_int * 4)(*dims), -1)
    act = G.Action(0.0, 1.0, 1.0, 0, 1.0, 1.0, 3, 0, 0.0)
    import torch
    # small real buffers: the size check rejects the call before any kernel could read them
    bufs = [torch.zeros(8, dtype=torch.float64, device="cuda") for _ in range(5)]
    p = [b.data_ptr() for b in bufs]
    rc = lib.gbc_apply_meo_noalloc(C.byref(geom), C.byref(act), p[0], p[1], p[2], 1, p[3], p[4], None)
    assert rc == 1  # GBC_ERR_ARGS
    assert torch.count_nonzero(bufs[3]).item() == 0


@pytest.mark.parametrize("dims", [(8, 7, 8, 8), (8, 8, 8, 5)])
def test_noalloc_rejects_odd_extent(dims):
    lib = G.load()
    lib.gbc_apply_meo_noalloc.argtypes = [C.POINTER(G.Geom), C.POINTER(G.Action), C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    geom = G.Geom((C.c_int * 4)(*dims), -1)
    act = G.Action(0.0, 1.0, 1.0, 0, 1.0, 1.0, 3, 0, 0.0)
    import torch
    bufs = [torch.zeros(8, dtype=torch.float64, device="cuda") for _ in range(5)]
    p = [b.data_ptr() for b in bufs]
    rc = lib.gbc_apply_meo_noalloc(C.byref(geom), C.byref(act), p[0], p[1], p[2], 1, p[3], p[4], None)
    assert rc == 1  # GBC_ERR_ARGS, before any kernel
    assert torch.count_nonzero(bufs[3]).item() == 0
