"""ctypes wrapper of the CPU oracle (test infrastructure only).

Arrays use the canonical host layouts of ``oracle.cc``: complex128 gauge links of
shape (V, 4, 3, 3), spinors of shape (V, 4, 3) (or (V, 12)), site index
``x + Lx*(y + Ly*(z + Lz*t))``.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

PRECOND_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_void_p)

OP_DSLASH, OP_CLOVER, OP_CLOVER_INV, OP_MEO, OP_MDAGM, OP_UNPREC, OP_SYM, OP_SYM_MDAGM = range(8)
(SOLVER_CG, SOLVER_RELIABLE_CG, SOLVER_FGMRES, SOLVER_BICGSTAB, SOLVER_RELIABLE_BICGSTAB,
 SOLVER_RICHARDSON_BICGSTAB) = range(6)


def load():
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    lib = C.CDLL(path)
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    lib.orc_gauge_hot.argtypes = [ip, C.c_double, C.c_uint64, dp]
    lib.orc_reunit.argtypes = [ip, dp]
    lib.orc_stout.argtypes = [ip, dp, C.c_double, C.c_int, ip]
    lib.orc_apply_bc.argtypes = [ip, dp, ip]
    lib.orc_plaquette.argtypes = [ip, dp, dp, dp]
    lib.orc_mesfield.argtypes = [ip, dp, dp]
    lib.orc_create.restype = C.c_void_p
    lib.orc_create.argtypes = [ip, dp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double,
                               C.c_double, C.c_int, C.c_int, C.c_double]
    lib.orc_destroy.argtypes = [C.c_void_p]
    lib.orc_volume.restype = C.c_long
    lib.orc_volume.argtypes = [C.c_void_p]
    lib.orc_logdet_even.restype = C.c_double
    lib.orc_logdet_even.argtypes = [C.c_void_p]
    lib.orc_logdet_odd.restype = C.c_double
    lib.orc_logdet_odd.argtypes = [C.c_void_p]
    lib.orc_neg_eigs.argtypes = [C.c_void_p]
    lib.orc_get_clover.argtypes = [C.c_void_p, dp, dp]
    lib.orc_clover_invert_packed.restype = C.c_double
    lib.orc_clover_invert_packed.argtypes = [C.c_long, dp]
    lib.orc_apply.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, dp, dp]
    lib.orc_apply_f32.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float),
                                  C.POINTER(C.c_float)]
    lib.orc_norm2_cb.restype = C.c_double
    lib.orc_norm2_cb.argtypes = [C.c_void_p, dp, C.c_int]
    lib.orc_inner_cb.argtypes = [C.c_void_p, dp, dp, C.c_int, dp]
    lib.orc_solve.argtypes = [C.c_void_p, C.c_int, dp, dp, C.c_double, C.c_int, C.c_double, C.c_int,
                              PRECOND_FN, C.c_void_p, dp]
    lib.orc_qprop.argtypes = [C.c_void_p, dp, dp, C.c_double, C.c_int, dp]
    lib.orc_read_nersc.argtypes = [C.c_char_p, ip, dp, C.c_long, dp, dp]
    lib.orc_gamma.argtypes = [dp]
    lib.orc_uniform.restype = C.c_double
    lib.orc_uniform.argtypes = [C.c_uint64, C.c_uint64]
    lib.orc_normal.restype = C.c_double
    lib.orc_normal.argtypes = [C.c_uint64, C.c_uint64]
    lib.orc_num_threads.restype = C.c_int
    lib.orc_set_threads.argtypes = [C.c_int]
    lib.orc_givens.argtypes = [C.c_int, C.c_int, dp, C.c_int, ip, C.c_int, dp]
    lib.orc_least_squares.argtypes = [C.c_int, C.c_int, dp, dp, C.c_int, dp]
    lib.orc_arnoldi.argtypes = [C.c_void_p, C.c_int, dp, C.c_double, dp, dp, dp, dp]
    _lib = lib
    return lib


def _dp(a):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int))


def givens(H, col, cols, vec=None):
    """Build the FGMRES Givens rotation on column ``col`` of H (complex, shape (ncols, nrows):
    Chroma's H(col, row)), apply it to the listed columns and to ``vec``; returns the new H, vec."""
    lib = load()
    H = np.array(H, dtype=np.complex128, order="C")
    ncols, nrows = H.shape
    cols_a, cols_p = _ip(np.asarray(cols, dtype=np.int32).reshape(-1))
    v = None if vec is None else np.array(vec, dtype=np.complex128).reshape(nrows)
    rc = lib.orc_givens(ncols, nrows, _dp(H.view(np.float64)), int(col), cols_p, len(cols_a),
                        None if v is None else _dp(v.view(np.float64)))
    if rc != 0:
        raise ValueError("bad Givens column")
    return H, v


def least_squares(R, b, n_cols):
    """x with R[:n_cols] x = b[:n_cols] for the upper-triangular R of shape (ncols, nrows)."""
    lib = load()
    R = np.ascontiguousarray(R, dtype=np.complex128)
    ncols, nrows = R.shape
    b = np.ascontiguousarray(b, dtype=np.complex128).reshape(nrows)
    x = np.zeros(n_cols, dtype=np.complex128)
    if lib.orc_least_squares(ncols, nrows, _dp(R.view(np.float64)), _dp(b.view(np.float64)), int(n_cols),
                             _dp(x.view(np.float64))) != 0:
        raise ValueError("bad least-squares sizes")
    return x


def volume(dims):
    return int(np.prod(dims))


class Oracle:
    """Stateless helpers: field generation, smearing, boundary conditions, plaquette, NERSC."""

    def __init__(self):
        self.lib = load()

    def threads(self, n=None):
        if n:
            self.lib.orc_set_threads(int(n))
        return self.lib.orc_num_threads()

    def gamma(self):
        out = np.zeros(80, dtype=np.complex128)
        self.lib.orc_gamma(_dp(out.view(np.float64)))
        return out[:64].reshape(4, 4, 4), out[64:].reshape(4, 4)

    def gauge_hot(self, dims, eps, seed):
        V = volume(dims)
        u = np.zeros((V, 4, 3, 3), dtype=np.complex128)
        d, dp = _ip(dims)
        self.lib.orc_gauge_hot(dp, float(eps), int(seed), _dp(u.view(np.float64)))
        return u

    def reunit(self, dims, u):
        u = np.ascontiguousarray(u, dtype=np.complex128).copy()
        d, dp = _ip(dims)
        self.lib.orc_reunit(dp, _dp(u.view(np.float64)))
        return u

    def stout(self, dims, u, rho, n_smear, smear_dirs=(1, 1, 1, 1)):
        u = np.ascontiguousarray(u, dtype=np.complex128).copy()
        d, dp = _ip(dims)
        s, sp = _ip(smear_dirs)
        self.lib.orc_stout(dp, _dp(u.view(np.float64)), float(rho), int(n_smear), sp)
        return u

    def apply_bc(self, dims, u, bc=(1, 1, 1, -1)):
        u = np.ascontiguousarray(u, dtype=np.complex128).copy()
        d, dp = _ip(dims)
        b, bp = _ip(bc)
        self.lib.orc_apply_bc(dp, _dp(u.view(np.float64)), bp)
        return u

    def plaquette(self, dims, u):
        u = np.ascontiguousarray(u, dtype=np.complex128)
        d, dp = _ip(dims)
        p = C.c_double()
        t = C.c_double()
        self.lib.orc_plaquette(dp, _dp(u.view(np.float64)), C.byref(p), C.byref(t))
        return p.value, t.value

    def mesfield(self, dims, u):
        u = np.ascontiguousarray(u, dtype=np.complex128)
        V = volume(dims)
        f = np.zeros((V, 6, 3, 3), dtype=np.complex128)
        d, dp = _ip(dims)
        self.lib.orc_mesfield(dp, _dp(u.view(np.float64)), _dp(f.view(np.float64)))
        return f

    def invert_packed(self, packed):
        packed = np.ascontiguousarray(packed, dtype=np.float64).copy()
        ld = self.lib.orc_clover_invert_packed(packed.size // 72, _dp(packed))
        return packed, ld

    def read_nersc(self, path):
        dims = np.zeros(4, dtype=np.int32)
        p = C.c_double()
        t = C.c_double()
        rc = self.lib.orc_read_nersc(path.encode(), dims.ctypes.data_as(C.POINTER(C.c_int)), None, 0,
                                     C.byref(p), C.byref(t))
        if rc < 0:
            raise IOError(f"cannot read NERSC header of {path}: {rc}")
        V = int(np.prod(dims))
        u = np.zeros((V, 4, 3, 3), dtype=np.complex128)
        rc = self.lib.orc_read_nersc(path.encode(), dims.ctypes.data_as(C.POINTER(C.c_int)),
                                     _dp(u.view(np.float64)), V, C.byref(p), C.byref(t))
        if rc != 0:
            raise IOError(f"cannot read NERSC payload of {path}: {rc}")
        return tuple(int(x) for x in dims), u, p.value, t.value


class OracleOp:
    """The even-odd clover operator built from BC-applied links (Chroma's EvenOddPrecCloverLinOp)."""

    def __init__(self, dims, u, mass, csw_r, csw_t=None, aniso=False, xi_0=1.0, nu=1.0, t_dir=3,
                 twisted_m=None):
        self.lib = load()
        self.dims = tuple(int(x) for x in dims)
        self.V = volume(dims)
        u = np.ascontiguousarray(u, dtype=np.complex128)
        d, dp = _ip(dims)
        self.h = self.lib.orc_create(dp, _dp(u.view(np.float64)), float(mass), float(csw_r),
                                     float(csw_r if csw_t is None else csw_t), int(bool(aniso)),
                                     float(xi_0), float(nu), int(t_dir), int(twisted_m is not None),
                                     float(twisted_m or 0.0))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def _vec(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128).reshape(self.V, 12)
        return x

    def apply(self, opcode, x, isign=+1, cb=1):
        x = self._vec(x)
        out = np.zeros_like(x)
        rc = self.lib.orc_apply(self.h, int(opcode), int(isign), int(cb), _dp(out.view(np.float64)),
                                _dp(x.view(np.float64)))
        if rc != 0:
            raise ValueError("bad oracle apply")
        return out

    def apply_f32(self, opcode, x, isign=+1, cb=1):
        x = np.ascontiguousarray(x, dtype=np.complex64).reshape(self.V, 12)
        out = np.zeros_like(x)
        fp = C.POINTER(C.c_float)
        rc = self.lib.orc_apply_f32(self.h, int(opcode), int(isign), int(cb),
                                    out.view(np.float32).ctypes.data_as(fp),
                                    x.view(np.float32).ctypes.data_as(fp))
        if rc != 0:
            raise ValueError("bad oracle apply")
        return out

    def clover(self):
        c = np.zeros((self.V, 72))
        ci = np.zeros((self.V, 72))
        self.lib.orc_get_clover(self.h, _dp(c), _dp(ci))
        return c, ci

    def logdet_even(self):
        return self.lib.orc_logdet_even(self.h)

    def logdet_odd(self):
        return self.lib.orc_logdet_odd(self.h)

    def neg_eigs(self):
        return self.lib.orc_neg_eigs(self.h)

    def norm2(self, x, cb=1):
        return self.lib.orc_norm2_cb(self.h, _dp(self._vec(x).view(np.float64)), int(cb))

    def inner(self, x, y, cb=1):
        out = np.zeros(2)
        self.lib.orc_inner_cb(self.h, _dp(self._vec(x).view(np.float64)), _dp(self._vec(y).view(np.float64)),
                              int(cb), _dp(out))
        return complex(out[0], out[1])

    def solve(self, chi, solver=SOLVER_CG, rsd=1e-10, maxit=10000, delta=0.1, nkrylov=16, psi0=None,
              precond=None):
        chi = self._vec(chi)
        psi = np.zeros_like(chi) if psi0 is None else self._vec(psi0).copy()
        res = np.zeros(4)  # n_count, resid, rel_resid, outer steps (multi-precision Richardson)
        V = self.V
        if precond is not None:
            def _cb(user, out, inp):
                o = np.ctypeslib.as_array(C.cast(out, C.POINTER(C.c_double)), shape=(V * 24,))
                i = np.ctypeslib.as_array(C.cast(inp, C.POINTER(C.c_double)), shape=(V * 24,))
                o[:] = precond(i.view(np.complex128).reshape(V, 12)).view(np.float64).reshape(-1)
            cbf = PRECOND_FN(_cb)
        else:
            cbf = PRECOND_FN()
        self.lib.orc_solve(self.h, int(solver), _dp(psi.view(np.float64)), _dp(chi.view(np.float64)),
                           float(rsd), int(maxit), float(delta), int(nkrylov), cbf, None, _dp(res))
        return psi, {"n_count": int(res[0]), "resid": float(res[1]), "rel_resid": float(res[2]),
                     "n_outer": int(res[3])}

    def arnoldi(self, chi, nkrylov, rsd=1e-6):
        """One flexible Arnoldi cycle of M~ (identity preconditioner) from chi / |chi|: returns
        V (nkrylov+1, V, 12), H and R (nkrylov, nkrylov+1; H[col, row]), g (nkrylov+1) and the dimension."""
        chi = self._vec(chi)
        nk = int(nkrylov)
        Vs = np.zeros((nk + 1, self.V, 12), dtype=np.complex128)
        H = np.zeros((nk, nk + 1), dtype=np.complex128)
        R = np.zeros_like(H)
        g = np.zeros(nk + 1, dtype=np.complex128)
        dim = self.lib.orc_arnoldi(self.h, nk, _dp(chi.view(np.float64)), float(rsd), _dp(Vs.view(np.float64)),
                                   _dp(H.view(np.float64)), _dp(R.view(np.float64)), _dp(g.view(np.float64)))
        if dim < 0:
            raise ValueError("bad Krylov size")
        return Vs, H, R, g, dim

    def full_residuals(self, psi, chi):
        """FP64 true relative residuals |chi_k - M psi_k| / |chi_k| of the unpreconditioned operator
        (both parities) for every right-hand side k of psi, chi (shape (n, V, 12) or (V, 12))."""
        psi = np.asarray(psi).reshape(-1, self.V, 12)
        chi = np.asarray(chi).reshape(-1, self.V, 12)
        out = []
        for p, c in zip(psi, chi):
            r = c - self.apply(OP_UNPREC, p)
            out.append(float(np.sqrt(np.vdot(r, r).real / np.vdot(c, c).real)))
        return np.array(out)

    def qprop(self, chi, rsd=1e-10, maxit=10000):
        chi = self._vec(chi)
        psi = np.zeros_like(chi)
        res = np.zeros(3)
        self.lib.orc_qprop(self.h, _dp(psi.view(np.float64)), _dp(chi.view(np.float64)), float(rsd), int(maxit),
                           _dp(res))
        return psi, {"n_count": int(res[0]), "resid": float(res[1]), "rel_resid": float(res[2])}
