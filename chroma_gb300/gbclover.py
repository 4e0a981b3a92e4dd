"""ctypes binding of ``libgbclover.so`` (include/gbclover.h).

Plain host arrays only: complex128 numpy arrays in the canonical layouts of the header
(links (V, 4, 3, 3), spinors (nrhs, V, 4, 3) or (V, 4, 3)).  Device pointers (for the
resident-input path) are passed as integers.  There is no CPU fallback: if the library
cannot be loaded, or no CUDA device is present, the calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgbclover.so")

GBC_OK = 0
ERRORS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "solver did not converge", 4: "Krylov breakdown",
          5: "non-finite value", 6: "invalid call order", 7: "12-real reconstruction not possible",
          8: "learned preconditioner unavailable"}
PREC_HALF, PREC_SINGLE, PREC_DOUBLE = 2, 4, 8
PREC_DF64 = 16  # operator arithmetic of apply / time_operator: FP64 fields, double-float arithmetic
RECON_18, RECON_12 = 18, 12
OP_DSLASH, OP_CLOVER, OP_CLOVINV, OP_MEO, OP_MDAGM, OP_UNPREC, OP_SYM, OP_SYM_MDAGM = range(8)
TIME_PRECOND = 100  # gbc_time_operator: one application of the learned preconditioner
SOLVER_CG, SOLVER_RELIABLE_CG, SOLVER_MIXED, SOLVER_FGMRES, SOLVER_BICGSTAB = range(5)
SYS_MEO, SYS_MDAGM, SYS_FULL, SYS_SYM, SYS_SYM_MDAGM = range(5)
BLAS_NORM2, BLAS_CDOT, BLAS_CG_UPDATE, BLAS_XPAY, BLAS_BICG_XR = range(5)
# status codes (GBC_OK, GBC_ERR_*)
(OK, ERR_ARGS, ERR_CUDA, ERR_NOT_CONVERGED, ERR_BREAKDOWN, ERR_NONFINITE, ERR_STATE, ERR_RECON,
 ERR_PRECOND) = range(9)

# every entry point include/gbclover.h declares
EXPORTS = ["gbc_create", "gbc_destroy", "gbc_strerror", "gbc_last_error", "gbc_load_gauge", "gbc_load_clover",
           "gbc_get_clover", "gbc_get_logdet", "gbc_apply", "gbc_solve", "gbc_solve_device", "gbc_load_precond",
           "gbc_gauge_synthetic", "gbc_time_operator", "gbc_tune_report", "gbc_apply_meo_noalloc",
           "gbc_precond_init", "gbc_precond_save", "gbc_precond_weights", "gbc_precond_set_weights",
           "gbc_precond_apply", "gbc_precond_loss_grad", "gbc_precond_train", "gbc_batch_create",
           "gbc_batch_destroy", "gbc_batch_solve", "gbc_batch_last_error", "gbc_stout_smear",
           "gbc_solve_multishift", "gbc_blas"]


class Geom(C.Structure):
    _fields_ = [("dims", C.c_int * 4), ("t_boundary", C.c_int)]


class Action(C.Structure):
    _fields_ = [("mass", C.c_double), ("clov_coeff_r", C.c_double), ("clov_coeff_t", C.c_double),
                ("aniso", C.c_int), ("xi_0", C.c_double), ("nu", C.c_double), ("t_dir", C.c_int),
                ("twisted", C.c_int), ("twisted_m", C.c_double)]


class Opts(C.Structure):
    _fields_ = [("sloppy_precision", C.c_int), ("sloppy_reconstruct", C.c_int), ("max_rhs", C.c_int),
                ("verbose", C.c_int)]


class SolveParams(C.Structure):
    _fields_ = [("solver", C.c_int), ("system", C.c_int), ("rsd_target", C.c_double), ("max_iter", C.c_int),
                ("delta", C.c_double), ("rsd_tolerance_factor", C.c_double), ("sloppy_precision", C.c_int),
                ("inner_tol", C.c_double), ("inner_max_iter", C.c_int), ("nkrylov", C.c_int),
                ("use_precond", C.c_int), ("zero_guess", C.c_int), ("ndefl", C.c_int)]


class Result(C.Structure):
    _fields_ = [("n_count", C.c_int), ("status", C.c_int), ("resid", C.c_double), ("rel_resid", C.c_double),
                ("seconds", C.c_double), ("n_outer", C.c_int), ("n_reliable", C.c_int),
                ("device_seconds", C.c_double), ("launches", C.c_longlong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load(path=LIB_PATH):
    """Load the CUDA library (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} missing: run __graft_entry__.build() (nvcc, sm_103a) first")
    lib = C.CDLL(path)
    dp = C.POINTER(C.c_double)
    lib.gbc_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(Geom), C.POINTER(Action), C.POINTER(Opts)]
    lib.gbc_destroy.argtypes = [C.c_void_p]
    lib.gbc_destroy.restype = None
    lib.gbc_strerror.restype = C.c_char_p
    lib.gbc_strerror.argtypes = [C.c_int]
    lib.gbc_last_error.restype = C.c_char_p
    lib.gbc_last_error.argtypes = [C.c_void_p]
    lib.gbc_tune_report.restype = C.c_char_p
    lib.gbc_tune_report.argtypes = [C.c_void_p]
    lib.gbc_load_gauge.argtypes = [C.c_void_p, dp]
    lib.gbc_load_clover.argtypes = [C.c_void_p, dp, dp]
    lib.gbc_get_clover.argtypes = [C.c_void_p, dp, dp, dp, C.POINTER(C.c_int)]
    lib.gbc_get_logdet.argtypes = [C.c_void_p, dp, dp]
    lib.gbc_apply.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, dp, dp]
    lib.gbc_solve.argtypes = [C.c_void_p, C.POINTER(SolveParams), C.c_int, dp, dp, C.POINTER(Result)]
    lib.gbc_solve_device.argtypes = [C.c_void_p, C.POINTER(SolveParams), C.c_int, C.c_void_p, C.c_void_p,
                                     C.POINTER(Result)]
    lib.gbc_load_precond.argtypes = [C.c_void_p, C.c_char_p]
    lib.gbc_time_operator.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, dp, dp]
    fp = C.POINTER(C.c_float)
    lib.gbc_precond_init.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_ulonglong]
    lib.gbc_precond_save.argtypes = [C.c_void_p, C.c_char_p]
    lib.gbc_precond_weights.argtypes = [C.c_void_p, fp, C.c_int, C.POINTER(C.c_int)]
    lib.gbc_precond_set_weights.argtypes = [C.c_void_p, fp, C.c_int]
    lib.gbc_precond_apply.argtypes = [C.c_void_p, C.c_int, dp, dp]
    lib.gbc_precond_loss_grad.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, fp, C.c_int]
    lib.gbc_precond_train.argtypes = [C.c_void_p, C.c_int, dp, dp, C.c_int, C.c_int, C.c_double, C.c_ulonglong, dp]
    lib.gbc_gauge_synthetic.argtypes = [C.POINTER(C.c_int), C.c_double, C.c_ulonglong, C.c_int, C.c_double,
                                        C.POINTER(C.c_int), C.c_int, dp]
    lib.gbc_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]
    lib.gbc_batch_destroy.argtypes = [C.c_void_p]
    lib.gbc_batch_destroy.restype = None
    lib.gbc_batch_solve.argtypes = [C.c_void_p, C.POINTER(SolveParams), C.POINTER(dp), C.POINTER(dp),
                                    C.POINTER(Result)]
    lib.gbc_batch_last_error.restype = C.c_char_p
    lib.gbc_batch_last_error.argtypes = [C.c_void_p]
    lib.gbc_stout_smear.argtypes = [C.POINTER(Geom), C.c_int, C.c_double, C.POINTER(C.c_int), dp, dp]
    lib.gbc_blas.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, dp, C.POINTER(dp), dp]
    lib.gbc_solve_multishift.argtypes = [C.c_void_p, C.POINTER(SolveParams), C.c_int, dp, dp, C.POINTER(dp), dp,
                                         C.POINTER(Result)]
    _lib = lib
    return lib


class GBCError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def _dp(a):
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data_as(C.POINTER(C.c_double))


def gauge_synthetic(dims, eps, seed, n_stout=0, rho=0.0, smear_dirs=(1, 1, 1, 1), t_boundary=-1):
    """Seeded hot-start links (host generator of the library), shape (V, 4, 3, 3) complex128."""
    lib = load()
    V = int(np.prod(dims))
    u = np.empty((V, 4, 3, 3), dtype=np.complex128)
    d = (C.c_int * 4)(*dims)
    sd = (C.c_int * 4)(*smear_dirs)
    rc = lib.gbc_gauge_synthetic(d, float(eps), int(seed), int(n_stout), float(rho), sd, int(t_boundary),
                                 _dp(u.view(np.float64)))
    if rc != GBC_OK:
        raise GBCError(rc, "gauge_synthetic")
    return u


def stout_smear(dims, links, n_steps, rho, smear_dirs=(1, 1, 1, 1)):
    """n_steps stout steps of weight rho on the GPU (FP64); links (V, 4, 3, 3) complex128, no BC."""
    lib = load()
    u = np.ascontiguousarray(links, dtype=np.complex128).copy()
    g = Geom((C.c_int * 4)(*dims), 1)
    sd = (C.c_int * 4)(*smear_dirs)
    rc = lib.gbc_stout_smear(C.byref(g), int(n_steps), float(rho), sd, _dp(u.view(np.float64)),
                             _dp(u.view(np.float64)))
    if rc != GBC_OK:
        raise GBCError(rc, "stout_smear")
    return u


class Context:
    """One solver context: links, clover term and workspaces on the GPU (one CUDA stream)."""

    def __init__(self, dims, mass, clov_coeff, clov_coeff_t=None, t_boundary=-1, sloppy_precision=PREC_HALF,
                 sloppy_reconstruct=RECON_12, max_rhs=12, aniso=None, twisted_m=None, verbose=False):
        self.lib = load()
        self.dims = tuple(int(d) for d in dims)
        self.V = int(np.prod(self.dims))
        g = Geom((C.c_int * 4)(*self.dims), int(t_boundary))
        a = Action(float(mass), float(clov_coeff), float(clov_coeff if clov_coeff_t is None else clov_coeff_t),
                   0, 1.0, 1.0, 3, int(twisted_m is not None), float(twisted_m or 0.0))
        if aniso is not None:
            a.aniso, a.xi_0, a.nu, a.t_dir = 1, float(aniso["xi_0"]), float(aniso["nu"]), int(aniso.get("t_dir", 3))
        o = Opts(int(sloppy_precision), int(sloppy_reconstruct), int(max_rhs), int(bool(verbose)))
        h = C.c_void_p()
        rc = self.lib.gbc_create(C.byref(h), C.byref(g), C.byref(a), C.byref(o))
        if rc != GBC_OK:
            raise GBCError(rc, "gbc_create")
        self.h = h
        self.max_rhs = max_rhs

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != GBC_OK:
            raise GBCError(rc, f"{what}: {self.lib.gbc_last_error(self.h).decode()}")

    def load_gauge(self, links):
        u = np.ascontiguousarray(links, dtype=np.complex128).reshape(self.V, 4, 3, 3)
        self._check(self.lib.gbc_load_gauge(self.h, _dp(u.view(np.float64))), "load_gauge")

    def load_clover(self, clov, invclov):
        a = np.ascontiguousarray(clov, dtype=np.float64)
        b = np.ascontiguousarray(invclov, dtype=np.float64)
        self._check(self.lib.gbc_load_clover(self.h, _dp(a), _dp(b)), "load_clover")

    def get_clover(self):
        a = np.zeros((self.V, 72))
        b = np.zeros((self.V, 72))
        ld = C.c_double()
        nn = C.c_int()
        self._check(self.lib.gbc_get_clover(self.h, _dp(a), _dp(b), C.byref(ld), C.byref(nn)), "get_clover")
        return a, b, ld.value, nn.value

    def logdet(self):
        """(sum_even, sum_odd) of log|d| over the clover blocks' LDL^dag factors."""
        e = C.c_double()
        o = C.c_double()
        self._check(self.lib.gbc_get_logdet(self.h, C.byref(e), C.byref(o)), "get_logdet")
        return e.value, o.value

    def _fields(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        if x.size % (self.V * 12):
            raise ValueError("spinor size")
        return x.reshape(-1, self.V, 12)

    def apply(self, op, x, isign=+1, cb=1, prec=PREC_DOUBLE, out=None):
        x = self._fields(x)
        nrhs = x.shape[0]
        out = np.zeros_like(x) if out is None else self._fields(out).copy()
        self._check(self.lib.gbc_apply(self.h, int(op), int(isign), int(cb), int(prec), nrhs,
                                       _dp(out.view(np.float64)), _dp(x.view(np.float64))), "apply")
        return out

    def solve(self, chi, solver=SOLVER_CG, system=SYS_MEO, rsd_target=1e-10, max_iter=10000, delta=0.1,
              sloppy_precision=0, inner_tol=0.0, nkrylov=16, use_precond=0, psi0=None, tol_factor=10.0,
              raise_on_error=True, ndefl=0):
        chi = self._fields(chi)
        nrhs = chi.shape[0]
        psi = np.zeros_like(chi) if psi0 is None else self._fields(psi0).copy()
        p = SolveParams(int(solver), int(system), float(rsd_target), int(max_iter), float(delta), float(tol_factor),
                        int(sloppy_precision), float(inner_tol), 0, int(nkrylov), int(use_precond),
                        int(psi0 is None), int(ndefl))
        res = (Result * nrhs)()
        rc = self.lib.gbc_solve(self.h, C.byref(p), nrhs, _dp(psi.view(np.float64)), _dp(chi.view(np.float64)), res)
        if rc != GBC_OK and raise_on_error:
            self._check(rc, "solve")
        return psi, [r.as_dict() for r in res], rc

    def solve_multishift(self, chi, shifts, rsd_target=1e-10, rsd_targets=None, max_iter=10000, tol_factor=10.0,
                         raise_on_error=True, sloppy_precision=0):
        """(M~^dag M~ + shift_s) psi_s = chi for every shift (odd sites); returns psi (ns, V, 12).
        sloppy_precision PREC_HALF / PREC_SINGLE: FP32 recursion plus per-shift FP64 refinement."""
        chi = np.ascontiguousarray(chi, dtype=np.complex128).reshape(self.V, 12)
        ns = len(shifts)
        psi = np.zeros((ns, self.V, 12), dtype=np.complex128)
        sh = (C.c_double * ns)(*[float(x) for x in shifts])
        rt = None if rsd_targets is None else (C.c_double * ns)(*[float(x) for x in rsd_targets])
        pp = (C.POINTER(C.c_double) * ns)(*[_dp(psi[k].view(np.float64)) for k in range(ns)])
        p = SolveParams(SOLVER_CG, SYS_MDAGM, float(rsd_target), int(max_iter), 0.1, float(tol_factor),
                        int(sloppy_precision), 0.0, 0, 16, 0, 1)
        res = (Result * ns)()
        rc = self.lib.gbc_solve_multishift(self.h, C.byref(p), ns, sh, rt, pp, _dp(chi.view(np.float64)), res)
        if rc != GBC_OK and raise_on_error:
            self._check(rc, "solve_multishift")
        return psi, [r.as_dict() for r in res], rc

    def solve_device(self, psi_ptr, chi_ptr, nrhs, solver=SOLVER_CG, system=SYS_MEO, rsd_target=1e-10,
                     max_iter=10000, delta=0.1, sloppy_precision=0, inner_tol=0.0, nkrylov=16, use_precond=0,
                     zero_guess=True, tol_factor=10.0, ndefl=0):
        p = SolveParams(int(solver), int(system), float(rsd_target), int(max_iter), float(delta), float(tol_factor),
                        int(sloppy_precision), float(inner_tol), 0, int(nkrylov), int(use_precond),
                        int(bool(zero_guess)), int(ndefl))
        res = (Result * nrhs)()
        rc = self.lib.gbc_solve_device(self.h, C.byref(p), int(nrhs), C.c_void_p(psi_ptr), C.c_void_p(chi_ptr), res)
        return [r.as_dict() for r in res], rc

    def time_operator(self, op, prec, nrhs=1, iters=20, flush_l2=True):
        """Mean seconds per application and algorithmic bytes (CUDA events on the context stream)."""
        sec = C.c_double()
        byt = C.c_double()
        self._check(self.lib.gbc_time_operator(self.h, int(op), int(prec), int(nrhs), int(iters), int(bool(flush_l2)),
                                               C.byref(sec), C.byref(byt)), "time_operator")
        return sec.value, byt.value

    def blas(self, op, fields, coef=None, prec_acc=PREC_DOUBLE, prec_op=PREC_DOUBLE):
        """One BLAS-1 kernel of the solvers on host fields (gbc_blas); fields are updated in place.
        Returns the reductions, shape (nrhs, nq)."""
        fs = [self._fields(f) for f in fields]
        for f, orig in zip(fs, fields):
            if not np.shares_memory(f, orig):
                raise ValueError("fields must be C-contiguous complex128 arrays (updated in place)")
        nrhs = fs[0].shape[0]
        nq = {BLAS_NORM2: 1, BLAS_CDOT: 2, BLAS_CG_UPDATE: 1, BLAS_XPAY: 0, BLAS_BICG_XR: 3}[op]
        res = np.zeros(max(1, nq * nrhs))
        cf = None if coef is None else np.ascontiguousarray(coef, dtype=np.float64)
        fp = (C.POINTER(C.c_double) * len(fs))(*[_dp(f.view(np.float64)) for f in fs])
        self._check(self.lib.gbc_blas(self.h, int(op), int(prec_acc), int(prec_op), nrhs,
                                      None if cf is None else _dp(cf), fp, _dp(res)), "blas")
        return res[:nq * nrhs].reshape(nrhs, nq)

    def tune_report(self):
        return self.lib.gbc_tune_report(self.h).decode()

    def load_precond(self, path):
        self._check(self.lib.gbc_load_precond(self.h, path.encode()), "load_precond")

    # ---- learned preconditioner -------------------------------------------------------------
    def precond_init(self, hidden=12, layers=4, seed=0):
        self._check(self.lib.gbc_precond_init(self.h, int(hidden), int(layers), int(seed)), "precond_init")

    def precond_save(self, path):
        self._check(self.lib.gbc_precond_save(self.h, path.encode()), "precond_save")

    def precond_weights(self):
        n = C.c_int()
        self._check(self.lib.gbc_precond_weights(self.h, None, 0, C.byref(n)), "precond_weights")
        w = np.zeros(n.value, dtype=np.float32)
        self._check(self.lib.gbc_precond_weights(self.h, w.ctypes.data_as(C.POINTER(C.c_float)), n.value, None),
                    "precond_weights")
        return w

    def precond_set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._check(self.lib.gbc_precond_set_weights(self.h, w.ctypes.data_as(C.POINTER(C.c_float)), w.size),
                    "precond_set_weights")

    def precond_apply(self, x):
        x = self._fields(x)
        out = np.zeros_like(x)
        self._check(self.lib.gbc_precond_apply(self.h, x.shape[0], _dp(out.view(np.float64)),
                                               _dp(x.view(np.float64))), "precond_apply")
        return out

    def precond_loss_grad(self, xs, es):
        xs = self._fields(xs)
        es = self._fields(es)
        n = self.precond_weights().size
        g = np.zeros(n, dtype=np.float32)
        loss = C.c_double()
        self._check(self.lib.gbc_precond_loss_grad(self.h, xs.shape[0], _dp(xs.view(np.float64)),
                                                   _dp(es.view(np.float64)), C.byref(loss),
                                                   g.ctypes.data_as(C.POINTER(C.c_float)), n), "precond_loss_grad")
        return loss.value, g

    def precond_train(self, xs, es, epochs=10, batch=8, lr=1e-3, seed=0):
        xs = self._fields(xs)
        es = self._fields(es)
        losses = np.zeros(epochs)
        self._check(self.lib.gbc_precond_train(self.h, xs.shape[0], _dp(xs.view(np.float64)),
                                               _dp(es.view(np.float64)), int(epochs), int(batch), float(lr), int(seed),
                                               _dp(losses)), "precond_train")
        return losses


class Batch:
    """Independent lattices solved together (gbc_batch_*): one stencil launch covers all of them."""

    def __init__(self, contexts):
        self.lib = load()
        self.contexts = list(contexts)
        arr = (C.c_void_p * len(self.contexts))(*[c.h.value for c in self.contexts])
        h = C.c_void_p()
        rc = self.lib.gbc_batch_create(C.byref(h), len(self.contexts), arr)
        if rc != GBC_OK:
            raise GBCError(rc, "gbc_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, chis, rsd_target=1e-10, max_iter=10000, delta=0.1, sloppy_precision=0, inner_tol=0.0):
        n = len(self.contexts)
        chis = [np.ascontiguousarray(x, dtype=np.complex128).reshape(ctx.V, 12) for x, ctx in zip(chis, self.contexts)]
        psis = [np.zeros_like(x) for x in chis]
        p = SolveParams(SOLVER_MIXED, SYS_MEO, float(rsd_target), int(max_iter), float(delta), 10.0,
                        int(sloppy_precision), float(inner_tol), 0, 16, 0, 1)
        cp = (C.POINTER(C.c_double) * n)(*[_dp(x.view(np.float64)) for x in chis])
        pp = (C.POINTER(C.c_double) * n)(*[_dp(x.view(np.float64)) for x in psis])
        res = (Result * n)()
        rc = self.lib.gbc_batch_solve(self.h, C.byref(p), pp, cp, res)
        if rc != GBC_OK:
            raise GBCError(rc, "batch_solve: " + self.lib.gbc_batch_last_error(self.h).decode())
        return psis, [r.as_dict() for r in res]
