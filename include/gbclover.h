/*
 * gbclover.h -- C ABI of the GB300-native even-odd Wilson-clover solver.
 *
 * The library replaces the hot path of Chroma's propagator and HMC solves: the even-odd
 * preconditioned clover operator (Chroma lib/actions/ferm/linop/eoprec_clover_linop_w.cc) and
 * the solvers registered in TheLinOpFermSystemSolverFactory / TheMdagMFermSystemSolverFactory
 * (lib/actions/ferm/invert/syssolver_linop_factory.h:29-39, syssolver_mdagm_factory.h:28-39).
 * A Chroma-side adapter (chroma_plugin/) gathers QDP++ fields by lattice coordinate into the
 * host layouts below and calls these entry points; the context owns every device allocation.
 *
 * Host layouts (all complex numbers are interleaved re, im doubles):
 *   site index   s = x + Lx*(y + Ly*(z + Lz*t))                  (x fastest; NERSC order)
 *   gauge links  double[V][4][3][3][2]   u[s][mu][row][col]      BC already applied
 *   spinor       double[V][4][3][2]      psi[s][spin][colour]    DeGrand-Rossi gamma basis
 *   clover       double[V][72]           Chroma's PrimitiveClovTriang per site
 *                                        {diag[2][6], offd[2][15] complex}
 *   nrhs fields are stored back to back (rhs stride = V*24 doubles).
 * Parity of a site = (x+y+z+t) mod 2; parity 0 = Chroma's rb[0] (even), 1 = rb[1] (odd).
 *
 * Threading: one context = one CUDA stream; calls on one context must not overlap; separate
 * contexts are independent.  Every call returns a status (GBC_OK = 0).
 */
#ifndef GBCLOVER_H
#define GBCLOVER_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (gbc_strerror) --------------------------------------------------------- */
#define GBC_OK 0
#define GBC_ERR_ARGS 1          /* invalid argument / unsupported geometry */
#define GBC_ERR_CUDA 2          /* CUDA runtime error (message in gbc_last_error) */
#define GBC_ERR_NOT_CONVERGED 3 /* MaxIter reached above RsdToleranceFactor*RsdTarget */
#define GBC_ERR_BREAKDOWN 4     /* Krylov breakdown */
#define GBC_ERR_NONFINITE 5     /* NaN/Inf in a source, field or residual */
#define GBC_ERR_STATE 6         /* call order (e.g. solve before gauge load) */
#define GBC_ERR_RECON 7         /* 12-real reconstruction requested for non-SU(3) links */
#define GBC_ERR_PRECOND 8       /* learned preconditioner weights missing or corrupt */

/* ---- enums ------------------------------------------------------------------------------- */
/* precisions: QUDA_..._PRECISION of syssolver_quda_clover_params.cc (HALF/SINGLE/DOUBLE) */
#define GBC_PREC_HALF 2
#define GBC_PREC_SINGLE 4
#define GBC_PREC_DOUBLE 8
/* operator arithmetic of gbc_apply and gbc_time_operator only (not a storage precision): the FP64
   fields in double-float arithmetic (two floats per value, ~48-bit significand), the arithmetic of
   the solvers' Schur prep and intermediate defect-correction residuals */
#define GBC_PREC_DF64 16
/* gauge reconstruction: RECONS_NONE = 18 reals, RECONS_12 */
#define GBC_RECON_18 18
#define GBC_RECON_12 12
/* operators for gbc_apply (parity tests; mirror the EvenOddPrecLinearOperator blocks) */
#define GBC_OP_DSLASH 0   /* D' on output parity cb (lwldslash_w.h:226-303)                         */
#define GBC_OP_CLOVER 1   /* A on parity cb (clover_term_qdp_w.h:2138-2160)                         */
#define GBC_OP_CLOVINV 2  /* A^-1 on parity cb (invclov, eoprec_clover_linop_w.cc:75-86; odd: seoprec) */
#define GBC_OP_MEO 3      /* M~ = A_oo - 1/4 D_oe A_ee^-1 D_eo on odd sites (eoprec_clover_linop_w.cc:142-187) */
#define GBC_OP_MDAGM 4    /* M~^dag M~ (lib/lmdagm.h)                                                */
#define GBC_OP_UNPREC 5   /* full unpreconditioned M (lib/eoprec_linop.h:147-165)                    */
#define GBC_OP_SYM 6      /* M_s = 1 - 1/4 A_oo^-1 D_oe A_ee^-1 D_eo on odd sites
                             (SymEvenOddPrecCloverLinOp, seoprec_clover_linop_w.cc:145-187)          */
#define GBC_OP_SYM_MDAGM 7 /* M_s^dag M_s                                                           */
/* solvers (Chroma invType they stand in for) */
#define GBC_SOLVER_CG 0           /* CG_INVERTER: CGNE, InvCG2 (invcg2.cc:70-232), FP64           */
#define GBC_SOLVER_RELIABLE_CG 1  /* RELIABLE_CG_MP_CLOVER_INVERTER (reliable_cg.cc:10-188)         */
#define GBC_SOLVER_MIXED 2        /* RICHARDSON_MP_CLOVER_INVERTER pattern: FP64 defect correction
                                     around a reliable-update CGNE in sloppy precision
                                     (inv_multiprec_richardson.cc:13-107)                            */
#define GBC_SOLVER_FGMRES 3       /* FGMRESDR_INVERTER (syssolver_linop_fgmres_dr.cc): NKrylov, NDefl
                                     (deflated restarts), preconditioned by the learned network when
                                     loaded                                                          */
#define GBC_SOLVER_BICGSTAB 4     /* FP64 defect correction around a reliable BiCGStab on M~ in the
                                     sloppy precision: RELIABLE_BICGSTAB_MP_CLOVER_INVERTER
                                     (reliable_bicgstab.cc:93-277), QUDA SolverType BICGSTAB.  The
                                     MdagM systems run the inner CGNE; a BiCGStab breakdown switches
                                     the rest of the solve to it                                    */
/* linear systems */
#define GBC_SYS_MEO 0    /* M~ psi_o = chi_o           (LinOpSystemSolver, syssolver_linop.h)          */
#define GBC_SYS_MDAGM 1  /* M~^dag M~ psi_o = chi_o    (MdagMSystemSolver, syssolver_mdagm.h:25-35)    */
#define GBC_SYS_FULL 2   /* M psi = chi on both parities: Schur prep, odd solve, even reconstruction
                            (PrecFermActQprop, eoprec_fermact_qprop.cc:41-80)                        */
#define GBC_SYS_SYM 3    /* M_s psi_o = chi_o for the symmetric operator SEOPREC_CLOVER
                            (SymEvenOddPrecCloverLinOp, seoprec_clover_linop_w.cc:145-187), with
                            + isign i mu gamma_5 when twisted (:174-184)                            */
#define GBC_SYS_SYM_MDAGM 4 /* M_s^dag M_s psi_o = chi_o (MdagM solver of a SEOPREC action)            */

/* ---- parameter structs ------------------------------------------------------------------- */
typedef struct gbc_geom {
  int dims[4];    /* Lx, Ly, Lz, Lt; every extent even and >= 2 (QDP++'s rb checkerboard) */
  int t_boundary; /* +1 periodic, -1 antiperiodic in time: the sign already folded into the links
                     at t = Lt-1 (SimpleFermBC::modify, simple_fermbc.h:87-104); used by the
                     12-real reconstruction */
} gbc_geom;

/* CloverFermActParams (clover_fermact_params_w.cc:27-99) */
typedef struct gbc_action {
  double mass;          /* Mass = 1/(2 Kappa) - 4  (param_io.cc:12-15)            */
  double clov_coeff_r;  /* clovCoeffR (= clovCoeff when isotropic)                */
  double clov_coeff_t;  /* clovCoeffT                                             */
  int aniso;            /* AnisoParam.anisoP                                       */
  double xi_0, nu;      /* AnisoParam.xi_0, AnisoParam.nu                          */
  int t_dir;            /* AnisoParam.t_dir (3)                                    */
  int twisted;          /* TwistedM present                                       */
  double twisted_m;     /* TwistedM                                               */
} gbc_action;

typedef struct gbc_opts {
  int sloppy_precision;   /* CudaSloppyPrecision: GBC_PREC_HALF / SINGLE / DOUBLE  */
  int sloppy_reconstruct; /* CudaSloppyReconstruct: GBC_RECON_12 / GBC_RECON_18    */
  int max_rhs;            /* largest nrhs a solve will be given (workspace sizing) */
  int verbose;
} gbc_opts;

/* per-call solve parameters (SysSolverQUDACloverParams fields, syssolver_quda_clover_params.h:15-90) */
typedef struct gbc_solve_params {
  int solver;                 /* GBC_SOLVER_*                                       */
  int system;                 /* GBC_SYS_*                                          */
  double rsd_target;          /* RsdTarget: relative residual |chi - A psi| / |chi| */
  int max_iter;               /* MaxIter                                            */
  double delta;               /* Delta (reliable-update trigger)                    */
  double rsd_tolerance_factor;/* RsdToleranceFactor: failure threshold (default 10)  */
  int sloppy_precision;       /* 0 = context default                                */
  double inner_tol;           /* GBC_SOLVER_MIXED inner relative tolerance (0 = 1e-6)*/
  int inner_max_iter;         /* 0 = max_iter                                       */
  int nkrylov;                /* FGMRES NKrylov (0 = 16)                            */
  int use_precond;            /* FGMRES: apply the loaded learned preconditioner     */
  int zero_guess;             /* 1: ignore psi on entry (qprop passes zero)          */
  int ndefl;                  /* FGMRES NDefl: harmonic Ritz vectors carried across
                                 restarts (FGMRES-DR); 0 = plain restarts; at most
                                 32 - NKrylov                                      */
} gbc_solve_params;

/* SystemSolverResults_t (lib/syssolver.h:16-23) plus what the adapter logs */
typedef struct gbc_result {
  int n_count;        /* iterations (operator applications / 2 for CGNE)      */
  int status;         /* GBC_OK or an error code for this right-hand side     */
  double resid;       /* |chi - A psi| on the system's sites, FP64             */
  double rel_resid;   /* resid / |chi|                                         */
  double seconds;     /* wall time of the whole call                           */
  int n_outer;        /* outer (FP64) iterations of the mixed solvers          */
  int n_reliable;     /* reliable updates                                      */
  double device_seconds; /* CUDA-event time of the solve on the context stream  */
  long long launches;    /* kernels this library launched during the solve      */
} gbc_result;

typedef struct gbc_ctx gbc_ctx;

/* ---- lifecycle -------------------------------------------------------------------------- */
/* Replaces the constructor of the solver adapter (cf. LinOpSysSolverQUDAClover ctor,
   syssolver_linop_clover_quda_w.h:50-566).  opts may be NULL (defaults: HALF, RECON_12, 12). */
int gbc_create(gbc_ctx** ctx, const gbc_geom* geom, const gbc_action* act, const gbc_opts* opts);
/* Replaces ~LinOpSysSolverQUDAClover (syssolver_linop_clover_quda_w.h:570-575). */
void gbc_destroy(gbc_ctx* ctx);
/* Text of a status code, and the message of the context's last failure.  Chroma reports a failed
   solve on QDPIO::cerr before QDP_abort (syssolver_linop_clover_quda_w.h:636-643); the adapter
   prints these strings there. */
const char* gbc_strerror(int status);
const char* gbc_last_error(gbc_ctx* ctx);
/* The stencil launch shapes the autotuner picked so far, one line per kernel configuration
   (the role of QUDA's AutotuneDslash tag; GBC_AUTOTUNE=0 in the environment disables tuning). */
const char* gbc_tune_report(gbc_ctx* ctx);

/* ---- fields ------------------------------------------------------------------------------ */
/* Links from FermState::getLinks() (BC applied, possibly smeared); builds the clover term and
   its even-parity inverse on the device (QDPCloverTermT::create + choles(0),
   clover_term_qdp_w.h:244-294, 560-571; cf. loadGaugeQuda/loadCloverQuda of
   syssolver_linop_clover_quda_w.h:523,552). */
int gbc_load_gauge(gbc_ctx* ctx, const double* links);
/* Optional: replace the clover term with host-packed A (all sites) and A^-1 (even sites),
   e.g. from QDPCloverTermT::packForQUDA's source (clover_term_qdp_w.h:2221-2228). */
int gbc_load_clover(gbc_ctx* ctx, const double* clov, const double* invclov_even);
/* Packed A and A^-1 (even sites; odd sites zero) and sum_even log|d| (cholesDet(0),
   clover_term_qdp_w.h:580-606); any output pointer may be NULL. */
int gbc_get_clover(gbc_ctx* ctx, double* clov, double* invclov, double* logdet_even, int* n_negative);
/* Log determinants of the clover blocks of the field gbc_load_gauge built: sum_even log|d|
   (EvenOddPrecCloverLinOp::logDetEvenEvenLinOp, eoprec_clover_linop_w.cc:310-312) and sum_odd
   log|d| (SymEvenOddPrecCloverLinOp::logDetOddOddLinOp, seoprec_clover_linop_w.cc:490-492);
   either pointer may be NULL, not both. */
int gbc_get_logdet(gbc_ctx* ctx, double* logdet_even, double* logdet_odd);

/* ---- operators (parity tests; LinearOperator<LatticeFermion>::operator(), lib/linearop.h:25-49) */
/* out/in: nrhs host spinors (full lattice); only the parity the operator reads/writes matters;
   sites of the other parity in out are left untouched.  prec selects the storage precision
   the operator runs in (GBC_PREC_DOUBLE for the FP64 path), or GBC_PREC_DF64 (not for the
   symmetric operators). */
int gbc_apply(gbc_ctx* ctx, int op, int isign, int cb, int prec, int nrhs, double* out, const double* in);

/* ---- BLAS-1 (parity tests of the reductions and fused updates the solvers run) -------------- */
/* The QDP++ reductions over rb[1] that Chroma's solvers call, and the fused vector updates that
   stand in for InvCG2's and BiCGStab's separate QDP++ expressions.  fields[k] are nrhs canonical
   full-lattice host spinors back to back; the odd sites are used and updated fields are written
   back there.  Each field is held in the precision the solvers keep it in: the accumulator
   precision prec_acc (x, r, r0) or the operator precision prec_op (p, q, v, t).  res holds nq values
   per right-hand side, res[rhs * nq + q]; coef holds the per-right-hand-side coefficients. */
#define GBC_BLAS_NORM2 0     /* fields {x}: res = norm2(x, rb[1]) (invcg2.cc:121,165,182); nq 1, prec_op */
#define GBC_BLAS_CDOT 1      /* fields {x, y}: res = Re, Im innerProduct(x, y, rb[1]) (invbicgstab.cc:77,106);
                                nq 2; x in prec_acc, y in prec_op                                            */
#define GBC_BLAS_CG_UPDATE 2 /* fields {x, p, r, q}: x += a p, r -= a q, res = norm2(r) with a = coef[rhs]
                                (invcg2.cc:176-182); nq 1                                                     */
#define GBC_BLAS_XPAY 3      /* fields {r, p}: p = r + b p with b = coef[rhs] (invcg2.cc:220)                */
#define GBC_BLAS_BICG_XR 4   /* fields {x, r, p, v, t, r0}: x += alpha p + omega (r - alpha v),
                                r -= alpha v + omega t, res = norm2(r), Re, Im innerProduct(r0, r)
                                (invbicgstab.cc:142-160, 77); coef = re, im of alpha then of omega per
                                right-hand side; nq 3; precision pairs (DOUBLE, DOUBLE), (SINGLE, SINGLE),
                                (SINGLE, HALF)                                                               */
int gbc_blas(gbc_ctx* ctx, int op, int prec_acc, int prec_op, int nrhs, const double* coef, double* const* fields,
             double* res);

/* ---- solves (LinOpSystemSolver::operator()(psi, chi), lib/syssolver.h:32-50) --------------- */
/* psi, chi: nrhs host spinors, full lattice.  GBC_SYS_MEO / MDAGM read chi and psi on the odd
   sites and write psi there; GBC_SYS_FULL reads chi everywhere and writes psi everywhere.
   res: nrhs results.  Returns the worst status over the right-hand sides. */
int gbc_solve(gbc_ctx* ctx, const gbc_solve_params* p, int nrhs, double* psi, const double* chi, gbc_result* res);
/* Same with psi and chi already in device memory (same canonical layout). */
int gbc_solve_device(gbc_ctx* ctx, const gbc_solve_params* p, int nrhs, double* psi_dev, const double* chi_dev,
                     gbc_result* res);

/* ---- batches of independent lattices ------------------------------------------------------- */
/* No Chroma counterpart (Chroma solves one lattice at a time).  A batch groups contexts of
   different lattices (each loaded with its gauge field, same sloppy reconstruction); a batch solve
   runs the outer FP64 defect correction per lattice and the inner reliable-update CGNE for all
   lattices together, each stencil application one launch over a work table of (lattice, block)
   pairs.  psi[l], chi[l]: host spinors of lattice l (odd sites, as GBC_SYS_MEO). */
typedef struct gbc_batch gbc_batch;
int gbc_batch_create(gbc_batch** batch, int n, gbc_ctx* const* ctxs);
void gbc_batch_destroy(gbc_batch* batch);
int gbc_batch_solve(gbc_batch* batch, const gbc_solve_params* p, double* const* psi, const double* const* chi,
                    gbc_result* res);
const char* gbc_batch_last_error(gbc_batch* batch);

/* ---- measurement (the timing loops of Chroma's t_clover.cc:16-212 / t_lwldslash_sse.cc:20-215) */
/* Times `iters` applications of op (GBC_OP_DSLASH: one hopping launch; GBC_OP_MEO: the two fused
   launches of M~) on device-resident pseudo-random fields of nrhs right-hand sides in precision
   prec, with CUDA events on the context stream.  flush_l2 != 0 overwrites a 256 MiB buffer
   between launches, outside the timed events.  seconds = mean per application; bytes = the
   compulsory (algorithmic) DRAM bytes of one application:
     D'  : Vh (8 L + 2 n S)        M~ : Vh (16 L + 2 C + 5 n S)
   with L, S, C the stored bytes of a link, a spinor (+ its norm in half) and a clover site. */
int gbc_time_operator(gbc_ctx* ctx, int op, int prec, int nrhs, int iters, int flush_l2, double* seconds,
                      double* bytes);
/* op code of gbc_time_operator for one application of the loaded learned preconditioner to nrhs
   odd-site fields (no Chroma counterpart); bytes = per layer the FP32 links of every site once and
   the FP32 activations in and out of every right-hand side, plus the input and output spinors */
#define GBC_TIME_PRECOND 100

/* ---- no-allocation operator ----------------------------------------------------------------- */
/* No counterpart in the reference.  The even-odd operator M~ (as gbc_apply with GBC_OP_MEO and
   GBC_PREC_DOUBLE) for callers that cannot allocate device memory while they run -- e.g. Chroma
   on QDP-JIT, whose pool allocator reserves most of the GPU at start-up, or code that must not
   let a cudaMalloc/cudaFree synchronise the device mid-pipeline.  It allocates nothing: every
   input and output is a caller-owned device pointer in the canonical host layouts above
   (links_dev: the hopping-term links, BC and any anisotropy factors applied; clov_dev: packed A
   on the odd sites; invclov_dev: packed A^-1 on the even sites; in_dev/out_dev: full-lattice
   spinors, odd sites read/written, even sites of out_dev untouched).  Its one temporary, the
   even-parity intermediate, lives in a static device array of GBC_NOALLOC_MAX_VH sites per
   checkerboard (12 MiB).  CUDA loads the library's modules lazily by default, so that array is
   taken on a device when the first gbc_create or gbc_apply_meo_noalloc runs there (with that
   device current), and held until exit: a caller whose allocator will later hold the GPU makes
   one of those calls first.  Lattices with more than GBC_NOALLOC_MAX_VH sites per checkerboard,
   or an odd extent, return GBC_ERR_ARGS (the size case with a message on stderr).  The first
   call on a device also looks up that array's device address (once per device), so make the
   first call before any stream capture.  Work is issued
   on `stream` (a cudaStream_t; NULL = the default stream); every call shares the one array, so
   calls that overlap on the GPU race -- serialise them. */
#define GBC_NOALLOC_MAX_VH 65536
int gbc_apply_meo_noalloc(const gbc_geom* geom, const gbc_action* act, const double* links_dev,
                          const double* clov_dev, const double* invclov_dev, int isign, double* out_dev,
                          const double* in_dev, void* stream);

/* ---- learned preconditioner --------------------------------------------------------------- */
/* No Chroma counterpart: FGMRESDR_INVERTER takes any factory solver as its preconditioner
   (syssolver_linop_fgmres_dr.h:173-184); this one is a gauge-covariant linear network K ~ M~^-1
   of `layers` link-weighted nearest-neighbour layers with `hidden` complex channels per colour
   (4 or 12), channel mixing on the tensor cores (BF16 in, FP32 accumulate).  Its input/output
   are odd-site spinors.  Weights file: "GBCW", version 1, layers, hidden, per layer cin, cout,
   9*cout*cin complex float32, then an FNV-1a 64-bit checksum of everything before it. */
int gbc_precond_init(gbc_ctx* ctx, int hidden, int layers, unsigned long long seed);
/* Load network weights for use inside FGMRES (GBC_ERR_PRECOND if missing or corrupt). */
int gbc_load_precond(gbc_ctx* ctx, const char* path);
int gbc_precond_save(gbc_ctx* ctx, const char* path);
/* Weights as interleaved (re, im) floats, layer after layer, W[l][(d*cout + o)*cin + i] with
   d = 0 self, 1 + 2 mu the +mu hop U_mu(x) h(x+mu), 2 + 2 mu the -mu hop U_mu(x-mu)^dag h(x-mu). */
int gbc_precond_weights(gbc_ctx* ctx, float* out, int capacity, int* count);
int gbc_precond_set_weights(gbc_ctx* ctx, const float* in, int count);
/* out = K(in) for nrhs host spinors (odd sites; even sites of out set to zero). */
int gbc_precond_apply(gbc_ctx* ctx, int nrhs, double* out, const double* in);
/* loss = sum_b |K(in_b) - target_b|^2 / |target_b|^2 over odd sites, and dL/dRe W + i dL/dIm W. */
int gbc_precond_loss_grad(gbc_ctx* ctx, int nb, const double* in, const double* target, double* loss, float* grad,
                          int capacity);
/* Adam on minibatches of (input, target) pairs on the current gauge field (forward and backward
   kernels on the device); loss_per_epoch[epochs] may be NULL. */
int gbc_precond_train(gbc_ctx* ctx, int nsamples, const double* in, const double* target, int epochs, int batch,
                      double lr, unsigned long long seed, double* loss_per_epoch);

/* ---- synthetic inputs ---------------------------------------------------------------------- */
/* Seeded hot-start links U = reunit(exp(i eps H)), H traceless Hermitian with Gaussian entries,
   then n_stout stout steps of size rho in the directions with smear_dirs[mu] != 0
   (stout_utils.cc:105-180, 936-966), then the time boundary sign t_boundary at t = Lt-1.
   Host code (OpenMP); the counter-based recipe is given in the implementation. */
int gbc_gauge_synthetic(const int dims[4], double eps, unsigned long long seed, int n_stout, double rho,
                        const int smear_dirs[4], int t_boundary, double* links);

/* ---- multi-shift solves (RHMC) --------------------------------------------------------------- */
/* (M~^dag M~ + shifts[s]) psi[s] = chi on the odd sites for s = 0..nshift-1 in one Krylov space:
   replaces MdagMMultiSysSolverCG::operator()(psi, shifts, chi)
   (lib/actions/ferm/invert/multi_syssolver_mdagm_cg.h:58-80) and its MInvCG2
   (lib/actions/ferm/invert/minvcg2.cc:70-357), same recursion and stopping rule, FP64.
   shifts[s] >= 0; rsd_targets[s] is RsdCG per shift (NULL: p->rsd_target for all); p->max_iter,
   p->rsd_tolerance_factor and p->sloppy_precision are used, the other fields of p are ignored.
   sloppy_precision GBC_PREC_HALF or GBC_PREC_SINGLE selects the mixed-precision form (the
   multiprec pattern of Chroma's multi-shift solvers): the shared-Krylov recursion on FP32 fields to
   a relative 1e-6, then an FP64 defect correction of every shift, batched over the shifts, with
   corrections from CG on the shifted system in the sloppy operator (n_count adds those iterations);
   0 or GBC_PREC_DOUBLE runs the recursion in FP64 to the targets.  chi and every psi[s]
   are canonical host arrays (only their odd sites are read / written); res[s] per shift, with the
   FP64 true relative residual of that shifted system. */
int gbc_solve_multishift(gbc_ctx* ctx, const gbc_solve_params* p, int nshift, const double* shifts,
                         const double* rsd_targets, double* const* psi, const double* chi, gbc_result* res);

/* ---- gauge-field setup on the device ------------------------------------------------------- */
/* n_steps stout-smearing steps of weight rho in the directions with smear_dirs[mu] != 0 (NULL =
   all four), on the GPU in FP64: replaces smear_links / StoutFermState::create
   (lib/util/gauge/stout_utils.cc:936-966, lib/actions/ferm/fermstates/stout_fermstate_w.h:137-176)
   for a solver's setup.  links_in and links_out are host arrays in the canonical layout of
   gbc_load_gauge (they may be the same array); geom->t_boundary is not applied (Chroma applies
   the fermion boundary after smearing).  Allocates two link fields on the device for the call. */
int gbc_stout_smear(const gbc_geom* geom, int n_steps, double rho, const int smear_dirs[4], const double* links_in,
                    double* links_out);

#ifdef __cplusplus
}
#endif
#endif /* GBCLOVER_H */
