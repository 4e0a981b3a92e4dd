// Host-visible kernel interface of the GB300 clover solver library (internal, not the C-ABI).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace gbc {

// every host wrapper that launches a kernel of this library adds to this counter
void count_launch(long long n = 1);
long long launch_count();

enum { HOP_PLAIN = 0, HOP_CLOV = 1, HOP_XPAY = 2 };
// reductions fused into the stencil epilogue: none; |out|^2; (out, self) and |out|^2 of the XPAY
// epilogue (BiCGStab's (t, s), (t, t) for t = M~ s), three partial rows per right-hand side;
// (aux, out) of the XPAY epilogue with aux an FP32 field (BiCGStab's (r0, v) for v = M~ p), two rows
enum { RED_NONE = 0, RED_NORM = 1, RED_DOT_SELF = 2, RED_DOT_AUX = 3 };
inline int red_rows(int reduce) { return reduce == RED_DOT_SELF ? 3 : reduce == RED_DOT_AUX ? 2 : reduce ? 1 : 0; }
enum { PREC_HALF = 2, PREC_SINGLE = 4, PREC_DOUBLE = 8 };
// internal arithmetic mode, not a storage precision: FP64-stored fields, double-float arithmetic
// (the PrecDF kernels on the split copies of the FP64 links and clover)
enum { PREC_DF = 16 };

struct Geom {
  int L[4];
  int Lxh;
  int Vh;
  int stride;  // padded plane length (multiple of 64 sites)
  int t_sign;  // -1 when the links at t = Lt-1 carry the antiperiodic sign (12-real reconstruction)
};

// One checkerboard spinor field holding nrhs right-hand sides in precision prec.
struct Spinor {
  int prec = 0;
  int nrhs = 0;
  int stride = 0;
  void* v = nullptr;
  float* norm = nullptr;        // half precision only
  size_t rhs_bytes = 0;         // bytes between right-hand sides in v
  size_t norm_rhs_stride = 0;   // floats between right-hand sides in norm
};

struct HopArgs {
  Geom g;
  int out_parity;
  int nrhs;
  const void* in;
  const float* in_norm;
  size_t in_rhs_bytes;
  void* out;
  float* out_norm;
  size_t out_rhs_bytes;
  const void* self;
  const float* self_norm;
  size_t self_rhs_bytes;
  size_t norm_rhs_stride;
  const void* gauge_fwd[4];  // links U_mu(x) of the output parity
  const void* gauge_bwd[4];  // links U_mu(x) of the input parity (used as U_mu^dag(x - mu))
  const void* clov;          // packed clover of the output parity (HOP_CLOV, HOP_XPAY)
  double a;                  // coefficient of D' psi
  double twist;              // HOP_XPAY: twisted-mass mu (0 = none)
  double* partials;          // RED_*: sums per block, [quantity][rhs][part_stride]
  int part_stride;
  // optional per-right-hand-side flags (active[r * active_stride] != 0): a right-hand side whose
  // flag is 0 is skipped (no loads, no store, zero partials); nullptr = all active
  const int* active;
  int active_stride;
  // RED_DOT_AUX: the FP32 field (per right-hand side, planes of stride g.stride) dotted with out
  const void* aux;
  size_t aux_rhs_bytes;
};

// Launch geometry chosen by the caller (autotuned): TX sites x NRB right-hand sides per block,
// MINB resident blocks per SM requested from the register allocator.  pair = 1: the fp16 kernel
// with two sites per thread (TX threads cover 2 TX sites; fp16 storage and even Lt only);
// pair = 2: the fp16 kernel that streams the next hops through a shared-memory ring (cp.async);
// pair = 3: the fp16 kernel with two right-hand sides per thread (TX sites x NRB right-hand sides,
// TX NRB / 2 threads; even nrhs only).
struct HopShape {
  int tx;
  int nrb;
  int minb;
  int pair;
};
// the compiled candidates (dslash_inst.cuh)
constexpr HopShape kHopShapes[] = {{128, 1, 1, 0}, {128, 1, 6, 0}, {32, 4, 1, 0},  {32, 4, 5, 0},
                                   {64, 2, 4, 0},  {32, 12, 2, 0}, {128, 1, 2, 1}, {128, 1, 3, 1},
                                   {64, 1, 6, 1},  {128, 1, 3, 2}, {128, 1, 4, 2}, {64, 1, 8, 2},
                                   {32, 12, 2, 3}, {16, 12, 5, 3}, {16, 12, 4, 3}, {16, 4, 10, 3}};
constexpr int kNumHopShapes = 16;
// whether shape sh can run the hopping term of precision prec over nrhs right-hand sides of a
// lattice with time extent lt
inline bool hop_shape_valid(const HopShape& sh, int prec, int nrhs, int lt) {
  if (sh.pair == 1) return prec == PREC_HALF && lt % 2 == 0;
  if (sh.pair == 2) return prec == PREC_HALF;
  if (sh.pair == 3) return prec == PREC_HALF && nrhs % 2 == 0 && sh.nrb <= nrhs;
  return !(sh.nrb > 1 && sh.nrb > nrhs);  // a block would be mostly idle
}

// site blocks of one right-hand-side group (the partials each launch writes per right-hand side)
inline int hop_blocks(const HopShape& sh, int Vh) {
  const int sites = sh.pair == 1 ? 2 * sh.tx : sh.tx;
  return (Vh + sites - 1) / sites;
}

// Returns the number of x-blocks launched (partials per right-hand side), or -1 if the
// (precision, recon, shape) combination is not compiled.
int hop_launch_d(int recon, int mode, bool dag, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s);
int hop_launch_s(int recon, int mode, bool dag, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s);
int hop_launch_h(int recon, int mode, bool dag, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s);

// One launch over several lattices: args[l] in device memory, work[b] = (lattice, 128-site block).
int hop_multi_launch_d(int recon, int mode, bool dag, int reduce, const HopArgs* args, const int2* work, int nwork,
                       cudaStream_t s);
int hop_multi_launch_s(int recon, int mode, bool dag, int reduce, const HopArgs* args, const int2* work, int nwork,
                       cudaStream_t s);
int hop_multi_launch_h(int recon, int mode, bool dag, int reduce, const HopArgs* args, const int2* work, int nwork,
                       cudaStream_t s);
inline int hop_multi_launch(int prec, int recon, int mode, bool dag, int reduce, const HopArgs* args,
                            const int2* work, int nwork, cudaStream_t s) {
  switch (prec) {
    case PREC_DOUBLE: return hop_multi_launch_d(recon, mode, dag, reduce, args, work, nwork, s);
    case PREC_SINGLE: return hop_multi_launch_s(recon, mode, dag, reduce, args, work, nwork, s);
    case PREC_HALF: return hop_multi_launch_h(recon, mode, dag, reduce, args, work, nwork, s);
  }
  return -1;
}

int hop_launch_df(int recon, int mode, bool dag, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s);
inline int hop_launch(int prec, int recon, int mode, bool dag, int reduce, const HopArgs& a, HopShape sh,
                      cudaStream_t s) {
  switch (prec) {
    case PREC_DF: return hop_launch_df(recon, mode, dag, reduce, a, sh, s);
    case PREC_DOUBLE: return hop_launch_d(recon, mode, dag, reduce, a, sh, s);
    case PREC_SINGLE: return hop_launch_s(recon, mode, dag, reduce, a, sh, s);
    case PREC_HALF: return hop_launch_h(recon, mode, dag, reduce, a, sh, s);
  }
  return -1;
}

// ---- field import / export / packing (fields.cu) ---------------------------------------------
// canonical complex128 links [V][4][3][3] -> planes of (parity, mu) in prec/recon, links of
// direction mu scaled by coeff[mu]; max |row2 - sign*conj(row0 x row1)| written to *recon_err.
void pack_gauge(const Geom& g, const double* canon, int prec, int recon, void* const planes[2][4],
                const double coeff[4], float* recon_err, cudaStream_t s);
// canonical packed clover [V][72] -> per-parity planes (only parity p_mask bit set: 1 even, 2 odd)
void pack_clover(const Geom& g, const double* canon, int prec, void* const planes[2], int p_mask, cudaStream_t s);
// canonical spinor [V][12] complex128 of rhs r at canon + r*canon_rhs (doubles) <-> parity cb field
void import_spinor(const Geom& g, const double* canon, size_t canon_rhs, int cb, const Spinor& f, cudaStream_t s);
void export_spinor(const Geom& g, double* canon, size_t canon_rhs, int cb, const Spinor& f, cudaStream_t s);

// ---- clover construction on the device (clover.cu) --------------------------------------------
struct CloverCoeffs {
  double diag_mass;
  double coef[6];  // clover coefficient (with the 1/2) of the planes 01,02,03,12,13,23
};
// clov[V][72] = packed A (all sites); inv[V][72] = packed A^-1 on the sites of parity inv_parity
// (2: both parities; zero elsewhere); logdet[V] = sum log|d_i| of the LDL^dag factors on those
// sites, nneg[V] the number of negative d_i.
void clover_build(const int dims[4], const double* canon_links, const CloverCoeffs& cc, double* clov, double* inv,
                  double* logdet, int* nneg, int inv_parity, cudaStream_t s);
void clover_invert(long nsites, double* packed, double* logdet, int* nneg, cudaStream_t s);
// inv = A^-1 on the sites of one parity, from the packed clov of all sites (canonical order)
void clover_invert_parity(const int dims[4], const double* clov, double* inv, int parity, cudaStream_t s);

// ---- BLAS-1 and reductions (blas.cu) ----------------------------------------------------------
// Every vector argument is a Spinor of Vh sites and nrhs right-hand sides; coefficient arrays
// live in device memory, one value (double) or complex (double2) per right-hand side.
struct Red {
  double* partials;  // [nred][nrhs][part_stride]
  int part_stride;
  double* result;    // [nred][nrhs]
};
int blas_blocks(const Geom& g);  // blocks per right-hand side of the reduction kernels

void blas_copy(const Geom& g, const Spinor& y, const Spinor& x, cudaStream_t s);       // y = x (any precisions)
void blas_zero(const Geom& g, const Spinor& y, cudaStream_t s);
void blas_axpby(const Geom& g, const double2* a, const Spinor& x, const double2* b, const Spinor& y,
                cudaStream_t s);                                                           // y = a x + b y
void blas_norm2(const Geom& g, const Spinor& x, const Red& r, cudaStream_t s);             // result[0][rhs]
void blas_cdot(const Geom& g, const Spinor& x, const Spinor& y, const Red& r, cudaStream_t s);  // <x,y> -> result[0..1]
// CG update: x += a p;  r -= a q;  result = |r|^2      (a per rhs, real)
void blas_cg_update(const Geom& g, const double* a, const Spinor& x, const Spinor& p, const Spinor& r,
                    const Spinor& q, const Red& red, cudaStream_t s);
// p = r + b p  (b per rhs, real)
void blas_xpay(const Geom& g, const Spinor& r, const double* b, const Spinor& p, cudaStream_t s);
// y = x - y, result = |y|^2    (residual from a source and M psi)
void blas_xmy_norm2(const Geom& g, const Spinor& x, const Spinor& y, const Red& red, cudaStream_t s);
// y = x - y + tw i gamma_5 x, result = |y|^2   (tw real, the same for every right-hand side)
void blas_xmy_twist_norm2(const Geom& g, const Spinor& x, const Spinor& y, double tw, const Red& red,
                          cudaStream_t s);
// y += sigma_r x and result = Re <x, y> (x, y same precision; sigma per rhs, device)
void blas_shift_dot(const Geom& g, const double* sigma, const Spinor& x, const Spinor& y, const Red& red,
                    cudaStream_t s);
// y += sigma_r x (x, y same precision; sigma per rhs, device)
void blas_shift_axpy(const Geom& g, const double* sigma, const Spinor& x, const Spinor& y, cudaStream_t s);
// x += y (y may be lower precision)
void blas_xpy(const Geom& g, const Spinor& x, const Spinor& y, cudaStream_t s);
// x -= y (y may be lower precision), result = |x|^2
void blas_xsub_norm2(const Geom& g, const Spinor& x, const Spinor& y, const Red& red, cudaStream_t s);
// finalize the partial sums of nred quantities x nrhs into red.result
void reduce_finalize(const Red& red, int nred, int nrhs, int nblocks, cudaStream_t s);

// ---- CG scalar control on the device (blas.cu) ------------------------------------------------
struct CGScalars {
  double c, d, a, b, cp, rsd_sq, c_prev;
  int active, iters;
};
// after |M p|^2 is in red_d: d = red_d[r]; a = active ? c/d : 0
void cg_alpha(CGScalars* st, const double* red_d, double* a_out, int nrhs, cudaStream_t s);
// after |r|^2 is in red_r: cp; converged -> active = 0; b = active ? cp/c : 0; c = cp; iters++
void cg_beta(CGScalars* st, const double* red_r, double* b_out, int nrhs, cudaStream_t s);

// One lattice of a batched CGNE (batch_kernels.cu): its inner vectors, scalars and partial sums.
struct LatCg {
  int Vh;
  int nblk;                 // 128-site blocks = partials per sum
  Spinor e, r;              // correction and residual (accumulator precision)
  Spinor p, q;              // search vector and M~^dag M~ p (sloppy precision)
  CGScalars* cg;
  const double* hop_part;   // |M~ p|^2 per block, written by the stencil launch
  double* upd_part;         // |r|^2 per block, written by batch_cg_update
};
// every lattice at once: one launch each (lat in device memory, work = the batch's work table)
void batch_cg_alpha(const LatCg* lat, int n, cudaStream_t s);
void batch_cg_update(int pa, int po, const LatCg* lat, const int2* work, int nwork, cudaStream_t s);
void batch_cg_beta(const LatCg* lat, int n, cudaStream_t s);
void batch_xpay(int pa, int po, const LatCg* lat, const int2* work, int nwork, cudaStream_t s);

// ---- the same iterations as one persistent kernel (batch_persistent.cuh) -----------------------
// Software grid barrier of a cooperative launch: arrival counter, generation, error flag (a wait
// that gave up).  Zeroed before every launch.
struct GridBar {
  unsigned count;
  unsigned gen;
  int err;
  int where;  // barrier index of the first wait that gave up
};
// per lattice: the largest |r| since the last reliable update and |r| at that update (the
// reliable-update trigger of the host loop), read and written back by the kernel
struct PersistLat {
  double maxrr, at_update;
};
constexpr int kPersistMaxLattices = 32;
// Runs up to kmax CGNE iterations of every active lattice in one cooperative launch (grid = the
// co-resident blocks, at most nwork): the four stencil passes, the update and p = r + b p walk the
// work table (the update fused into the second M~^dag pass), alpha and beta are summed by every
// block from the partials (identical sums in every block, so no scalar is shared), 5 grid
// barriers per iteration.  Stops when no lattice is active, or after an iteration (every fourth of
// the launch) in which an active lattice's |r| fell below delta * maxrr or rose above at_update (a
// reliable update is due); writes the CGScalars and PersistLat back and out[0] = iterations run.
// Returns 0, -1 when (pa, po, recon) has no persistent variant or the
// cooperative launch is refused (the caller then uses the per-launch path), or the CUDA error.
int batch_cg_persistent(int pa, int po, int recon, const HopArgs* args, const LatCg* lat, const int2* work,
                        int nwork, int n, int kmax, double delta, PersistLat* pl, GridBar* bar, int* out,
                        cudaStream_t s);

}  // namespace gbc

namespace gbc {
// out = T in (T = packed clover blocks of the field's parity, prec of the spinors)
// (df: FP64 spinors, clover as the double-float split copy, double-float arithmetic)
void blas_clover(const Geom& g, const void* clov, const Spinor& out, const Spinor& in, cudaStream_t s,
                 bool df = false);
// out[i] = (hi, lo) floats of in[i]: the double-float copy of an FP64 field (n doubles)
void split_df64(const double* in, float2* out, size_t n, cudaStream_t s);
}  // namespace gbc
