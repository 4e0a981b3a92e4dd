// Wilson hopping term for fp16 storage over many right-hand sides, one site and one right-hand
// side per thread, the two half spinors of each hop packed into FFMA2 pairs.
//
// On GB300 the multi-right-hand-side stencil is bound by the FP32 pipes and by latency, not by
// HBM: with the links shared by 12 right-hand sides each stored byte carries ~10 flops, and a packed
// FFMA2 occupies both FMA half-pipes, so it does the FP32 work of two scalar FFMAs in one issue slot
// but no more per clock.  The design therefore minimises FMA-pipe work per site and right-hand
// side and keeps registers low enough for many resident warps:
//   - the two half spinors (1 -+ gamma_mu) psi of a hop are multiplied by the same link, so each
//     link element m = a + ib feeds both of them in one FFMA2: the pair (Re h0_c, Re h1_c) etc.
//     The element is staged once per block in shared memory as (a, a, b', b') with b' = -b for a
//     forward hop and +b for a backward one (U^dag), so that Re(m h) = a Re h + b' Im h and
//     Im(m h) = a Im h - b' Re h for both: four FFMA2 per element for both half spinors;
//   - the results, pairs (upper spin 0, spin 1), are accumulated with the neighbour's site norm by
//     FFMA2; the lower spins, which the projector's B matrix builds from the same pairs either in
//     order (mu = 2, 3) or swapped (mu = 0, 1), go to two pair accumulators summed at the end;
//   - one right-hand side per thread (~100 registers) instead of two (168), and the neighbour
//     spinors of the next two hops are loaded while the current hop is computed.
//
// Block: TS sites (16 or 32) x NRB right-hand sides; thread t works on site t % TS and right-hand
// side t / TS of the block's group, so a warp holds 32 / TS right-hand sides of the same TS sites
// and every shared-memory link word it reads serves 32 / TS lanes.  The links and neighbour indices
// of the block's sites are staged once (8 hops x 9 elements x TS sites x 16 B) and read by all its
// right-hand sides.
#pragma once
#include "dslash.cuh"

namespace gbc {

template <int TS>
struct MrLinks {
  float4 e[8][9][TS];  // element k = 3 r + c of the matrix applied by hop d: (a, a, b', b')
  int nb[8][TS];       // neighbour (input parity) of hop d
};

template <int RECON, int TS>
__device__ __forceinline__ void stage_links_mr(MrLinks<TS>& L, const HopArgs& a, int sblock) {
  const Geom& g = a.g;
  for (int p = threadIdx.x; p < 8 * TS; p += blockDim.x) {
    const int s = p % TS, d = p / TS;
    const int idx = sblock * TS + s;
    if (idx >= g.Vh) continue;
    const int mu = d >> 1;
    const bool bwd = d & 1;
    const Coord c = cb_coords(g, idx, a.out_parity);
    cplx<float> u[9];
    if (!bwd) {
      const float sign = (mu == 3 && c.x[3] == g.L[3] - 1) ? (float)g.t_sign : 1.0f;
      load_link<PrecH, RECON>(u, a.gauge_fwd[mu], idx, g.stride, sign);
      Coord n = c;
      n.x[mu] = c.x[mu] + 1 == g.L[mu] ? 0 : c.x[mu] + 1;
      L.nb[d][s] = cb_index(g, n);
    } else {
      Coord n = c;
      n.x[mu] = c.x[mu] == 0 ? g.L[mu] - 1 : c.x[mu] - 1;
      const float sign = (mu == 3 && n.x[3] == g.L[3] - 1) ? (float)g.t_sign : 1.0f;
      const int j = cb_index(g, n);
      load_link<PrecH, RECON>(u, a.gauge_bwd[mu], j, g.stride, sign);
      L.nb[d][s] = j;
    }
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        // element multiplying h[k] in row r: U[r][k] (forward) or conj(U[k][r]) (backward), stored
        // as (a, a, b', b') with b' = -Im for the forward element, +Im(U[k][r]) for the backward one
        const float re = bwd ? u[3 * k + r].re : u[3 * r + k].re;
        const float bp = bwd ? u[3 * k + r].im : -u[3 * r + k].im;
        L.e[d][3 * r + k][s] = make_float4(re, re, bp, bp);
      }
  }
}

// the stored fp16 words of one neighbour and its site norm
struct MrNbr {
  uint32_t w[12];
  float n;
};

__device__ __forceinline__ void mr_load(MrNbr& d, const char* in, const float* nrm, int j, int stride) {
  const uint4* p = reinterpret_cast<const uint4*>(in);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const uint4 v = ldg(p + (size_t)k * stride + j);
    d.w[4 * k] = v.x;
    d.w[4 * k + 1] = v.y;
    d.w[4 * k + 2] = v.z;
    d.w[4 * k + 3] = v.w;
  }
  d.n = ldg(nrm + j);
}

// accumulators: upper spins as (spin 0, spin 1) pairs, lower spins as (spin 2, spin 3) and (spin 3,
// spin 2) pairs, real and imaginary parts separately, per colour
struct MrAcc {
  float2 ur[3], ui[3], sr[3], si[3], xr[3], xi[3];
};

// hop of direction MU with projector sign S (DeGrand-Rossi tables of project<> / reconstruct<>)
template <int MU, int S, int TS>
__device__ __forceinline__ void mr_hop(MrAcc& A, const MrLinks<TS>& L, int d, int s, const MrNbr& nb) {
  // projected half spinors as pairs (half spinor 0, half spinor 1) of real and imaginary parts
  float2 hr[3], hi[3], nhr[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    __half2 x, y;
    project_h2<MU, S>(nb.w, c, x, y);
    hr[c] = make_float2(__low2float(x), __low2float(y));
    hi[c] = make_float2(__high2float(x), __high2float(y));
    nhr[c] = make_float2(-hr[c].x, -hr[c].y);
  }
  const float n = nb.n;
  const float2 pp = make_float2(n, n), mm = make_float2(-n, -n);
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    float2 yr, yi;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float4 e = L.e[d][3 * r + c][s];
      const float2 ea = make_float2(e.x, e.y), eb = make_float2(e.z, e.w);
      yr = c == 0 ? __fmul2_rn(ea, hr[0]) : __ffma2_rn(ea, hr[c], yr);
      yr = __ffma2_rn(eb, hi[c], yr);
      yi = c == 0 ? __fmul2_rn(ea, hi[0]) : __ffma2_rn(ea, hi[c], yi);
      yi = __ffma2_rn(eb, nhr[c], yi);
    }
    A.ur[r] = __ffma2_rn(pp, yr, A.ur[r]);
    A.ui[r] = __ffma2_rn(pp, yi, A.ui[r]);
    if constexpr (MU == 0) {  // (spin 3, spin 2) += -S i (y0, y1)
      A.xr[r] = __ffma2_rn(S > 0 ? pp : mm, yi, A.xr[r]);
      A.xi[r] = __ffma2_rn(S > 0 ? mm : pp, yr, A.xi[r]);
    } else if constexpr (MU == 1) {  // (spin 3, spin 2) += S (-y0, y1)
      const float2 sg = S > 0 ? make_float2(-n, n) : make_float2(n, -n);
      A.xr[r] = __ffma2_rn(sg, yr, A.xr[r]);
      A.xi[r] = __ffma2_rn(sg, yi, A.xi[r]);
    } else if constexpr (MU == 2) {  // (spin 2, spin 3) += i S (-y0, y1)
      const float2 sg = S > 0 ? make_float2(-n, n) : make_float2(n, -n);
      const float2 ng = make_float2(-sg.x, -sg.y);
      A.sr[r] = __ffma2_rn(ng, yi, A.sr[r]);
      A.si[r] = __ffma2_rn(sg, yr, A.si[r]);
    } else {  // (spin 2, spin 3) += S (y0, y1)
      A.sr[r] = __ffma2_rn(S > 0 ? pp : mm, yr, A.sr[r]);
      A.si[r] = __ffma2_rn(S > 0 ? pp : mm, yi, A.si[r]);
    }
  }
}

template <bool DAG, int H, int TS>
__device__ __forceinline__ void mr_hop_h(MrAcc& A, const MrLinks<TS>& L, int s, const MrNbr& nb) {
  constexpr int MU = H >> 1;
  constexpr bool BWD = (H & 1) != 0;
  constexpr int S = BWD ? (DAG ? -1 : +1) : (DAG ? +1 : -1);  // (1 +- isign gamma)
  mr_hop<MU, S, TS>(A, L, H, s, nb);
}

// Grid: ceil(Vh / TS) site blocks x ceil(nrhs / NRB) right-hand-side groups, groups fastest.
template <int RECON, int MODE, bool DAG, int REDUCE, int TS, int NRB, int MINB>
__global__ void __launch_bounds__(TS * NRB, MINB) hop_kernel_mr(const HopArgs a) {
  static_assert(TS == 16 || TS == 32, "a warp holds whole right-hand sides of TS sites");
  const int ng = (a.nrhs + NRB - 1) / NRB;
  const int sblock = blockIdx.x / ng;
  const int group = blockIdx.x - sblock * ng;
  const int tid = threadIdx.x;
  const int s = tid % TS;
  const int rhs = group * NRB + tid / TS;
  const int idx = sblock * TS + s;
  const Geom& g = a.g;
  __shared__ MrLinks<TS> L;
  stage_links_mr<RECON, TS>(L, a, sblock);
  __syncthreads();
  Sums3<float> local{{0.f, 0.f, 0.f}};
  const bool live = idx < g.Vh && rhs < a.nrhs && (!a.active || a.active[(size_t)rhs * a.active_stride]);
  if (live) {
    const char* in = (const char*)a.in + (size_t)rhs * a.in_rhs_bytes;
    const float* nrm = a.in_norm + (size_t)rhs * a.norm_rhs_stride;
    MrAcc A;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      A.ur[c] = A.ui[c] = A.sr[c] = A.si[c] = A.xr[c] = A.xi[c] = make_float2(0.f, 0.f);
    }
    // the neighbours of the next two hops are in flight while a hop is computed
    MrNbr n0, n1, n2;
    mr_load(n0, in, nrm, L.nb[0][s], g.stride);
    mr_load(n1, in, nrm, L.nb[1][s], g.stride);
    mr_load(n2, in, nrm, L.nb[2][s], g.stride);
    mr_hop_h<DAG, 0, TS>(A, L, s, n0);
    mr_load(n0, in, nrm, L.nb[3][s], g.stride);
    mr_hop_h<DAG, 1, TS>(A, L, s, n1);
    mr_load(n1, in, nrm, L.nb[4][s], g.stride);
    mr_hop_h<DAG, 2, TS>(A, L, s, n2);
    mr_load(n2, in, nrm, L.nb[5][s], g.stride);
    mr_hop_h<DAG, 3, TS>(A, L, s, n0);
    mr_load(n0, in, nrm, L.nb[6][s], g.stride);
    mr_hop_h<DAG, 4, TS>(A, L, s, n1);
    mr_load(n1, in, nrm, L.nb[7][s], g.stride);
    mr_hop_h<DAG, 5, TS>(A, L, s, n2);
    mr_hop_h<DAG, 6, TS>(A, L, s, n0);
    mr_hop_h<DAG, 7, TS>(A, L, s, n1);
    cplx<float> acc[12];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      acc[c] = {A.ur[c].x, A.ui[c].x};
      acc[3 + c] = {A.ur[c].y, A.ui[c].y};
      acc[6 + c] = {A.sr[c].x + A.xr[c].y, A.si[c].x + A.xi[c].y};
      acc[9 + c] = {A.sr[c].y + A.xr[c].x, A.si[c].y + A.xi[c].x};
    }
    local = hop_epilogue<PrecH, MODE, DAG, REDUCE>(a, rhs, idx, acc);
  }
  if constexpr (REDUCE != RED_NONE) {
    // the TS lanes of one right-hand side are TS consecutive lanes of one warp: a fixed butterfly
    // over them, then one FP64 partial per (quantity, right-hand side, site block)
    constexpr int NQ = red_count<REDUCE>();
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      float v = local.q[q];
#pragma unroll
      for (int off = TS / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      if (s == 0 && rhs < a.nrhs) a.partials[((size_t)q * a.nrhs + rhs) * a.part_stride + sblock] = (double)v;
    }
  }
}

}  // namespace gbc
