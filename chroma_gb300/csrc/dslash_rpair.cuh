// Wilson hopping term for fp16 storage with two right-hand sides per thread.
//
// The multi-right-hand-side stencil is bound by the FP32 pipe and the load/store unit, not by
// HBM: with one site and one right-hand side per thread every thread reads the whole link of each
// hop from shared memory, and the complex arithmetic needs swapped copies of the spinor.  Here a
// thread holds right-hand sides r and r + 1 of one site in the two lanes of each float2 (the C2
// form of the two-sites-per-thread kernel): the link, identical for both lanes, is read once per
// thread from shared memory as (ur, ur, ui, ui) and feeds both right-hand sides; the factors +-i
// of the projectors only relabel real and imaginary parts; the two neighbour norms fold into the
// accumulation FMAs.  The 8 neighbour indices are staged in shared memory with the links, once
// per block.  Lanes 2k and 2k + 1 of a warp work on the same site (two pairs of right-hand sides),
// so each 16-byte link word read from shared memory serves two lanes.
//
// Block: TS sites x NRB right-hand sides, TS * NRB / 2 threads; nrhs must be even.
#pragma once
#include "dslash.cuh"
#include "dslash_async.cuh"

namespace gbc {

// the 8 links of a block's TS sites, reconstructed once, as (ur, ur, ui, ui); backward hops hold
// U^dag of the neighbour's link.  Layout [hop][element][site]; the neighbour index of each hop in
// nsm[hop][site].
template <int RECON, int TS>
__device__ __forceinline__ void stage_links_rp(float4 (*lsm)[9][TS], int (*nsm)[TS], const HopArgs& a, int sblock) {
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
      nsm[d][s] = cb_index(g, n);
    } else {
      Coord n = c;
      n.x[mu] = c.x[mu] == 0 ? g.L[mu] - 1 : c.x[mu] - 1;
      const float sign = (mu == 3 && n.x[3] == g.L[3] - 1) ? (float)g.t_sign : 1.0f;
      const int j = cb_index(g, n);
      load_link<PrecH, RECON>(u, a.gauge_bwd[mu], j, g.stride, sign);
      nsm[d][s] = j;
    }
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const cplx<float> e = bwd ? conj(u[3 * k + r]) : u[3 * r + k];
        lsm[d][3 * r + k][s] = make_float4(e.re, e.re, e.im, e.im);
      }
  }
}

// neighbour j of right-hand sides r (lane x) and r + 1 (lane y), projected in half2 arithmetic
template <int MU, int S>
__device__ __forceinline__ void load_project_rp(C2 (&h)[2][3], const void* b0, const void* b1, int j, int stride) {
  const uint4* p0 = reinterpret_cast<const uint4*>(b0);
  const uint4* p1 = reinterpret_cast<const uint4*>(b1);
  uint32_t w0[12], w1[12];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const uint4 v0 = ldg(p0 + (size_t)k * stride + j);
    const uint4 v1 = ldg(p1 + (size_t)k * stride + j);
    w0[4 * k] = v0.x; w0[4 * k + 1] = v0.y; w0[4 * k + 2] = v0.z; w0[4 * k + 3] = v0.w;
    w1[4 * k] = v1.x; w1[4 * k + 1] = v1.y; w1[4 * k + 2] = v1.z; w1[4 * k + 3] = v1.w;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    __half2 a0, b0h, a1, b1h;
    project_h2<MU, S>(w0, c, a0, b0h);
    project_h2<MU, S>(w1, c, a1, b1h);
    h[0][c] = C2{make_float2(__low2float(a0), __low2float(a1)), make_float2(__high2float(a0), __high2float(a1))};
    h[1][c] = C2{make_float2(__low2float(b0h), __low2float(b1h)), make_float2(__high2float(b0h), __high2float(b1h))};
  }
}

// uh = U h row by row as mult_rebuild_pair, the three link elements of each row read from shared
// memory just before use (a whole link would hold 36 registers)
template <int MU, int S, int TS>
__device__ __forceinline__ void mult_rebuild_rp(C2 (&acc)[12], const float4 (*lk)[TS], int s, const C2 (&h)[2][3],
                                                float2 n) {
  const float2 nn = make_float2(-n.x, -n.y);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    C2 u[9];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float4 v = lk[3 * c + k][s];
      u[3 * c + k] = C2{make_float2(v.x, v.y), make_float2(v.z, v.w)};
    }
    const C2 a = mv_row<false>(u, c, h[0]);
    const C2 b = mv_row<false>(u, c, h[1]);
    acc_scaled<0>(acc[c], a, n, nn);
    acc_scaled<0>(acc[3 + c], b, n, nn);
    constexpr int P1 = S > 0 ? 0 : 1, M1 = S > 0 ? 1 : 0;  // +-1
    constexpr int PI = S > 0 ? 2 : 3, MI = S > 0 ? 3 : 2;  // +-i
    if constexpr (MU == 0) {
      acc_scaled<MI>(acc[6 + c], b, n, nn);
      acc_scaled<MI>(acc[9 + c], a, n, nn);
    } else if constexpr (MU == 1) {
      acc_scaled<P1>(acc[6 + c], b, n, nn);
      acc_scaled<M1>(acc[9 + c], a, n, nn);
    } else if constexpr (MU == 2) {
      acc_scaled<MI>(acc[6 + c], a, n, nn);
      acc_scaled<PI>(acc[9 + c], b, n, nn);
    } else {
      acc_scaled<P1>(acc[6 + c], a, n, nn);
      acc_scaled<P1>(acc[9 + c], b, n, nn);
    }
  }
}

template <int MU, bool DAG, int TS>
__device__ __forceinline__ void hop_dir_rp(C2 (&acc)[12], const float4 (*lsm)[9][TS], const int (*nsm)[TS], int s,
                                           const char* in0, const char* in1, const float* nm0, const float* nm1,
                                           int stride) {
  constexpr int SF = DAG ? +1 : -1;  // forward:  (1 - isign gamma)
  constexpr int SB = DAG ? -1 : +1;  // backward: (1 + isign gamma)
  C2 h[2][3];
  {
    const int j = nsm[2 * MU][s];
    load_project_rp<MU, SF>(h, in0, in1, j, stride);
    const float2 n = make_float2(ldg(nm0 + j), ldg(nm1 + j));
    mult_rebuild_rp<MU, SF, TS>(acc, lsm[2 * MU], s, h, n);
  }
  {
    const int j = nsm[2 * MU + 1][s];
    load_project_rp<MU, SB>(h, in0, in1, j, stride);
    const float2 n = make_float2(ldg(nm0 + j), ldg(nm1 + j));
    mult_rebuild_rp<MU, SB, TS>(acc, lsm[2 * MU + 1], s, h, n);
  }
}

// fused-reduction partials of a two-RHS block: lanes of one parity share a pair group, so a
// butterfly over the even lane offsets leaves the even-lane sums in lane 0 and the odd-lane sums in
// lane 1; then a fixed-order sum over the TS/16 warps of each pair group (bitwise repeatable).
// Partial rows q * nrhs + rhs.
template <int TS, int NRB, int NQ>
__device__ __forceinline__ void rp_block_sums(const HopArgs& a, Sums3<float> l0, Sums3<float> l1, int group,
                                              int sblock) {
  constexpr int SW = TS / 16;
  const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
  __shared__ double wsum[NQ][TS * NRB / 64][2][2];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    float v0 = l0.q[q], v1 = l1.q[q];
#pragma unroll
    for (int off = 16; off >= 2; off >>= 1) {
      v0 += __shfl_xor_sync(0xffffffffu, v0, off);
      v1 += __shfl_xor_sync(0xffffffffu, v1, off);
    }
    if (l < 2) {
      wsum[q][w][l][0] = (double)v0;
      wsum[q][w][l][1] = (double)v1;
    }
  }
  __syncthreads();
  if (tid < NRB) {
    const int pgp = tid >> 1;
    const int r = group * NRB + tid;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double sum = 0.0;
#pragma unroll
      for (int k = 0; k < SW; ++k) sum += wsum[q][(pgp >> 1) * SW + k][pgp & 1][tid & 1];
      if (r < a.nrhs) a.partials[((size_t)q * a.nrhs + r) * a.part_stride + sblock] = sum;
    }
  }
}


// Grid: ceil(Vh / TS) site blocks x ceil(nrhs / NRB) right-hand-side groups, groups fastest.
// Thread t: warp w = t / 32, lane l; site (w % (TS/16)) * 16 + l / 2 of the block, pair group
// (w / (TS/16)) * 2 + (l & 1), i.e. right-hand sides 2 pg and 2 pg + 1 of the group.
template <int RECON, int MODE, bool DAG, int REDUCE, int TS, int NRB, int MINB>
__global__ void __launch_bounds__(TS * NRB / 2, MINB) hop_kernel_rp(const HopArgs a) {
  static_assert(TS % 16 == 0 && NRB % 4 == 0, "TS sites in half-warps, pair groups in lane pairs");
  constexpr int SW = TS / 16;
  const int ng = (a.nrhs + NRB - 1) / NRB;
  const int sblock = blockIdx.x / ng;
  const int group = blockIdx.x - sblock * ng;
  const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
  const int s = (w % SW) * 16 + (l >> 1);
  const int pg = (w / SW) * 2 + (l & 1);
  const int r0 = group * NRB + 2 * pg;
  const int idx = sblock * TS + s;
  const Geom& g = a.g;
  __shared__ float4 lsm[8][9][TS];
  __shared__ int nsm[8][TS];
  stage_links_rp<RECON, TS>(lsm, nsm, a, sblock);
  __syncthreads();
  Sums3<float> l0{{0.f, 0.f, 0.f}}, l1{{0.f, 0.f, 0.f}};  // thread and warp sums in FP32, block sums in FP64
  // a pair with one live right-hand side computes both (the other's output is simply refreshed)
  const bool live = r0 < a.nrhs && (!a.active || a.active[(size_t)r0 * a.active_stride] ||
                                    a.active[(size_t)(r0 + 1) * a.active_stride]);
  if (idx < g.Vh && live) {
    const char* in0 = (const char*)a.in + (size_t)r0 * a.in_rhs_bytes;
    const char* in1 = in0 + a.in_rhs_bytes;
    const float* nm0 = a.in_norm + (size_t)r0 * a.norm_rhs_stride;
    const float* nm1 = nm0 + a.norm_rhs_stride;
    C2 acc[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    hop_dir_rp<0, DAG, TS>(acc, lsm, nsm, s, in0, in1, nm0, nm1, g.stride);
    hop_dir_rp<1, DAG, TS>(acc, lsm, nsm, s, in0, in1, nm0, nm1, g.stride);
    hop_dir_rp<2, DAG, TS>(acc, lsm, nsm, s, in0, in1, nm0, nm1, g.stride);
    hop_dir_rp<3, DAG, TS>(acc, lsm, nsm, s, in0, in1, nm0, nm1, g.stride);
    cplx<float> sa[12], sb[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      sa[k] = {acc[k].r.x, acc[k].i.x};
      sb[k] = {acc[k].r.y, acc[k].i.y};
    }
    l0 = hop_epilogue<PrecH, MODE, DAG, REDUCE>(a, r0, idx, sa);
    l1 = hop_epilogue<PrecH, MODE, DAG, REDUCE>(a, r0 + 1, idx, sb);
  }
  if constexpr (REDUCE != RED_NONE) rp_block_sums<TS, NRB, red_count<REDUCE>()>(a, l0, l1, group, sblock);
}

}  // namespace gbc
