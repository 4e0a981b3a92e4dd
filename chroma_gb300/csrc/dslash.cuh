// Wilson hopping term with fused clover epilogues, one output checkerboard, n right-hand sides.
//
//   D' psi(x) = sum_mu U_mu(x) (1 - isign gamma_mu) psi(x+mu) + U_mu^dag(x-mu) (1 + isign gamma_mu) psi(x-mu)
//   (Chroma lib/actions/ferm/linop/lwldslash_w.h:16-44, 226-303; DeGrand-Rossi gamma basis)
//
// The projector (1 + s gamma_mu) has rank 2: with gamma_mu = [[0, A], [B, 0]] in 2x2 spin
// blocks, the top half is h = psi_top + s A psi_bot and the bottom half is s B h.  Each hop
// therefore multiplies only two colour vectors by the link and rebuilds the lower spins.
//
// Epilogues (MODE):
//   HOP_PLAIN  out = a * D' psi
//   HOP_CLOV   out = T (a * D' psi)                  T = packed clover blocks at the output parity
//                                                    (A_ee^-1 for  A_ee^-1 D_eo psi_o)
//   HOP_XPAY   out = T self + a * D' psi  [+ isign * i * mu * gamma_5 self]
//                                                    (A_oo psi_o - 1/4 D_oe t_e, eoprec_clover_linop_w.cc:142-187)
//   REDUCE adds per-block partial sums of |out|^2 for each right-hand side.
//
// Thread mapping: a block holds TX sites x NRB right-hand sides; the NRB threads that share a
// site read the same links, so the links come from DRAM once and from L1 for the others.
#pragma once
#include "gbc_device.cuh"
#include "gbc_kernels.h"

namespace gbc {

// top half of (1 + s gamma_mu) psi, s = +-1 (compile time)
template <int MU, int S, typename T>
__device__ __forceinline__ void project(cplx<T> (&h)[2][3], const cplx<T> (&p)[12]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    cplx<T> p0 = p[c], p1 = p[3 + c], p2 = p[6 + c], p3 = p[9 + c];
    if constexpr (MU == 0) {  // A = [[0, i], [i, 0]]
      h[0][c] = S > 0 ? p0 + timesI(p3) : p0 - timesI(p3);
      h[1][c] = S > 0 ? p1 + timesI(p2) : p1 - timesI(p2);
    } else if constexpr (MU == 1) {  // A = [[0, -1], [1, 0]]
      h[0][c] = S > 0 ? p0 - p3 : p0 + p3;
      h[1][c] = S > 0 ? p1 + p2 : p1 - p2;
    } else if constexpr (MU == 2) {  // A = [[i, 0], [0, -i]]
      h[0][c] = S > 0 ? p0 + timesI(p2) : p0 - timesI(p2);
      h[1][c] = S > 0 ? p1 - timesI(p3) : p1 + timesI(p3);
    } else {  // A = 1
      h[0][c] = S > 0 ? p0 + p2 : p0 - p2;
      h[1][c] = S > 0 ? p1 + p3 : p1 - p3;
    }
  }
}

// acc_top += uh, acc_bot += s B uh
template <int MU, int S, typename T>
__device__ __forceinline__ void reconstruct(cplx<T> (&acc)[12], const cplx<T> (&uh)[2][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    cplx<T> a = uh[0][c], b = uh[1][c];
    acc[c] = acc[c] + a;
    acc[3 + c] = acc[3 + c] + b;
    if constexpr (MU == 0) {  // B = [[0, -i], [-i, 0]]
      acc[6 + c] = S > 0 ? acc[6 + c] - timesI(b) : acc[6 + c] + timesI(b);
      acc[9 + c] = S > 0 ? acc[9 + c] - timesI(a) : acc[9 + c] + timesI(a);
    } else if constexpr (MU == 1) {  // B = [[0, 1], [-1, 0]]
      acc[6 + c] = S > 0 ? acc[6 + c] + b : acc[6 + c] - b;
      acc[9 + c] = S > 0 ? acc[9 + c] - a : acc[9 + c] + a;
    } else if constexpr (MU == 2) {  // B = [[-i, 0], [0, i]]
      acc[6 + c] = S > 0 ? acc[6 + c] - timesI(a) : acc[6 + c] + timesI(a);
      acc[9 + c] = S > 0 ? acc[9 + c] + timesI(b) : acc[9 + c] - timesI(b);
    } else {  // B = 1
      acc[6 + c] = S > 0 ? acc[6 + c] + a : acc[6 + c] - a;
      acc[9 + c] = S > 0 ? acc[9 + c] + b : acc[9 + c] - b;
    }
  }
}

template <typename T>
__device__ __forceinline__ void mat_vec2(cplx<T> (&uh)[2][3], const cplx<T> (&u)[9], const cplx<T> (&h)[2][3]) {
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      cplx<T> v = u[3 * r] * h[s][0];
      cmac(v, u[3 * r + 1], h[s][1]);
      cmac(v, u[3 * r + 2], h[s][2]);
      uh[s][r] = v;
    }
}

template <typename T>
__device__ __forceinline__ void adj_mat_vec2(cplx<T> (&uh)[2][3], const cplx<T> (&u)[9], const cplx<T> (&h)[2][3]) {
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      cplx<T> v = {0, 0};
      cmacc(v, u[r], h[s][0]);
      cmacc(v, u[3 + r], h[s][1]);
      cmacc(v, u[6 + r], h[s][2]);
      uh[s][r] = v;
    }
}

template <typename P, int RECON, int MU, bool DAG>
__device__ __forceinline__ void hop_dir(cplx<typename P::real> (&acc)[12], const HopArgs& a, const Coord& c, int idx,
                                        const char* in, const float* in_norm) {
  using T = typename P::real;
  constexpr int SF = DAG ? +1 : -1;  // forward:  (1 - isign gamma)
  constexpr int SB = DAG ? -1 : +1;  // backward: (1 + isign gamma)
  const Geom& g = a.g;
  cplx<T> s[12], h[2][3], uh[2][3], u[9];
  // forward neighbour
  {
    Coord n = c;
    n.x[MU] = c.x[MU] + 1 == g.L[MU] ? 0 : c.x[MU] + 1;
    int ni = cb_index(g, n);
    load_spinor<P>(s, in, in_norm, ni, g.stride);
    project<MU, SF>(h, s);
    T sign = (MU == 3 && c.x[3] == g.L[3] - 1) ? (T)g.t_sign : (T)1;
    load_link<P, RECON>(u, a.gauge_fwd[MU], idx, g.stride, sign);
    mat_vec2(uh, u, h);
    reconstruct<MU, SF>(acc, uh);
  }
  // backward neighbour
  {
    Coord n = c;
    n.x[MU] = c.x[MU] == 0 ? g.L[MU] - 1 : c.x[MU] - 1;
    int ni = cb_index(g, n);
    load_spinor<P>(s, in, in_norm, ni, g.stride);
    project<MU, SB>(h, s);
    T sign = (MU == 3 && n.x[3] == g.L[3] - 1) ? (T)g.t_sign : (T)1;
    load_link<P, RECON>(u, a.gauge_bwd[MU], ni, g.stride, sign);
    adj_mat_vec2(uh, u, h);
    reconstruct<MU, SB>(acc, uh);
  }
}

template <typename P, int RECON, int MODE, bool DAG, bool REDUCE, int TX, int NRB>
__global__ void __launch_bounds__(TX * NRB) hop_kernel(const HopArgs a) {
  using T = typename P::real;
  const int tid = threadIdx.x;
  const int rl = tid / TX;
  const int rhs = blockIdx.y * NRB + rl;
  const int idx = blockIdx.x * TX + (tid % TX);
  const Geom& g = a.g;
  const bool active = idx < g.Vh && rhs < a.nrhs;
  double local = 0.0;
  if (active) {
    Coord c = cb_coords(g, idx, a.out_parity);
    const char* in = (const char*)a.in + (size_t)rhs * a.in_rhs_bytes;
    const float* in_norm = a.in_norm ? a.in_norm + (size_t)rhs * a.norm_rhs_stride : nullptr;
    cplx<T> acc[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = {0, 0};
    hop_dir<P, RECON, 0, DAG>(acc, a, c, idx, in, in_norm);
    hop_dir<P, RECON, 1, DAG>(acc, a, c, idx, in, in_norm);
    hop_dir<P, RECON, 2, DAG>(acc, a, c, idx, in, in_norm);
    hop_dir<P, RECON, 3, DAG>(acc, a, c, idx, in, in_norm);
    const T coef = (T)a.a;
    cplx<T> out[12];
    if constexpr (MODE == HOP_PLAIN) {
#pragma unroll
      for (int k = 0; k < 12; ++k) out[k] = coef * acc[k];
    } else if constexpr (MODE == HOP_CLOV) {
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        T d[6];
        cplx<T> o[15], x[6], y[6];
        load_clover_block<P>(d, o, a.clov, idx, g.stride, b);
#pragma unroll
        for (int k = 0; k < 6; ++k) x[k] = coef * acc[6 * b + k];
        clover_block_mul(y, d, o, x);
#pragma unroll
        for (int k = 0; k < 6; ++k) out[6 * b + k] = y[k];
      }
    } else {  // HOP_XPAY
      cplx<T> self[12];
      const char* sp = (const char*)a.self + (size_t)rhs * a.self_rhs_bytes;
      load_spinor<P>(self, sp, a.self_norm ? a.self_norm + (size_t)rhs * a.norm_rhs_stride : nullptr, idx, g.stride);
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        T d[6];
        cplx<T> o[15], x[6], y[6];
        load_clover_block<P>(d, o, a.clov, idx, g.stride, b);
#pragma unroll
        for (int k = 0; k < 6; ++k) x[k] = self[6 * b + k];
        clover_block_mul(y, d, o, x);
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          cplx<T> v = y[k];
          v.re = fmadd(coef, acc[6 * b + k].re, v.re);
          v.im = fmadd(coef, acc[6 * b + k].im, v.im);
          out[6 * b + k] = v;
        }
      }
      if (a.twist != 0.0) {
        // + isign * i * mu * gamma_5 self,  gamma_5 = diag(1, 1, -1, -1)
        const T tw = (T)(DAG ? -a.twist : a.twist);
#pragma unroll
        for (int k = 0; k < 12; ++k) {
          T s5 = k < 6 ? tw : -tw;
          out[k] = out[k] + s5 * timesI(self[k]);
        }
      }
    }
    char* op = (char*)a.out + (size_t)rhs * a.out_rhs_bytes;
    store_spinor<P>(op, a.out_norm ? a.out_norm + (size_t)rhs * a.norm_rhs_stride : nullptr, idx, g.stride, out);
    if constexpr (REDUCE) {
#pragma unroll
      for (int k = 0; k < 12; ++k) local += (double)out[k].re * out[k].re + (double)out[k].im * out[k].im;
    }
  }
  if constexpr (REDUCE) {
    // warps never straddle two right-hand sides (TX is a multiple of 32)
    __shared__ double wsum[TX * NRB / 32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) local += __shfl_down_sync(0xffffffffu, local, off);
    if ((tid & 31) == 0) wsum[tid >> 5] = local;
    __syncthreads();
    if (tid < NRB) {
      const int r = blockIdx.y * NRB + tid;
      double s = 0.0;
#pragma unroll
      for (int w = 0; w < TX / 32; ++w) s += wsum[tid * (TX / 32) + w];
      if (r < a.nrhs) a.partials[(size_t)r * a.part_stride + blockIdx.x] = s;
    }
  }
}

}  // namespace gbc
