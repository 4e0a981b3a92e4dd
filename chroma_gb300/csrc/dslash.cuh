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

// Double-float colour products with one renormalisation per output component: the exact products
// of the high parts are summed by TwoSum and their rounding errors, with the cross terms, in a plain
// float (the compensated dot product Dot2 of Ogita, Rump and Oishi, SIAM J. Sci. Comput. 26, 2005):
// 12 FP32 operations per product instead of 15, and a shorter dependency chain.
struct Dot2 {
  float s, c;
};
__device__ __forceinline__ void dot2_add(Dot2& d, df64 a, df64 b) {  // d += a b
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const df64 t = two_sum(d.s, p);
  d.s = t.hi;
  d.c = __fadd_rn(d.c, __fadd_rn(t.lo, e));
}
__device__ __forceinline__ df64 dot2_value(const Dot2& d) { return quick_two_sum(d.s, d.c); }

template <>
__device__ __forceinline__ void mat_vec2<df64>(cplx<df64> (&uh)[2][3], const cplx<df64> (&u)[9],
                                              const cplx<df64> (&h)[2][3]) {
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      Dot2 re{0.f, 0.f}, im{0.f, 0.f};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const cplx<df64> x = u[3 * r + k], y = h[s][k];
        dot2_add(re, x.re, y.re);
        dot2_add(re, -x.im, y.im);
        dot2_add(im, x.re, y.im);
        dot2_add(im, x.im, y.re);
      }
      uh[s][r] = {dot2_value(re), dot2_value(im)};
    }
}

template <>
__device__ __forceinline__ void adj_mat_vec2<df64>(cplx<df64> (&uh)[2][3], const cplx<df64> (&u)[9],
                                                  const cplx<df64> (&h)[2][3]) {
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      Dot2 re{0.f, 0.f}, im{0.f, 0.f};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const cplx<df64> x = u[3 * k + r], y = h[s][k];  // conj(u[k][r]) h[k]
        dot2_add(re, x.re, y.re);
        dot2_add(re, x.im, y.im);
        dot2_add(im, x.re, y.im);
        dot2_add(im, -x.im, y.re);
      }
      uh[s][r] = {dot2_value(re), dot2_value(im)};
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

// Double-float arithmetic: the 8 hops as one rolled loop, so that the long double-float code of
// the spin projection, the colour product and the accumulation exists once instead of 8 times
// (the fully unrolled form stalled on instruction fetch).  Per hop only data movement depends on
// the direction: the projection is h = p_top + w with w = s A p_bot, the accumulation
// acc_top += uh, acc_bot += v with v = s B uh, and A, B are permutations with factors +-1, +-i;
// a backward hop multiplies by U^dag, the conjugate transpose of the loaded link.  The operations
// and their order are those of hop_dir, so the results are bit for bit the same.
template <typename P, int RECON, bool DAG>
__device__ __forceinline__ void hop_rolled_df(cplx<df64> (&acc)[12], const HopArgs& a, const Coord& c, int idx,
                                              const char* in, const float* in_norm) {
  const Geom& g = a.g;
#pragma unroll 1
  for (int hp = 0; hp < 8; ++hp) {
    const int mu = hp >> 1;
    const bool fwd = (hp & 1) == 0;
    const bool neg = fwd ? !DAG : DAG;  // s = -1: forward (1 - isign gamma), backward (1 + isign gamma)
    Coord n = c;
    int xm = c.x[0], lm = g.L[0];
#pragma unroll
    for (int d = 1; d < 4; ++d)
      if (mu == d) {
        xm = c.x[d];
        lm = g.L[d];
      }
    const int xn = fwd ? (xm + 1 == lm ? 0 : xm + 1) : (xm == 0 ? lm - 1 : xm - 1);
#pragma unroll
    for (int d = 0; d < 4; ++d)
      if (mu == d) n.x[d] = xn;
    const int ni = cb_index(g, n);
    cplx<df64> s[12], h[2][3], uh[2][3], u[9], w0[3], w1[3];
    load_spinor<P>(s, in, in_norm, ni, g.stride);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const cplx<df64> p2 = s[6 + k], p3 = s[9 + k];
      if (mu == 0) {
        w0[k] = timesI(p3);
        w1[k] = timesI(p2);
      } else if (mu == 1) {
        w0[k] = -p3;
        w1[k] = p2;
      } else if (mu == 2) {
        w0[k] = timesI(p2);
        w1[k] = -timesI(p3);
      } else {
        w0[k] = p2;
        w1[k] = p3;
      }
      if (neg) {
        w0[k] = -w0[k];
        w1[k] = -w1[k];
      }
      h[0][k] = s[k] + w0[k];
      h[1][k] = s[3 + k] + w1[k];
    }
    const int tm = fwd ? c.x[3] : n.x[3];
    const df64 sign = (mu == 3 && tm == g.L[3] - 1) ? (df64)g.t_sign : (df64)1;
    load_link<P, RECON>(u, fwd ? a.gauge_fwd[mu] : a.gauge_bwd[mu], fwd ? idx : ni, g.stride, sign);
    if (!fwd) {
      // U^dag: transpose and conjugate
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int k = r + 1; k < 3; ++k) {
          const cplx<df64> t = u[3 * r + k];
          u[3 * r + k] = u[3 * k + r];
          u[3 * k + r] = t;
        }
#pragma unroll
      for (int k = 0; k < 9; ++k) u[k].im = -u[k].im;
    }
    mat_vec2(uh, u, h);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const cplx<df64> ua = uh[0][k], ub = uh[1][k];
      acc[k] = acc[k] + ua;
      acc[3 + k] = acc[3 + k] + ub;
      cplx<df64> v6, v9;
      if (mu == 0) {
        v6 = -timesI(ub);
        v9 = -timesI(ua);
      } else if (mu == 1) {
        v6 = ub;
        v9 = -ua;
      } else if (mu == 2) {
        v6 = -timesI(ua);
        v9 = timesI(ub);
      } else {
        v6 = ua;
        v9 = ub;
      }
      if (neg) {
        v6 = -v6;
        v9 = -v9;
      }
      acc[6 + k] = acc[6 + k] + v6;
      acc[9 + k] = acc[9 + k] + v9;
    }
  }
}

// ---- FP32-arithmetic path on packed float2 instructions (FFMA2/FADD2/FMUL2 of sm_100+) ----------
// A complex number is one float2; u*h = (ur, ur)*h + (-ui, ui)*swap(h), so every complex
// multiply-add is two FFMA2 and every complex add one FADD2: half the instructions of scalar code.
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 f2addi(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.y, b.x)); }  // a + i b
__device__ __forceinline__ float2 f2subi(float2 a, float2 b) { return __fadd2_rn(a, make_float2(b.y, -b.x)); }  // a - i b

template <typename P>
__device__ __forceinline__ void load_spinor_f2(float2 (&s)[12], float& n, const void* base, const float* norm, int idx,
                                               int stride) {
  if constexpr (std::is_same<P, PrecS>::value) {
    const float4* p = reinterpret_cast<const float4*>(base);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      float4 v = ldw(p + (size_t)k * stride + idx);
      s[2 * k] = make_float2(v.x, v.y);
      s[2 * k + 1] = make_float2(v.z, v.w);
    }
    n = 1.0f;
  } else {
    const uint4* p = reinterpret_cast<const uint4*>(base);
    n = ldw(norm + idx);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      uint4 v = ldw(p + (size_t)k * stride + idx);
      s[4 * k + 0] = h2f(v.x);
      s[4 * k + 1] = h2f(v.y);
      s[4 * k + 2] = h2f(v.z);
      s[4 * k + 3] = h2f(v.w);
    }
  }
}

// top half of (1 + S gamma_mu) psi on packed complex values
template <int MU, int S>
__device__ __forceinline__ void project_f2(float2 (&h)[2][3], const float2 (&p)[12]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float2 p0 = p[c], p1 = p[3 + c], p2 = p[6 + c], p3 = p[9 + c];
    if constexpr (MU == 0) {
      h[0][c] = S > 0 ? f2addi(p0, p3) : f2subi(p0, p3);
      h[1][c] = S > 0 ? f2addi(p1, p2) : f2subi(p1, p2);
    } else if constexpr (MU == 1) {
      h[0][c] = S > 0 ? f2sub(p0, p3) : f2add(p0, p3);
      h[1][c] = S > 0 ? f2add(p1, p2) : f2sub(p1, p2);
    } else if constexpr (MU == 2) {
      h[0][c] = S > 0 ? f2addi(p0, p2) : f2subi(p0, p2);
      h[1][c] = S > 0 ? f2subi(p1, p3) : f2addi(p1, p3);
    } else {
      h[0][c] = S > 0 ? f2add(p0, p2) : f2sub(p0, p2);
      h[1][c] = S > 0 ? f2add(p1, p3) : f2sub(p1, p3);
    }
  }
}

// acc_top += uh, acc_bot += S B uh (same B tables as reconstruct<>)
template <int MU, int S>
__device__ __forceinline__ void reconstruct_f2(float2 (&acc)[12], const float2 (&uh)[2][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float2 a = uh[0][c], b = uh[1][c];
    acc[c] = f2add(acc[c], a);
    acc[3 + c] = f2add(acc[3 + c], b);
    if constexpr (MU == 0) {
      acc[6 + c] = S > 0 ? f2subi(acc[6 + c], b) : f2addi(acc[6 + c], b);
      acc[9 + c] = S > 0 ? f2subi(acc[9 + c], a) : f2addi(acc[9 + c], a);
    } else if constexpr (MU == 1) {
      acc[6 + c] = S > 0 ? f2add(acc[6 + c], b) : f2sub(acc[6 + c], b);
      acc[9 + c] = S > 0 ? f2sub(acc[9 + c], a) : f2add(acc[9 + c], a);
    } else if constexpr (MU == 2) {
      acc[6 + c] = S > 0 ? f2subi(acc[6 + c], a) : f2addi(acc[6 + c], a);
      acc[9 + c] = S > 0 ? f2addi(acc[9 + c], b) : f2subi(acc[9 + c], b);
    } else {
      acc[6 + c] = S > 0 ? f2add(acc[6 + c], a) : f2sub(acc[6 + c], a);
      acc[9 + c] = S > 0 ? f2add(acc[9 + c], b) : f2sub(acc[9 + c], b);
    }
  }
}

// uh = U h (ADJ: U^dag h) for the two half-spinor colour vectors, h scaled by n
template <bool ADJ>
__device__ __forceinline__ void matvec_f2(float2 (&uh)[2][3], const cplx<float> (&u)[9], const float2 (&h)[2][3]) {
  float2 hs[2][3];
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int c = 0; c < 3; ++c) hs[s][c] = make_float2(h[s][c].y, h[s][c].x);
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      // element multiplying h[.][k] in row r: U[r][k] or conj(U[k][r])
      const cplx<float> e = ADJ ? u[3 * k + r] : u[3 * r + k];
      const float2 A = make_float2(e.re, e.re);
      const float2 B = ADJ ? make_float2(e.im, -e.im) : make_float2(-e.im, e.im);
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        float2 v = k == 0 ? __fmul2_rn(A, h[s][0]) : __ffma2_rn(A, h[s][k], uh[s][r]);
        uh[s][r] = __ffma2_rn(B, hs[s][k], v);
      }
    }
  }
}

// fp16 storage: project the neighbour in half2 arithmetic straight from the stored words and
// convert only the 6 projected colour components (12 conversions instead of 24). The sum of two
// fp16 components is rounded once more to fp16, an error of the same size as their storage
// rounding. Same tables as project<>.
__device__ __forceinline__ __half2 as_h2(uint32_t w) { return *reinterpret_cast<__half2*>(&w); }
__device__ __forceinline__ __half2 h2addi(__half2 a, __half2 b) {  // a + i b
  return __hfma2(__lowhigh2highlow(b), __floats2half2_rn(-1.f, 1.f), a);
}
__device__ __forceinline__ __half2 h2subi(__half2 a, __half2 b) {  // a - i b
  return __hfma2(__lowhigh2highlow(b), __floats2half2_rn(1.f, -1.f), a);
}

// colour c of the top half of (1 + S gamma_mu) psi from the stored fp16 words w
template <int MU, int S>
__device__ __forceinline__ void project_h2(const uint32_t (&w)[12], int c, __half2& a, __half2& b) {
  const __half2 p0 = as_h2(w[c]), p1 = as_h2(w[3 + c]), p2 = as_h2(w[6 + c]), p3 = as_h2(w[9 + c]);
  if constexpr (MU == 0) {
    a = S > 0 ? h2addi(p0, p3) : h2subi(p0, p3);
    b = S > 0 ? h2addi(p1, p2) : h2subi(p1, p2);
  } else if constexpr (MU == 1) {
    a = S > 0 ? __hsub2(p0, p3) : __hadd2(p0, p3);
    b = S > 0 ? __hadd2(p1, p2) : __hsub2(p1, p2);
  } else if constexpr (MU == 2) {
    a = S > 0 ? h2addi(p0, p2) : h2subi(p0, p2);
    b = S > 0 ? h2subi(p1, p3) : h2addi(p1, p3);
  } else {
    a = S > 0 ? __hadd2(p0, p2) : __hsub2(p0, p2);
    b = S > 0 ? __hadd2(p1, p3) : __hsub2(p1, p3);
  }
}

template <int MU, int S>
__device__ __forceinline__ void load_project_h(float2 (&h)[2][3], float& n, const void* base, const float* norm,
                                               int idx, int stride) {
  const uint4* p = reinterpret_cast<const uint4*>(base);
  uint32_t w[12];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const uint4 v = ldw(p + (size_t)k * stride + idx);
    w[4 * k] = v.x;
    w[4 * k + 1] = v.y;
    w[4 * k + 2] = v.z;
    w[4 * k + 3] = v.w;
  }
  n = ldw(norm + idx);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    __half2 a, b;
    project_h2<MU, S>(w, c, a, b);
    h[0][c] = __half22float2(a);
    h[1][c] = __half22float2(b);
  }
}

// load the neighbour and project it: half2 projection for fp16 storage, FP32 otherwise
template <typename P, int MU, int S>
__device__ __forceinline__ void load_project(float2 (&h)[2][3], float& n, const void* base, const float* norm, int idx,
                                             int stride) {
  if constexpr (std::is_same<P, PrecH>::value) {
    load_project_h<MU, S>(h, n, base, norm, idx, stride);
  } else {
    float2 s[12];
    load_spinor_f2<P>(s, n, base, norm, idx, stride);
    project_f2<MU, S>(h, s);
  }
}

// fp16 spinors are stored divided by their site norm: scale the projected half spinor back
template <typename P>
__device__ __forceinline__ void scale_f2(float2 (&h)[2][3], float n) {
  if constexpr (std::is_same<P, PrecH>::value) {
    const float2 nn = make_float2(n, n);
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
      for (int c = 0; c < 3; ++c) h[s][c] = __fmul2_rn(h[s][c], nn);
  }
}

template <typename P, int RECON, int MU, bool DAG>
__device__ __forceinline__ void hop_dir_f2(float2 (&acc)[12], const HopArgs& a, const Coord& c, int idx,
                                           const char* in, const float* in_norm) {
  constexpr int SF = DAG ? +1 : -1;
  constexpr int SB = DAG ? -1 : +1;
  const Geom& g = a.g;
  float2 h[2][3], uh[2][3];
  cplx<float> u[9];
  float n;
  {
    Coord nb = c;
    nb.x[MU] = c.x[MU] + 1 == g.L[MU] ? 0 : c.x[MU] + 1;
    const int ni = cb_index(g, nb);
    load_project<P, MU, SF>(h, n, in, in_norm, ni, g.stride);
    scale_f2<P>(h, n);
    const float sign = (MU == 3 && c.x[3] == g.L[3] - 1) ? (float)g.t_sign : 1.0f;
    load_link<P, RECON>(u, a.gauge_fwd[MU], idx, g.stride, sign);
    matvec_f2<false>(uh, u, h);
    reconstruct_f2<MU, SF>(acc, uh);
  }
  {
    Coord nb = c;
    nb.x[MU] = c.x[MU] == 0 ? g.L[MU] - 1 : c.x[MU] - 1;
    const int ni = cb_index(g, nb);
    load_project<P, MU, SB>(h, n, in, in_norm, ni, g.stride);
    scale_f2<P>(h, n);
    const float sign = (MU == 3 && nb.x[3] == g.L[3] - 1) ? (float)g.t_sign : 1.0f;
    load_link<P, RECON>(u, a.gauge_bwd[MU], ni, g.stride, sign);
    matvec_f2<true>(uh, u, h);
    reconstruct_f2<MU, SB>(acc, uh);
  }
}

// ---- links shared by the right-hand sides of a block (NRB > 1) ----------------------------------
// Each (site, direction) link is loaded and reconstructed once per block and kept in shared memory
// as the pairs (ur, ur, -ui, ui) that the packed complex multiply consumes; without this every
// right-hand side would redo the 12-real reconstruction.  Layout [dir][element][site] keeps a
// warp's 32 sites on consecutive 16-byte words.  The neighbour index of each hop goes to nsm
// [dir][site], so the threads of the block's right-hand sides need no coordinate arithmetic.
template <typename P, int RECON, int TX>
__device__ __forceinline__ void stage_links(float4 (*lsm)[9][TX], int (*nsm)[TX], const HopArgs& a, int sblock) {
  const Geom& g = a.g;
  for (int p = threadIdx.x; p < 8 * TX; p += blockDim.x) {
    const int s = p % TX, d = p / TX;
    const int idx = sblock * TX + s;
    if (idx >= g.Vh) continue;
    const int mu = d >> 1;
    const bool bwd = d & 1;
    const Coord c = cb_coords(g, idx, a.out_parity);
    cplx<float> u[9];
    if (!bwd) {
      const float sign = (mu == 3 && c.x[3] == g.L[3] - 1) ? (float)g.t_sign : 1.0f;
      load_link<P, RECON>(u, a.gauge_fwd[mu], idx, g.stride, sign);
      Coord n = c;
      n.x[mu] = c.x[mu] + 1 == g.L[mu] ? 0 : c.x[mu] + 1;
      nsm[d][s] = cb_index(g, n);
    } else {
      Coord n = c;
      n.x[mu] = c.x[mu] == 0 ? g.L[mu] - 1 : c.x[mu] - 1;
      const float sign = (mu == 3 && n.x[3] == g.L[3] - 1) ? (float)g.t_sign : 1.0f;
      const int j = cb_index(g, n);
      load_link<P, RECON>(u, a.gauge_bwd[mu], j, g.stride, sign);
      nsm[d][s] = j;
    }
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        // element multiplying h[k] in row r: U[r][k] (forward) or conj(U[k][r]) (backward)
        const cplx<float> e = bwd ? conj(u[3 * k + r]) : u[3 * r + k];
        lsm[d][3 * r + k][s] = make_float4(e.re, e.re, -e.im, e.im);
      }
  }
}

template <int TX>
__device__ __forceinline__ void matvec_sm(float2 (&uh)[2][3], const float4 (*lsm)[9][TX], int d, int s,
                                          const float2 (&h)[2][3]) {
  float2 hs[2][3];
#pragma unroll
  for (int q = 0; q < 2; ++q)
#pragma unroll
    for (int c = 0; c < 3; ++c) hs[q][c] = make_float2(h[q][c].y, h[q][c].x);
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float4 ab = lsm[d][3 * r + k][s];
      const float2 A = make_float2(ab.x, ab.y), B = make_float2(ab.z, ab.w);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        float2 v = k == 0 ? __fmul2_rn(A, h[q][0]) : __ffma2_rn(A, h[q][k], uh[q][r]);
        uh[q][r] = __ffma2_rn(B, hs[q][k], v);
      }
    }
}

template <typename P, int MU, bool DAG, int TX>
__device__ __forceinline__ void hop_dir_sm(float2 (&acc)[12], const float4 (*lsm)[9][TX], const int (*nsm)[TX], int s,
                                           const HopArgs& a, const char* in, const float* in_norm) {
  constexpr int SF = DAG ? +1 : -1;
  constexpr int SB = DAG ? -1 : +1;
  const Geom& g = a.g;
  float2 h[2][3], uh[2][3];
  float n;
  {
    load_project<P, MU, SF>(h, n, in, in_norm, nsm[2 * MU][s], g.stride);
    scale_f2<P>(h, n);
    matvec_sm<TX>(uh, lsm, 2 * MU, s, h);
    reconstruct_f2<MU, SF>(acc, uh);
  }
  {
    load_project<P, MU, SB>(h, n, in, in_norm, nsm[2 * MU + 1][s], g.stride);
    scale_f2<P>(h, n);
    matvec_sm<TX>(uh, lsm, 2 * MU + 1, s, h);
    reconstruct_f2<MU, SB>(acc, uh);
  }
}

// Grid: one dimension, right-hand-side groups fastest (block b covers sites (b / ng) * TX ... and
// right-hand sides (b % ng) * NRB ...), so the groups that share a site range run together and
// their link reads after the first come from L2.  MINB caps the registers (MINB resident blocks).
template <typename P, int RECON, int MODE, bool DAG, int REDUCE, int TX, int NRB>
__device__ __forceinline__ void hop_body(const HopArgs& a, int sblock, int group);

// site sums of a fused reduction (RED_NORM: q[0] = |out|^2; RED_DOT_SELF: q = Re, Im (out, self),
// |out|^2; RED_DOT_AUX: q = Re, Im (aux, out)), in the compute precision
template <typename T>
struct Sums3 {
  T q[3];
};
template <int RED>
__host__ __device__ constexpr int red_count() {
  return RED == RED_DOT_SELF ? 3 : RED == RED_DOT_AUX ? 2 : RED == RED_NORM ? 1 : 0;
}
template <typename T>
__device__ __forceinline__ Sums3<T> operator+(Sums3<T> a, const Sums3<T>& b) {
#pragma unroll
  for (int q = 0; q < 3; ++q) a.q[q] += b.q[q];
  return a;
}

// Store one output site in the output precision and return its site sums of the REDUCE kind
// (self: the XPAY operand, for RED_DOT_SELF).
template <typename P, int REDUCE>
__device__ __forceinline__ Sums3<typename P::real> store_site(const HopArgs& a, int rhs, int idx,
                                                              const cplx<typename P::real> (&out)[12],
                                                              const cplx<typename P::real> (&self)[12]) {
  using T = typename P::real;
  char* op = (char*)a.out + (size_t)rhs * a.out_rhs_bytes;
  store_spinor<P>(op, a.out_norm ? a.out_norm + (size_t)rhs * a.norm_rhs_stride : nullptr, idx, a.g.stride, out);
  // site sums in the compute precision (FP64 is slow on this part), block sums in FP64
  Sums3<T> site{{0, 0, 0}};
  if constexpr (REDUCE != RED_NONE) {
    T nn = 0;
#pragma unroll
    for (int k = 0; k < 12; ++k) nn = fmadd(out[k].re, out[k].re, fmadd(out[k].im, out[k].im, nn));
    site.q[REDUCE == RED_DOT_SELF ? 2 : 0] = nn;
  }
  if constexpr (REDUCE == RED_DOT_AUX) {
    // (aux, out) = sum conj(aux) out, aux an FP32 field at the output site
    cplx<float> x[12];
    load_spinor<PrecS>(x, (const char*)a.aux + (size_t)rhs * a.aux_rhs_bytes, nullptr, idx, a.g.stride);
    T re = 0, im = 0;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      re = fmadd((T)x[k].re, out[k].re, fmadd((T)x[k].im, out[k].im, re));
      im = fmadd((T)x[k].re, out[k].im, fmadd(-(T)x[k].im, out[k].re, im));
    }
    site.q[0] = re;
    site.q[1] = im;
  }
  if constexpr (REDUCE == RED_DOT_SELF) {
    T re = 0, im = 0;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      re = fmadd(out[k].re, self[k].re, fmadd(out[k].im, self[k].im, re));
      im = fmadd(out[k].re, self[k].im, fmadd(-out[k].im, self[k].re, im));
    }
    site.q[0] = re;
    site.q[1] = im;
  }
  return site;
}

template <typename P, int MODE, bool DAG>
__device__ __forceinline__ void hop_epilogue_value(const HopArgs& a, int rhs, int idx,
                                                   const cplx<typename P::real> (&acc)[12],
                                                   cplx<typename P::real> (&out)[12],
                                                   cplx<typename P::real> (&self)[12]);

// The MODE epilogue of one output site: out = a D' psi, T (a D' psi) or T self + a D' psi
// (+ twist), stored in the output precision; returns the site sums of the REDUCE kind.
template <typename P, int MODE, bool DAG, int REDUCE>
__device__ __forceinline__ Sums3<typename P::real> hop_epilogue(const HopArgs& a, int rhs, int idx,
                                                                const cplx<typename P::real> (&acc)[12]) {
  static_assert((REDUCE != RED_DOT_SELF && REDUCE != RED_DOT_AUX) || MODE == HOP_XPAY,
                "the dot-product reductions are fused into the XPAY epilogue");
  using T = typename P::real;
  cplx<T> out[12];
  cplx<T> self[12];
  hop_epilogue_value<P, MODE, DAG>(a, rhs, idx, acc, out, self);
  return store_site<P, REDUCE>(a, rhs, idx, out, self);
}

// The output value of the MODE epilogue at one site (self: the XPAY operand, loaded here)
template <typename P, int MODE, bool DAG>
__device__ __forceinline__ void hop_epilogue_value(const HopArgs& a, int rhs, int idx,
                                                   const cplx<typename P::real> (&acc)[12],
                                                   cplx<typename P::real> (&out)[12],
                                                   cplx<typename P::real> (&self)[12]) {
  using T = typename P::real;
  const Geom& g = a.g;
  const T coef = (T)a.a;
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
}

template <typename P, int RECON, int MODE, bool DAG, int REDUCE, int TX, int NRB, int MINB>
__global__ void __launch_bounds__(TX * NRB, MINB) hop_kernel(const HopArgs a) {
  const int ng = (a.nrhs + NRB - 1) / NRB;
  const int sblock = blockIdx.x / ng;
  hop_body<P, RECON, MODE, DAG, REDUCE, TX, NRB>(a, sblock, blockIdx.x - sblock * ng);
}

// One launch over several independent lattices (each its own HopArgs: geometry, fields,
// partials): block b works on lattice work[b].x, site block work[b].y.
template <typename P, int RECON, int MODE, bool DAG, int REDUCE>
__global__ void __launch_bounds__(128) hop_kernel_multi(const HopArgs* __restrict__ args, const int2* __restrict__ work) {
  const int2 w = work[blockIdx.x];
  hop_body<P, RECON, MODE, DAG, REDUCE, 128, 1>(args[w.x], w.y, 0);
}

template <typename P, int RECON, int MODE, bool DAG, int REDUCE, int TX, int NRB>
__device__ __forceinline__ void hop_body(const HopArgs& a, int sblock, int group) {
  using T = typename P::real;
  const int tid = threadIdx.x;
  const int rl = tid / TX;
  const int rhs = group * NRB + rl;
  const int idx = sblock * TX + (tid % TX);
  const Geom& g = a.g;
  const bool active = idx < g.Vh && rhs < a.nrhs && (!a.active || a.active[(size_t)rhs * a.active_stride]);
  // 8 x 9 x 32 x 16 B = 36 KiB of static shared memory for 32-site blocks
  constexpr bool kShared = NRB > 1 && TX == 32 && std::is_same<T, float>::value;
  __shared__ float4 lsm[kShared ? 8 : 1][9][kShared ? TX : 1];
  __shared__ int nsm[kShared ? 8 : 1][kShared ? TX : 1];
  if constexpr (kShared) {
    stage_links<P, RECON, TX>(lsm, nsm, a, sblock);
    __syncthreads();
  }
  // fused reductions: thread and warp sums in the compute precision, block sums in FP64
  Sums3<T> local{{0, 0, 0}};
  if (active) {
    Coord c = cb_coords(g, idx, a.out_parity);
    const char* in = (const char*)a.in + (size_t)rhs * a.in_rhs_bytes;
    const float* in_norm = a.in_norm ? a.in_norm + (size_t)rhs * a.norm_rhs_stride : nullptr;
    cplx<T> acc[12];
    if constexpr (std::is_same<T, float>::value) {
      float2 accf[12];
#pragma unroll
      for (int k = 0; k < 12; ++k) accf[k] = make_float2(0.f, 0.f);
      if constexpr (kShared) {
        const int s = tid % TX;
        hop_dir_sm<P, 0, DAG, TX>(accf, lsm, nsm, s, a, in, in_norm);
        hop_dir_sm<P, 1, DAG, TX>(accf, lsm, nsm, s, a, in, in_norm);
        hop_dir_sm<P, 2, DAG, TX>(accf, lsm, nsm, s, a, in, in_norm);
        hop_dir_sm<P, 3, DAG, TX>(accf, lsm, nsm, s, a, in, in_norm);
      } else {
        hop_dir_f2<P, RECON, 0, DAG>(accf, a, c, idx, in, in_norm);
        hop_dir_f2<P, RECON, 1, DAG>(accf, a, c, idx, in, in_norm);
        hop_dir_f2<P, RECON, 2, DAG>(accf, a, c, idx, in, in_norm);
        hop_dir_f2<P, RECON, 3, DAG>(accf, a, c, idx, in, in_norm);
      }
#pragma unroll
      for (int k = 0; k < 12; ++k) acc[k] = {accf[k].x, accf[k].y};
    } else if constexpr (std::is_same<T, df64>::value) {
#pragma unroll
      for (int k = 0; k < 12; ++k) acc[k] = {0, 0};
      hop_rolled_df<P, RECON, DAG>(acc, a, c, idx, in, in_norm);
    } else {
#pragma unroll
      for (int k = 0; k < 12; ++k) acc[k] = {0, 0};
      hop_dir<P, RECON, 0, DAG>(acc, a, c, idx, in, in_norm);
      hop_dir<P, RECON, 1, DAG>(acc, a, c, idx, in, in_norm);
      hop_dir<P, RECON, 2, DAG>(acc, a, c, idx, in, in_norm);
      hop_dir<P, RECON, 3, DAG>(acc, a, c, idx, in, in_norm);
    }
    local = hop_epilogue<P, MODE, DAG, REDUCE>(a, rhs, idx, acc);
  }
  if constexpr (REDUCE != RED_NONE) {
    // warps never straddle two right-hand sides (TX is a multiple of 32)
    constexpr int NQ = red_count<REDUCE>();
    __shared__ double wsum[NQ][TX * NRB / 32];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      T v = local.q[q];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
      if ((tid & 31) == 0) wsum[q][tid >> 5] = (double)v;
    }
    __syncthreads();
    if (tid < NRB) {
      const int r = group * NRB + tid;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < TX / 32; ++w) s += wsum[q][tid * (TX / 32) + w];
        if (r < a.nrhs) a.partials[((size_t)q * a.nrhs + r) * a.part_stride + sblock] = s;
      }
    }
  }
}

// block sums of a one-right-hand-side block of NT threads (pair and ring kernels): partial rows
// q * nrhs + rhs
template <int NQ, int NT, typename T>
__device__ __forceinline__ void block_sums_1rhs(const HopArgs& a, Sums3<T> local, int rhs, int sblock) {
  __shared__ double wsum[NQ][NT / 32];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    T v = local.q[q];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) wsum[q][threadIdx.x >> 5] = (double)v;
  }
  __syncthreads();
  if (threadIdx.x < NQ) {
    const int q = threadIdx.x;
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) s += wsum[q][w];
    a.partials[((size_t)q * a.nrhs + rhs) * a.part_stride + sblock] = s;
  }
}

// ---- fp16 storage, two sites per thread ---------------------------------------------------------
// The sites A = (x, y, z, t) and B = (x', y, z, t + Lt/2) of the output checkerboard (cb indices
// i and i + Vh/2, same x/2) share one thread, and every float2 holds one real component of both
// (.x = A, .y = B).  Complex arithmetic then becomes real FFMA2/FADD2 arithmetic on pairs with no
// lane swaps or sign shuffles, the factors +-i of the projectors only relabel real and imaginary
// parts, the fp16 conversions land directly in the pair registers, and the site norm folds into
// the accumulation FMAs.  Needs Lt even (the checkerboard already needs Lx even).
struct C2 {
  float2 r, i;
};

// a - b on both lanes (sub.rn.f32x2, sm_100 and later)
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
  unsigned long long ra = *reinterpret_cast<unsigned long long*>(&a), rb = *reinterpret_cast<unsigned long long*>(&b),
                     rd;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
  return *reinterpret_cast<float2*>(&rd);
}

__device__ __forceinline__ C2 c2_from_h2(uint32_t wa, uint32_t wb) {
  const __half2 ha = *reinterpret_cast<const __half2*>(&wa);
  const __half2 hb = *reinterpret_cast<const __half2*>(&wb);
  return C2{make_float2(__low2float(ha), __low2float(hb)), make_float2(__high2float(ha), __high2float(hb))};
}

// project the fp16 neighbours of both sites in half2 arithmetic (as load_project_h), then convert
// the projected components into the pair registers
template <int MU, int S>
__device__ __forceinline__ void load_project_pair(C2 (&h)[2][3], const void* base, int ja, int jb, int stride) {
  const uint4* p = reinterpret_cast<const uint4*>(base);
  uint32_t wa[12], wb[12];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const uint4 va = ldg(p + (size_t)k * stride + ja);
    const uint4 vb = ldg(p + (size_t)k * stride + jb);
    wa[4 * k] = va.x; wa[4 * k + 1] = va.y; wa[4 * k + 2] = va.z; wa[4 * k + 3] = va.w;
    wb[4 * k] = vb.x; wb[4 * k + 1] = vb.y; wb[4 * k + 2] = vb.z; wb[4 * k + 3] = vb.w;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    __half2 aa, ba, ab, bb;
    project_h2<MU, S>(wa, c, aa, ba);
    project_h2<MU, S>(wb, c, ab, bb);
    h[0][c] = C2{make_float2(__low2float(aa), __low2float(ab)), make_float2(__high2float(aa), __high2float(ab))};
    h[1][c] = C2{make_float2(__low2float(ba), __low2float(bb)), make_float2(__high2float(ba), __high2float(bb))};
  }
}

// sign * conj(a b - c d): the third link row from the first two
__device__ __forceinline__ C2 conj_cross(C2 a, C2 b, C2 c, C2 d) {
  const float2 p = __ffma2_rn(c.i, d.i, __fmul2_rn(a.r, b.r));
  const float2 q = __ffma2_rn(a.i, b.i, __fmul2_rn(c.r, d.r));
  const float2 s = __ffma2_rn(c.r, d.i, __fmul2_rn(c.i, d.r));
  const float2 t = __ffma2_rn(a.r, b.i, __fmul2_rn(a.i, b.r));
  return {fsub2(p, q), fsub2(s, t)};
}

template <int RECON, bool SIGN>
__device__ __forceinline__ void load_link_pair(C2 (&u)[9], const void* base, int ja, int jb, int stride, float2 sign) {
  constexpr int NC = RECON == 18 ? 9 : 6;
  const uint2* p = reinterpret_cast<const uint2*>(base);
#pragma unroll
  for (int k = 0; k < (NC + 1) / 2; ++k) {
    const uint2 va = ldg(p + (size_t)k * stride + ja);
    const uint2 vb = ldg(p + (size_t)k * stride + jb);
    u[2 * k] = c2_from_h2(va.x, vb.x);
    if (2 * k + 1 < NC) u[2 * k + 1] = c2_from_h2(va.y, vb.y);
  }
  if constexpr (RECON == 12) {
    u[6] = conj_cross(u[1], u[5], u[2], u[4]);
    u[7] = conj_cross(u[2], u[3], u[0], u[5]);
    u[8] = conj_cross(u[0], u[4], u[1], u[3]);
    if constexpr (SIGN) {
#pragma unroll
      for (int k = 6; k < 9; ++k) u[k] = {__fmul2_rn(sign, u[k].r), __fmul2_rn(sign, u[k].i)};
    }
  }
}

// row r of U h (ADJ: of U^dag h) for one colour vector h
template <bool ADJ>
__device__ __forceinline__ C2 mv_row(const C2 (&u)[9], int r, const C2 (&h)[3]) {
  const C2 e0 = ADJ ? u[r] : u[3 * r], e1 = ADJ ? u[3 + r] : u[3 * r + 1], e2 = ADJ ? u[6 + r] : u[3 * r + 2];
  float2 a = __fmul2_rn(e0.r, h[0].r);
  a = __ffma2_rn(e1.r, h[1].r, a);
  a = __ffma2_rn(e2.r, h[2].r, a);
  float2 b = __fmul2_rn(e0.i, h[0].i);
  b = __ffma2_rn(e1.i, h[1].i, b);
  b = __ffma2_rn(e2.i, h[2].i, b);
  float2 c = __fmul2_rn(e0.r, h[0].i);
  c = __ffma2_rn(e1.r, h[1].i, c);
  c = __ffma2_rn(e2.r, h[2].i, c);
  float2 d = __fmul2_rn(e0.i, h[0].r);
  d = __ffma2_rn(e1.i, h[1].r, d);
  d = __ffma2_rn(e2.i, h[2].r, d);
  // U h: (a - b, c + d);  U^dag h: (a + b, c - d)
  return ADJ ? C2{__fadd2_rn(a, b), fsub2(c, d)} : C2{fsub2(a, b), __fadd2_rn(c, d)};
}

// acc += K n v,  K = +1, -1, +i, -i (0, 1, 2, 3);  nn = -n
template <int K>
__device__ __forceinline__ void acc_scaled(C2& acc, C2 v, float2 n, float2 nn) {
  if constexpr (K == 0) {
    acc.r = __ffma2_rn(n, v.r, acc.r);
    acc.i = __ffma2_rn(n, v.i, acc.i);
  } else if constexpr (K == 1) {
    acc.r = __ffma2_rn(nn, v.r, acc.r);
    acc.i = __ffma2_rn(nn, v.i, acc.i);
  } else if constexpr (K == 2) {
    acc.r = __ffma2_rn(nn, v.i, acc.r);
    acc.i = __ffma2_rn(n, v.r, acc.i);
  } else {
    acc.r = __ffma2_rn(n, v.i, acc.r);
    acc.i = __ffma2_rn(nn, v.r, acc.i);
  }
}

// uh = U h (or U^dag h) row by row, each row rebuilt into the four spins at once (the B tables
// of reconstruct<>), scaled by the neighbours' site norms n
template <int MU, int S, bool ADJ>
__device__ __forceinline__ void mult_rebuild_pair(C2 (&acc)[12], const C2 (&u)[9], const C2 (&h)[2][3], float2 n) {
  const float2 nn = make_float2(-n.x, -n.y);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const C2 a = mv_row<ADJ>(u, c, h[0]);
    const C2 b = mv_row<ADJ>(u, c, h[1]);
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

template <int RECON, int MU, bool DAG>
__device__ __forceinline__ void hop_dir_pair(C2 (&acc)[12], const HopArgs& a, const Coord& ca, const Coord& cb,
                                             int ia, int ib, const char* in, const float* in_norm) {
  constexpr int SF = DAG ? +1 : -1;  // forward:  (1 - isign gamma)
  constexpr int SB = DAG ? -1 : +1;  // backward: (1 + isign gamma)
  const Geom& g = a.g;
  const int last = g.L[MU] - 1;
  C2 h[2][3], u[9];
  {
    Coord na = ca, nb = cb;
    na.x[MU] = ca.x[MU] == last ? 0 : ca.x[MU] + 1;
    nb.x[MU] = cb.x[MU] == last ? 0 : cb.x[MU] + 1;
    const int ja = cb_index(g, na), jb = cb_index(g, nb);
    load_project_pair<MU, SF>(h, in, ja, jb, g.stride);
    const float2 n = make_float2(ldg(in_norm + ja), ldg(in_norm + jb));
    const float ts = (float)g.t_sign;
    const float2 sign = make_float2(ca.x[3] == g.L[3] - 1 ? ts : 1.f, cb.x[3] == g.L[3] - 1 ? ts : 1.f);
    load_link_pair<RECON, MU == 3>(u, a.gauge_fwd[MU], ia, ib, g.stride, sign);
    mult_rebuild_pair<MU, SF, false>(acc, u, h, n);
  }
  {
    Coord na = ca, nb = cb;
    na.x[MU] = ca.x[MU] == 0 ? last : ca.x[MU] - 1;
    nb.x[MU] = cb.x[MU] == 0 ? last : cb.x[MU] - 1;
    const int ja = cb_index(g, na), jb = cb_index(g, nb);
    load_project_pair<MU, SB>(h, in, ja, jb, g.stride);
    const float2 n = make_float2(ldg(in_norm + ja), ldg(in_norm + jb));
    const float ts = (float)g.t_sign;
    const float2 sign = make_float2(na.x[3] == g.L[3] - 1 ? ts : 1.f, nb.x[3] == g.L[3] - 1 ? ts : 1.f);
    load_link_pair<RECON, MU == 3>(u, a.gauge_bwd[MU], ja, jb, g.stride, sign);
    mult_rebuild_pair<MU, SB, true>(acc, u, h, n);
  }
}

// Grid: Vh/2 / TX site blocks x nrhs, right-hand sides fastest (as hop_kernel with NRB = 1).
template <int RECON, int MODE, bool DAG, int REDUCE, int TX, int MINB>
__global__ void __launch_bounds__(TX, MINB) hop_kernel_pair(const HopArgs a) {
  const int sblock = blockIdx.x / a.nrhs;
  const int rhs = blockIdx.x - sblock * a.nrhs;
  const Geom& g = a.g;
  const int half = g.Vh >> 1;
  const int ia = sblock * TX + threadIdx.x;
  Sums3<float> local{{0.f, 0.f, 0.f}};  // thread and warp sums in FP32, block sums in FP64
  if (ia < half && (!a.active || a.active[(size_t)rhs * a.active_stride])) {
    const int ib = ia + half;
    const Coord ca = cb_coords(g, ia, a.out_parity);
    Coord cb = ca;
    cb.x[3] = ca.x[3] + (g.L[3] >> 1);
    cb.x[0] = (ca.x[0] & ~1) + ((a.out_parity + ca.x[1] + ca.x[2] + cb.x[3]) & 1);
    const char* in = (const char*)a.in + (size_t)rhs * a.in_rhs_bytes;
    const float* in_norm = a.in_norm + (size_t)rhs * a.norm_rhs_stride;
    C2 acc[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    hop_dir_pair<RECON, 0, DAG>(acc, a, ca, cb, ia, ib, in, in_norm);
    hop_dir_pair<RECON, 1, DAG>(acc, a, ca, cb, ia, ib, in, in_norm);
    hop_dir_pair<RECON, 2, DAG>(acc, a, ca, cb, ia, ib, in, in_norm);
    hop_dir_pair<RECON, 3, DAG>(acc, a, ca, cb, ia, ib, in, in_norm);
    cplx<float> sa[12], sb[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      sa[k] = {acc[k].r.x, acc[k].i.x};
      sb[k] = {acc[k].r.y, acc[k].i.y};
    }
    local = hop_epilogue<PrecH, MODE, DAG, REDUCE>(a, rhs, ia, sa) + hop_epilogue<PrecH, MODE, DAG, REDUCE>(a, rhs, ib, sb);
  }
  if constexpr (REDUCE != RED_NONE) block_sums_1rhs<red_count<REDUCE>(), TX>(a, local, rhs, sblock);
}

}  // namespace gbc
