// Device-side building blocks shared by the stencil, clover and BLAS kernels:
// complex arithmetic, the checkerboard geometry, and the packed field formats.
//
// Field formats in HBM (one checkerboard = Vh sites; "stride" = padded Vh):
//   spinor  double : double2 [12][stride]  one complex per plane (component k = spin*3 + colour)
//           single : float4  [ 6][stride]  two complex per plane
//           half   : uint4   [ 3][stride]  four complex per plane (fp16) + float norm[stride];
//                    stored value = component / norm(site), norm = max |re|,|im| over the site
//   gauge   per (parity, mu), 12-real (rows 0,1; row 2 = sign * conj(row0 x row1)) or 18-real
//           double : double2 planes, one complex each   (6 or 9 planes)
//           single : float4  planes, two complex each   (3 or 5 planes)
//           half   : uint2   planes, two complex each   (3 or 5 planes)
//   clover  per parity, Chroma's packed Hermitian blocks (clover_term_qdp_w.h:19-24) in the order
//           block0 {diag[6], offd[15] complex}, block1 {...}: 36 reals per block
//           double : double2 [36][stride]
//           single : float4  [18][stride]
//           half   : per block uint4[4] + uint2[1]  -> uint4 [8][stride] then uint2 [2][stride]
//   double-float copies of the FP64 links and clover (PrecDF): the FP64 planes with every double
//   split into (hi, lo) floats, a double2 (re, im) becoming a float4 (re.hi, re.lo, im.hi, im.lo)
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "gbc_kernels.h"

namespace gbc {

template <typename T>
struct cplx {
  T re, im;
};

template <typename T>
__device__ __forceinline__ cplx<T> mk(T r, T i) { return cplx<T>{r, i}; }
template <typename T>
__device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <typename T>
__device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <typename T>
__device__ __forceinline__ cplx<T> operator-(cplx<T> a) { return {-a.re, -a.im}; }
template <typename T>
__device__ __forceinline__ cplx<T> operator*(cplx<T> a, cplx<T> b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
template <typename T>
__device__ __forceinline__ cplx<T> operator*(T s, cplx<T> a) { return {s * a.re, s * a.im}; }
template <typename T>
__device__ __forceinline__ cplx<T> conj(cplx<T> a) { return {a.re, -a.im}; }
template <typename T>
__device__ __forceinline__ cplx<T> timesI(cplx<T> a) { return {-a.im, a.re}; }
template <typename T>
__device__ __forceinline__ cplx<T> timesMinusI(cplx<T> a) { return {a.im, -a.re}; }
__device__ __forceinline__ double fmadd(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fmadd(float a, float b, float c) { return __fmaf_rn(a, b, c); }
// acc += a * b
template <typename T>
__device__ __forceinline__ void cmac(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fmadd(a.re, b.re, acc.re);
  acc.re = fmadd(-a.im, b.im, acc.re);
  acc.im = fmadd(a.re, b.im, acc.im);
  acc.im = fmadd(a.im, b.re, acc.im);
}
// acc += conj(a) * b
template <typename T>
__device__ __forceinline__ void cmacc(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fmadd(a.re, b.re, acc.re);
  acc.re = fmadd(a.im, b.im, acc.re);
  acc.im = fmadd(a.re, b.im, acc.im);
  acc.im = fmadd(-a.im, b.re, acc.im);
}

// --------------------------------------------------------------------------------------------
// Geometry of one checkerboard.  cb index i <-> (x, y, z, t) with x = 2*xh + ((p+y+z+t)&1),
// xh = i % (Lx/2): the canonical site index x + Lx*(y + Ly*(z + Lz*t)) halved.
// --------------------------------------------------------------------------------------------
struct Coord {
  int x[4];
};

__device__ __forceinline__ Coord cb_coords(const Geom& g, int i, int parity) {
  Coord c;
  int xh = i % g.Lxh;
  int r = i / g.Lxh;
  c.x[1] = r % g.L[1];
  r /= g.L[1];
  c.x[2] = r % g.L[2];
  c.x[3] = r / g.L[2];
  c.x[0] = 2 * xh + ((parity + c.x[1] + c.x[2] + c.x[3]) & 1);
  return c;
}

__device__ __forceinline__ int cb_index(const Geom& g, const Coord& c) {
  return (c.x[0] >> 1) + g.Lxh * (c.x[1] + g.L[1] * (c.x[2] + g.L[2] * c.x[3]));
}

__device__ __forceinline__ int full_index(const Geom& g, const Coord& c) {
  return c.x[0] + g.L[0] * (c.x[1] + g.L[1] * (c.x[2] + g.L[2] * c.x[3]));
}

// --------------------------------------------------------------------------------------------
// Double-float arithmetic: a value is hi + lo with two floats (a 48-bit significand), built from
// the error-free transformations TwoSum (Knuth), QuickTwoSum (Dekker) and TwoProduct by FMA, in the
// "sloppy" addition of the published double-double libraries (Bailey's DD, Hida-Li-Bailey QD):
// the error of a sum is of the order 2^-46 of its largest operand.  GB300 runs FP32 at many times
// its FP64 rate, so FP64-stored fields go through stencils in this arithmetic where ~1e-14 of
// accuracy suffices.  Every operation uses the _rn intrinsics, which the compiler never contracts
// into FMAs (contraction would break the error-free transformations).
// --------------------------------------------------------------------------------------------
struct df64 {
  float hi, lo;
  df64() = default;
  __device__ __forceinline__ df64(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ df64(int v) : hi((float)v), lo(0.f) {}
  __device__ __forceinline__ df64(float v) : hi(v), lo(0.f) {}
  __device__ __forceinline__ df64(double v);
};

__device__ __forceinline__ df64 quick_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return df64(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ df64 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  return df64(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v)));
}
__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  const df64 s = two_sum(a.hi, b.hi);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}
__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }
// a * b + c with one renormalisation
__device__ __forceinline__ df64 fmadd(df64 a, df64 b, df64 c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const df64 s = two_sum(p, c.hi);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo)));
}

// double -> hi + lo by integer operations (GB300's FP64 pipe, which the conversion instructions
// would use, is the slow part this arithmetic avoids): hi = the leading 24 bits of the significand,
// lo = the remaining 29 bits rounded to 24, then renormalised.  |x| below 2^-126 maps to zero (far
// below any field value the solvers carry); |x| above float's range is not a lattice field value.
__device__ __forceinline__ df64 df64_from_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff);
  if (e < 897) return df64(0.f, 0.f);
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  const float hi = __uint_as_float(sgn | ((unsigned)(e - 896) << 23) | (unsigned)(m >> 29));
  const unsigned ml = (unsigned)(m & 0x1FFFFFFFull);
  float lo = 0.f;
  if (e >= 949) {
    // ml = mh 2^23 + mlow with both parts exact in float (magic-number conversion), then one rounding
    const float mlow = __fsub_rn(__uint_as_float(0x4B000000u | (ml & 0x7FFFFFu)), 8388608.f);
    const float mh = __fsub_rn(__uint_as_float(0x4B000000u | (ml >> 23)), 8388608.f);
    const float mf = __fmaf_rn(mh, 8388608.f, mlow);
    lo = __uint_as_float(__float_as_uint(__fmul_rn(mf, __uint_as_float((unsigned)(e - 948) << 23))) | sgn);
  }
  return quick_two_sum(hi, lo);
}
__device__ __forceinline__ df64::df64(double v) { *this = df64_from_bits(v); }

// float -> double by integer operations (exact; zero and subnormal floats map to zero)
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0) return 0.0;
  const unsigned long long b = ((unsigned long long)(u & 0x80000000u) << 32) |
                               ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)b);
}
__device__ __forceinline__ double df64_to_double(df64 v) { return f2d_bits(v.hi) + f2d_bits(v.lo); }

// --------------------------------------------------------------------------------------------
// Precision tags
// --------------------------------------------------------------------------------------------
struct PrecD { using real = double; static constexpr int bytes = 8; };
struct PrecS { using real = float; static constexpr int bytes = 4; };
struct PrecH { using real = float; static constexpr int bytes = 2; };  // fp16 storage, fp32 arithmetic
// FP64 storage, double-float arithmetic: spinors are the FP64 fields; links and clover come from
// a copy whose every FP64 value is split once into (hi, lo) floats (same bytes, same plane layout,
// a double2 (re, im) becoming a float4 (re.hi, re.lo, im.hi, im.lo))
struct PrecDF { using real = df64; static constexpr int bytes = 8; };

// Accumulator of a site functor's reductions: F::Acc when the functor declares one (its compute
// precision), else double.  The reduction drivers sum a thread's sites and the lanes of a warp in
// Acc and only the per-warp results in FP64: GB300's FP64 pipe is slow enough that one FP64
// conversion and add per site and quantity made a bandwidth-bound reduction FP64-bound.
template <class F, class = void>
struct AccOf {
  using type = double;
};
template <class F>
struct AccOf<F, std::void_t<typename F::Acc>> {
  using type = typename F::Acc;
};

template <typename P> struct Store;
template <> struct Store<PrecD> { using vec = double2; };
template <> struct Store<PrecS> { using vec = float4; };
template <> struct Store<PrecH> { using vec = uint4; };
template <> struct Store<PrecDF> { using vec = double2; };

// Spinor views: base pointer of one right-hand side, plus norm for half
template <typename P>
struct SpinorRef {
  void* v;
  float* norm;  // half only
};

__device__ __forceinline__ float2 h2f(uint32_t w) {
  __half2 h = *reinterpret_cast<__half2*>(&w);
  return __half22float2(h);
}
__device__ __forceinline__ uint32_t f2h(float a, float b) {
  __half2 h = __floats2half2_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

// Loads of data that no kernel writes while it runs (links, clover, tables): the read-only path.
template <typename T>
__device__ __forceinline__ T ldg(const T* p) { return __ldg(p); }
// Loads of spinor fields and their norms.  Translation units whose kernels read fields that other
// blocks of the same launch wrote (the persistent batch kernel, between its grid barriers) define
// GBC_COHERENT_LOADS: plain loads, which the barrier's gpu-scope fences order after those writes;
// the read-only path (ld.global.nc) requires data that no one writes while the kernel runs.
#ifdef GBC_COHERENT_LOADS
template <typename T>
__device__ __forceinline__ T ldw(const T* p) { return *p; }
#else
template <typename T>
__device__ __forceinline__ T ldw(const T* p) { return __ldg(p); }
#endif

// ---- spinor load/store -------------------------------------------------------------------------
template <typename P>
__device__ __forceinline__ void load_spinor(cplx<typename P::real> (&s)[12], const void* base, const float* norm,
                                            int idx, int stride);

template <>
__device__ __forceinline__ void load_spinor<PrecD>(cplx<double> (&s)[12], const void* base, const float*, int idx,
                                                   int stride) {
  const double2* p = reinterpret_cast<const double2*>(base);
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    double2 v = ldw(p + (size_t)k * stride + idx);
    s[k] = {v.x, v.y};
  }
}
template <>
__device__ __forceinline__ void load_spinor<PrecS>(cplx<float> (&s)[12], const void* base, const float*, int idx,
                                                   int stride) {
  const float4* p = reinterpret_cast<const float4*>(base);
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    float4 v = ldw(p + (size_t)k * stride + idx);
    s[2 * k] = {v.x, v.y};
    s[2 * k + 1] = {v.z, v.w};
  }
}
template <>
__device__ __forceinline__ void load_spinor<PrecH>(cplx<float> (&s)[12], const void* base, const float* norm, int idx,
                                                   int stride) {
  const uint4* p = reinterpret_cast<const uint4*>(base);
  float n = ldw(norm + idx);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    uint4 v = ldw(p + (size_t)k * stride + idx);
    float2 a = h2f(v.x), b = h2f(v.y), c = h2f(v.z), d = h2f(v.w);
    s[4 * k + 0] = {a.x * n, a.y * n};
    s[4 * k + 1] = {b.x * n, b.y * n};
    s[4 * k + 2] = {c.x * n, c.y * n};
    s[4 * k + 3] = {d.x * n, d.y * n};
  }
}

// A double-float kernel reads its spinor operands from their split copies (made once per launch by
// split_df64: every double2 (re, im) of the FP64 field as a float4 (re.hi, re.lo, im.hi, im.lo),
// same bytes and index), so a neighbour spinor costs no conversion at each of its 8 uses; results
// are stored as FP64.
template <>
__device__ __forceinline__ void load_spinor<PrecDF>(cplx<df64> (&s)[12], const void* base, const float*, int idx,
                                                    int stride) {
  const float4* p = reinterpret_cast<const float4*>(base);
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    float4 v = ldw(p + (size_t)k * stride + idx);
    s[k] = {df64(v.x, v.y), df64(v.z, v.w)};
  }
}

template <typename P>
__device__ __forceinline__ void store_spinor(void* base, float* norm, int idx, int stride,
                                             const cplx<typename P::real> (&s)[12]);
template <>
__device__ __forceinline__ void store_spinor<PrecDF>(void* base, float*, int idx, int stride,
                                                     const cplx<df64> (&s)[12]) {
  double2* p = reinterpret_cast<double2*>(base);
#pragma unroll
  for (int k = 0; k < 12; ++k)
    p[(size_t)k * stride + idx] = make_double2(df64_to_double(s[k].re), df64_to_double(s[k].im));
}

template <>
__device__ __forceinline__ void store_spinor<PrecD>(void* base, float*, int idx, int stride,
                                                    const cplx<double> (&s)[12]) {
  double2* p = reinterpret_cast<double2*>(base);
#pragma unroll
  for (int k = 0; k < 12; ++k) p[(size_t)k * stride + idx] = make_double2(s[k].re, s[k].im);
}
template <>
__device__ __forceinline__ void store_spinor<PrecS>(void* base, float*, int idx, int stride,
                                                    const cplx<float> (&s)[12]) {
  float4* p = reinterpret_cast<float4*>(base);
#pragma unroll
  for (int k = 0; k < 6; ++k) p[(size_t)k * stride + idx] = make_float4(s[2 * k].re, s[2 * k].im, s[2 * k + 1].re, s[2 * k + 1].im);
}
template <>
__device__ __forceinline__ void store_spinor<PrecH>(void* base, float* norm, int idx, int stride,
                                                    const cplx<float> (&s)[12]) {
  uint4* p = reinterpret_cast<uint4*>(base);
  float m = 0.f;
#pragma unroll
  for (int k = 0; k < 12; ++k) m = fmaxf(m, fmaxf(fabsf(s[k].re), fabsf(s[k].im)));
  // a site whose largest component is below 1e-30 is stored as zero: 1/m would overflow for
  // subnormal m (and 0 * inf = NaN), and such a site is far below fp16 resolution of any field
  // the solvers carry
  const bool live = m >= 1e-30f;
  float inv = live ? 1.0f / m : 0.f;
  norm[idx] = live ? m : 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    uint4 v;
    v.x = f2h(s[4 * k].re * inv, s[4 * k].im * inv);
    v.y = f2h(s[4 * k + 1].re * inv, s[4 * k + 1].im * inv);
    v.z = f2h(s[4 * k + 2].re * inv, s[4 * k + 2].im * inv);
    v.w = f2h(s[4 * k + 3].re * inv, s[4 * k + 3].im * inv);
    p[(size_t)k * stride + idx] = v;
  }
}

// ---- gauge links --------------------------------------------------------------------------------
template <typename P, int RECON>
struct LinkPlanes;
template <> struct LinkPlanes<PrecD, 18> { static constexpr int n = 9; };
template <> struct LinkPlanes<PrecD, 12> { static constexpr int n = 6; };
template <> struct LinkPlanes<PrecS, 18> { static constexpr int n = 5; };
template <> struct LinkPlanes<PrecS, 12> { static constexpr int n = 3; };
template <> struct LinkPlanes<PrecH, 18> { static constexpr int n = 5; };
template <> struct LinkPlanes<PrecH, 12> { static constexpr int n = 3; };
template <> struct LinkPlanes<PrecDF, 18> { static constexpr int n = 9; };

template <typename P>
struct LinkVec;
template <> struct LinkVec<PrecD> { using vec = double2; };
template <> struct LinkVec<PrecS> { using vec = float4; };
template <> struct LinkVec<PrecH> { using vec = uint2; };
template <> struct LinkVec<PrecDF> { using vec = float4; };

// Load link (row-major 3x3) from its planes; for RECON 12 rebuild row 2 = sign * conj(row0 x row1).
template <typename P, int RECON>
__device__ __forceinline__ void load_link(cplx<typename P::real> (&u)[9], const void* base, int idx, int stride,
                                          typename P::real sign) {
  using T = typename P::real;
  constexpr int NC = RECON == 18 ? 9 : 6;
  if constexpr (std::is_same<P, PrecD>::value) {
    const double2* p = reinterpret_cast<const double2*>(base);
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      double2 v = ldg(p + (size_t)k * stride + idx);
      u[k] = {v.x, v.y};
    }
  } else if constexpr (std::is_same<P, PrecDF>::value) {
    static_assert(RECON == 18, "FP64-stored links keep 18 reals");
    const float4* p = reinterpret_cast<const float4*>(base);
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      float4 v = ldg(p + (size_t)k * stride + idx);
      u[k] = {df64(v.x, v.y), df64(v.z, v.w)};
    }
  } else if constexpr (std::is_same<P, PrecS>::value) {
    const float4* p = reinterpret_cast<const float4*>(base);
#pragma unroll
    for (int k = 0; k < (NC + 1) / 2; ++k) {
      float4 v = ldg(p + (size_t)k * stride + idx);
      u[2 * k] = {v.x, v.y};
      if (2 * k + 1 < NC) u[2 * k + 1] = {v.z, v.w};
    }
  } else {
    const uint2* p = reinterpret_cast<const uint2*>(base);
#pragma unroll
    for (int k = 0; k < (NC + 1) / 2; ++k) {
      uint2 v = ldg(p + (size_t)k * stride + idx);
      float2 a = h2f(v.x), b = h2f(v.y);
      u[2 * k] = {a.x, a.y};
      if (2 * k + 1 < NC) u[2 * k + 1] = {b.x, b.y};
    }
  }
  if constexpr (RECON == 12) {
    // row2 = sign * conj(row0 x row1)
    u[6] = sign * conj(u[1] * u[5] - u[2] * u[4]);
    u[7] = sign * conj(u[2] * u[3] - u[0] * u[5]);
    u[8] = sign * conj(u[0] * u[4] - u[1] * u[3]);
  }
  (void)sizeof(T);
}

// ---- clover blocks ----------------------------------------------------------------------------
// Load one 36-real packed block b into (diag[6], offd[15]) in compute precision.
template <typename P>
__device__ __forceinline__ void load_clover_block(typename P::real (&d)[6], cplx<typename P::real> (&o)[15],
                                                  const void* base, int idx, int stride, int b) {
  if constexpr (std::is_same<P, PrecD>::value) {
    const double2* p = reinterpret_cast<const double2*>(base) + (size_t)(18 * b) * stride + idx;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double2 v = ldg(p + (size_t)k * stride);
      d[2 * k] = v.x;
      d[2 * k + 1] = v.y;
    }
#pragma unroll
    for (int k = 0; k < 15; ++k) {
      double2 v = ldg(p + (size_t)(3 + k) * stride);
      o[k] = {v.x, v.y};
    }
  } else if constexpr (std::is_same<P, PrecDF>::value) {
    const float4* p = reinterpret_cast<const float4*>(base) + (size_t)(18 * b) * stride + idx;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float4 v = ldg(p + (size_t)k * stride);
      d[2 * k] = df64(v.x, v.y);
      d[2 * k + 1] = df64(v.z, v.w);
    }
#pragma unroll
    for (int k = 0; k < 15; ++k) {
      float4 v = ldg(p + (size_t)(3 + k) * stride);
      o[k] = {df64(v.x, v.y), df64(v.z, v.w)};
    }
  } else if constexpr (std::is_same<P, PrecS>::value) {
    const float4* p = reinterpret_cast<const float4*>(base) + (size_t)(9 * b) * stride + idx;
    float r[36];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      float4 v = ldg(p + (size_t)k * stride);
      r[4 * k] = v.x; r[4 * k + 1] = v.y; r[4 * k + 2] = v.z; r[4 * k + 3] = v.w;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) d[k] = r[k];
#pragma unroll
    for (int k = 0; k < 15; ++k) o[k] = {r[6 + 2 * k], r[7 + 2 * k]};
  } else {
    const uint4* p4 = reinterpret_cast<const uint4*>(base) + (size_t)(4 * b) * stride + idx;
    const uint2* p2 = reinterpret_cast<const uint2*>(reinterpret_cast<const uint4*>(base) + (size_t)8 * stride) +
                      (size_t)b * stride + idx;
    float r[36];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      uint4 v = ldg(p4 + (size_t)k * stride);
      float2 a = h2f(v.x), bb = h2f(v.y), c = h2f(v.z), e = h2f(v.w);
      r[8 * k] = a.x; r[8 * k + 1] = a.y; r[8 * k + 2] = bb.x; r[8 * k + 3] = bb.y;
      r[8 * k + 4] = c.x; r[8 * k + 5] = c.y; r[8 * k + 6] = e.x; r[8 * k + 7] = e.y;
    }
    uint2 v = ldg(p2);
    float2 a = h2f(v.x), bb = h2f(v.y);
    r[32] = a.x; r[33] = a.y; r[34] = bb.x; r[35] = bb.y;
#pragma unroll
    for (int k = 0; k < 6; ++k) d[k] = r[k];
#pragma unroll
    for (int k = 0; k < 15; ++k) o[k] = {r[6 + 2 * k], r[7 + 2 * k]};
  }
}

// y[6] = T x[6] for one Hermitian block (diag, lower offd packed i*(i-1)/2+j)
template <typename T>
__device__ __forceinline__ void clover_block_mul(cplx<T> (&y)[6], const T (&d)[6], const cplx<T> (&o)[15],
                                                 const cplx<T> (&x)[6]) {
#pragma unroll
  for (int i = 0; i < 6; ++i) y[i] = d[i] * x[i];
  int k = 0;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
#pragma unroll
    for (int j = 0; j < i; ++j) {
      cmac(y[i], o[k], x[j]);
      cmacc(y[j], o[k], x[i]);
      ++k;
    }
  }
}

}  // namespace gbc
