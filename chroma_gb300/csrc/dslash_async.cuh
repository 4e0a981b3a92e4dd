// Wilson hopping term for fp16 storage with the loads of the next hops in flight: one site and one
// right-hand side per thread, as hop_kernel with NRB = 1, but the neighbour spinor, its norm and
// the link of each of the 8 hops are copied into a per-thread ring of 4 shared-memory slots by
// cp.async, issued four hops ahead of the arithmetic.  The single-right-hand-side stencil is
// latency-bound (few resident warps, each with one or two hops of loads outstanding): the ring
// keeps four hops of loads in flight per thread without holding them in registers.  Each thread
// reads back only the slots it wrote, so no block barrier is needed; a slot is refilled only
// after the hop that used it has been computed.
#pragma once
#include "dslash.cuh"

namespace gbc {

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// [slot][word][thread]: a warp's accesses to one word are 32 consecutive elements
template <int RECON, int TX>
struct HopRing {
  static constexpr int LK = RECON == 18 ? 5 : 3;  // uint2 link planes
  uint4 sp[4][3][TX];
  uint2 lk[4][LK][TX];
  float nm[4][TX];
};

// the neighbour site and link site of hop h = 2 mu + backward
struct HopSites {
  int j[8];     // neighbour (input parity)
  float sg[2];  // sign of the reconstructed third row for the two time hops (12-real links)
};

__device__ __forceinline__ HopSites hop_sites(const Geom& g, const Coord& c) {
  HopSites hs;
#pragma unroll
  for (int mu = 0; mu < 4; ++mu) {
    Coord f = c, b = c;
    f.x[mu] = c.x[mu] + 1 == g.L[mu] ? 0 : c.x[mu] + 1;
    b.x[mu] = c.x[mu] == 0 ? g.L[mu] - 1 : c.x[mu] - 1;
    hs.j[2 * mu] = cb_index(g, f);
    hs.j[2 * mu + 1] = cb_index(g, b);
    if (mu == 3) {
      hs.sg[0] = c.x[3] == g.L[3] - 1 ? (float)g.t_sign : 1.0f;
      hs.sg[1] = b.x[3] == g.L[3] - 1 ? (float)g.t_sign : 1.0f;
    }
  }
  return hs;
}

template <int RECON, int TX>
__device__ __forceinline__ void issue_hop(HopRing<RECON, TX>& R, int slot, int h, const HopArgs& a, const HopSites& hs,
                                          int idx, const char* in, const float* in_norm) {
  constexpr int LK = HopRing<RECON, TX>::LK;
  const int t = threadIdx.x;
  const int stride = a.g.stride;
  const int mu = h >> 1;
  const bool bwd = h & 1;
  const int j = hs.j[h];
  const uint4* p = reinterpret_cast<const uint4*>(in);
#pragma unroll
  for (int k = 0; k < 3; ++k) cp_async16(&R.sp[slot][k][t], p + (size_t)k * stride + j);
  cp_async4(&R.nm[slot][t], in_norm + j);
  const uint2* l = reinterpret_cast<const uint2*>(bwd ? a.gauge_bwd[mu] : a.gauge_fwd[mu]);
  const int li = bwd ? j : idx;
#pragma unroll
  for (int k = 0; k < LK; ++k) cp_async8(&R.lk[slot][k][t], l + (size_t)k * stride + li);
  cp_commit();
}

// hop H from its slot: half2 projection, site norm, link (12 or 18 reals), packed FP32 colour
// products and reconstruction, as hop_dir_f2
template <int RECON, int H, bool DAG, int TX>
__device__ __forceinline__ void compute_hop(float2 (&acc)[12], const HopRing<RECON, TX>& R, const HopSites& hs) {
  constexpr int MU = H >> 1;
  constexpr bool BWD = (H & 1) != 0;
  constexpr int S = BWD ? (DAG ? -1 : +1) : (DAG ? +1 : -1);
  constexpr int slot = H & 3;
  constexpr int LK = HopRing<RECON, TX>::LK;
  constexpr int NC = RECON == 18 ? 9 : 6;
  const int t = threadIdx.x;
  uint32_t w[12];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const uint4 v = R.sp[slot][k][t];
    w[4 * k] = v.x;
    w[4 * k + 1] = v.y;
    w[4 * k + 2] = v.z;
    w[4 * k + 3] = v.w;
  }
  float2 h[2][3], uh[2][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    __half2 x, y;
    project_h2<MU, S>(w, c, x, y);
    h[0][c] = __half22float2(x);
    h[1][c] = __half22float2(y);
  }
  scale_f2<PrecH>(h, R.nm[slot][t]);
  cplx<float> u[9];
#pragma unroll
  for (int k = 0; k < LK; ++k) {
    const uint2 v = R.lk[slot][k][t];
    const float2 e0 = h2f(v.x), e1 = h2f(v.y);
    u[2 * k] = {e0.x, e0.y};
    if (2 * k + 1 < NC) u[2 * k + 1] = {e1.x, e1.y};
  }
  if constexpr (RECON == 12) {
    const float sign = MU == 3 ? hs.sg[BWD ? 1 : 0] : 1.0f;
    u[6] = sign * conj(u[1] * u[5] - u[2] * u[4]);
    u[7] = sign * conj(u[2] * u[3] - u[0] * u[5]);
    u[8] = sign * conj(u[0] * u[4] - u[1] * u[3]);
  }
  matvec_f2<BWD>(uh, u, h);
  reconstruct_f2<MU, S>(acc, uh);
}

// wait for hop H's copies, compute it, and refill its slot with hop H + 4
template <int RECON, int H, bool DAG, int TX>
__device__ __forceinline__ void ring_step(float2 (&acc)[12], HopRing<RECON, TX>& R, const HopArgs& a,
                                          const HopSites& hs, int idx, const char* in, const float* in_norm) {
  cp_wait<(H < 4 ? 3 : 7 - H)>();
  compute_hop<RECON, H, DAG, TX>(acc, R, hs);
  if constexpr (H + 4 < 8) issue_hop<RECON, TX>(R, H & 3, H + 4, a, hs, idx, in, in_norm);
}

// Grid: Vh / TX site blocks x nrhs, right-hand sides fastest (as hop_kernel with NRB = 1).
template <int RECON, int MODE, bool DAG, int REDUCE, int TX, int MINB>
__global__ void __launch_bounds__(TX, MINB) hop_kernel_async(const HopArgs a) {
  __shared__ HopRing<RECON, TX> R;
  const int sblock = blockIdx.x / a.nrhs;
  const int rhs = blockIdx.x - sblock * a.nrhs;
  const Geom& g = a.g;
  const int idx = sblock * TX + threadIdx.x;
  Sums3<float> local{{0.f, 0.f, 0.f}};  // thread and warp sums in FP32, block sums in FP64
  if (idx < g.Vh && (!a.active || a.active[(size_t)rhs * a.active_stride])) {
    const Coord c = cb_coords(g, idx, a.out_parity);
    const HopSites hs = hop_sites(g, c);
    const char* in = (const char*)a.in + (size_t)rhs * a.in_rhs_bytes;
    const float* in_norm = a.in_norm + (size_t)rhs * a.norm_rhs_stride;
#pragma unroll
    for (int h = 0; h < 4; ++h) issue_hop<RECON, TX>(R, h, h, a, hs, idx, in, in_norm);
    float2 acc[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = make_float2(0.f, 0.f);
    ring_step<RECON, 0, DAG, TX>(acc, R, a, hs, idx, in, in_norm);
    ring_step<RECON, 1, DAG, TX>(acc, R, a, hs, idx, in, in_norm);
    ring_step<RECON, 2, DAG, TX>(acc, R, a, hs, idx, in, in_norm);
    ring_step<RECON, 3, DAG, TX>(acc, R, a, hs, idx, in, in_norm);
    ring_step<RECON, 4, DAG, TX>(acc, R, a, hs, idx, in, in_norm);
    ring_step<RECON, 5, DAG, TX>(acc, R, a, hs, idx, in, in_norm);
    ring_step<RECON, 6, DAG, TX>(acc, R, a, hs, idx, in, in_norm);
    ring_step<RECON, 7, DAG, TX>(acc, R, a, hs, idx, in, in_norm);
    cplx<float> out[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) out[k] = {acc[k].x, acc[k].y};
    local = hop_epilogue<PrecH, MODE, DAG, REDUCE>(a, rhs, idx, out);
  }
  if constexpr (REDUCE != RED_NONE) block_sums_1rhs<red_count<REDUCE>(), TX>(a, local, rhs, sblock);
}

}  // namespace gbc
