// The inner CGNE of a batch of lattices as a persistent kernel: one cooperative launch runs many
// iterations for every lattice (InvCG2's recursion, invcg2.cc:153-221, on M~^dag M~ of each
// lattice), walking the batch's work table of (lattice, 128-site block) pairs with a grid-stride
// loop, so the GPU stays busy across lattices of different sizes without a launch per step.
//
// Per iteration, 5 grid barriers separate the passes that read another block's output:
//   te = A_ee^-1 D_eo p | mp = A_oo p - 1/4 D_oe te, |mp|^2 partials | alpha (every block) |
//   te = (..)^dag mp | q = (..)^dag mp in registers, e += a p, r -= a q, |r|^2 partials |
//   beta (every block) | p = r + b p |
// Every block keeps its own copy of every lattice's scalars in shared memory and sums the partials
// of each lattice in the same fixed order (one warp per lattice), so all blocks hold
// bitwise-identical scalars and take identical decisions (skip a converged lattice, stop for a
// reliable update or when every lattice has converged) without sharing them.
//
// The grid barrier spins on a generation counter with a time limit (about 2 s of SM clock): a wait
// that runs out sets an error flag, after which every block leaves at its next barrier and the
// host reports the solve as failed; no wait is unbounded.  A cooperative launch guarantees that
// every block is resident, so the barrier is only a guard against the unexpected.
//
// This file is compiled with GBC_COHERENT_LOADS: spinor fields, which other blocks of the same
// launch wrote before a barrier, are read with plain loads instead of ld.global.nc (links and
// clover, which nothing writes, keep the read-only path).
#pragma once
#include <algorithm>

#include "batch_ops.cuh"
#include "dslash.cuh"

namespace gbc {
namespace persistent {

constexpr long long kWaitCycles = 4000000000LL;  // SM clock cycles (~2 s at 2 GHz)

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// returns false when this barrier or an earlier one of the launch gave up waiting.  Arrival is a
// release-ordered atomic on the counter; the last block resets it and bumps the generation, which
// the others poll with acquire loads (busy for the first polls, then with short sleeps); the error
// flag and the clock are looked at every 64 polls only.
__device__ __forceinline__ bool grid_barrier(GridBar* gb, unsigned nblocks, int where) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile int* errp = &gb->err;
    const unsigned g = ld_acquire(&gb->gen);
    __threadfence();
    const unsigned arrived = atomicAdd(&gb->count, 1u) + 1u;
    int good = 1;
    if (arrived == nblocks) {
      gb->count = 0;
      __threadfence();
      atomicAdd(&gb->gen, 1u);
    } else {
      const long long t0 = clock64();
      for (unsigned polls = 1; ld_acquire(&gb->gen) == g; ++polls) {
        if ((polls & 63) == 0 && (*errp || clock64() - t0 > kWaitCycles)) {
          if (atomicCAS(&gb->err, 0, 1) == 0) gb->where = where;
          good = 0;
          break;
        }
        if (polls > 256) __nanosleep(20);
      }
    }
    __threadfence();
    ok = good && !*errp;
  }
  __syncthreads();
  return ok;
}

// FP64 sum of n partials by one warp, identical in every block (fixed lane mapping and order);
// every lane of the warp gets the total.  The lattices of a batch are summed by different warps
// side by side, so a reduction phase costs one round of loads whatever the number of lattices.
__device__ __forceinline__ double warp_total(const double* part, int n, int lane) {
  double s = 0.0;
  for (int i = lane; i < n; i += 32) s += part[i];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  return s;
}

// q = M~^dag mp at the block's odd sites (the isign-MINUS XPAY epilogue of a, kept in registers)
// fused with the CG update e += alpha p, r -= alpha q, and |r|^2 of the block -> l.upd_part
template <typename PA, typename PO, int RECON>
__device__ __forceinline__ void xpay_dag_update_block(const HopArgs& a, const LatCg& l, int sblock, double alpha) {
  static_assert(std::is_same<typename PO::real, float>::value && std::is_same<typename PA::real, float>::value,
                "FP32-arithmetic stencil and accumulators");
  const int idx = sblock * kBatchSites + threadIdx.x;
  float accr = 0.f;
  if (idx < a.g.Vh) {
    const Coord c = cb_coords(a.g, idx, a.out_parity);
    const char* in = (const char*)a.in;
    float2 accf[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) accf[k] = make_float2(0.f, 0.f);
    hop_dir_f2<PO, RECON, 0, true>(accf, a, c, idx, in, a.in_norm);
    hop_dir_f2<PO, RECON, 1, true>(accf, a, c, idx, in, a.in_norm);
    hop_dir_f2<PO, RECON, 2, true>(accf, a, c, idx, in, a.in_norm);
    hop_dir_f2<PO, RECON, 3, true>(accf, a, c, idx, in, a.in_norm);
    cplx<float> acc[12], q[12], self[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = {accf[k].x, accf[k].y};
    hop_epilogue_value<PO, HOP_XPAY, true>(a, 0, idx, acc, q, self);
    cplx<float> es[12], rs[12], ps[12];
    ldf<PA>(es, l.e, idx);
    ldf<PA>(rs, l.r, idx);
    ldf<PO>(ps, l.p, idx);
    const float al = (float)alpha;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      es[k].re = fmadd(al, ps[k].re, es[k].re);
      es[k].im = fmadd(al, ps[k].im, es[k].im);
      rs[k].re = fmadd(-al, q[k].re, rs[k].re);
      rs[k].im = fmadd(-al, q[k].im, rs[k].im);
      accr = fmadd(rs[k].re, rs[k].re, fmadd(rs[k].im, rs[k].im, accr));
    }
    stf<PA>(l.e, idx, es);
    stf<PA>(l.r, idx, rs);
  }
  __shared__ double sh[kBatchSites / 32];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) accr += __shfl_down_sync(0xffffffffu, accr, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)accr;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
#pragma unroll
    for (int q = 0; q < kBatchSites / 32; ++q) t += sh[q];
    l.upd_part[sblock] = t;
  }
  __syncthreads();  // sh is reused by the next call
}

template <typename PA, typename PO, int RECON, int MINB>
__global__ void __launch_bounds__(kBatchSites, MINB)
cg_kernel(const HopArgs* __restrict__ args, const LatCg* __restrict__ lat, const int2* __restrict__ work, int nwork,
          int n, int kmax, double delta, PersistLat* pl, GridBar* gb, int* out) {
  constexpr int L = kPersistMaxLattices;
  __shared__ double s_c[L], s_d[L], s_a[L], s_b[L], s_cp[L], s_cprev[L], s_rsd[L], s_max[L], s_atu[L];
  __shared__ int s_act[L], s_it[L];
  __shared__ int s_stop;
  const int tid = threadIdx.x;
  if (tid < n) {
    const CGScalars st = *lat[tid].cg;
    s_c[tid] = st.c;
    s_d[tid] = st.d;
    s_a[tid] = st.a;
    s_b[tid] = st.b;
    s_cp[tid] = st.cp;
    s_cprev[tid] = st.c_prev;
    s_rsd[tid] = st.rsd_sq;
    s_act[tid] = st.active;
    s_it[tid] = st.iters;
    s_max[tid] = pl[tid].maxrr;
    s_atu[tid] = pl[tid].at_update;
  }
  if (tid == 0) s_stop = 0;
  __syncthreads();
  const unsigned nb = gridDim.x;
  int k = 0;
  int bar = 0;
  bool ok = true;
  while (k < kmax) {
    // te = A_ee^-1 D_eo p
    for (int w = blockIdx.x; w < nwork; w += nb) {
      const int2 wk = work[w];
      if (s_act[wk.x]) hop_body<PO, RECON, HOP_CLOV, false, RED_NONE, kBatchSites, 1>(args[wk.x], wk.y, 0);
    }
    if (!(ok = grid_barrier(gb, nb, bar++))) break;
    // mp = A_oo p - 1/4 D_oe te with |mp|^2 per block
    for (int w = blockIdx.x; w < nwork; w += nb) {
      const int2 wk = work[w];
      if (s_act[wk.x]) hop_body<PO, RECON, HOP_XPAY, false, RED_NORM, kBatchSites, 1>(args[n + wk.x], wk.y, 0);
    }
    if (!(ok = grid_barrier(gb, nb, bar++))) break;
    // alpha = |r|^2 / |M~ p|^2 per lattice (warp w sums lattices w, w + 4, ...)
    for (int l = tid >> 5; l < n; l += kBatchSites / 32) {
      if (!s_act[l]) continue;
      const double d = warp_total(lat[l].hop_part, lat[l].nblk, tid & 31);
      if ((tid & 31) == 0) {
        s_d[l] = d;
        s_a[l] = d > 0.0 ? s_c[l] / d : 0.0;
      }
    }
    __syncthreads();
    // te = (A_ee^-1 D_eo)^dag mp ; q = M~^dag mp
    for (int w = blockIdx.x; w < nwork; w += nb) {
      const int2 wk = work[w];
      if (s_act[wk.x]) hop_body<PO, RECON, HOP_CLOV, true, RED_NONE, kBatchSites, 1>(args[2 * n + wk.x], wk.y, 0);
    }
    if (!(ok = grid_barrier(gb, nb, bar++))) break;
    // with q = M~^dag mp in registers: e += a p ; r -= a q with |r|^2 per block
    for (int w = blockIdx.x; w < nwork; w += nb) {
      const int2 wk = work[w];
      if (s_act[wk.x]) xpay_dag_update_block<PA, PO, RECON>(args[3 * n + wk.x], lat[wk.x], wk.y, s_a[wk.x]);
    }
    if (!(ok = grid_barrier(gb, nb, bar++))) break;
    // beta, convergence and the reliable-update trigger per lattice (warp w: lattices w, w + 4, ...)
    for (int l = tid >> 5; l < n; l += kBatchSites / 32) {
      if (!s_act[l]) continue;
      const double cp = warp_total(lat[l].upd_part, lat[l].nblk, tid & 31);
      if ((tid & 31) == 0) {
        const double c = s_c[l];
        const int act = cp > s_rsd[l];
        s_cp[l] = cp;
        s_it[l] += 1;
        s_b[l] = (act && c > 0.0) ? cp / c : 0.0;
        s_cprev[l] = c;
        s_c[l] = cp;
        s_act[l] = act;
        // the reliable-update test at the cadence of the per-launch path (after every 4th
        // iteration): the CG residual is not monotone, and a test after every iteration would
        // stop on its short rises above |r| at the last update
        if (((k + 1) & 3) == 0) {
          const double rn = sqrt(cp);
          s_max[l] = fmax(s_max[l], rn);
          if (act && (rn < delta * s_max[l] || rn > s_atu[l])) s_stop = 1;
        }
      }
    }
    __syncthreads();  // every lattice's scalars updated
    if (tid == 0) {
      int any = 0;
      for (int l = 0; l < n; ++l) any |= s_act[l];
      if (!any) s_stop = 1;
    }
    __syncthreads();
    // p = r + b p for the lattices still iterating
    for (int w = blockIdx.x; w < nwork; w += nb) {
      const int2 wk = work[w];
      if (s_act[wk.x]) batch_xpay_block<PA, PO>(lat[wk.x], wk.y, s_b[wk.x]);
    }
    if (!(ok = grid_barrier(gb, nb, bar++))) break;
    ++k;
    if (s_stop) break;
  }
  if (!ok) return;
  if (blockIdx.x == 0) {
    if (tid < n) {
      CGScalars st;
      st.c = s_c[tid];
      st.d = s_d[tid];
      st.a = s_a[tid];
      st.b = s_b[tid];
      st.cp = s_cp[tid];
      st.rsd_sq = s_rsd[tid];
      st.c_prev = s_cprev[tid];
      st.active = s_act[tid];
      st.iters = s_it[tid];
      *lat[tid].cg = st;
      pl[tid].maxrr = s_max[tid];
    }
    if (tid == 0) out[0] = k;
  }
}

template <typename PA, typename PO, int RECON, int MINB = 4>
int launch(const HopArgs* args, const LatCg* lat, const int2* work, int nwork, int n, int kmax, double delta,
           PersistLat* pl, GridBar* bar, int* out, cudaStream_t s) {
  auto kern = cg_kernel<PA, PO, RECON, MINB>;
  static int per_sm = -1, sms = 0;
  if (per_sm < 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBatchSites, 0) != cudaSuccess)
      per_sm = 0;
  }
  if (per_sm <= 0) return -1;
  const int grid = std::min(nwork, per_sm * sms);
  cudaError_t e = cudaMemsetAsync(bar, 0, sizeof(GridBar), s);
  if (e != cudaSuccess) return (int)e;
  void* kargs[] = {(void*)&args, (void*)&lat, (void*)&work, (void*)&nwork, (void*)&n, (void*)&kmax,
                   (void*)&delta, (void*)&pl, (void*)&bar, (void*)&out};
  e = cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(kBatchSites), kargs, 0, s);
  if (e == cudaErrorCooperativeLaunchTooLarge || e == cudaErrorNotSupported) {
    (void)cudaGetLastError();
    return -1;
  }
  return (int)e;
}

}  // namespace persistent
}  // namespace gbc
