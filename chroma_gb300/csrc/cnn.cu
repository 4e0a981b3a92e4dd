// Learned preconditioner: a gauge-covariant convolutional network approximating M~^-1.
//
// Fields live on the whole lattice in even-odd order (site j = parity * Vh + cb index) as
// [site][channel][colour] complex FP32.  A layer maps C_in to C_out channels:
//
//     out(x)[o][a] = sum_{d=0..8} sum_i W_d[o][i] (T_d h)(x)[i][a]
//     T_0 h(x) = h(x),  T_{+mu} h(x) = U_mu(x) h(x+mu),  T_{-mu} h(x) = U_mu(x-mu)^dag h(x-mu)
//
// W acts on channels only and the links on colour only, so every layer (and the network) is
// gauge covariant.  The channel mixing is a GEMM over the rows (site, colour): the gathered
// T_d h form a 9*C_in complex row, staged in shared memory as BF16 in the tensor cores' core-matrix
// layout, and tcgen05.mma (BF16 in, FP32 accumulate in tensor memory) multiplies it by the real
// form of W.  The network is linear; it takes the odd-site input as channels = spins with zero
// even sites and returns its odd sites.
//
// Backward: the input gradient of a layer is the same layer with W'_{+mu} = W_{-mu}^H,
// W'_{-mu} = W_{+mu}^H, W'_0 = W_0^H (T_{+mu}^dag = T_{-mu}), and the weight gradient is
// sum over rows of delta_out (x) conj(gathered input), with mma.sync m16n8k16 (a reduction over
// the rows into a small matrix, accumulated across blocks with atomics).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <string>
#include <vector>

#include "cnn.h"
#include "ctx.h"
#include "gbc_device.cuh"

namespace gbc {
namespace {

constexpr int CT = 128;     // threads per block
constexpr int SITES = 32;   // sites per block -> 96 rows (site, colour)
constexpr int ROWS = SITES * 3;
constexpr int DP = ROWS + 8;  // pitch of the transposed delta tile: 52 words = 4 mod 8 (conflict-free)

__host__ __device__ constexpr int kpad(int cin) { return ((9 * cin * 2 + 15) / 16) * 16; }
__host__ __device__ constexpr int npad(int cout) { return ((2 * cout + 7) / 8) * 8; }

__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ Coord eo_coords(const Geom& g, int j) {
  const int par = j >= g.Vh ? 1 : 0;
  return cb_coords(g, j - par * g.Vh, par);
}
__device__ __forceinline__ int eo_index(const Geom& g, const Coord& c) {
  const int par = (c.x[0] + c.x[1] + c.x[2] + c.x[3]) & 1;
  return par * g.Vh + cb_index(g, c);
}

// Row pitch (bf16 elements) of the staged tiles: at least kpad(cin), with the pitch in 32-bit words
// = 4 mod 8, so that the 8 rows x 4 column pairs an mma fragment load touches fall in 32 distinct
// shared-memory banks (a pitch of 224 elements put them on 8 banks: 4-way conflicts).
__host__ __device__ constexpr int gpitch(int cin) {
  return kpad(cin) + ((4 - (kpad(cin) / 2) % 8 + 8) % 8) * 2;
}

// Where element (row, k) of a staged bf16 tile lives, in elements from the tile base:
//  - PitchLayout: row-major at pitch gpitch(cin) (the mma.sync fragments of the weight gradient);
//  - CoreLayout: the tensor cores' canonical K-major layout without swizzle, read by tcgen05.mma
//    through a shared-memory descriptor: 8 x 8 core matrices (8 rows of 16 bytes, 128 contiguous
//    bytes), the core matrices of a row group along K 128 bytes apart (the descriptor's leading
//    byte offset), row groups KP * 16 bytes apart (its stride byte offset).
template <int CIN>
struct PitchLayout {
  __device__ __forceinline__ int operator()(int row, int k) const { return row * gpitch(CIN) + k; }
};
template <int CIN>
struct CoreLayout {
  __device__ __forceinline__ int operator()(int row, int k) const {
    return (row >> 3) * (kpad(CIN) * 8) + (k >> 3) * 64 + (row & 7) * 8 + (k & 7);
  }
};

// the 9 sites each site of the tile reads (d = 0 itself, 1 + 2 mu forward, 2 + 2 mu backward)
__device__ void tile_neighbours(int (*nbr)[9], const Geom& g, int V, int site0) {
  for (int p = threadIdx.x; p < SITES * 9; p += blockDim.x) {
    const int s = p / 9, d = p % 9, j = site0 + s;
    int n = j;
    if (j < V && d > 0) {
      Coord c = eo_coords(g, j);
      const int mu = (d - 1) >> 1;
      if (((d - 1) & 1) == 0) c.x[mu] = c.x[mu] + 1 == g.L[mu] ? 0 : c.x[mu] + 1;
      else c.x[mu] = c.x[mu] == 0 ? g.L[mu] - 1 : c.x[mu] - 1;
      n = eo_index(g, c);
    }
    nbr[s][d] = n;
  }
}

// G[row = s*3 + a][k = (d*CIN + i)*2 + re/im] = (T_d h)(site)[i][a] in BF16, row pitch GP; the K
// padding zeroed.  One task per (site, direction, channel), channel fastest: consecutive threads
// read consecutive channel vectors and write consecutive 32-bit words (re, im packed), and the
// link of a (site, direction) is shared through L1 by the threads of its channels.
template <int CIN, class Lay>
__device__ void gather_tile(__nv_bfloat16* G, const int (*nbr)[9], int V, const float2* links, const float2* h,
                            int site0, Lay lay) {
  for (int p = threadIdx.x; p < SITES * 9 * CIN; p += blockDim.x) {
    const int i = p % CIN, sd = p / CIN, s = sd % SITES, d = sd / SITES;
    const int j = site0 + s;
    const int k = (d * CIN + i) * 2;
    auto put = [&](int a, uint32_t v) { *reinterpret_cast<uint32_t*>(G + lay(s * 3 + a, k)) = v; };
    if (j >= V) {
      put(0, 0u);
      put(1, 0u);
      put(2, 0u);
      continue;
    }
    const int n = nbr[s][d];
    const float2* src = h + ((size_t)n * CIN + i) * 3;
    const float2 x0 = src[0], x1 = src[1], x2 = src[2];
    if (d == 0) {
      put(0, bf16x2(x0.x, x0.y));
      put(1, bf16x2(x1.x, x1.y));
      put(2, bf16x2(x2.x, x2.y));
      continue;
    }
    const int mu = (d - 1) >> 1;
    const bool bwd = ((d - 1) & 1) != 0;
    // T_{+mu} h = U_mu(x) h(x+mu);  T_{-mu} h = U_mu(x-mu)^dag h(x-mu)
    const float2* L = links + ((size_t)(bwd ? n : j) * 4 + mu) * 9;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float2 u0, u1, u2;
      if (!bwd) {
        u0 = L[3 * a];
        u1 = L[3 * a + 1];
        u2 = L[3 * a + 2];
      } else {
        u0 = make_float2(L[a].x, -L[a].y);
        u1 = make_float2(L[3 + a].x, -L[3 + a].y);
        u2 = make_float2(L[6 + a].x, -L[6 + a].y);
      }
      const float re = u0.x * x0.x - u0.y * x0.y + u1.x * x1.x - u1.y * x1.y + u2.x * x2.x - u2.y * x2.y;
      const float im = u0.x * x0.y + u0.y * x0.x + u1.x * x1.y + u1.y * x1.x + u2.x * x2.y + u2.y * x2.x;
      put(a, bf16x2(re, im));
    }
  }
  // zero the K padding
  constexpr int K = 9 * CIN * 2, KP = kpad(CIN);
  if (KP > K)
    for (int p = threadIdx.x; p < ROWS * (KP - K); p += blockDim.x) {
      const int r = p / (KP - K), k = K + p % (KP - K);
      G[lay(r, k)] = __float2bfloat16(0.f);
    }
}

// The block's transports staged once: lk[s][d - 1][3 a + k] = M_d[a][k] with M_{+mu} = U_mu(x) and
// M_{-mu} = U_mu(x - mu)^dag, for every direction d = 1..8 of the SITES sites.  The forward layer
// reads them for every right-hand side of the batch instead of reloading the link per channel.
__device__ void stage_transports(float2 (*lk)[8][9], const int (*nbr)[9], int V, const float2* links, int site0) {
  for (int p = threadIdx.x; p < SITES * 8 * 9; p += blockDim.x) {
    const int e = p % 9, sd = p / 9, s = sd / 8, d = sd % 8 + 1;
    const int j = site0 + s;
    if (j >= V) continue;
    const int mu = (d - 1) >> 1;
    const bool bwd = ((d - 1) & 1) != 0;
    const int a = e / 3, k = e % 3;
    const float2* L = links + ((size_t)(bwd ? nbr[s][d] : j) * 4 + mu) * 9;
    const float2 u = bwd ? L[3 * k + a] : L[3 * a + k];
    lk[s][d - 1][e] = bwd ? make_float2(u.x, -u.y) : u;
  }
}

// G as gather_tile, from staged transports: one task per (site, direction, channel), channel
// fastest, so that consecutive threads read consecutive channel vectors of a neighbour and write
// consecutive words of a row; the transport comes from shared memory instead of the links.
template <int CIN, class Lay>
__device__ void gather_tile_staged(__nv_bfloat16* G, const int (*nbr)[9], const float2 (*lk)[8][9], int V,
                                   const float2* h, int site0, Lay lay) {
  for (int p = threadIdx.x; p < SITES * 9 * CIN; p += blockDim.x) {
    const int i = p % CIN, sd = p / CIN, s = sd % SITES, d = sd / SITES;
    const int j = site0 + s;
    const int k = (d * CIN + i) * 2;
    auto put = [&](int a, uint32_t v) { *reinterpret_cast<uint32_t*>(G + lay(s * 3 + a, k)) = v; };
    if (j >= V) {
      put(0, 0u);
      put(1, 0u);
      put(2, 0u);
      continue;
    }
    const float2* src = h + ((size_t)nbr[s][d] * CIN + i) * 3;
    const float2 x0 = src[0], x1 = src[1], x2 = src[2];
    if (d == 0) {
      put(0, bf16x2(x0.x, x0.y));
      put(1, bf16x2(x1.x, x1.y));
      put(2, bf16x2(x2.x, x2.y));
      continue;
    }
    const float2* m = lk[s][d - 1];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float2 u0 = m[3 * a], u1 = m[3 * a + 1], u2 = m[3 * a + 2];
      const float re = u0.x * x0.x - u0.y * x0.y + u1.x * x1.x - u1.y * x1.y + u2.x * x2.x - u2.y * x2.y;
      const float im = u0.x * x0.y + u0.y * x0.x + u1.x * x1.y + u1.y * x1.x + u2.x * x2.y + u2.y * x2.x;
      put(a, bf16x2(re, im));
    }
  }
  // zero the K padding
  constexpr int K = 9 * CIN * 2, KP = kpad(CIN);
  if (KP > K)
    for (int p = threadIdx.x; p < ROWS * (KP - K); p += blockDim.x) {
      const int r = p / (KP - K), k = K + p % (KP - K);
      G[lay(r, k)] = __float2bfloat16(0.f);
    }
}

__device__ __forceinline__ uint32_t ld_bf16x2(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }
__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// ---- 5th-generation tensor cores (tcgen05) for the forward channel mixing ----------------------
// One thread issues tcgen05.mma (kind::f16, BF16 in, FP32 accumulate in tensor memory) on
// shared-memory descriptors of the gathered tile G (the MMA's M = 128 rows: the block's 96
// (site, colour) rows, then 32 rows that overlap the weights and are discarded) and the weights W
// (NU rows = output channels x re/im, padded to a multiple of 16); completion is signalled through
// an mbarrier by tcgen05.commit, and each warp reads its 32 accumulator lanes back with tcgen05.ld.

__device__ int g_tc_wait_errors;  // waits for tensor-core completion that gave up (host-checked)

// shared-memory matrix descriptor, K-major without swizzle: start, leading byte offset (between
// K-adjacent core matrices), stride byte offset (between 8-row groups), descriptor version 1
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, N and M
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// thread 0 waits for phase `parity` of the mbarrier, for about 1 s of SM clock at most
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > 2000000000LL) return false;
  }
}

template <int NU>
__device__ __forceinline__ void tmem_load_row(uint32_t taddr, float (&v)[NU]) {
  uint32_t r[NU];
  if constexpr (NU == 32) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
  } else {
    static_assert(NU == 16, "16 or 32 accumulator columns");
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
  }
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int q = 0; q < NU; ++q) v[q] = __uint_as_float(r[q]);
}

__host__ __device__ constexpr int nump(int cout) { return ((2 * cout + 15) / 16) * 16; }  // N of the MMA
constexpr int kTmemCols = 32;  // tensor-memory columns allocated per block (>= nump, power of 2)

// out[b][j][o][a] = (G W^T)[row][2o + re/im] for every right-hand side b of the batch: the
// weights and (for batches) the block's transports are staged once, then per b the gathered tile G
// and its GEMM on the tensor cores
template <int CIN, int COUT>
__global__ void __launch_bounds__(CT) layer_kernel(Geom g, int V, int batch, const float2* links, const float2* hin,
                                                   float2* hout, const __nv_bfloat16* Wr) {
  constexpr int KP = kpad(CIN), NP = npad(COUT), NU = nump(COUT);
  constexpr int MROWS = 128;  // the MMA's M: the 96 rows of the tile and 32 discarded rows
  static_assert(ROWS <= MROWS && NU <= kTmemCols, "tile does not fit the MMA");
  extern __shared__ __align__(128) unsigned char smem[];
  // G holds the tile's 96 rows; the MMA's rows 96..127 read whatever follows (the weights, the
  // staged transports or the padding the launch adds): their results are never read back
  // (likewise the MMA's weight rows NP..NU-1, whose result columns are never read back)
  __nv_bfloat16* G = reinterpret_cast<__nv_bfloat16*>(smem);  // CoreLayout, ROWS x KP
  __nv_bfloat16* W = G + ROWS * KP;                           // CoreLayout, NP x KP
  float2(*lk)[8][9] = reinterpret_cast<float2(*)[8][9]>(W + NP * KP);
  __shared__ int nbr[SITES][9];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_ok;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int site0 = blockIdx.x * SITES;
  const CoreLayout<CIN> lay{};
  for (int p = tid; p < NP * KP; p += blockDim.x) W[lay(p / KP, p % KP)] = Wr[p];
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  tile_neighbours(nbr, g, V, site0);
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  // one right-hand side reads each transport once: it gathers straight from the links (the staged
  // copy only costs shared memory and occupancy there)
  const bool staged = batch > 1;
  if (staged) stage_transports(lk, nbr, V, links, site0);
  const uint64_t adesc = umma_desc(smem_u32(G), 128, KP * 16);
  const uint64_t bdesc = umma_desc(smem_u32(W), 128, KP * 16);
  constexpr uint32_t idesc = umma_idesc_bf16(MROWS, NU);
  bool ok = true;
  for (int b = 0; b < batch && ok; ++b) {
    __syncthreads();  // transports staged; the previous right-hand side's accumulators are read
    if (staged) gather_tile_staged<CIN>(G, nbr, lk, V, hin + (size_t)b * V * CIN * 3, site0, lay);
    else gather_tile<CIN>(G, nbr, V, links, hin + (size_t)b * V * CIN * 3, site0, lay);
    // the tensor cores read G through the async proxy
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
      for (int ks = 0; ks < KP / 16; ++ks) {
        // K steps of 16 elements: two core matrices along K, 256 bytes
        const uint64_t da = adesc + (uint64_t)((ks * 256) >> 4), db = bdesc + (uint64_t)((ks * 256) >> 4);
        const uint32_t acc = ks > 0 ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(da), "l"(db), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       smem_u32(&mbar))
                   : "memory");
      s_ok = mbar_wait(smem_u32(&mbar), (uint32_t)(b & 1));
      if (!s_ok) {
        atomicAdd(&g_tc_wait_errors, 1);
        // give the MMAs in flight one more bounded wait before their tensor memory is freed
        (void)mbar_wait(smem_u32(&mbar), (uint32_t)(b & 1));
      }
    }
    __syncthreads();
    ok = s_ok != 0;
    if (!ok) break;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const int row = warp * 32 + lane;
    if (warp * 32 < ROWS) {  // warp 3 holds only padding rows
      float v[NU];
      tmem_load_row<NU>(tmem + ((uint32_t)(warp * 32) << 16), v);
      const int s = row / 3, a = row % 3, j = site0 + s;
      if (row < ROWS && j < V) {
        float2* out = hout + (size_t)b * V * COUT * 3;
#pragma unroll
        for (int o = 0; o < COUT; ++o) out[((size_t)j * COUT + o) * 3 + a] = make_float2(v[2 * o], v[2 * o + 1]);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  }
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
}

// gradient of the real-form weights: dW[n][k] += sum_rows delta[row][n] * G[row][k]
template <int CIN, int COUT>
__global__ void __launch_bounds__(CT) wgrad_kernel(Geom g, int V, const float2* links, const float2* hin,
                                                   const float2* delta, float* dW) {
  constexpr int KP = kpad(CIN), NP = npad(COUT), MP = ((NP + 15) / 16) * 16, GP = gpitch(CIN);
  extern __shared__ __align__(16) unsigned char smem[];
  __nv_bfloat16* G = reinterpret_cast<__nv_bfloat16*>(smem);
  __nv_bfloat16* Dt = G + ROWS * GP;  // [MP][DP]: delta transposed (A operand, row-major M x K)
  __shared__ int nbr[SITES][9];
  const int b = blockIdx.y;
  const int site0 = blockIdx.x * SITES;
  tile_neighbours(nbr, g, V, site0);
  __syncthreads();
  gather_tile<CIN>(G, nbr, V, links, hin + (size_t)b * V * CIN * 3, site0, PitchLayout<CIN>{});
  const float2* dl = delta + (size_t)b * V * COUT * 3;
  for (int p = threadIdx.x; p < MP * ROWS; p += blockDim.x) {
    const int n = p / ROWS, row = p % ROWS;
    const int s = row / 3, a = row % 3, j = site0 + s, o = n >> 1;
    float v = 0.f;
    if (n < 2 * COUT && j < V) {
      const float2 d = dl[((size_t)j * COUT + o) * 3 + a];
      v = (n & 1) ? d.y : d.x;
    }
    Dt[(size_t)n * DP + row] = __float2bfloat16(v);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = lane >> 2, tig = lane & 3;
  constexpr int MT = MP / 16, NT = KP / 8;
  for (int t = warp; t < MT * NT; t += CT / 32) {
    const int mt = t % MT, nt = t / MT;
    float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int ks = 0; ks < ROWS / 16; ++ks) {
      const __nv_bfloat16* A0 = Dt + (size_t)(mt * 16 + gid) * DP + ks * 16 + 2 * tig;
      const __nv_bfloat16* A1 = A0 + 8 * DP;
      uint32_t a[4] = {ld_bf16x2(A0), ld_bf16x2(A1), ld_bf16x2(A0 + 8), ld_bf16x2(A1 + 8)};
      // B (K = rows x N = k columns), col-major fragment: (k = 2 tig + {0,1}, n = gid)
      const int col = nt * 8 + gid;
      const int r0 = ks * 16 + 2 * tig;
      uint32_t bb[2] = {pack_bf16(G[(size_t)r0 * GP + col], G[(size_t)(r0 + 1) * GP + col]),
                        pack_bf16(G[(size_t)(r0 + 8) * GP + col], G[(size_t)(r0 + 9) * GP + col])};
      mma_bf16(c, a, bb);
    }
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int n = mt * 16 + gid + 8 * half;
      const int k = nt * 8 + 2 * tig;
      if (n < 2 * COUT) {
        atomicAdd(&dW[(size_t)n * KP + k], c[2 * half]);
        atomicAdd(&dW[(size_t)n * KP + k + 1], c[2 * half + 1]);
      }
    }
  }
}

// odd-site spinor field (precision P) -> layer-0 activations (even sites zero)
template <typename P>
__global__ void embed_kernel(Geom g, int V, Spinor f, float2* act) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (j >= V) return;
  float2* out = act + ((size_t)b * V + j) * 12;
  if (j < g.Vh) {
    for (int k = 0; k < 12; ++k) out[k] = make_float2(0.f, 0.f);
    return;
  }
  cplx<typename P::real> v[12];
  load_spinor<P>(v, (const char*)f.v + (size_t)b * f.rhs_bytes, f.norm ? f.norm + (size_t)b * f.norm_rhs_stride : nullptr,
                 j - g.Vh, f.stride);
  for (int k = 0; k < 12; ++k) out[k] = make_float2((float)v[k].re, (float)v[k].im);
}

template <typename P>
__global__ void extract_kernel(Geom g, int V, const float2* act, Spinor f) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (i >= g.Vh) return;
  const float2* src = act + ((size_t)b * V + g.Vh + i) * 12;
  cplx<typename P::real> v[12];
  for (int k = 0; k < 12; ++k) v[k] = {(typename P::real)src[k].x, (typename P::real)src[k].y};
  store_spinor<P>((char*)f.v + (size_t)b * f.rhs_bytes, f.norm ? f.norm + (size_t)b * f.norm_rhs_stride : nullptr, i,
                  f.stride, v);
}

// canonical complex128 [V][12] (rhs b at offset b*V*12) -> activations, odd sites only
__global__ void embed_canon_kernel(Geom g, int V, const double2* canon, float2* act) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (j >= V) return;
  float2* out = act + ((size_t)b * V + j) * 12;
  if (j < g.Vh) {
    for (int k = 0; k < 12; ++k) out[k] = make_float2(0.f, 0.f);
    return;
  }
  const Coord c = eo_coords(g, j);
  const double2* src = canon + ((size_t)b * V + full_index(g, c)) * 12;
  for (int k = 0; k < 12; ++k) out[k] = make_float2((float)src[k].x, (float)src[k].y);
}

__global__ void extract_canon_kernel(Geom g, int V, const float2* act, double2* canon) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (j >= V) return;
  const Coord c = eo_coords(g, j);
  double2* dst = canon + ((size_t)b * V + full_index(g, c)) * 12;
  const float2* src = act + ((size_t)b * V + j) * 12;
  for (int k = 0; k < 12; ++k)
    dst[k] = j < g.Vh ? make_double2(0.0, 0.0) : make_double2((double)src[k].x, (double)src[k].y);
}

// loss = sum_b sum_odd |y - e|^2 / |e|^2 ; delta = 2 (y - e) / |e|^2 on odd sites, 0 elsewhere
__global__ void loss_kernel(Geom g, int V, const float2* y, const float2* e, const double* enorm2, float2* delta,
                            double* partial) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  double l = 0.0;
  if (j < V) {
    const size_t o = ((size_t)b * V + j) * 12;
    const float inv = (float)(1.0 / enorm2[b]);
    for (int k = 0; k < 12; ++k) {
      float2 d = make_float2(0.f, 0.f);
      if (j >= g.Vh) {
        d = make_float2(y[o + k].x - e[o + k].x, y[o + k].y - e[o + k].y);
        l += (double)(d.x * d.x + d.y * d.y) * inv;
        d = make_float2(2.f * d.x * inv, 2.f * d.y * inv);
      }
      delta[o + k] = d;
    }
  }
  __shared__ double sh[256];
  sh[threadIdx.x] = l;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(partial, sh[0]);
}

__global__ void links_kernel(Geom g, int V, const double2* canon, float2* links) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= V) return;
  const Coord c = eo_coords(g, j);
  const long s = full_index(g, c);
  for (int m = 0; m < 4; ++m)
    for (int k = 0; k < 9; ++k) {
      const double2 v = canon[(s * 4 + m) * 9 + k];
      links[((size_t)j * 4 + m) * 9 + k] = make_float2((float)v.x, (float)v.y);
    }
}

template <int CIN, int COUT>
void launch_layer(const Geom& g, int V, int batch, const float2* links, const float2* in, float2* out,
                  const __nv_bfloat16* W, cudaStream_t s) {
  // tile G (128 rows) and weights W (nump rows), bf16 in the tensor cores' core-matrix layout
  // (their bytes are a multiple of 128), then the staged transports (float2)
  // G (96 rows) and W (npad rows) in the core-matrix layout, then the staged transports; at least
  // the 128 rows x kpad that the MMA's A operand (and its B operand, ending earlier) spans
  const size_t tile = (size_t)(ROWS * kpad(CIN) + npad(COUT) * kpad(CIN)) * 2;
  const size_t span = (size_t)128 * kpad(CIN) * 2;
  const size_t lkb = sizeof(float2) * SITES * 8 * 9;
  const size_t smem = std::max(batch > 1 ? tile + lkb : tile, span);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(layer_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)std::max(tile + lkb, span));
    attr = true;
  }
  dim3 grid((V + SITES - 1) / SITES);
  layer_kernel<CIN, COUT><<<grid, CT, smem, s>>>(g, V, batch, links, in, out, W);
  count_launch();
}

template <int CIN, int COUT>
void launch_wgrad(const Geom& g, int V, int batch, const float2* links, const float2* in, const float2* delta,
                  float* dW, cudaStream_t s) {
  constexpr int MP = ((npad(COUT) + 15) / 16) * 16;
  const size_t smem = (size_t)(ROWS * gpitch(CIN) + MP * DP) * 2;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(wgrad_kernel<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  dim3 grid((V + SITES - 1) / SITES, batch);
  wgrad_kernel<CIN, COUT><<<grid, CT, smem, s>>>(g, V, links, in, delta, dW);
  count_launch();
}

void layer(const Geom& g, int V, int batch, int cin, int cout, const float2* links, const float2* in, float2* out,
           const __nv_bfloat16* W, cudaStream_t s) {
  if (cin == 4 && cout == 12) launch_layer<4, 12>(g, V, batch, links, in, out, W, s);
  else if (cin == 12 && cout == 12) launch_layer<12, 12>(g, V, batch, links, in, out, W, s);
  else if (cin == 12 && cout == 4) launch_layer<12, 4>(g, V, batch, links, in, out, W, s);
  else if (cin == 4 && cout == 4) launch_layer<4, 4>(g, V, batch, links, in, out, W, s);
  else throw std::string("network layer shape not compiled");
}

void wgrad(const Geom& g, int V, int batch, int cin, int cout, const float2* links, const float2* in,
           const float2* delta, float* dW, cudaStream_t s) {
  if (cin == 4 && cout == 12) launch_wgrad<4, 12>(g, V, batch, links, in, delta, dW, s);
  else if (cin == 12 && cout == 12) launch_wgrad<12, 12>(g, V, batch, links, in, delta, dW, s);
  else if (cin == 12 && cout == 4) launch_wgrad<12, 4>(g, V, batch, links, in, delta, dW, s);
  else if (cin == 4 && cout == 4) launch_wgrad<4, 4>(g, V, batch, links, in, delta, dW, s);
  else throw std::string("network layer shape not compiled");
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// host model
// ---------------------------------------------------------------------------------------------
using cf = std::complex<float>;

int Cnn::cin(int l) const { return l == 0 ? 4 : hidden; }
int Cnn::cout(int l) const { return l == nlayers - 1 ? 4 : hidden; }

void Cnn::init(int hidden_, int layers_, unsigned long long seed) {
  hidden = hidden_;
  nlayers = layers_;
  W.assign(nlayers, {});
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.f, 1.f);
  for (int l = 0; l < nlayers; ++l) {
    const int ci = cin(l), co = cout(l);
    W[l].assign((size_t)9 * co * ci, cf(0, 0));
    // start near the identity map through the self term, with small random hops (scaled so a
    // layer roughly preserves norms)
    const float sc = 0.1f / std::sqrt((float)(9 * ci));
    for (auto& w : W[l]) w = cf(sc * nd(rng), sc * nd(rng));
    for (int o = 0; o < co; ++o)
      for (int i = 0; i < ci; ++i)
        if (o % ci == i || (ci > co && i % co == o)) W[l][(size_t)o * ci + i] += cf(ci > co ? 1.0f / (ci / co) : 1.0f, 0);
  }
  m1.assign(nlayers, {});
  m2.assign(nlayers, {});
  for (int l = 0; l < nlayers; ++l) {
    m1[l].assign(W[l].size() * 2, 0.f);
    m2[l].assign(W[l].size() * 2, 0.f);
  }
  step = 0;
  dirty = true;
}

static void real_form(const std::vector<cf>& Wc, int ci, int co, bool adjoint, std::vector<__nv_bfloat16>& out) {
  // forward: rows 2*COUT (re/im of output o), K = (d*CIN + i)*2 + re/im
  // adjoint: out channels = ci, in channels = co, W'_d = (W_{swap d})^H
  const int oc = adjoint ? ci : co, ic = adjoint ? co : ci;
  const int KP = kpad(ic), NP = npad(oc);
  out.assign((size_t)NP * KP, __float2bfloat16(0.f));
  for (int d = 0; d < 9; ++d) {
    const int ds = adjoint ? (d == 0 ? 0 : (((d - 1) ^ 1) + 1)) : d;
    for (int o = 0; o < oc; ++o)
      for (int i = 0; i < ic; ++i) {
        cf w = adjoint ? std::conj(Wc[((size_t)ds * co + i) * ci + o]) : Wc[((size_t)d * co + o) * ci + i];
        const int k = (d * ic + i) * 2;
        out[(size_t)(2 * o) * KP + k] = __float2bfloat16(w.real());
        out[(size_t)(2 * o) * KP + k + 1] = __float2bfloat16(-w.imag());
        out[(size_t)(2 * o + 1) * KP + k] = __float2bfloat16(w.imag());
        out[(size_t)(2 * o + 1) * KP + k + 1] = __float2bfloat16(w.real());
      }
  }
}

void Cnn::upload(cudaStream_t s) {
  if (!dirty) return;
  for (int l = 0; l < nlayers; ++l) {
    std::vector<__nv_bfloat16> a, b;
    real_form(W[l], cin(l), cout(l), false, a);
    real_form(W[l], cin(l), cout(l), true, b);
    if (!dW[l]) {
      GBC_CUDA(cudaMalloc(&dW[l], a.size() * 2));
      GBC_CUDA(cudaMalloc(&dWadj[l], b.size() * 2));
      GBC_CUDA(cudaMalloc(&dG[l], sizeof(float) * (size_t)npad(cout(l)) * kpad(cin(l))));
    }
    GBC_CUDA(cudaMemcpyAsync(dW[l], a.data(), a.size() * 2, cudaMemcpyHostToDevice, s));
    GBC_CUDA(cudaMemcpyAsync(dWadj[l], b.data(), b.size() * 2, cudaMemcpyHostToDevice, s));
  }
  GBC_CUDA(cudaStreamSynchronize(s));
  dirty = false;
}

void Cnn::release() {
  for (int l = 0; l < 8; ++l) {
    if (dW[l]) cudaFree(dW[l]);
    if (dWadj[l]) cudaFree(dWadj[l]);
    if (dG[l]) cudaFree(dG[l]);
    dW[l] = dWadj[l] = nullptr;
    dG[l] = nullptr;
  }
  for (auto& p : act) if (p) cudaFree(p);
  act.clear();
  if (links) cudaFree(links);
  links = nullptr;
  if (delta[0]) cudaFree(delta[0]);
  if (delta[1]) cudaFree(delta[1]);
  delta[0] = delta[1] = nullptr;
  act_batch = 0;
}

void Cnn::ensure(gbc_ctx* c, int batch) {
  const int V = (int)c->V;
  if (!links || links_version != c->gauge_version) {
    if (!links) GBC_CUDA(cudaMalloc(&links, sizeof(float2) * (size_t)V * 36));
    links_kernel<<<(V + 127) / 128, 128, 0, c->stream>>>(c->g, V, reinterpret_cast<const double2*>(c->d_links), links);
    count_launch();
    links_version = c->gauge_version;
  }
  if (act_batch < batch) {
    for (auto& p : act) if (p) cudaFree(p);
    act.assign(nlayers + 1, nullptr);
    for (int l = 0; l <= nlayers; ++l) {
      const int ch = l == 0 ? 4 : cout(l - 1);
      GBC_CUDA(cudaMalloc(&act[l], sizeof(float2) * (size_t)batch * V * std::max(ch, 12) * 3));
    }
    for (int q = 0; q < 2; ++q) {
      if (delta[q]) cudaFree(delta[q]);
      GBC_CUDA(cudaMalloc(&delta[q], sizeof(float2) * (size_t)batch * V * std::max(hidden, 4) * 3));
    }
    act_batch = batch;
  }
  upload(c->stream);
}

void Cnn::forward(gbc_ctx* c, int batch) {
  const int V = (int)c->V;
  for (int l = 0; l < nlayers; ++l) layer(c->g, V, batch, cin(l), cout(l), links, act[l], act[l + 1], dW[l], c->stream);
}

// A layer whose wait for its tensor-core results gave up (it then frees its tensor memory and
// returns) counts in g_tc_wait_errors: read and reset it, and fail the call that ran the layers.
static void check_tc_waits(cudaStream_t s) {
  int n = 0;
  GBC_CUDA(cudaMemcpyFromSymbolAsync(&n, g_tc_wait_errors, sizeof(int), 0, cudaMemcpyDeviceToHost, s));
  GBC_CUDA(cudaStreamSynchronize(s));
  if (n) {
    const int zero = 0;
    GBC_CUDA(cudaMemcpyToSymbol(g_tc_wait_errors, &zero, sizeof(int)));
    throw std::string("network layer: a wait for the tensor cores gave up");
  }
}

double Cnn::loss_and_grad(gbc_ctx* c, int batch, const float2* target, const double* enorm2) {
  const int V = (int)c->V;
  cudaStream_t s = c->stream;
  forward(c, batch);
  double* dl = nullptr;
  GBC_CUDA(cudaMalloc(&dl, sizeof(double)));
  GBC_CUDA(cudaMemsetAsync(dl, 0, sizeof(double), s));
  dim3 grid((V + 255) / 256, batch);
  loss_kernel<<<grid, 256, 0, s>>>(c->g, V, act[nlayers], target, enorm2, delta[0], dl);
  count_launch();
  for (int l = 0; l < nlayers; ++l)
    GBC_CUDA(cudaMemsetAsync(dG[l], 0, sizeof(float) * (size_t)npad(cout(l)) * kpad(cin(l)), s));
  int cur = 0;
  for (int l = nlayers - 1; l >= 0; --l) {
    wgrad(c->g, V, batch, cin(l), cout(l), links, act[l], delta[cur], dG[l], s);
    if (l > 0) {
      layer(c->g, V, batch, cout(l), cin(l), links, delta[cur], delta[1 - cur], dWadj[l], s);
      cur = 1 - cur;
    }
  }
  double loss = 0;
  GBC_CUDA(cudaMemcpyAsync(&loss, dl, sizeof(double), cudaMemcpyDeviceToHost, s));
  GBC_CUDA(cudaStreamSynchronize(s));
  cudaFree(dl);
  check_tc_waits(s);
  return loss;
}

// complex gradient dL/dRe W + i dL/dIm W from the real-form gradient
void Cnn::download_grad(cudaStream_t s, std::vector<std::vector<cf>>& grad) {
  grad.assign(nlayers, {});
  for (int l = 0; l < nlayers; ++l) {
    const int ci = cin(l), co = cout(l), KP = kpad(ci);
    std::vector<float> gr((size_t)npad(co) * KP);
    GBC_CUDA(cudaMemcpyAsync(gr.data(), dG[l], gr.size() * 4, cudaMemcpyDeviceToHost, s));
    GBC_CUDA(cudaStreamSynchronize(s));
    grad[l].assign((size_t)9 * co * ci, cf(0, 0));
    for (int d = 0; d < 9; ++d)
      for (int o = 0; o < co; ++o)
        for (int i = 0; i < ci; ++i) {
          const int k = (d * ci + i) * 2;
          const float dre = gr[(size_t)(2 * o) * KP + k] + gr[(size_t)(2 * o + 1) * KP + k + 1];
          const float dim = gr[(size_t)(2 * o + 1) * KP + k] - gr[(size_t)(2 * o) * KP + k + 1];
          grad[l][((size_t)d * co + o) * ci + i] = cf(dre, dim);
        }
  }
}

void Cnn::adam(const std::vector<std::vector<cf>>& grad, double lr) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  ++step;
  const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
  for (int l = 0; l < nlayers; ++l)
    for (size_t q = 0; q < W[l].size(); ++q) {
      const float gq[2] = {grad[l][q].real(), grad[l][q].imag()};
      float wq[2] = {W[l][q].real(), W[l][q].imag()};
      for (int r = 0; r < 2; ++r) {
        float& m = m1[l][2 * q + r];
        float& v = m2[l][2 * q + r];
        m = b1 * m + (1 - b1) * gq[r];
        v = b2 * v + (1 - b2) * gq[r] * gq[r];
        wq[r] -= (float)lr * (m / c1) / (std::sqrt(v / c2) + eps);
      }
      W[l][q] = cf(wq[0], wq[1]);
    }
  dirty = true;
}

// file: "GBCW" u32 version=1, u32 layers, u32 hidden, then per layer u32 cin, u32 cout,
// 9*cout*cin complex float32, then u64 FNV-1a of everything before it
static uint64_t fnv1a(const unsigned char* p, size_t n) {
  uint64_t h = 1469598103934665603ULL;
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ULL;
  }
  return h;
}

bool Cnn::save(const std::string& path) const {
  std::vector<unsigned char> buf;
  auto put = [&](const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    buf.insert(buf.end(), c, c + n);
  };
  const char magic[4] = {'G', 'B', 'C', 'W'};
  const uint32_t ver = 1, L = nlayers, H = hidden;
  put(magic, 4);
  put(&ver, 4);
  put(&L, 4);
  put(&H, 4);
  for (int l = 0; l < nlayers; ++l) {
    const uint32_t ci = cin(l), co = cout(l);
    put(&ci, 4);
    put(&co, 4);
    put(W[l].data(), W[l].size() * sizeof(cf));
  }
  const uint64_t h = fnv1a(buf.data(), buf.size());
  put(&h, 8);
  std::ofstream f(path, std::ios::binary);
  if (!f) return false;
  f.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)buf.size());
  return (bool)f;
}

int Cnn::load(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return GBC_ERR_PRECOND;
  std::vector<unsigned char> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  if (buf.size() < 16 + 8 || std::memcmp(buf.data(), "GBCW", 4) != 0) return GBC_ERR_PRECOND;
  uint64_t h;
  std::memcpy(&h, buf.data() + buf.size() - 8, 8);
  if (fnv1a(buf.data(), buf.size() - 8) != h) return GBC_ERR_PRECOND;
  uint32_t ver, L, H;
  std::memcpy(&ver, buf.data() + 4, 4);
  std::memcpy(&L, buf.data() + 8, 4);
  std::memcpy(&H, buf.data() + 12, 4);
  if (ver != 1 || L < 1 || L > 8 || (H != 4 && H != 12)) return GBC_ERR_PRECOND;
  init((int)H, (int)L, 0);
  size_t off = 16;
  for (int l = 0; l < nlayers; ++l) {
    uint32_t ci, co;
    if (off + 8 > buf.size() - 8) return GBC_ERR_PRECOND;
    std::memcpy(&ci, buf.data() + off, 4);
    std::memcpy(&co, buf.data() + off + 4, 4);
    off += 8;
    if ((int)ci != cin(l) || (int)co != cout(l)) return GBC_ERR_PRECOND;
    const size_t n = W[l].size() * sizeof(cf);
    if (off + n > buf.size() - 8) return GBC_ERR_PRECOND;
    std::memcpy(W[l].data(), buf.data() + off, n);
    off += n;
  }
  if (off != buf.size() - 8) return GBC_ERR_PRECOND;
  dirty = true;
  return GBC_OK;
}

void cnn_apply_spinor(gbc_ctx* c, Cnn& net, const Spinor& in, const Spinor& out) {
  const int V = (int)c->V;
  net.ensure(c, in.nrhs);
  dim3 grid((V + 127) / 128, in.nrhs);
  if (in.prec == PREC_DOUBLE) embed_kernel<PrecD><<<grid, 128, 0, c->stream>>>(c->g, V, in, net.act[0]);
  else if (in.prec == PREC_SINGLE) embed_kernel<PrecS><<<grid, 128, 0, c->stream>>>(c->g, V, in, net.act[0]);
  else embed_kernel<PrecH><<<grid, 128, 0, c->stream>>>(c->g, V, in, net.act[0]);
  count_launch();
  net.forward(c, in.nrhs);
  dim3 g2((c->g.Vh + 127) / 128, in.nrhs);
  if (out.prec == PREC_DOUBLE) extract_kernel<PrecD><<<g2, 128, 0, c->stream>>>(c->g, V, net.act[net.nlayers], out);
  else if (out.prec == PREC_SINGLE) extract_kernel<PrecS><<<g2, 128, 0, c->stream>>>(c->g, V, net.act[net.nlayers], out);
  else extract_kernel<PrecH><<<g2, 128, 0, c->stream>>>(c->g, V, net.act[net.nlayers], out);
  count_launch();
  check_tc_waits(c->stream);
}

void cnn_embed_canon(gbc_ctx* c, Cnn& net, int batch, const double* canon_dev, float2* act) {
  const int V = (int)c->V;
  dim3 grid((V + 127) / 128, batch);
  embed_canon_kernel<<<grid, 128, 0, c->stream>>>(c->g, V, reinterpret_cast<const double2*>(canon_dev), act);
  count_launch();
}

void cnn_extract_canon(gbc_ctx* c, Cnn& net, int batch, const float2* act, double* canon_dev) {
  const int V = (int)c->V;
  dim3 grid((V + 127) / 128, batch);
  extract_canon_kernel<<<grid, 128, 0, c->stream>>>(c->g, V, act, reinterpret_cast<double2*>(canon_dev));
  count_launch();
}

}  // namespace gbc
