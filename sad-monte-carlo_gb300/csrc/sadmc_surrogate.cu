// Learned surrogate for delayed-acceptance LJ moves: a radial-descriptor MLP
// (32 Gaussian radial basis functions per atom -> 64 -> 64 -> 1, SiLU), per-atom energies
// summed over the cluster.  The reference has no learned part; this is the surrogate the
// delayed-acceptance moves screen with, trained online on configurations the walkers
// themselves visit.
//
//   descriptor  G[i,k] = sum_{j != i} exp(-(r_ij - c_k)^2 / (2 w^2)), c_k = 0.8 + 2.2 k/31,
//               w = 0.1 (binary32)
//   forward     fifth-generation tensor cores (tcgen05.mma, BF16 operands in shared memory,
//               FP32 accumulators in tensor memory), 128-row tiles; the last layer
//               (64 -> 1) and the SiLUs in FP32.  The delayed-acceptance move kernel runs
//               the same network per walker on mma.sync fragments (sadmc_mma.cuh).
//   training    one fused kernel per tile of whole configurations: the forward, the
//               per-configuration residual, and the backward's three contractions on the
//               tensor cores (d1 = d2 W2^T; the weight gradients W2 and W1 with the bias
//               gradients from a ones column, one M = 128, N = 112, K = 128 MMA); then
//               one kernel sums the tiles in a fixed order and takes the Adam step
//   update      Adam with bias correction on FP32 master weights; bf16 copies refreshed
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "sadmc_common.cuh"
#include "sadmc_mma.cuh"
#include "sadmc_surrogate.h"
#include "sadmc_tc05.cuh"

namespace sadmc {
namespace dev {

constexpr uint32_t kPolls = 1u << 24;  // bounded mbarrier waits (never expected to run out)

// Descriptors of rows [0, rows): row r = atom (r % n) of configuration (r / n); positions
// [configs][n][3] binary32.  Four threads per row, eight RBF columns each (one 16-byte
// bf16 store per thread).  Writes bf16 G (the forward operand) and, if requested, FP32 G.
constexpr int DESC_TPR = 4;
__global__ void descriptor_kernel(const float* pos, int n, int rows, __nv_bfloat16* gq, float* gf) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = tid / DESC_TPR, part = tid % DESC_TPR;
  if (r >= rows) return;
  constexpr int K = SG_RBF / DESC_TPR;
  const int c = r / n, i = r % n;
  const float* p = pos + (size_t)c * n * 3;
  const float xi = p[3 * i], yi = p[3 * i + 1], zi = p[3 * i + 2];
  float g[K];
#pragma unroll
  for (int k = 0; k < K; ++k) g[k] = 0.0f;
  const float inv2w2 = 1.0f / (2.0f * 0.1f * 0.1f);
  for (int j = 0; j < n; ++j) {
    if (j == i) continue;
    const float dx = p[3 * j] - xi, dy = p[3 * j + 1] - yi, dz = p[3 * j + 2] - zi;
    const float rij = sqrtf(dx * dx + dy * dy + dz * dz);
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const float d = rij - rbf_centre(part * K + k);
      g[k] += __expf(-d * d * inv2w2);
    }
  }
  *reinterpret_cast<uint4*>(gq + (size_t)r * SG_RBF + part * K) =
      make_uint4(pack_bf16(g[0], g[1]), pack_bf16(g[2], g[3]), pack_bf16(g[4], g[5]), pack_bf16(g[6], g[7]));
  if (gf) {
#pragma unroll
    for (int k = 0; k < K; ++k) gf[(size_t)r * SG_RBF + part * K + k] = g[k];
  }
}

// After a bounded wait ran out, wait (bounded again) for the asynchronous work this CTA
// still has in flight before its tensor memory is freed: the weights' bulk copies
// (copies_pending) and the MMAs of the last commit (parity last_parity, if any).
__device__ void drain_async(uint64_t* wbar, bool copies_pending, uint64_t* mbar, int last_parity) {
  if (copies_pending) tc05::mbar_wait(wbar, 0, kPolls);
  if (last_parity >= 0) tc05::mbar_wait(mbar, (uint32_t)last_parity, kPolls);
}

// Forward pass on the fifth-generation tensor cores: one CTA of 4 warps per 128-row tile.
// G (128 x 32), W1^T (64 x 32), h1 (128 x 64) and W2^T (64 x 64) sit in shared memory as
// BF16 core matrices (K-major, no swizzle); thread 0 issues the tcgen05 MMAs of each
// layer (M = 128, N = 64, K = 16 per instruction) into FP32 accumulators in tensor
// memory (layer 1 in columns 0-63, layer 2 in 64-127) and commits them to an mbarrier;
// each warp reads its 32 rows back with tcgen05.ld for the bias, SiLU and, after layer 2,
// the 64 -> 1 output in FP32.  Writes per-row energies.  A wait that runs out (it never
// should) writes NaN energies and sets *timeout when timeout is not null.
__global__ void __launch_bounds__(128, 1) forward_tc_kernel(const __nv_bfloat16* gq, int rows,
                                                            SgWeights wts, float* e_out,
                                                            unsigned int* timeout) {
  constexpr int M = SG_TILE;
  __shared__ __align__(1024) uint4 sA1[M * SG_RBF / 8];     // G tile, 4 core matrices along K
  __shared__ __align__(1024) uint4 sB1[SG_H1 * SG_RBF / 8];  // W1^T
  __shared__ __align__(1024) uint4 sA2[M * SG_H1 / 8];      // h1 tile, 8 core matrices along K
  __shared__ __align__(1024) uint4 sB2[SG_H2 * SG_H1 / 8];  // W2^T
  __shared__ float sb1[SG_H1], sb2[SG_H2], sw3[SG_H2];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ __align__(8) uint64_t wbar;  // the weights' bulk copies
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * M;
  unsigned char* a1 = reinterpret_cast<unsigned char*>(sA1);
  unsigned char* b1 = reinterpret_cast<unsigned char*>(sB1);
  unsigned char* a2 = reinterpret_cast<unsigned char*>(sA2);
  unsigned char* b2 = reinterpret_cast<unsigned char*>(sB2);
  // operands into shared memory, 16-byte chunks = one core-matrix row
  const uint4* G = reinterpret_cast<const uint4*>(gq);
  for (int c = tid; c < M * (SG_RBF / 8); c += 128) {
    const int r = c / (SG_RBF / 8), kg = c % (SG_RBF / 8);
    const uint4 v = row0 + r < rows ? G[(size_t)(row0 + r) * (SG_RBF / 8) + kg] : make_uint4(0, 0, 0, 0);
    *reinterpret_cast<uint4*>(a1 + tc05::core_offset(r, kg, SG_RBF / 8)) = v;
  }
  for (int k = tid; k < SG_H1; k += 128) { sb1[k] = wts.b1[k]; sb2[k] = wts.b2[k]; sw3[k] = wts.w3[k]; }
  // 256 columns: the two 64-column accumulators with room to spare (two CTAs per SM)
  if (warp == 0) tc05::tmem_alloc(&tbase, 256);
  constexpr uint32_t kW1Bytes = SG_H1 * SG_RBF * 2, kW2Bytes = SG_H2 * SG_H1 * 2;
  if (tid == 0) {
    tc05::mbar_init(&mbar, 1);
    tc05::mbar_init(&wbar, 1);
    // the weights come already in core-matrix order: two bulk copies by the copy engine
    tc05::mbar_expect_tx(&wbar, kW1Bytes + kW2Bytes);
    tc05::bulk_g2s(b1, wts.wc + SG_WC_W1T, kW1Bytes, &wbar);
    tc05::bulk_g2s(b2, wts.wc + SG_WC_W2T, kW2Bytes, &wbar);
  }
  tc05::fence_smem_async();
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
  const uint32_t tmem = tbase;
  constexpr uint32_t idesc = tc05::idesc_bf16(M, SG_H1);
  int last_parity = -1;  // thread 0: parity of the last commit issued
  // layer 1: D1 = G W1 (two K = 16 steps, 2 core matrices = 256 bytes apart), once the
  // weights have landed
  const bool wok = tid == 0 ? tc05::mbar_wait(&wbar, 0, kPolls) : true;
  if (tid == 0 && wok) {
#pragma unroll
    for (int ks = 0; ks < SG_RBF / 16; ++ks)
      tc05::mma_bf16(tmem, tc05::sdesc(tc05::smem_u32(a1) + 256 * ks, 128, 128 * (SG_RBF / 8)),
                     tc05::sdesc(tc05::smem_u32(b1) + 256 * ks, 128, 128 * (SG_RBF / 8)), idesc, ks > 0);
    tc05::commit(&mbar);
    last_parity = 0;
  }
  bool ok = __syncthreads_and(wok);
  if (ok) ok = tc05::mbar_wait(&mbar, 0, kPolls);
  tc05::fence_after();
  const int r = warp * 32 + lane;  // this thread's row of the tile
  const uint32_t lane_addr = (uint32_t)(warp * 32) << 16;
  if (ok) {
    // bias and SiLU of layer 1, h1 into shared memory as the layer-2 A operand
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float acc[32];
      tc05::ld32(tmem + lane_addr + 32 * half, acc);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        uint32_t pk[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int j = 32 * half + 8 * q + 2 * u;
          pk[u] = pack_bf16(silu32(acc[8 * q + 2 * u] + sb1[j]), silu32(acc[8 * q + 2 * u + 1] + sb1[j + 1]));
        }
        *reinterpret_cast<uint4*>(a2 + tc05::core_offset(r, 4 * half + q, SG_H1 / 8)) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
  }
  tc05::fence_smem_async();
  tc05::fence_before();
  // the CTA agrees on the layer-1 outcome before the layer-2 MMAs are issued
  ok = __syncthreads_and(ok);
  tc05::fence_after();
  // layer 2: D2 = h1 W2 (four K = 16 steps) into columns 64-127
  if (tid == 0 && ok) {
#pragma unroll
    for (int ks = 0; ks < SG_H1 / 16; ++ks)
      tc05::mma_bf16(tmem + SG_H1, tc05::sdesc(tc05::smem_u32(a2) + 256 * ks, 128, 128 * (SG_H1 / 8)),
                     tc05::sdesc(tc05::smem_u32(b2) + 256 * ks, 128, 128 * (SG_H1 / 8)), idesc, ks > 0);
    tc05::commit(&mbar);
    last_parity = 1;
  }
  if (ok) ok = tc05::mbar_wait(&mbar, 1, kPolls);
  ok = __syncthreads_and(ok);
  tc05::fence_after();
  float e = 0.f;
  if (ok) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float acc[32];
      tc05::ld32(tmem + lane_addr + SG_H1 + 32 * half, acc);
#pragma unroll
      for (int q = 0; q < 32; ++q) e += silu32(acc[q] + sb2[32 * half + q]) * sw3[32 * half + q];
    }
    e += wts.b3[0];
  } else {
    e = __int_as_float(0x7fc00000);
    if (tid == 0) {
      if (timeout) atomicOr(timeout, 1u);
      drain_async(&wbar, !wok, &mbar, last_parity);
    }
  }
  if (row0 + r < rows) e_out[row0 + r] = e;
  tc05::fence_before();
  __syncthreads();
  if (warp == 0) tc05::tmem_dealloc(tmem, 256);
}

// ---- fused training step ------------------------------------------------------------
// Shared memory of train_tc_kernel (byte offsets from a 1024-byte aligned base).  Every
// operand is bf16 in core matrices (8 rows x 16 bytes, K-major, no swizzle):
//   A1  G tile                    [128 rows r][K = 32 k]       layer 1 A
//   B1  W1^T                      [64 n][32 k]                 layer 1 B
//   A2  h1 tile, later d2 tile    [128 r][64]                  layer 2 A, then d1's A
//   B2  W2^T                      [64 n][64 k]                 layer 2 B
//   B3  W2                        [64 k][64 n]                 d1 = d2 W2^T, B
//   A4  [d2^T ; d1^T]             [128: n then k][K = 128 r]   weight-gradient A
//   B4  [h1^T ; G^T ; 1 ; 0]      [112: k, k', ones][128 r]    weight-gradient B
constexpr uint32_t TT_A1 = 0, TT_B1 = TT_A1 + SG_TILE * SG_RBF * 2, TT_A2 = TT_B1 + SG_H1 * SG_RBF * 2,
                   TT_B2 = TT_A2 + SG_TILE * SG_H1 * 2, TT_B3 = TT_B2 + SG_H2 * SG_H1 * 2,
                   TT_A4 = TT_B3 + SG_H1 * SG_H2 * 2, TT_B4 = TT_A4 + SG_TILE * SG_TILE * 2,
                   TT_N4 = 112, TT_END = TT_B4 + TT_N4 * SG_TILE * 2;
constexpr size_t TT_SMEM = TT_END + 1024;  // + the alignment slack of the dynamic base

__device__ __forceinline__ void st_bf16(unsigned char* base, uint32_t off, float v) {
  *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}
// Byte offset of element (row, K = r) of a [rows][K = 128 r] operand.
__device__ __forceinline__ uint32_t tt_off(int row, int r) {
  return tc05::core_offset(row, r >> 3, SG_TILE / 8) + 2 * (r & 7);
}

// Sum v[0..63] over the 32 lanes of the warp by a butterfly reduce-scatter: lane l ends
// with the sums of entries 2 l and 2 l + 1 (62 shuffles).
__device__ __forceinline__ float2 warp_reduce_scatter64(float v[64], int lane) {
#pragma unroll
  for (int o = 16, len = 32; o >= 1; o >>= 1, len >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int j = 0; j < len; ++j) {
      const float keep = up ? v[len + j] : v[j];
      const float give = up ? v[j] : v[len + j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, give, o);
    }
  }
  return make_float2(v[0], v[1]);
}

// One CTA (4 warps, thread t = tile row t) per tile of cpt = floor(128 / n) whole
// configurations.  Forward as forward_tc_kernel; then, with de = dL/de_row =
// 2 (E_s - E) / C for the rows of a configuration (0 for the padding rows):
//   d2 = de w3 silu'(z2)                      (FP32, then bf16 operands)
//   d1 = (d2 W2^T) silu'(z1)                  tcgen05, M = 128, N = 64, K = 64
//   [dW2^T | db2 ; dW1^T | db1] = [d2^T ; d1^T] [h1 | G | 1]
//                                             tcgen05, M = 128, N = 112, K = 128
//   dw3 = sum_r de h2, db3 = sum_r de         warp reduce-scatters
// and writes the tile's gradient sums (part[tile]) and loss sum (lpart[tile]).  Tensor
// memory: z1 in columns 0-63, z2 in 64-127, d2 W2^T in 128-191, the weight-gradient
// accumulator in 0-111 once z1 and z2 are consumed.
__global__ void __launch_bounds__(128, 1) train_tc_kernel(const __nv_bfloat16* gq, const float* target,
                                                          int n, int configs, double loss_scale,
                                                          SgWeights wts, float* part, double* lpart,
                                                          unsigned int* timeout) {
  extern __shared__ unsigned char tt_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)tt_raw + 1023) & ~(uintptr_t)1023);
  __shared__ float sb1[SG_H1], sb2[SG_H2], sw3[SG_H2];
  __shared__ float se[SG_TILE];       // per-row energies
  __shared__ float sde[SG_TILE];      // per-configuration dL/de
  __shared__ double sl[SG_TILE];      // per-configuration loss terms
  __shared__ float2 sred[4][32];      // dw3 per warp (lane l: entries 2 l, 2 l + 1)
  __shared__ float sdb3[4];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ __align__(8) uint64_t wbar;
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int cpt = SG_TILE / n;
  const int c0 = blockIdx.x * cpt;
  const int nc = min(cpt, configs - c0);
  const int rows_t = nc * n;
  const size_t row0 = (size_t)c0 * n;
  const int r = tid;
  const uint32_t base = tc05::smem_u32(sm);
  if (tid == 0) {
    tc05::mbar_init(&mbar, 1);
    tc05::mbar_init(&wbar, 1);
    constexpr uint32_t kW1 = SG_H1 * SG_RBF * 2, kW2 = SG_H2 * SG_H1 * 2;
    tc05::mbar_expect_tx(&wbar, kW1 + 2 * kW2);
    tc05::bulk_g2s(sm + TT_B1, wts.wc + SG_WC_W1T, kW1, &wbar);
    tc05::bulk_g2s(sm + TT_B2, wts.wc + SG_WC_W2T, kW2, &wbar);
    tc05::bulk_g2s(sm + TT_B3, wts.wc + SG_WC_W2, kW2, &wbar);
  }
  // G row r into A1 (K-major) and, transposed, into B4 rows 64-95; B4 row 96 = ones,
  // rows 97-111 = 0 (their columns of the weight-gradient accumulator are unused)
  {
    uint4 gv[SG_RBF / 8];
    const uint4* G = reinterpret_cast<const uint4*>(gq);
#pragma unroll
    for (int kg = 0; kg < SG_RBF / 8; ++kg) {
      gv[kg] = r < rows_t ? G[(row0 + r) * (SG_RBF / 8) + kg] : make_uint4(0, 0, 0, 0);
      *reinterpret_cast<uint4*>(sm + TT_A1 + tc05::core_offset(r, kg, SG_RBF / 8)) = gv[kg];
    }
    const __nv_bfloat16* gb = reinterpret_cast<const __nv_bfloat16*>(gv);
#pragma unroll
    for (int k = 0; k < SG_RBF; ++k)
      *reinterpret_cast<__nv_bfloat16*>(sm + TT_B4 + tt_off(64 + k, r)) = gb[k];
    st_bf16(sm, TT_B4 + tt_off(96, r), 1.0f);
#pragma unroll
    for (int k = 97; k < TT_N4; ++k) st_bf16(sm, TT_B4 + tt_off(k, r), 0.0f);
  }
  for (int k = tid; k < SG_H1; k += 128) { sb1[k] = wts.b1[k]; sb2[k] = wts.b2[k]; sw3[k] = wts.w3[k]; }
  if (warp == 0) tc05::tmem_alloc(&tbase, 256);
  tc05::fence_smem_async();
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
  const uint32_t tmem = tbase;
  const uint32_t lane_addr = (uint32_t)(warp * 32) << 16;
  const uint32_t trow = tmem + lane_addr;
  int last_parity = -1;
  // layer 1: z1 = G W1 -> columns 0-63
  const bool wok = tid == 0 ? tc05::mbar_wait(&wbar, 0, kPolls) : true;
  if (tid == 0 && wok) {
    constexpr uint32_t id = tc05::idesc_bf16(SG_TILE, SG_H1);
#pragma unroll
    for (int ks = 0; ks < SG_RBF / 16; ++ks)
      tc05::mma_bf16(tmem, tc05::sdesc(base + TT_A1 + 256 * ks, 128, 128 * (SG_RBF / 8)),
                     tc05::sdesc(base + TT_B1 + 256 * ks, 128, 128 * (SG_RBF / 8)), id, ks > 0);
    tc05::commit(&mbar);
    last_parity = 0;
  }
  bool ok = __syncthreads_and(wok);
  if (ok) ok = tc05::mbar_wait(&mbar, 0, kPolls);
  tc05::fence_after();
  // h1 = silu(z1 + b1) -> A2 (K-major) and B4 rows 0-63 (h1^T)
  if (ok) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float acc[32];
      tc05::ld32(trow + 32 * half, acc);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        uint32_t pk[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int j = 32 * half + 8 * q + 2 * u;
          pk[u] = pack_bf16(silu32(acc[8 * q + 2 * u] + sb1[j]), silu32(acc[8 * q + 2 * u + 1] + sb1[j + 1]));
        }
        *reinterpret_cast<uint4*>(sm + TT_A2 + tc05::core_offset(r, 4 * half + q, SG_H1 / 8)) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
        const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(pk);
#pragma unroll
        for (int u = 0; u < 8; ++u)
          *reinterpret_cast<__nv_bfloat16*>(sm + TT_B4 + tt_off(32 * half + 8 * q + u, r)) = hb[u];
      }
    }
  }
  tc05::fence_smem_async();
  tc05::fence_before();
  ok = __syncthreads_and(ok);
  tc05::fence_after();
  // layer 2: z2 = h1 W2 -> columns 64-127
  if (tid == 0 && ok) {
    constexpr uint32_t id = tc05::idesc_bf16(SG_TILE, SG_H2);
#pragma unroll
    for (int ks = 0; ks < SG_H1 / 16; ++ks)
      tc05::mma_bf16(tmem + SG_H1, tc05::sdesc(base + TT_A2 + 256 * ks, 128, 128 * (SG_H1 / 8)),
                     tc05::sdesc(base + TT_B2 + 256 * ks, 128, 128 * (SG_H1 / 8)), id, ks > 0);
    tc05::commit(&mbar);
    last_parity = 1;
  }
  if (ok) ok = tc05::mbar_wait(&mbar, 1, kPolls);
  tc05::fence_after();
  float e = 0.f;
  if (ok) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float acc[32];
      tc05::ld32(trow + SG_H1 + 32 * half, acc);
#pragma unroll
      for (int q = 0; q < 32; ++q) e += silu32(acc[q] + sb2[32 * half + q]) * sw3[32 * half + q];
    }
    e += wts.b3[0];
  }
  se[r] = e;
  ok = __syncthreads_and(ok);
  // per configuration: E_s = sum of its rows (FP64, row order), residual, dL/de
  if (tid < nc) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += (double)se[tid * n + i];
    const double res = s - (double)target[c0 + tid];
    sde[tid] = (float)(2.0 * res * loss_scale);
    sl[tid] = res * res * loss_scale;
  }
  __syncthreads();
  const float de = r < rows_t ? sde[r / n] : 0.0f;
  // d2 = de w3 silu'(z2 + b2) -> A2 (the d1 MMA's A, K-major) and A4 rows 0-63 (d2^T);
  // dw3 terms de silu(z2 + b2), reduced over the warp
  if (ok) {
    float dw[64];
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float acc[32];
      tc05::ld32(trow + SG_H1 + 32 * half, acc);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        uint32_t pk[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int j = 32 * half + 8 * q + 2 * u;
          const float za = acc[8 * q + 2 * u] + sb2[j], zb = acc[8 * q + 2 * u + 1] + sb2[j + 1];
          const float da = de * sw3[j] * dsilu32(za), db = de * sw3[j + 1] * dsilu32(zb);
          dw[j] = de * silu32(za);
          dw[j + 1] = de * silu32(zb);
          pk[u] = pack_bf16(da, db);
        }
        *reinterpret_cast<uint4*>(sm + TT_A2 + tc05::core_offset(r, 4 * half + q, SG_H2 / 8)) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
        const __nv_bfloat16* db = reinterpret_cast<const __nv_bfloat16*>(pk);
#pragma unroll
        for (int u = 0; u < 8; ++u)
          *reinterpret_cast<__nv_bfloat16*>(sm + TT_A4 + tt_off(32 * half + 8 * q + u, r)) = db[u];
      }
    }
    sred[warp][lane] = warp_reduce_scatter64(dw, lane);
    float d3 = de;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) d3 += __shfl_xor_sync(0xffffffffu, d3, o);
    if (lane == 0) sdb3[warp] = d3;
  }
  tc05::fence_smem_async();
  tc05::fence_before();
  ok = __syncthreads_and(ok);
  tc05::fence_after();
  // d2 W2^T -> columns 128-191
  if (tid == 0 && ok) {
    constexpr uint32_t id = tc05::idesc_bf16(SG_TILE, SG_H1);
#pragma unroll
    for (int ks = 0; ks < SG_H2 / 16; ++ks)
      tc05::mma_bf16(tmem + 128, tc05::sdesc(base + TT_A2 + 256 * ks, 128, 128 * (SG_H2 / 8)),
                     tc05::sdesc(base + TT_B3 + 256 * ks, 128, 128 * (SG_H2 / 8)), id, ks > 0);
    tc05::commit(&mbar);
    last_parity = 0;
  }
  if (ok) ok = tc05::mbar_wait(&mbar, 0, kPolls);
  tc05::fence_after();
  // d1 = (d2 W2^T) silu'(z1 + b1) -> A4 rows 64-127 (d1^T)
  if (ok) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float a3[32], a1[32];
      tc05::ld32(trow + 128 + 32 * half, a3);
      tc05::ld32(trow + 32 * half, a1);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int k = 32 * half + j;
        st_bf16(sm, TT_A4 + tt_off(64 + k, r), a3[j] * dsilu32(a1[j] + sb1[k]));
      }
    }
  }
  tc05::fence_smem_async();
  tc05::fence_before();
  ok = __syncthreads_and(ok);
  tc05::fence_after();
  // weight gradients: [d2^T ; d1^T] [h1 | G | 1 | 0] -> columns 0-111
  if (tid == 0 && ok) {
    constexpr uint32_t id = tc05::idesc_bf16(SG_TILE, TT_N4);
#pragma unroll
    for (int ks = 0; ks < SG_TILE / 16; ++ks)
      tc05::mma_bf16(tmem, tc05::sdesc(base + TT_A4 + 256 * ks, 128, 128 * (SG_TILE / 8)),
                     tc05::sdesc(base + TT_B4 + 256 * ks, 128, 128 * (SG_TILE / 8)), id, ks > 0);
    tc05::commit(&mbar);
    last_parity = 1;
  }
  if (ok) ok = tc05::mbar_wait(&mbar, 1, kPolls);
  ok = __syncthreads_and(ok);
  tc05::fence_after();
  float* P = part + (size_t)blockIdx.x * SG_NPARAM;
  if (ok) {
    float acc[32];
    if (r < 64) {  // accumulator row n = r: dW2[k][n] in columns k, db2[n] in column 96
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        tc05::ld32(trow + 32 * c, acc);
#pragma unroll
        for (int j = 0; j < 32; ++j) P[SG_OFF_W2 + (32 * c + j) * SG_H2 + r] = acc[j];
      }
      tc05::ld32(trow + 96, acc);
      P[SG_OFF_B2 + r] = acc[0];
    } else {       // row 64 + k: dW1[k'][k] in columns 64 + k', db1[k] in column 96
      const int k = r - 64;
      tc05::ld32(trow + 64, acc);
#pragma unroll
      for (int j = 0; j < 32; ++j) P[SG_OFF_W1 + j * SG_H1 + k] = acc[j];
      tc05::ld32(trow + 96, acc);
      P[SG_OFF_B1 + k] = acc[0];
    }
    if (tid < 32) {
      float2 s = sred[0][tid];
#pragma unroll
      for (int w = 1; w < 4; ++w) { s.x += sred[w][tid].x; s.y += sred[w][tid].y; }
      P[SG_OFF_W3 + 2 * tid] = s.x;
      P[SG_OFF_W3 + 2 * tid + 1] = s.y;
    }
    if (tid == 0) {
      P[SG_OFF_B3] = sdb3[0] + sdb3[1] + sdb3[2] + sdb3[3];
      double l = 0.0;
      for (int c = 0; c < nc; ++c) l += sl[c];
      lpart[blockIdx.x] = l;
    }
  } else {
    const float nan = __int_as_float(0x7fc00000);
    for (int p = tid; p < SG_NPARAM; p += 128) P[p] = nan;
    if (tid == 0) {
      lpart[blockIdx.x] = __longlong_as_double(0x7ff8000000000000ll);
      if (timeout) atomicOr(timeout, 1u);
      drain_async(&wbar, !wok, &mbar, last_parity);
    }
  }
  tc05::fence_before();
  __syncthreads();
  if (warp == 0) tc05::tmem_dealloc(tmem, 256);
}

// Write parameter p's bf16 copies: W1^T / W2^T row-major (mma.sync operands) and the
// tcgen05 core-matrix orders (W1^T, W2^T, W2).
__device__ __forceinline__ void refresh_one(int p, float val, __nv_bfloat16* w1t, __nv_bfloat16* w2t,
                                            __nv_bfloat16* wc) {
  const __nv_bfloat16 v = __float2bfloat16_rn(val);
  if (p >= SG_OFF_W1 && p < SG_OFF_B1) {
    const int q = p - SG_OFF_W1, k = q / SG_H1, n = q % SG_H1;  // W1[k][n]
    w1t[n * SG_RBF + k] = v;
    wc[SG_WC_W1T + (tc05::core_offset(n, k / 8, SG_RBF / 8) + 2 * (k % 8)) / 2] = v;
  } else if (p >= SG_OFF_W2 && p < SG_OFF_B2) {
    const int q = p - SG_OFF_W2, k = q / SG_H2, n = q % SG_H2;  // W2[k][n]
    w2t[n * SG_H1 + k] = v;
    wc[SG_WC_W2T + (tc05::core_offset(n, k / 8, SG_H1 / 8) + 2 * (k % 8)) / 2] = v;
    wc[SG_WC_W2 + (tc05::core_offset(k, n / 8, SG_H2 / 8) + 2 * (n % 8)) / 2] = v;
  }
}

// grad[p] = sum over tiles (fixed order) of part[t][p]; thread 0 sums the loss.  With
// adam.step > 0, Adam (Kingma & Ba 2015) updates master[p] and the bf16 copies.
__global__ void reduce_adam_kernel(const float* part, const double* lpart, int tiles, float* grad,
                                   double* loss, SgAdam adam, __nv_bfloat16* w1t, __nv_bfloat16* w2t,
                                   __nv_bfloat16* wc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p == 0) {
    double l = 0.0;
    for (int t = 0; t < tiles; ++t) l += lpart[t];
    *loss = l;
  }
  if (p >= SG_NPARAM) return;
  // eight independent partial sums (tiles t = k mod 8), combined in a fixed order: the
  // loads overlap, and the result depends only on the number of tiles
  float a[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  int t = 0;
  for (; t + 8 <= tiles; t += 8) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] += part[(size_t)(t + k) * SG_NPARAM + p];
  }
  for (int k = 0; t + k < tiles; ++k) a[k] += part[(size_t)(t + k) * SG_NPARAM + p];
  const float s = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
  grad[p] = s;
  if (adam.step > 0) {
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    const float mm = beta1 * adam.m[p] + (1.f - beta1) * s;
    const float vv = beta2 * adam.v[p] + (1.f - beta2) * s * s;
    adam.m[p] = mm;
    adam.v[p] = vv;
    const float mh = mm / (1.f - powf(beta1, (float)adam.step));
    const float vh = vv / (1.f - powf(beta2, (float)adam.step));
    const float w = adam.master[p] - adam.lr * mh / (sqrtf(vh) + eps);
    adam.master[p] = w;
    refresh_one(p, w, w1t, w2t, wc);
  }
}

__global__ void refresh_bf16_kernel(const float* w, __nv_bfloat16* w1t, __nv_bfloat16* w2t,
                                    __nv_bfloat16* wc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < SG_NPARAM) refresh_one(p, w[p], w1t, w2t, wc);
}

// Copy the walkers' current configurations (LJ double-single planes) into the training
// ring as binary32 [n][3] records with their energies.
__global__ void collect_kernel(const float* lj_pos, int np, int n, const WalkerCore* cores, int walkers,
                               float* ring_pos, float* ring_e, int ring_cap, int ring_head) {
  const int w = blockIdx.x;
  if (w >= walkers) return;
  const int slot = (ring_head + w) % ring_cap;
  const float* p = lj_pos + (size_t)w * 6 * np;
  for (int j = threadIdx.x; j < n; j += blockDim.x)
    for (int a = 0; a < 3; ++a)
      ring_pos[((size_t)slot * n + j) * 3 + a] = (float)((double)p[a * np + j] + (double)p[(3 + a) * np + j]);
  if (threadIdx.x == 0) ring_e[slot] = (float)cores[w].E;
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void gather_kernel(const float* ring_pos, const float* ring_e, int n, int ring_count,
                              uint64_t seed, uint64_t step, int count, float* out_pos, float* out_e) {
  const int c = blockIdx.x;
  if (c >= count) return;
  const uint64_t h = splitmix64(seed ^ splitmix64(step * 0x100000001B3ull + (uint64_t)c));
  const int s = (int)((h >> 11) % (uint64_t)ring_count);
  for (int k = threadIdx.x; k < 3 * n; k += blockDim.x)
    out_pos[(size_t)c * 3 * n + k] = ring_pos[(size_t)s * 3 * n + k];
  if (threadIdx.x == 0) out_e[c] = ring_e[s];
}

__global__ void take_flag_kernel(unsigned int* flag, unsigned int* out) { *out = atomicExch(flag, 0u); }

}  // namespace dev

cudaError_t sg_descriptors(const float* pos, int n, int rows, __nv_bfloat16* gq, float* gf,
                           cudaStream_t st) {
  const long long threads = (long long)rows * dev::DESC_TPR;
  dev::descriptor_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(pos, n, rows, gq, gf);
  return cudaGetLastError();
}

namespace {
// Set by the tensor-core kernels of the allocating entry points when a wait ran out
// (their energies or gradients are NaN).
__device__ unsigned int g_sg_tc_timeout;
}  // namespace

cudaError_t sg_timeout_flag(unsigned int** flag) {
  return cudaGetSymbolAddress((void**)flag, g_sg_tc_timeout);
}

cudaError_t sg_take_flag(unsigned int* flag, unsigned int* out, cudaStream_t st) {
  dev::take_flag_kernel<<<1, 1, 0, st>>>(flag, out);
  return cudaGetLastError();
}

cudaError_t sg_forward(const __nv_bfloat16* gq, int rows, const SgWeights& w, float* e,
                       unsigned int* timeout, cudaStream_t st) {
  dev::forward_tc_kernel<<<(rows + SG_TILE - 1) / SG_TILE, 128, 0, st>>>(gq, rows, w, e, timeout);
  return cudaGetLastError();
}

namespace {
// Scratch of sadmc_surrogate_loss_grads_noalloc: SgScratch for SG_STATIC_ROWS rows
// (about 2 MB), one copy per device, never allocated or freed at run time.
static __device__ __align__(256) unsigned char g_sg_static_scratch[SgScratch::bytes(SG_STATIC_ROWS)];
constexpr int kStaticDevices = 64;
std::mutex g_static_mu;
void* g_static_addr[kStaticDevices] = {};
std::atomic<bool> g_train_attr[kStaticDevices] = {};
}  // namespace

cudaError_t sg_static_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kStaticDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sg_static_scratch);  // with `dev` current
    if (e != cudaSuccess) return e;
    g_static_addr[dev] = p;
  }
  *out = g_static_addr[dev];
  return cudaSuccess;
}

cudaError_t sg_prepare_train(void) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < kStaticDevices && g_train_attr[dev].load(std::memory_order_acquire)) return cudaSuccess;
  e = cudaFuncSetAttribute(dev::train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dev::TT_SMEM);
  if (e == cudaSuccess && dev >= 0 && dev < kStaticDevices) g_train_attr[dev].store(true, std::memory_order_release);
  return e;
}

cudaError_t sg_train_step(const float* pos, const float* target, int configs, int n,
                          const SgWeights& w, float* grad, const SgAdam& adam, SgScratch s,
                          double* loss_dev, unsigned int* timeout, cudaStream_t st) {
  if (n < 1 || n > SG_MAX_ATOMS || configs < 1) return cudaErrorInvalidValue;
  const int rows = configs * n;
  const int tiles = sg_tiles(configs, n);
  cudaError_t e = sg_prepare_train();
  if (e == cudaSuccess) e = sg_descriptors(pos, n, rows, s.gq, nullptr, st);
  if (e == cudaSuccess) {
    dev::train_tc_kernel<<<tiles, 128, dev::TT_SMEM, st>>>(s.gq, target, n, configs, 1.0 / (double)configs,
                                                           w, s.part, s.lpart, timeout);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    dev::reduce_adam_kernel<<<(SG_NPARAM + 127) / 128, 128, 0, st>>>(s.part, s.lpart, tiles, grad, loss_dev,
                                                                    adam, w.w1t, w.w2t, w.wc);
    e = cudaGetLastError();
  }
  return e;
}

cudaError_t sg_refresh(const float* master, const SgWeights& w, cudaStream_t st) {
  dev::refresh_bf16_kernel<<<(SG_NPARAM + 127) / 128, 128, 0, st>>>(master, w.w1t, w.w2t, w.wc);
  return cudaGetLastError();
}

cudaError_t sg_collect(const float* lj_pos, int np, int n, const WalkerCore* cores, int walkers,
                       float* ring_pos, float* ring_e, int ring_cap, int ring_head, cudaStream_t st) {
  dev::collect_kernel<<<walkers, 64, 0, st>>>(lj_pos, np, n, cores, walkers, ring_pos, ring_e, ring_cap, ring_head);
  return cudaGetLastError();
}

cudaError_t sg_gather(const float* ring_pos, const float* ring_e, int n, int ring_count,
                      uint64_t seed, uint64_t step, int count, float* out_pos, float* out_e,
                      cudaStream_t st) {
  dev::gather_kernel<<<count, 128, 0, st>>>(ring_pos, ring_e, n, ring_count, seed, step, count, out_pos, out_e);
  return cudaGetLastError();
}

}  // namespace sadmc
