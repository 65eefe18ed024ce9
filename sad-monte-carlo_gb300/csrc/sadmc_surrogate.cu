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
//   backward    FP32 per-row deltas, then weight gradients as row reductions
//   update      Adam with bias correction on FP32 master weights; bf16 copies refreshed
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <mutex>

#include "sadmc_common.cuh"
#include "sadmc_mma.cuh"
#include "sadmc_surrogate.h"
#include "sadmc_tc05.cuh"

namespace sadmc {
namespace dev {

// Descriptors of rows [row0, row0 + rows): row r = atom (r % n) of configuration (r / n);
// positions [configs][n][3] binary32.  Writes bf16 G (the forward operand) and, if
// requested, FP32 G.
__global__ void descriptor_kernel(const float* pos, int n, int rows, __nv_bfloat16* gq, float* gf) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const int c = r / n, i = r % n;
  const float* p = pos + (size_t)c * n * 3;
  const float xi = p[3 * i], yi = p[3 * i + 1], zi = p[3 * i + 2];
  float g[SG_RBF];
#pragma unroll
  for (int k = 0; k < SG_RBF; ++k) g[k] = 0.0f;
  const float inv2w2 = 1.0f / (2.0f * 0.1f * 0.1f);
  for (int j = 0; j < n; ++j) {
    if (j == i) continue;
    const float dx = p[3 * j] - xi, dy = p[3 * j + 1] - yi, dz = p[3 * j + 2] - zi;
    const float rij = sqrtf(dx * dx + dy * dy + dz * dz);
#pragma unroll
    for (int k = 0; k < SG_RBF; ++k) {
      const float d = rij - rbf_centre(k);
      g[k] += __expf(-d * d * inv2w2);
    }
  }
#pragma unroll
  for (int k = 0; k < SG_RBF; ++k) {
    gq[(size_t)r * SG_RBF + k] = __float2bfloat16_rn(g[k]);
    if (gf) gf[(size_t)r * SG_RBF + k] = g[k];
  }
}

// Forward pass on the fifth-generation tensor cores: one CTA of 4 warps per 128-row tile.
// G (128 x 32), W1^T (64 x 32), h1 (128 x 64) and W2^T (64 x 64) sit in shared memory as
// BF16 core matrices (K-major, no swizzle); thread 0 issues the tcgen05 MMAs of each
// layer (M = 128, N = 64, K = 16 per instruction) into FP32 accumulators in tensor
// memory (layer 1 in columns 0-63, layer 2 in 64-127) and commits them to an mbarrier;
// each warp reads its 32 rows back with tcgen05.ld for the bias, SiLU and, after layer 2,
// the 64 -> 1 output in FP32.  Writes per-row energies and, for training, z1 and z2.
// A wait that runs out (it never should) sets *timeout and writes NaN energies.
__global__ void __launch_bounds__(128, 1) forward_tc_kernel(const __nv_bfloat16* gq, int rows,
                                                            SgWeights wts, float* e_out,
                                                            float* z1_out, float* z2_out,
                                                            unsigned int* timeout) {
  constexpr int M = 128;
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
    tc05::bulk_g2s(b1, wts.wc, kW1Bytes, &wbar);
    tc05::bulk_g2s(b2, wts.wc + SG_H1 * SG_RBF, kW2Bytes, &wbar);
  }
  tc05::fence_smem_async();
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
  const uint32_t tmem = tbase;
  constexpr uint32_t idesc = tc05::idesc_bf16(M, SG_H1);
  constexpr uint32_t kPolls = 1u << 24;
  // layer 1: D1 = G W1 (two K = 16 steps, 2 core matrices = 256 bytes apart), once the
  // weights have landed
  const bool wok = tid == 0 ? tc05::mbar_wait(&wbar, 0, kPolls) : true;
  if (tid == 0 && wok) {
#pragma unroll
    for (int ks = 0; ks < SG_RBF / 16; ++ks)
      tc05::mma_bf16(tmem, tc05::sdesc(tc05::smem_u32(a1) + 256 * ks, 128, 128 * (SG_RBF / 8)),
                     tc05::sdesc(tc05::smem_u32(b1) + 256 * ks, 128, 128 * (SG_RBF / 8)), idesc, ks > 0);
    tc05::commit(&mbar);
  }
  bool ok = tc05::mbar_wait(&mbar, 0, kPolls);
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
          const float z0 = acc[8 * q + 2 * u] + sb1[j], zz1 = acc[8 * q + 2 * u + 1] + sb1[j + 1];
          if (z1_out && row0 + r < rows) {
            z1_out[(size_t)(row0 + r) * SG_H1 + j] = z0;
            z1_out[(size_t)(row0 + r) * SG_H1 + j + 1] = zz1;
          }
          pk[u] = pack_bf16(silu32(z0), silu32(zz1));
        }
        *reinterpret_cast<uint4*>(a2 + tc05::core_offset(r, 4 * half + q, SG_H1 / 8)) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
  }
  tc05::fence_smem_async();
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
  // layer 2: D2 = h1 W2 (four K = 16 steps) into columns 64-127
  if (tid == 0 && ok) {
#pragma unroll
    for (int ks = 0; ks < SG_H1 / 16; ++ks)
      tc05::mma_bf16(tmem + SG_H1, tc05::sdesc(tc05::smem_u32(a2) + 256 * ks, 128, 128 * (SG_H1 / 8)),
                     tc05::sdesc(tc05::smem_u32(b2) + 256 * ks, 128, 128 * (SG_H1 / 8)), idesc, ks > 0);
    tc05::commit(&mbar);
  }
  // every thread saw the same layer-1 outcome only if the CTA agrees on it
  ok = __syncthreads_and(ok);
  if (ok) ok = tc05::mbar_wait(&mbar, 1, kPolls);
  tc05::fence_after();
  float e = 0.f;
  if (ok) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      float acc[32];
      tc05::ld32(tmem + lane_addr + SG_H1 + 32 * half, acc);
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const int j = 32 * half + q;
        const float z = acc[q] + sb2[j];
        if (z2_out && row0 + r < rows) z2_out[(size_t)(row0 + r) * SG_H2 + j] = z;
        e += silu32(z) * sw3[j];
      }
    }
    e += wts.b3[0];
  } else {
    e = __int_as_float(0x7fc00000);
    if (tid == 0) atomicOr(timeout, 1u);
  }
  if (row0 + r < rows) e_out[row0 + r] = e;
  tc05::fence_before();
  __syncthreads();
  if (warp == 0) tc05::tmem_dealloc(tmem, 256);
}

// Per configuration: E_s = sum of its n row energies, residual against the target,
// dL/de = 2 (E_s - E) / C for each of its rows; the loss sum is accumulated.
__global__ void residual_kernel(const float* e, int n, int configs, const float* target,
                                float* de, float* es_out, double* loss_acc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= configs) return;
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += (double)e[(size_t)c * n + i];
  const double r = s - (double)target[c];
  if (es_out) es_out[c] = (float)s;
  const float d = (float)(2.0 * r / (double)configs);
  for (int i = 0; i < n; ++i) de[(size_t)c * n + i] = d;
  atomicAdd(loss_acc, r * r / (double)configs);
}

// Per-row deltas: d2 = de * w3 * silu'(z2); d1 = (d2 W2q^T) * silu'(z1).  FP32.
__global__ void delta_kernel(const float* z1, const float* z2, const float* de, int rows,
                             SgWeights wts, float* d1, float* d2) {
  __shared__ float sW2[SG_H1 * SG_H2];  // W2 rounded to bf16, [k][n]
  __shared__ float sw3[SG_H2];
  for (int k = threadIdx.x; k < SG_H1 * SG_H2; k += blockDim.x) sW2[k] = bf16r(wts.w2[k]);
  for (int k = threadIdx.x; k < SG_H2; k += blockDim.x) sw3[k] = wts.w3[k];
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  float dd2[SG_H2];
  const float e = de[r];
#pragma unroll 8
  for (int n = 0; n < SG_H2; ++n) {
    dd2[n] = e * sw3[n] * dsilu32(z2[(size_t)r * SG_H2 + n]);
    d2[(size_t)r * SG_H2 + n] = dd2[n];
  }
  for (int k = 0; k < SG_H1; ++k) {
    float s = 0.f;
#pragma unroll 8
    for (int n = 0; n < SG_H2; ++n) s += dd2[n] * sW2[k * SG_H2 + n];
    d1[(size_t)r * SG_H1 + k] = s * dsilu32(z1[(size_t)r * SG_H1 + k]);
  }
}

// Weight gradients as reductions over rows; one thread per parameter.
//   dW1[k][n] = sum_r Gq[r][k] d1[r][n]     dW2[k][n] = sum_r h1q[r][k] d2[r][n]
//   db1 = sum d1, db2 = sum d2, dw3[n] = sum de h2[r][n], db3 = sum de
__global__ void wgrad_kernel(const __nv_bfloat16* gq, const float* z1, const float* z2,
                             const float* d1, const float* d2, const float* de, int rows,
                             float* grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= SG_NPARAM) return;
  float s = 0.f;
  if (p < SG_OFF_B1) {                       // W1
    const int k = p / SG_H1, n = p % SG_H1;
    for (int r = 0; r < rows; ++r) s += __bfloat162float(gq[(size_t)r * SG_RBF + k]) * d1[(size_t)r * SG_H1 + n];
  } else if (p < SG_OFF_W2) {                // b1
    const int n = p - SG_OFF_B1;
    for (int r = 0; r < rows; ++r) s += d1[(size_t)r * SG_H1 + n];
  } else if (p < SG_OFF_B2) {                // W2
    const int q = p - SG_OFF_W2, k = q / SG_H2, n = q % SG_H2;
    for (int r = 0; r < rows; ++r) s += bf16r(silu32(z1[(size_t)r * SG_H1 + k])) * d2[(size_t)r * SG_H2 + n];
  } else if (p < SG_OFF_W3) {                // b2
    const int n = p - SG_OFF_B2;
    for (int r = 0; r < rows; ++r) s += d2[(size_t)r * SG_H2 + n];
  } else if (p < SG_OFF_B3) {                // w3
    const int n = p - SG_OFF_W3;
    for (int r = 0; r < rows; ++r) s += de[r] * silu32(z2[(size_t)r * SG_H2 + n]);
  } else {                                   // b3
    for (int r = 0; r < rows; ++r) s += de[r];
  }
  grad[p] = s;
}

// Adam (Kingma & Ba 2015) on the FP32 master weights, then the bf16 transposed copies.
__global__ void adam_kernel(float* w, const float* grad, float* m, float* v, int step, float lr,
                            float beta1, float beta2, float eps) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= SG_NPARAM) return;
  const float gr = grad[p];
  const float mm = beta1 * m[p] + (1.f - beta1) * gr;
  const float vv = beta2 * v[p] + (1.f - beta2) * gr * gr;
  m[p] = mm;
  v[p] = vv;
  const float mh = mm / (1.f - powf(beta1, (float)step));
  const float vh = vv / (1.f - powf(beta2, (float)step));
  w[p] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void refresh_bf16_kernel(const float* w, __nv_bfloat16* w1t, __nv_bfloat16* w2t,
                                    __nv_bfloat16* wc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < SG_RBF * SG_H1) {
    const int k = p / SG_H1, n = p % SG_H1;
    const __nv_bfloat16 v = __float2bfloat16_rn(w[SG_OFF_W1 + p]);
    w1t[n * SG_RBF + k] = v;
    wc[(tc05::core_offset(n, k / 8, SG_RBF / 8) + 2 * (k % 8)) / 2] = v;
  }
  if (p < SG_H1 * SG_H2) {
    const int k = p / SG_H2, n = p % SG_H2;
    const __nv_bfloat16 v = __float2bfloat16_rn(w[SG_OFF_W2 + p]);
    w2t[n * SG_H1 + k] = v;
    wc[SG_H1 * SG_RBF + (tc05::core_offset(n, k / 8, SG_H1 / 8) + 2 * (k % 8)) / 2] = v;
  }
}

// Copy the walkers' current configurations (LJ double-single planes) into the training
// ring as binary32 [n][3] records with their energies.
__global__ void collect_kernel(const float* lj_pos, int np, int n, const double* E, int walkers,
                               float* ring_pos, float* ring_e, int ring_cap, int ring_head) {
  const int w = blockIdx.x;
  if (w >= walkers) return;
  const int slot = (ring_head + w) % ring_cap;
  const float* p = lj_pos + (size_t)w * 6 * np;
  for (int j = threadIdx.x; j < n; j += blockDim.x)
    for (int a = 0; a < 3; ++a)
      ring_pos[((size_t)slot * n + j) * 3 + a] = (float)((double)p[a * np + j] + (double)p[(3 + a) * np + j]);
  if (threadIdx.x == 0) ring_e[slot] = (float)E[w];
}

__global__ void gather_kernel(const float* ring_pos, const float* ring_e, int n, const int* idx,
                              int count, float* out_pos, float* out_e) {
  const int c = blockIdx.x;
  if (c >= count) return;
  const int s = idx[c];
  for (int k = threadIdx.x; k < 3 * n; k += blockDim.x)
    out_pos[(size_t)c * 3 * n + k] = ring_pos[(size_t)s * 3 * n + k];
  if (threadIdx.x == 0) out_e[c] = ring_e[s];
}

}  // namespace dev

cudaError_t sg_descriptors(const float* pos, int n, int rows, __nv_bfloat16* gq, float* gf,
                           cudaStream_t st) {
  dev::descriptor_kernel<<<(rows + 127) / 128, 128, 0, st>>>(pos, n, rows, gq, gf);
  return cudaGetLastError();
}

namespace {
// Set by forward_tc_kernel when a tensor-core wait ran out (its energies are NaN).
__device__ unsigned int g_sg_tc_timeout;
}  // namespace

cudaError_t sg_forward(const __nv_bfloat16* gq, int rows, const SgWeights& w, float* e, float* z1,
                       float* z2, cudaStream_t st) {
  unsigned int* flag = nullptr;
  cudaError_t err = cudaGetSymbolAddress((void**)&flag, g_sg_tc_timeout);
  if (err != cudaSuccess) return err;
  dev::forward_tc_kernel<<<(rows + 127) / 128, 128, 0, st>>>(gq, rows, w, e, z1, z2, flag);
  return cudaGetLastError();
}

cudaError_t sg_forward_timeouts(unsigned int* count, cudaStream_t st) {
  unsigned int zero = 0;
  cudaError_t e = cudaMemcpyFromSymbolAsync(count, g_sg_tc_timeout, sizeof(unsigned int), 0,
                                            cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess && *count)
    e = cudaMemcpyToSymbolAsync(g_sg_tc_timeout, &zero, sizeof(unsigned int), 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

namespace {
// Scratch of sadmc_surrogate_loss_grads_noalloc: SgScratch for SG_STATIC_ROWS rows
// (about 4.3 MB), one copy per device, never allocated or freed at run time.
static __device__ __align__(256) unsigned char g_sg_static_scratch[SgScratch::bytes(SG_STATIC_ROWS)];
constexpr int kStaticDevices = 64;
std::mutex g_static_mu;
void* g_static_addr[kStaticDevices] = {};
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

cudaError_t sg_train_step(const float* pos, const float* target, int configs, int n,
                          const SgWeights& w, float* master, float* grad, float* m, float* v,
                          int step, float lr, SgScratch s, double* loss_dev, cudaStream_t st) {
  const int rows = configs * n;
  cudaError_t e = sg_descriptors(pos, n, rows, s.gq, nullptr, st);
  if (e == cudaSuccess) e = sg_forward(s.gq, rows, w, s.e, s.z1, s.z2, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(loss_dev, 0, sizeof(double), st);
  if (e == cudaSuccess) {
    dev::residual_kernel<<<(configs + 127) / 128, 128, 0, st>>>(s.e, n, configs, target, s.de, nullptr, loss_dev);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    dev::delta_kernel<<<(rows + 127) / 128, 128, 0, st>>>(s.z1, s.z2, s.de, rows, w, s.d1, s.d2);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    dev::wgrad_kernel<<<(SG_NPARAM + 127) / 128, 128, 0, st>>>(s.gq, s.z1, s.z2, s.d1, s.d2, s.de, rows, grad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && step > 0) {
    dev::adam_kernel<<<(SG_NPARAM + 127) / 128, 128, 0, st>>>(master, grad, m, v, step, lr, 0.9f, 0.999f, 1e-8f);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = sg_refresh(master, w, st);
  }
  return e;
}

cudaError_t sg_refresh(const float* master, const SgWeights& w, cudaStream_t st) {
  dev::refresh_bf16_kernel<<<(SG_H1 * SG_H2 + 127) / 128, 128, 0, st>>>(master, w.w1t, w.w2t, w.wc);
  return cudaGetLastError();
}

cudaError_t sg_collect(const float* lj_pos, int np, int n, const double* E, int walkers,
                       float* ring_pos, float* ring_e, int ring_cap, int ring_head, cudaStream_t st) {
  dev::collect_kernel<<<walkers, 64, 0, st>>>(lj_pos, np, n, E, walkers, ring_pos, ring_e, ring_cap, ring_head);
  return cudaGetLastError();
}

cudaError_t sg_gather(const float* ring_pos, const float* ring_e, int n, const int* idx, int count,
                      float* out_pos, float* out_e, cudaStream_t st) {
  dev::gather_kernel<<<count, 128, 0, st>>>(ring_pos, ring_e, n, idx, count, out_pos, out_e);
  return cudaGetLastError();
}

}  // namespace sadmc
