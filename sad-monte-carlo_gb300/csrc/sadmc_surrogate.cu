// Learned surrogate for delayed-acceptance LJ moves: a radial-descriptor MLP
// (32 Gaussian radial basis functions per atom -> 64 -> 64 -> 1, SiLU), per-atom energies
// summed over the cluster.  The reference has no learned part; this is the surrogate the
// delayed-acceptance moves screen with, trained online on configurations the walkers
// themselves visit.
//
//   descriptor  G[i,k] = sum_{j != i} exp(-(r_ij - c_k)^2 / (2 w^2)), c_k = 0.8 + 2.2 k/31,
//               w = 0.1 (binary32)
//   forward     tensor cores: mma.sync m16n8k16, bf16 operands (G, W1, h1, W2), FP32
//               accumulation; layer 1's accumulator fragments are re-packed in registers
//               as layer 2's A fragments; the last layer (64 -> 1) and the SiLUs in FP32
//   backward    FP32 per-row deltas, then weight gradients as row reductions
//   update      Adam with bias correction on FP32 master weights; bf16 copies refreshed
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <mutex>

#include "sadmc_common.cuh"
#include "sadmc_mma.cuh"
#include "sadmc_surrogate.h"

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

// Forward pass for 16-row tiles, one warp per tile.  Weights come from shared memory.
// Writes per-row energies and, for training, z1 and z2 (pre-activations).
__global__ void __launch_bounds__(128) forward_kernel(const __nv_bfloat16* gq, int rows,
                                                      SgWeights wts, float* e_out, float* z1_out,
                                                      float* z2_out) {
  __shared__ uint32_t sW1[SG_H1 * SG_RBF / 2];   // W1^T as bf16 pairs: [n][k/2]
  __shared__ uint32_t sW2[SG_H2 * SG_H1 / 2];    // W2^T: [n][k/2]
  __shared__ float sb1[SG_H1], sb2[SG_H2], sw3[SG_H2];
  for (int k = threadIdx.x; k < SG_H1 * SG_RBF / 2; k += blockDim.x)
    sW1[k] = reinterpret_cast<const uint32_t*>(wts.w1t)[k];
  for (int k = threadIdx.x; k < SG_H2 * SG_H1 / 2; k += blockDim.x)
    sW2[k] = reinterpret_cast<const uint32_t*>(wts.w2t)[k];
  for (int k = threadIdx.x; k < SG_H1; k += blockDim.x) { sb1[k] = wts.b1[k]; sb2[k] = wts.b2[k]; sw3[k] = wts.w3[k]; }
  __syncthreads();
  const float b3 = wts.b3[0];
  const int lane = threadIdx.x & 31;
  const int tile = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int row0 = tile * 16;
  if (row0 >= rows) return;
  const int g = lane >> 2, t = lane & 3;
  const int ra = row0 + g, rb = row0 + g + 8;
  const bool va = ra < rows, vb = rb < rows;
  // A fragments of G (16 x 32 = two k tiles)
  uint32_t aG[2][4];
  const uint32_t* G32 = reinterpret_cast<const uint32_t*>(gq);
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) {
    aG[kt][0] = va ? G32[(size_t)ra * (SG_RBF / 2) + 8 * kt + t] : 0u;
    aG[kt][1] = vb ? G32[(size_t)rb * (SG_RBF / 2) + 8 * kt + t] : 0u;
    aG[kt][2] = va ? G32[(size_t)ra * (SG_RBF / 2) + 8 * kt + 4 + t] : 0u;
    aG[kt][3] = vb ? G32[(size_t)rb * (SG_RBF / 2) + 8 * kt + 4 + t] : 0u;
  }
  // layer 1: 8 n tiles of 8
  float h1[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
      const int n = 8 * j + g;
      mma16816(c, aG[kt], sW1[n * (SG_RBF / 2) + 8 * kt + t], sW1[n * (SG_RBF / 2) + 8 * kt + 4 + t]);
    }
    const float bb0 = sb1[8 * j + 2 * t], bb1 = sb1[8 * j + 2 * t + 1];
    const float z[4] = {c[0] + bb0, c[1] + bb1, c[2] + bb0, c[3] + bb1};
    if (z1_out) {
      if (va) { z1_out[(size_t)ra * SG_H1 + 8 * j + 2 * t] = z[0]; z1_out[(size_t)ra * SG_H1 + 8 * j + 2 * t + 1] = z[1]; }
      if (vb) { z1_out[(size_t)rb * SG_H1 + 8 * j + 2 * t] = z[2]; z1_out[(size_t)rb * SG_H1 + 8 * j + 2 * t + 1] = z[3]; }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) h1[j][q] = silu32(z[q]);
  }
  // layer 2: A fragments from layer 1 accumulators (n tiles 2kt and 2kt+1 form k tile kt)
  float h2[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      const uint32_t a[4] = {pack_bf16(h1[2 * kt][0], h1[2 * kt][1]), pack_bf16(h1[2 * kt][2], h1[2 * kt][3]),
                             pack_bf16(h1[2 * kt + 1][0], h1[2 * kt + 1][1]),
                             pack_bf16(h1[2 * kt + 1][2], h1[2 * kt + 1][3])};
      const int n = 8 * j + g;
      mma16816(c, a, sW2[n * (SG_H1 / 2) + 8 * kt + t], sW2[n * (SG_H1 / 2) + 8 * kt + 4 + t]);
    }
    const float bb0 = sb2[8 * j + 2 * t], bb1 = sb2[8 * j + 2 * t + 1];
    const float z[4] = {c[0] + bb0, c[1] + bb1, c[2] + bb0, c[3] + bb1};
    if (z2_out) {
      if (va) { z2_out[(size_t)ra * SG_H2 + 8 * j + 2 * t] = z[0]; z2_out[(size_t)ra * SG_H2 + 8 * j + 2 * t + 1] = z[1]; }
      if (vb) { z2_out[(size_t)rb * SG_H2 + 8 * j + 2 * t] = z[2]; z2_out[(size_t)rb * SG_H2 + 8 * j + 2 * t + 1] = z[3]; }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) h2[j][q] = silu32(z[q]);
  }
  // layer 3 (FP32): e = h2 . w3 + b3, reduced over the quad sharing a row
  float ea = 0.f, eb = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float w0 = sw3[8 * j + 2 * t], w1 = sw3[8 * j + 2 * t + 1];
    ea += h2[j][0] * w0 + h2[j][1] * w1;
    eb += h2[j][2] * w0 + h2[j][3] * w1;
  }
  ea += __shfl_xor_sync(0xffffffffu, ea, 1);
  ea += __shfl_xor_sync(0xffffffffu, ea, 2);
  eb += __shfl_xor_sync(0xffffffffu, eb, 1);
  eb += __shfl_xor_sync(0xffffffffu, eb, 2);
  if (t == 0) {
    if (va) e_out[ra] = ea + b3;
    if (vb) e_out[rb] = eb + b3;
  }
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

__global__ void refresh_bf16_kernel(const float* w, __nv_bfloat16* w1t, __nv_bfloat16* w2t) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < SG_RBF * SG_H1) {
    const int k = p / SG_H1, n = p % SG_H1;
    w1t[n * SG_RBF + k] = __float2bfloat16_rn(w[SG_OFF_W1 + p]);
  }
  if (p < SG_H1 * SG_H2) {
    const int k = p / SG_H2, n = p % SG_H2;
    w2t[n * SG_H1 + k] = __float2bfloat16_rn(w[SG_OFF_W2 + p]);
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

cudaError_t sg_forward(const __nv_bfloat16* gq, int rows, const SgWeights& w, float* e, float* z1,
                       float* z2, cudaStream_t st) {
  const int tiles = (rows + 15) / 16;
  dev::forward_kernel<<<(tiles + 3) / 4, 128, 0, st>>>(gq, rows, w, e, z1, z2);
  return cudaGetLastError();
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
  dev::refresh_bf16_kernel<<<(SG_H1 * SG_H2 + 127) / 128, 128, 0, st>>>(master, w.w1t, w.w2t);
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
