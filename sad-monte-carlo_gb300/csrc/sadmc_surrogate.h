// Surrogate MLP layout and launchers (see sadmc_surrogate.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace sadmc {

constexpr int SG_RBF = 32, SG_H1 = 64, SG_H2 = 64;
// FP32 master parameters, one flat array: W1 [32][64], b1, W2 [64][64], b2, w3, b3
constexpr int SG_OFF_W1 = 0;
constexpr int SG_OFF_B1 = SG_OFF_W1 + SG_RBF * SG_H1;
constexpr int SG_OFF_W2 = SG_OFF_B1 + SG_H1;
constexpr int SG_OFF_B2 = SG_OFF_W2 + SG_H1 * SG_H2;
constexpr int SG_OFF_W3 = SG_OFF_B2 + SG_H2;
constexpr int SG_OFF_B3 = SG_OFF_W3 + SG_H2;
constexpr int SG_NPARAM = SG_OFF_B3 + 1;
constexpr int SG_WC_ELEMS = SG_H1 * SG_RBF + SG_H2 * SG_H1;

struct SgWeights {
  const float* w2;       // master W2 [k][n] (FP32)
  const float* b1;
  const float* b2;
  const float* w3;
  const float* b3;
  __nv_bfloat16* w1t;    // W1^T [n][k] bf16 (tensor-core B operand)
  __nv_bfloat16* w2t;    // W2^T [n][k] bf16
  // W1^T then W2^T in the tcgen05 shared-memory order (8-row x 16-byte core matrices,
  // K-major), SG_WC_ELEMS bf16: one bulk copy each lands them ready for the MMA
  __nv_bfloat16* wc;
  static SgWeights from(float* master, __nv_bfloat16* w1t, __nv_bfloat16* w2t,
                        __nv_bfloat16* wc) {
    return SgWeights{master + SG_OFF_W2, master + SG_OFF_B1, master + SG_OFF_B2,
                     master + SG_OFF_W3, master + SG_OFF_B3, w1t, w2t, wc};
  }
};

// Per-row scratch of a training step (rows = configurations * atoms).
struct SgScratch {
  __nv_bfloat16* gq;     // [rows][32]
  float* e;              // [rows]
  float* de;             // [rows]
  float* z1;             // [rows][64]
  float* z2;             // [rows][64]
  float* d1;             // [rows][64]
  float* d2;             // [rows][64]
  // bytes of scratch for `rows` rows
  static constexpr size_t bytes(size_t rows) {
    return rows * (SG_RBF * 2 + 4 + 4 + 4 * 4 * 64) + 6 * 256;
  }
  static SgScratch carve(void* base, size_t rows) {
    char* p = (char*)base;
    auto take = [&](size_t b) { char* q = p; p += (b + 255) / 256 * 256; return q; };
    SgScratch s;
    s.gq = (__nv_bfloat16*)take(rows * SG_RBF * 2);
    s.e = (float*)take(rows * 4);
    s.de = (float*)take(rows * 4);
    s.z1 = (float*)take(rows * 64 * 4);
    s.z2 = (float*)take(rows * 64 * 4);
    s.d1 = (float*)take(rows * 64 * 4);
    s.d2 = (float*)take(rows * 64 * 4);
    return s;
  }
};

// Rows (configurations x atoms) of the file-scope static scratch that serves callers
// which cannot allocate device memory (sadmc_surrogate_loss_grads_noalloc).
constexpr size_t SG_STATIC_ROWS = 4096;
// Device address of that static scratch on the current device.  The first call on a
// device resolves the symbol (cudaGetSymbolAddress, with the device current) and caches
// it; later calls on that device only read the cache.
cudaError_t sg_static_scratch(void** out);

cudaError_t sg_descriptors(const float* pos, int n, int rows, __nv_bfloat16* gq, float* gf,
                           cudaStream_t st);
cudaError_t sg_forward(const __nv_bfloat16* gq, int rows, const SgWeights& w, float* e, float* z1,
                       float* z2, cudaStream_t st);
// Tensor-core waits of sg_forward that ran out since the last call (then cleared);
// synchronizes st.
cudaError_t sg_forward_timeouts(unsigned int* count, cudaStream_t st);
// One training step on `configs` configurations of n atoms (positions [configs][n][3],
// binary32; target energies): loss into *loss_dev, gradients into grad; when step > 0
// an Adam step with that step number updates the master weights and their bf16 copies.
cudaError_t sg_train_step(const float* pos, const float* target, int configs, int n,
                          const SgWeights& w, float* master, float* grad, float* m, float* v,
                          int step, float lr, SgScratch s, double* loss_dev, cudaStream_t st);
cudaError_t sg_refresh(const float* master, const SgWeights& w, cudaStream_t st);
cudaError_t sg_collect(const float* lj_pos, int np, int n, const double* E, int walkers,
                       float* ring_pos, float* ring_e, int ring_cap, int ring_head,
                       cudaStream_t st);
cudaError_t sg_gather(const float* ring_pos, const float* ring_e, int n, const int* idx, int count,
                      float* out_pos, float* out_e, cudaStream_t st);

}  // namespace sadmc
