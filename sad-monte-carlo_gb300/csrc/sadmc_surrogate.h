// Surrogate MLP layout and launchers (see sadmc_surrogate.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace sadmc {

struct WalkerCore;

constexpr int SG_RBF = 32, SG_H1 = 64, SG_H2 = 64;
// FP32 master parameters, one flat array: W1 [32][64], b1, W2 [64][64], b2, w3, b3
constexpr int SG_OFF_W1 = 0;
constexpr int SG_OFF_B1 = SG_OFF_W1 + SG_RBF * SG_H1;
constexpr int SG_OFF_W2 = SG_OFF_B1 + SG_H1;
constexpr int SG_OFF_B2 = SG_OFF_W2 + SG_H1 * SG_H2;
constexpr int SG_OFF_W3 = SG_OFF_B2 + SG_H2;
constexpr int SG_OFF_B3 = SG_OFF_W3 + SG_H2;
constexpr int SG_NPARAM = SG_OFF_B3 + 1;
// bf16 copies in tcgen05 shared-memory order (8-row x 16-byte core matrices, K-major):
// W1^T [64][32] and W2^T [64][64] (the forward's B operands), then W2 [64][64] (the B
// operand of the backward's d1 = d2 W2^T)
constexpr int SG_WC_W1T = 0;
constexpr int SG_WC_W2T = SG_WC_W1T + SG_H1 * SG_RBF;
constexpr int SG_WC_W2 = SG_WC_W2T + SG_H2 * SG_H1;
constexpr int SG_WC_ELEMS = SG_WC_W2 + SG_H1 * SG_H2;
// Rows of one tensor-core tile; a training tile holds whole configurations (at most 128
// atoms each), floor(128 / n) of them.
constexpr int SG_TILE = 128;
constexpr int SG_MAX_ATOMS = SG_TILE;

struct SgWeights {
  const float* b1;
  const float* b2;
  const float* w3;
  const float* b3;
  __nv_bfloat16* w1t;    // W1^T [n][k] bf16 (the delayed-acceptance kernel's mma.sync B)
  __nv_bfloat16* w2t;    // W2^T [n][k] bf16
  __nv_bfloat16* wc;     // SG_WC_ELEMS bf16 in tcgen05 order (one bulk copy per matrix)
  static SgWeights from(float* master, __nv_bfloat16* w1t, __nv_bfloat16* w2t,
                        __nv_bfloat16* wc) {
    return SgWeights{master + SG_OFF_B1, master + SG_OFF_B2, master + SG_OFF_W3,
                     master + SG_OFF_B3, w1t, w2t, wc};
  }
};

// Training tiles of `configs` configurations of n atoms (n <= SG_MAX_ATOMS).
__host__ __device__ constexpr int sg_configs_per_tile(int n) { return SG_TILE / n; }
__host__ __device__ constexpr int sg_tiles(int configs, int n) {
  return (configs + sg_configs_per_tile(n) - 1) / sg_configs_per_tile(n);
}
// Upper bound of sg_tiles over n for configs * n <= rows: floor(128 / n) >= 64 / n.
__host__ __device__ constexpr size_t sg_max_tiles(size_t rows) { return rows / 64 + 1; }

// Scratch of a training step or a batched forward (rows = configurations * atoms).
struct SgScratch {
  __nv_bfloat16* gq;     // [rows][32] descriptors (the forward's A operand)
  float* e;              // [rows] per-atom energies (batched forward)
  float* part;           // [tiles][SG_NPARAM] per-tile gradient sums
  double* lpart;         // [tiles] per-tile loss sums
  static constexpr size_t round(size_t b) { return (b + 255) / 256 * 256; }
  static constexpr size_t bytes(size_t rows) {
    return round(rows * SG_RBF * 2) + round(rows * 4) +
           round(sg_max_tiles(rows) * SG_NPARAM * 4) + round(sg_max_tiles(rows) * 8);
  }
  static SgScratch carve(void* base, size_t rows) {
    char* p = (char*)base;
    auto take = [&](size_t b) { char* q = p; p += round(b); return q; };
    SgScratch s;
    s.gq = (__nv_bfloat16*)take(rows * SG_RBF * 2);
    s.e = (float*)take(rows * 4);
    s.part = (float*)take(sg_max_tiles(rows) * SG_NPARAM * 4);
    s.lpart = (double*)take(sg_max_tiles(rows) * 8);
    return s;
  }
};

// Adam state of the optimizer step folded into the gradient reduction.
struct SgAdam {
  float* master;  // FP32 parameters (updated in place)
  float* m;
  float* v;
  int step;       // Adam step number (>= 1); 0: gradients only, nothing updated
  float lr;
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
// Batched forward on the tensor cores: per-row energies.  A tensor-core wait that runs
// out writes NaN energies and, when timeout is not null, sets *timeout.
cudaError_t sg_forward(const __nv_bfloat16* gq, int rows, const SgWeights& w, float* e,
                       unsigned int* timeout, cudaStream_t st);
// Device address of the shared timeout flag of the allocating entry points.
cudaError_t sg_timeout_flag(unsigned int** flag);
// Read and clear *flag in one device atomic (into *out, a device word), stream-ordered.
cudaError_t sg_take_flag(unsigned int* flag, unsigned int* out, cudaStream_t st);
// One training step on `configs` configurations of n atoms (positions [configs][n][3],
// binary32; target energies): descriptors, the fused tensor-core forward and backward
// per tile of whole configurations, then the gradient reduction over tiles into grad
// and the loss (mean squared configuration-energy error) into *loss_dev; with
// adam.step > 0 the same kernel takes the Adam step and refreshes the bf16 copies.
// Deterministic: the tiles are summed in a fixed order.
cudaError_t sg_train_step(const float* pos, const float* target, int configs, int n,
                          const SgWeights& w, float* grad, const SgAdam& adam, SgScratch s,
                          double* loss_dev, unsigned int* timeout, cudaStream_t st);
cudaError_t sg_refresh(const float* master, const SgWeights& w, cudaStream_t st);
// Copy every walker's configuration (LJ double-single planes) and its energy (read from
// the walker state on the device) into the training ring at ring_head.
cudaError_t sg_collect(const float* lj_pos, int np, int n, const WalkerCore* cores, int walkers,
                       float* ring_pos, float* ring_e, int ring_cap, int ring_head,
                       cudaStream_t st);
// Minibatch of `count` ring entries drawn uniformly from the first ring_count with a
// counter-based hash of (seed, step, index).
cudaError_t sg_gather(const float* ring_pos, const float* ring_e, int n, int ring_count,
                      uint64_t seed, uint64_t step, int count, float* out_pos, float* out_e,
                      cudaStream_t st);
// Shared memory the fused training kernel asks for (set once per device).
cudaError_t sg_prepare_train(void);

}  // namespace sadmc
