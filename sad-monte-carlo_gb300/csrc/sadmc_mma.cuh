// Device helpers of the surrogate MLP: RBF centres, SiLU, bf16 packing and the
// mma.sync m16n8k16 bf16 tensor-core instruction (FP32 accumulation).
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace sadmc {
namespace dev {

__device__ __forceinline__ float rbf_centre(int k) { return 0.8f + (2.2f / 31.0f) * (float)k; }

// SiLU z / (1 + e^-z) for the batched forward and the training kernels, with the hardware
// reciprocal (__fdividef, a few ulp; 0 once the denominator passes 2^126, the SiLU's
// limit for large negative z) in place of an IEEE division: the kernels evaluate a few
// hundred SiLUs per thread in unrolled code, and the IEEE sequence's length made their
// instruction fetch the limiter.  The error is far below the BF16 rounding of the
// activations.
__device__ __forceinline__ float silu32(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
// SiLU as z/2 (1 + tanh(z/2)) on the hardware tanh (tanh.approx.f32, absolute error about
// 2^-11): one special-function operation and an FMA in place of an exponential and an
// IEEE division.  Used by the delayed-acceptance screen only, whose value decides no
// move by itself (the exact energy makes every final decision).
__device__ __forceinline__ float silu_fast(float z) {
  const float h = 0.5f * z;
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(h));
  return __fmaf_rn(h, t, h);
}
__device__ __forceinline__ float dsilu32(float z) {  // SiLU'(z), reciprocal as in silu32
  const float s = __fdividef(1.0f, 1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// D = A * B + C, m16n8k16, bf16 x bf16 -> f32
__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

}  // namespace dev
}  // namespace sadmc

namespace sadmc {
namespace dev {

// Weight layout of mlp16 in shared memory: for output unit n, the two 32-bit words a lane t
// of its quad passes to one m16n8k16 as B (K = 16 kt + 2t, 2t + 1 and 16 kt + 8 + 2t, +1) sit
// side by side, so one 64-bit load fetches them.  Units are MLP_S1 (layer 1) and MLP_S2
// (layer 2) words apart: the 8 units g of a load meet 32 different banks.
constexpr int MLP_S1 = 24, MLP_S2 = 40;
// Word index in that layout of word w (0 .. K/2 - 1) of unit n's row-major bf16 weights.
__host__ __device__ constexpr int mlp_wword(int n, int w, int stride) {
  return n * stride + (w >> 3) * 8 + 2 * (w & 3) + ((w >> 2) & 1);
}

// Surrogate energies of 16 rows (one warp): A fragments of G from a row-major bf16 tile
// in shared memory (32 bf16 = 16 words per row), weights in the mlp_wword layout and biases
// as float pairs in shared memory, SiLU in its tanh form (silu_fast).  Rows g and g+8 of
// the tile end in ea / eb (in the quad's lane t == 0 and the others alike).
template <int RW>  // 32-bit words between consecutive rows of the tile
__device__ __forceinline__ void mlp16(const uint32_t* gtile, const uint2* sW1, const uint2* sW2,
                                      const float2* sb1, const float2* sb2, const float2* sw3,
                                      float b3, float& ea, float& eb) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  uint32_t aG[2][4];
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) {
    aG[kt][0] = gtile[g * RW + 8 * kt + t];
    aG[kt][1] = gtile[(g + 8) * RW + 8 * kt + t];
    aG[kt][2] = gtile[g * RW + 8 * kt + 4 + t];
    aG[kt][3] = gtile[(g + 8) * RW + 8 * kt + 4 + t];
  }
  float h1[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    const int n = 8 * j + g;
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
      const uint2 b = sW1[(n * MLP_S1 + 8 * kt + 2 * t) >> 1];
      mma16816(c, aG[kt], b.x, b.y);
    }
    const float2 bb = sb1[4 * j + t];
    h1[j][0] = silu_fast(c[0] + bb.x); h1[j][1] = silu_fast(c[1] + bb.y);
    h1[j][2] = silu_fast(c[2] + bb.x); h1[j][3] = silu_fast(c[3] + bb.y);
  }
  ea = 0.f;
  eb = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    const int n = 8 * j + g;
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      const uint32_t a[4] = {pack_bf16(h1[2 * kt][0], h1[2 * kt][1]), pack_bf16(h1[2 * kt][2], h1[2 * kt][3]),
                             pack_bf16(h1[2 * kt + 1][0], h1[2 * kt + 1][1]),
                             pack_bf16(h1[2 * kt + 1][2], h1[2 * kt + 1][3])};
      const uint2 b = sW2[(n * MLP_S2 + 8 * kt + 2 * t) >> 1];
      mma16816(c, a, b.x, b.y);
    }
    const float2 bb = sb2[4 * j + t];
    const float2 ww = sw3[4 * j + t];
    ea = __fmaf_rn(silu_fast(c[0] + bb.x), ww.x, ea);
    ea = __fmaf_rn(silu_fast(c[1] + bb.y), ww.y, ea);
    eb = __fmaf_rn(silu_fast(c[2] + bb.x), ww.x, eb);
    eb = __fmaf_rn(silu_fast(c[3] + bb.y), ww.y, eb);
  }
  ea += __shfl_xor_sync(0xffffffffu, ea, 1);
  ea += __shfl_xor_sync(0xffffffffu, ea, 2);
  eb += __shfl_xor_sync(0xffffffffu, eb, 1);
  eb += __shfl_xor_sync(0xffffffffu, eb, 2);
  ea += b3;
  eb += b3;
}

}  // namespace dev
}  // namespace sadmc
