// Small device helpers shared by the system kernels.
#pragma once
#include <cstdint>

#include "sadmc_types.h"

namespace sadmc {
namespace dev {

// Double-single number hi + lo (|lo| <= ulp(hi)/2), about 48 significant bits, kept with
// binary32 arithmetic only (FP64 issue slots are scarce on GB300).
struct DS { float h, l; };

__device__ __forceinline__ DS ds_add(DS a, DS b) {  // Knuth two-sum + renormalisation
  float s = __fadd_rn(a.h, b.h);
  float bb = __fsub_rn(s, a.h);
  float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  float h = __fadd_rn(s, e);
  return DS{h, __fsub_rn(e, __fsub_rn(h, s))};
}
// g * (sh + sl) with g a binary32 value
__device__ __forceinline__ DS ds_scale(float g, float sh, float sl) {
  float p = __fmul_rn(g, sh);
  float pe = __fmaf_rn(g, sh, -p);  // exact low part of g*sh
  pe = __fadd_rn(pe, __fmul_rn(g, sl));
  float h = __fadd_rn(p, pe);
  return DS{h, __fsub_rn(pe, __fsub_rn(h, p))};
}
__device__ __forceinline__ DS ds_from_double(double x) {
  float h = (float)x;
  return DS{h, (float)(x - (double)h)};
}
__device__ __forceinline__ double ds_to_double(DS a) { return (double)a.h + (double)a.l; }

__device__ __forceinline__ bool finite64(double x) {
  return (__double_as_longlong(x) & 0x7ff0000000000000ll) != 0x7ff0000000000000ll;
}

template <int LPW>
__device__ __forceinline__ unsigned group_mask(int group) {
  return LPW == 32 ? 0xffffffffu : (((1u << LPW) - 1u) << (group * LPW));
}

template <int LPW>
__device__ __forceinline__ float group_sum(float v, unsigned gmask) {
#pragma unroll
  for (int o = LPW / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gmask, v, o, LPW);
  return v;
}
template <int LPW>
__device__ __forceinline__ double group_sum(double v, unsigned gmask) {
#pragma unroll
  for (int o = LPW / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gmask, v, o, LPW);
  return v;
}
template <int LPW>
__device__ __forceinline__ int group_sum(int v, unsigned gmask) {
#pragma unroll
  for (int o = LPW / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gmask, v, o, LPW);
  return v;
}

// "t % period == 0" for the move counter t = moves + 1, moves + 2, ... of one launch, as a
// countdown: one 64-bit remainder per launch instead of one per move.  period 0: never.
struct Every {
  uint32_t left, period;
  __device__ void init(uint64_t moves, uint64_t period_) {
    period = (uint32_t)period_;
    left = period ? period - (uint32_t)(moves % period_) : 0u;
  }
  // call once per move, after the move counter advanced
  __device__ bool tick() {
    if (period == 0) return false;
    if (--left == 0) { left = period; return true; }
    return false;
  }
};

// Rust's powi(6) / powi(3) as LLVM expands them (x2 = x*x; x6 = (x2*x2)*x2; x3 = x*x2).
__device__ __forceinline__ double powi6(double x) { double x2 = x * x; return (x2 * x2) * x2; }
__device__ __forceinline__ double powi3(double x) { return x * (x * x); }

}  // namespace dev
}  // namespace sadmc
