// Counter-based per-walker random draws: Philox4x32-10 (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011) keyed by (walker, seed),
// with the move counter as the counter.  It replaces the reference's sequential
// rand_xoshiro::Xoroshiro128Plus stream (src/rng.rs:27) so that any lane can draw any
// move's numbers without carrying state.
//
// Draw layout per move t (1-based move counter):
//   A = philox({t_lo, t_hi, 2s, seed_hi}),  B = philox({t_lo, t_hi, 2s+1, seed_hi}),
//   key = {walker, seed_lo}, s = 0 for moves and 1 for the initial descent.
//   continuous: which = mulhi(A.x, N); normals (g0,g1) <- (A.y,A.z), g2 <- (A.w,B.x);
//               uniform u = 53 bits of (B.y, B.z)
//   Ising:      i = mulhi(A.x, L), j = mulhi(A.y, L), u = 53 bits of (A.z, A.w)
// Normals are Box-Muller evaluated with explicitly rounded binary32 operations
// (__fmul_rn etc., never contracted) and series for ln and sin/cos, so the stream is
// reproducible bit for bit by any IEEE binary32 implementation of the same steps.
#pragma once
#include <cstdint>

#include "sadmc_types.h"

namespace sadmc {
namespace dev {

struct Philox4 { uint32_t x, y, z, w; };

__device__ __forceinline__ Philox4 philox4x32_10(Philox4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += W0; k1 += W1; }
    uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = Philox4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
  }
  return c;
}

__device__ __forceinline__ float u_open01(uint32_t x) {
  return __fmul_rn(__fadd_rn(__uint2float_rn(x >> 9), 0.5f), 1.0f / 8388608.0f);
}

// ln(x), x in (0,1]: x = m 2^e with m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh(s).
__device__ __forceinline__ float ln_series(float x) {
  uint32_t b = __float_as_uint(x);
  int e = (int)((b >> 23) & 0xffu) - 127;
  float m = __uint_as_float((b & 0x7fffffu) | 0x3f800000u);
  if (m > 1.41421356f) { m = __fmul_rn(m, 0.5f); e += 1; }
  float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  float s2 = __fmul_rn(s, s);
  float p = 1.0f / 11.0f;
  p = __fadd_rn(__fmul_rn(p, s2), 1.0f / 9.0f);
  p = __fadd_rn(__fmul_rn(p, s2), 1.0f / 7.0f);
  p = __fadd_rn(__fmul_rn(p, s2), 1.0f / 5.0f);
  p = __fadd_rn(__fmul_rn(p, s2), 1.0f / 3.0f);
  p = __fadd_rn(__fmul_rn(p, s2), 1.0f);
  return __fadd_rn(__fmul_rn(__int2float_rn(e), 0.693147182f), __fmul_rn(__fadd_rn(s, s), p));
}

__device__ __forceinline__ void sincos_quarter(float phi, float& s, float& c) {
  float x2 = __fmul_rn(phi, phi);
  float ps = -1.0f / 39916800.0f;
  ps = __fadd_rn(__fmul_rn(ps, x2), 1.0f / 362880.0f);
  ps = __fadd_rn(__fmul_rn(ps, x2), -1.0f / 5040.0f);
  ps = __fadd_rn(__fmul_rn(ps, x2), 1.0f / 120.0f);
  ps = __fadd_rn(__fmul_rn(ps, x2), -1.0f / 6.0f);
  ps = __fadd_rn(__fmul_rn(ps, x2), 1.0f);
  s = __fmul_rn(phi, ps);
  float pc = 1.0f / 479001600.0f;
  pc = __fadd_rn(__fmul_rn(pc, x2), -1.0f / 3628800.0f);
  pc = __fadd_rn(__fmul_rn(pc, x2), 1.0f / 40320.0f);
  pc = __fadd_rn(__fmul_rn(pc, x2), -1.0f / 720.0f);
  pc = __fadd_rn(__fmul_rn(pc, x2), 1.0f / 24.0f);
  pc = __fadd_rn(__fmul_rn(pc, x2), -0.5f);
  pc = __fadd_rn(__fmul_rn(pc, x2), 1.0f);
  c = pc;
}

__device__ __forceinline__ void normal_pair(uint32_t a, uint32_t b, float& z0, float& z1) {
  float u1 = u_open01(a);
  float u2 = u_open01(b);
  float r = __fsqrt_rn(__fmul_rn(-2.0f, ln_series(u1)));
  float q4 = __fmul_rn(u2, 4.0f);
  int q = __float2int_rz(q4);
  float f = __fsub_rn(q4, __int2float_rn(q));
  float phi = __fmul_rn(f, 1.57079637f);
  float s, c;
  sincos_quarter(phi, s, c);
  float cs, sn;
  switch (q & 3) {
    case 0: cs = c; sn = s; break;
    case 1: cs = -s; sn = c; break;
    case 2: cs = -c; sn = -s; break;
    default: cs = s; sn = -c; break;
  }
  z0 = __fmul_rn(r, cs);
  z1 = __fmul_rn(r, sn);
}

// The uniform is carried as its 53-bit integer; u = v * 2^-53.
__device__ __forceinline__ uint64_t u53_bits(uint32_t a, uint32_t b) {
  return ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
}

__device__ __forceinline__ uint32_t mulhi_range(uint32_t x, uint32_t n) { return __umulhi(x, n); }

struct Draws {
  uint32_t which, j;
  float g0, g1, g2;
  uint64_t u53;
};

__device__ __forceinline__ Draws draws_continuous(uint64_t seed, uint32_t walker, uint64_t t,
                                                  uint32_t n_atoms, uint32_t stream_pair) {
  const uint32_t k0 = walker, k1 = (uint32_t)seed, shi = (uint32_t)(seed >> 32);
  Philox4 A = philox4x32_10(Philox4{(uint32_t)t, (uint32_t)(t >> 32), 2u * stream_pair, shi}, k0, k1);
  Philox4 B = philox4x32_10(Philox4{(uint32_t)t, (uint32_t)(t >> 32), 2u * stream_pair + 1u, shi}, k0, k1);
  Draws d;
  d.which = mulhi_range(A.x, n_atoms);
  d.j = 0;
  float z3;
  normal_pair(A.y, A.z, d.g0, d.g1);
  normal_pair(A.w, B.x, d.g2, z3);
  d.u53 = u53_bits(B.y, B.z);
  return d;
}

// stream_pair 0: moves; 1: the initial descent (counter word 2 = 2 * stream_pair).
__device__ __forceinline__ Draws draws_ising(uint64_t seed, uint32_t walker, uint64_t t, uint32_t L,
                                             uint32_t stream_pair = 0) {
  const uint32_t k0 = walker, k1 = (uint32_t)seed, shi = (uint32_t)(seed >> 32);
  Philox4 A = philox4x32_10(Philox4{(uint32_t)t, (uint32_t)(t >> 32), 2u * stream_pair, shi}, k0, k1);
  Draws d;
  d.which = mulhi_range(A.x, L);
  d.j = mulhi_range(A.y, L);
  d.g0 = d.g1 = d.g2 = 0.0f;
  d.u53 = u53_bits(A.z, A.w);
  return d;
}

// Draws of one energy-number move (src/mc/energy_number.rs:540-606), Philox stream pair 2
// (counter word 2 = 4, 5, 6): translate iff u_choice > addremove probability, add iff
// add_bit == 0, the atom to move or remove is mulhi_range(pick, N), three normals, and
// the Metropolis uniform.
struct GrandDraws {
  uint64_t u_choice53, u53;
  uint32_t add_bit, pick;
  float g0, g1, g2;
};
__device__ __forceinline__ GrandDraws draws_grand(uint64_t seed, uint32_t walker, uint64_t t) {
  const uint32_t k0 = walker, k1 = (uint32_t)seed, shi = (uint32_t)(seed >> 32);
  const Philox4 A = philox4x32_10(Philox4{(uint32_t)t, (uint32_t)(t >> 32), 4u, shi}, k0, k1);
  const Philox4 B = philox4x32_10(Philox4{(uint32_t)t, (uint32_t)(t >> 32), 5u, shi}, k0, k1);
  const Philox4 C = philox4x32_10(Philox4{(uint32_t)t, (uint32_t)(t >> 32), 6u, shi}, k0, k1);
  GrandDraws d;
  d.u_choice53 = u53_bits(A.x, A.y);
  d.add_bit = A.z & 1u;
  d.pick = A.w;
  float z3;
  normal_pair(B.x, B.y, d.g0, d.g1);
  normal_pair(B.z, B.w, d.g2, z3);
  (void)z3;
  d.u53 = u53_bits(C.x, C.y);
  return d;
}
// Candidate k of an LJ add, uniform in (-1, 1)^3 (lj.rs:294-302), counter word 2 = 8 + 2k
// and 9 + 2k.
__device__ __forceinline__ void add_candidate(uint64_t seed, uint32_t walker, uint64_t t, int k,
                                              double& x, double& y, double& z) {
  const uint32_t k0 = walker, k1 = (uint32_t)seed, shi = (uint32_t)(seed >> 32);
  const Philox4 D = philox4x32_10(Philox4{(uint32_t)t, (uint32_t)(t >> 32), 8u + 2u * (uint32_t)k, shi}, k0, k1);
  const Philox4 E = philox4x32_10(Philox4{(uint32_t)t, (uint32_t)(t >> 32), 9u + 2u * (uint32_t)k, shi}, k0, k1);
  const double s53 = 1.0 / 9007199254740992.0;
  x = -1.0 + 2.0 * ((double)u53_bits(D.x, D.y) * s53);
  y = -1.0 + 2.0 * ((double)u53_bits(D.z, D.w) * s53);
  z = -1.0 + 2.0 * ((double)u53_bits(E.x, E.y) * s53);
}

// Lane glane of a walker's group holds the draws of move base + glane; a move reads its
// draws with six group shuffles, so Philox and Box-Muller run once per LPW moves.
template <int LPW, bool ISING>
struct DrawCache {
  uint32_t off;  // calls since the batch was drawn (LPW: draw the next batch)
  Draws mine;
  __device__ void init() { off = LPW; }
  // called once per move with consecutive t
  __device__ Draws get(uint64_t seed, uint32_t walker, uint64_t t, uint32_t n, unsigned gmask,
                       int glane) {
    if (SADMC_RARE(off >= (uint32_t)LPW)) {
      off = 0;
      mine = ISING ? draws_ising(seed, walker, t + (uint64_t)glane, n)
                   : draws_continuous(seed, walker, t + (uint64_t)glane, n, 0u);
    }
    const int src = (int)off++;
    if (LPW == 1) return mine;
    Draws d;
    d.which = __shfl_sync(gmask, mine.which, src, LPW);
    d.j = ISING ? __shfl_sync(gmask, mine.j, src, LPW) : 0u;
    d.g0 = ISING ? 0.0f : __shfl_sync(gmask, mine.g0, src, LPW);
    d.g1 = ISING ? 0.0f : __shfl_sync(gmask, mine.g1, src, LPW);
    d.g2 = ISING ? 0.0f : __shfl_sync(gmask, mine.g2, src, LPW);
    d.u53 = __shfl_sync(gmask, mine.u53, src, LPW);
    return d;
  }
};

}  // namespace dev
}  // namespace sadmc
