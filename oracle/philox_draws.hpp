// ORACLE / TEST INFRASTRUCTURE ONLY.  Nothing in the product path includes this file.
//
// Counter-based random draws shared (by specification, not by code) with the CUDA
// kernels in sad-monte-carlo_gb300/csrc/rng.cuh.  The reference draws from
// rand_xoshiro::Xoroshiro128Plus (src/rng.rs:27), a third-party crate (rand_xoshiro 0.4,
// rand 0.7, rand_distr 0.2; not vendored), so trajectory-level parity with the
// reference is impossible; the GPU and this oracle instead consume one common stream:
//
//   Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
//   1, 2, 3", SC 2011), key = {walker, seed_lo}, counter = {t_lo, t_hi, stream, seed_hi}.
//
// Per move t (the 1-based move counter after `moves += 1`, src/mc/energy.rs:905):
//   A = philox(t, stream 2*s),  B = philox(t, stream 2*s+1)   (s = 0 moves, 1 descent)
//   continuous systems: which = mulhi(A.x, N); (g0,g1) = normal_pair(A.y, A.z);
//                       (g2,-) = normal_pair(A.w, B.x); u = u53(B.y, B.z); B.w spare
//   Ising:             i = mulhi(A.x, L); j = mulhi(A.y, L); u = u53(A.z, A.w)
//
// The normal pair is Box-Muller evaluated in binary32 with only correctly rounded
// +,-,*,/,sqrt and a fixed operation order (series for ln and sin/cos written here
// from their Taylor/atanh expansions), so a compiler that does not contract a*b+c
// into an FMA (-ffp-contract=off here, __fmul_rn/__fadd_rn on the GPU) produces
// bit-identical draws on the CPU and the GPU.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

struct U4 { uint32_t x, y, z, w; };

inline void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

inline U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += W0; k1 += W1; }
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(M0, c.x, hi0, lo0);
    mulhilo32(M1, c.z, hi1, lo1);
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
  }
  return c;
}

inline float u_open01(uint32_t x) {  // (0,1), exact in binary32
  return ((float)(x >> 9) + 0.5f) * (1.0f / 8388608.0f);
}

inline float bits2f(uint32_t b) { float f; std::memcpy(&f, &b, 4); return f; }
inline uint32_t f2bits(float f) { uint32_t b; std::memcpy(&b, &f, 4); return b; }

// ln(x) for x in (0,1]: x = m 2^e, m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh(s), s=(m-1)/(m+1).
inline float ln_series(float x) {
  uint32_t b = f2bits(x);
  int e = (int)((b >> 23) & 0xffu) - 127;
  float m = bits2f((b & 0x7fffffu) | 0x3f800000u);
  if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float p = 1.0f / 11.0f;
  p = p * s2 + 1.0f / 9.0f;
  p = p * s2 + 1.0f / 7.0f;
  p = p * s2 + 1.0f / 5.0f;
  p = p * s2 + 1.0f / 3.0f;
  p = p * s2 + 1.0f;
  return (float)e * 0.693147182f + (s + s) * p;
}

// sin and cos of phi in [0, pi/2) by Taylor polynomials (Horner, fixed order).
inline void sincos_quarter(float phi, float& s, float& c) {
  float x2 = phi * phi;
  float ps = -1.0f / 39916800.0f;          // -1/11!
  ps = ps * x2 + 1.0f / 362880.0f;         //  1/9!
  ps = ps * x2 + -1.0f / 5040.0f;          // -1/7!
  ps = ps * x2 + 1.0f / 120.0f;            //  1/5!
  ps = ps * x2 + -1.0f / 6.0f;             // -1/3!
  ps = ps * x2 + 1.0f;
  s = phi * ps;
  float pc = 1.0f / 479001600.0f;          //  1/12!
  pc = pc * x2 + -1.0f / 3628800.0f;       // -1/10!
  pc = pc * x2 + 1.0f / 40320.0f;          //  1/8!
  pc = pc * x2 + -1.0f / 720.0f;           // -1/6!
  pc = pc * x2 + 1.0f / 24.0f;             //  1/4!
  pc = pc * x2 + -0.5f;
  pc = pc * x2 + 1.0f;
  c = pc;
}

// Box-Muller: two independent standard normals from two 32-bit words.
inline void normal_pair(uint32_t a, uint32_t b, float& z0, float& z1) {
  float u1 = u_open01(a);
  float u2 = u_open01(b);
  float r = std::sqrt(-2.0f * ln_series(u1));
  float q4 = u2 * 4.0f;              // exact
  int q = (int)q4;                   // quadrant 0..3
  float f = q4 - (float)q;           // exact, [0,1)
  float phi = f * 1.57079637f;
  float s, c;
  sincos_quarter(phi, s, c);
  float cs, sn;
  switch (q & 3) {
    case 0: cs = c; sn = s; break;
    case 1: cs = -s; sn = c; break;
    case 2: cs = -c; sn = -s; break;
    default: cs = s; sn = -c; break;
  }
  z0 = r * cs;
  z1 = r * sn;
}

inline double u53(uint32_t a, uint32_t b) {  // [0,1) with 53 random bits
  uint64_t v = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)v * (1.0 / 9007199254740992.0);
}

inline uint32_t mulhi_range(uint32_t x, uint32_t n) {
  return (uint32_t)(((uint64_t)x * (uint64_t)n) >> 32);
}

struct Draws {
  uint32_t which;   // atom index (continuous) or i (Ising)
  uint32_t j;       // Ising column
  float g[3];       // standard normals
  double u;         // uniform in [0,1) for the Metropolis test
};

// stream_pair: 0 for production moves, 1 for the initial descent (energy.rs:840-851)
inline Draws draws_continuous(uint64_t seed, uint32_t walker, uint64_t t, uint32_t n_atoms,
                              uint32_t stream_pair = 0) {
  uint32_t k0 = walker, k1 = (uint32_t)seed;
  uint32_t shi = (uint32_t)(seed >> 32);
  U4 A = philox4x32_10(U4{(uint32_t)t, (uint32_t)(t >> 32), 2u * stream_pair, shi}, k0, k1);
  U4 B = philox4x32_10(U4{(uint32_t)t, (uint32_t)(t >> 32), 2u * stream_pair + 1u, shi}, k0, k1);
  Draws d;
  d.which = mulhi_range(A.x, n_atoms);
  d.j = 0;
  float z3;
  normal_pair(A.y, A.z, d.g[0], d.g[1]);
  normal_pair(A.w, B.x, d.g[2], z3);
  (void)z3;
  d.u = u53(B.y, B.z);
  return d;
}

// stream_pair 0: moves; 1: the initial descent (counter word 2 = 2 * stream_pair).
inline Draws draws_ising(uint64_t seed, uint32_t walker, uint64_t t, uint32_t L,
                         uint32_t stream_pair = 0) {
  uint32_t k0 = walker, k1 = (uint32_t)seed;
  uint32_t shi = (uint32_t)(seed >> 32);
  U4 A = philox4x32_10(U4{(uint32_t)t, (uint32_t)(t >> 32), 2u * stream_pair, shi}, k0, k1);
  Draws d;
  d.which = mulhi_range(A.x, L);
  d.j = mulhi_range(A.y, L);
  d.g[0] = d.g[1] = d.g[2] = 0.0f;
  d.u = u53(A.z, A.w);
  return d;
}

}  // namespace orc
