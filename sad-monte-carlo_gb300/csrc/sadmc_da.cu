// Delayed-acceptance moves for LJ clusters (Christen & Fox, "Markov chain Monte Carlo
// using an approximation", J. Comput. Graph. Stat. 14, 2005), screened by the learned
// surrogate of sadmc_surrogate.cu.  One walker per warp, DA_WPB walkers per block sharing
// one shared-memory copy of the weights.
//
// Stage 1: the proposal of lj.rs:365-374 is screened with the surrogate energy
//   E~ = E + sum_i [e_s(G'_i) - e_s(G_i)], accepted with min(1, exp(ln w(E) - ln w(E~))).
//   The descriptors change incrementally: atom i != a gains phi(|r_i - to|) - phi(|r_i - from|),
//   the moved atom's row is rebuilt from the new distances; the MLP runs on all rows on the
//   tensor cores (mma.sync, 16-row tiles; SiLU in its tanh form).
// Stage 2: the exact binary32 pair energy e2 (as in lj_move_kernel) decides with the
//   Christen-Fox ratio min(1, [pi(y) a1(y,x)] / [pi(x) a1(x,y)]), where the reverse
//   screen a1(y,x) uses e2 - dS (the first stage's approximation depends on the state it
//   starts from), through the shared flat-histogram bookkeeping: the exact energy makes
//   every final decision and, for a fixed ln w, detailed balance holds.
// A stage-1 rejection is a rejected move (it is histogrammed like any other).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <atomic>

#include "sadmc_common.cuh"
#include "sadmc_fh.cuh"
#include "sadmc_launch.h"
#include "sadmc_lj_walker.cuh"
#include "sadmc_mma.cuh"
#include "sadmc_rng.cuh"
#include "sadmc_surrogate.h"

namespace sadmc {
namespace dev {

// Shared memory of a block: the weights once, then one region per walker.
constexpr int DA_WPB = 4;                                  // walkers (warps) per block
constexpr int DA_W_WORDS = SG_H1 * MLP_S1 + SG_H2 * MLP_S2 + 3 * SG_H1;  // mlp16's layout
// Per walker, for R descriptor rows (the atoms rounded up to 16, the MLP's row tile): two
// FP32 descriptor buffers, current and proposed, whose roles swap when a move is accepted
// (rows of 36 words: 16-byte aligned for float4, and 8 lanes on 8 rows of one float4 phase
// meet 32 different banks), the proposed bf16 copy (17 words a row) and two per-atom
// energy buffers.
constexpr int DA_GW = SG_RBF + 4;
constexpr int DA_BW = (SG_RBF + 2) / 2;  // bf16 descriptor row stride (words)
__host__ __device__ constexpr int da_rows(int n) { return (n + 15) & ~15; }
__host__ __device__ constexpr int da_walker_words(int R) { return R * (2 * DA_GW + (SG_RBF + 2) / 2 + 2); }
inline size_t da_smem_bytes(int R) {
  return 4 * ((size_t)DA_W_WORDS + (size_t)DA_WPB * (size_t)da_walker_words(R));
}

// 2^x on the special-function unit (ex2.approx.ftz.f32, relative error about 2^-22)
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Sum over the warp of v[l], left in lane l (a butterfly reduce-scatter: at each step a lane
// keeps the half of its vector its partner sends it and adds the partner's copy of it).
__device__ __forceinline__ float warp_reduce_scatter32(float (&v)[32], int lane) {
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool up = (lane & s) != 0;
#pragma unroll
    for (int j = 0; j < s; ++j) {
      const float send = up ? v[j] : v[j + s];
      const float keep = up ? v[j + s] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, s);
    }
  }
  return v[0];
}

// Stage-1 update of descriptor row i over columns [kb, kb + KPL): the proposed row, FP32 and
// bf16, from the current one plus the new-position minus the old-position RBF terms (ro, rn:
// the atom's old and new distances to the moved atom); the new-position terms are added to acc.
template <int KPL>
__device__ __forceinline__ void da_row_update(const float* sG, float* sGf, uint32_t* sGbw, int i, int kb,
                                              float ro, float rn, float l2w, float (&acc)[KPL]) {
  const float4* gsrc = reinterpret_cast<const float4*>(sG + i * DA_GW + kb);
  float4* gdst = reinterpret_cast<float4*>(sGf + i * DA_GW + kb);
#pragma unroll
  for (int k4 = 0; k4 < KPL / 4; ++k4) {
    const float4 g = gsrc[k4];
    float o[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float cn = rbf_centre(kb + 4 * k4 + u);
      const float pn = ex2_approx(-((rn - cn) * (rn - cn)) * l2w);
      const float po = ex2_approx(-((ro - cn) * (ro - cn)) * l2w);
      o[u] = (u == 0 ? g.x : u == 1 ? g.y : u == 2 ? g.z : g.w) + pn - po;
      acc[4 * k4 + u] += pn;
    }
    gdst[k4] = make_float4(o[0], o[1], o[2], o[3]);
    sGbw[i * DA_BW + kb / 2 + 2 * k4] = pack_bf16(o[0], o[1]);
    sGbw[i * DA_BW + kb / 2 + 2 * k4 + 1] = pack_bf16(o[2], o[3]);
  }
}

// Stage 1 for the second atom slot (atoms 32 ..) when it holds at most KPL atoms (KPL = 8:
// N <= 40): 32 / KPL lanes share a row, KPL columns each, so that a few atoms there do not
// leave most lanes idle.
// Adds the rows' new-position terms to col (column k of this lane's share).
template <int KPL, int APL>
__device__ __forceinline__ void da_slot1_packed(const LjWalker<32, APL>& lj, int lane, int n, int a,
                                                float fx, float fy, float fz, float tx, float ty,
                                                float tz, const float* sG, float* sGf, uint32_t* sGbw,
                                                float l2w, float (&col)[SG_RBF]) {
  constexpr int P = SG_RBF / KPL;  // lanes per row
  const int slot = lane / P, part = lane % P;
  const float xi = __shfl_sync(0xffffffffu, lj.x[APL - 1].h, slot);
  const float yi = __shfl_sync(0xffffffffu, lj.y[APL - 1].h, slot);
  const float zi = __shfl_sync(0xffffffffu, lj.z[APL - 1].h, slot);
  const int i = 32 + slot;
  if (i < n && i != a) {
    float dx = xi - fx, dy = yi - fy, dz = zi - fz;
    const float ro = sqrtf(dx * dx + dy * dy + dz * dz);
    dx = xi - tx; dy = yi - ty; dz = zi - tz;
    const float rn = sqrtf(dx * dx + dy * dy + dz * dz);
    float pk[KPL];
#pragma unroll
    for (int j = 0; j < KPL; ++j) pk[j] = 0.f;
    da_row_update<KPL>(sG, sGf, sGbw, i, part * KPL, ro, rn, l2w, pk);
#pragma unroll
    for (int b = 0; b < P; ++b)
      if (part == b) {
#pragma unroll
        for (int j = 0; j < KPL; ++j) col[b * KPL + j] += pk[j];
      }
  }
}

template <int APL>
__global__ void __launch_bounds__(32 * DA_WPB) lj_da_kernel(MoveLaunch m, LjSys s, SgWeights wts, int R,
                                                             int refresh_interval, uint64_t* stats) {
  constexpr int GW = DA_GW;             // FP32 descriptor row stride (words)
  constexpr int BW = (SG_RBF + 2) / 2;  // bf16 descriptor row stride (words)
  extern __shared__ __align__(16) uint32_t da_smem[];
  uint32_t* sW1 = da_smem;
  uint32_t* sW2 = sW1 + SG_H1 * MLP_S1;
  float* sb1 = reinterpret_cast<float*>(sW2 + SG_H2 * MLP_S2);
  float* sb2 = sb1 + SG_H1;
  float* sw3 = sb2 + SG_H2;
  for (int k = threadIdx.x; k < SG_H1 * SG_RBF / 2; k += blockDim.x)
    sW1[mlp_wword(k / (SG_RBF / 2), k % (SG_RBF / 2), MLP_S1)] = reinterpret_cast<const uint32_t*>(wts.w1t)[k];
  for (int k = threadIdx.x; k < SG_H2 * SG_H1 / 2; k += blockDim.x)
    sW2[mlp_wword(k / (SG_H1 / 2), k % (SG_H1 / 2), MLP_S2)] = reinterpret_cast<const uint32_t*>(wts.w2t)[k];
  for (int k = threadIdx.x; k < SG_H1; k += blockDim.x) { sb1[k] = wts.b1[k]; sb2[k] = wts.b2[k]; sw3[k] = wts.w3[k]; }
  __syncthreads();
  const float b3 = wts.b3[0];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int w = blockIdx.x * DA_WPB + wib;
  if (w >= m.n_walkers) return;
  Fh<32> fh;
  fh.load(m.cores, m.P, m.B, w, 0xffffffffu, lane, true);
  LjWalker<32, APL> lj;
  lj.set_radius2(s.radius2);
  lj.glane = lane;
  lj.gmask = 0xffffffffu;
  lj.n = fh.c.n;
  const int n = lj.n;  // <= R, the rows every walker region of the launch holds
  float* sG = reinterpret_cast<float*>(da_smem + DA_W_WORDS + (size_t)wib * da_walker_words(R));
  float* sGf = sG + R * GW;  // sG: current descriptors, sGf: proposed (swapped on acceptance)
  uint32_t* sGbw = reinterpret_cast<uint32_t*>(sGf + R * GW);
  __nv_bfloat16* sGb = reinterpret_cast<__nv_bfloat16*>(sGbw);
  float* sE = reinterpret_cast<float*>(sGbw + R * BW);
  float* sEn = sE + R;       // sE: current per-atom energies, sEn: proposed (swapped too)
  float* pw = s.pos + (size_t)w * 6 * (size_t)s.np;
  lj.load(pw, s.np);
  const float inv2w2 = 1.0f / (2.0f * 0.1f * 0.1f);
  const float l2w = inv2w2 * 1.4426950408889634f;  // the same Gaussian in base 2
  // high parts of the position of this lane's atom slot q (a runtime q without indexing the
  // register arrays)
  auto hi_of = [&](int q, float& xi, float& yi, float& zi) {
    xi = lj.x[0].h; yi = lj.y[0].h; zi = lj.z[0].h;
#pragma unroll
    for (int k = 1; k < APL; ++k)
      if (q == k) { xi = lj.x[k].h; yi = lj.y[k].h; zi = lj.z[k].h; }
  };

  // surrogate energies of all rows from sGb -> dst
  auto forward_rows = [&](float* dst) {
    for (int r0 = 0; r0 < n; r0 += 16) {
      float ea, eb;
      mlp16<BW>(sGbw + r0 * BW, reinterpret_cast<const uint2*>(sW1), reinterpret_cast<const uint2*>(sW2),
                reinterpret_cast<const float2*>(sb1), reinterpret_cast<const float2*>(sb2),
                reinterpret_cast<const float2*>(sw3), b3, ea, eb);
      const int g = lane >> 2;
      if ((lane & 3) == 0) {
        dst[r0 + g] = ea;
        dst[r0 + g + 8] = eb;
      }
    }
    __syncwarp();
  };
  // full descriptors of the current configuration, their bf16 copy and energies (rows
  // n..R-1 hold zeros)
  auto refresh = [&]() {
    for (int q = 0; q < APL; ++q) {
      float gacc[SG_RBF];
#pragma unroll
      for (int k = 0; k < SG_RBF; ++k) gacc[k] = 0.f;
      const int i = lane + 32 * q;
      const float xi = lj.x[q].h, yi = lj.y[q].h, zi = lj.z[q].h;
      for (int j = 0; j < n; ++j) {
        DS a, b, c;
        lj.fetch(j, a, b, c);
        if (i < n && j != i) {
          const float dx = a.h - xi, dy = b.h - yi, dz = c.h - zi;
          const float r = sqrtf(dx * dx + dy * dy + dz * dz);
#pragma unroll
          for (int k = 0; k < SG_RBF; ++k) {
            const float d = r - rbf_centre(k);
            gacc[k] += __expf(-d * d * inv2w2);
          }
        }
      }
      if (i < R) {
#pragma unroll
        for (int k = 0; k < SG_RBF; ++k) {
          sG[i * GW + k] = i < n ? gacc[k] : 0.f;
          sGb[i * 2 * BW + k] = __float2bfloat16_rn(i < n ? gacc[k] : 0.f);
        }
      }
    }
    __syncwarp();
    forward_rows(sE);
  };
  refresh();

  RecentScale rsb;
  rsb.init();
  DrawCache<32, false> dc;
  dc.init();
  DS sc = ds_from_double(fh.c.tscale);
  uint64_t screened_out = 0, exact_evals = 0;
  Every resum, refresh_every;
  resum.init(fh.c.moves, m.resum_interval > 0 ? (uint64_t)m.resum_interval : 0);
  refresh_every.init(fh.c.moves, refresh_interval > 0 ? (uint64_t)refresh_interval : 0);
  for (uint64_t it = 0; it < m.n_moves; ++it) {
    const uint64_t t = fh.c.moves + 1;
    double rs, omrs;
    rsb.get(t, lane, rs, omrs);
    fh.begin_move(omrs);
    const Draws d = dc.get(m.seed, (uint32_t)w, t, (uint32_t)n, 0xffffffffu, lane);
    // second-stage uniform: its own Philox stream (counter word 2 = 4)
    const Philox4 U = philox4x32_10(Philox4{(uint32_t)t, (uint32_t)(t >> 32), 4u, (uint32_t)(m.seed >> 32)},
                                    (uint32_t)w, (uint32_t)m.seed);
    const uint64_t u2 = u53_bits(U.x, U.y);
    const int a = (int)d.which;
    DS fx, fy, fz;
    lj.fetch(a, fx, fy, fz);
    const DS tx = ds_add(fx, ds_scale(d.g0, sc.h, sc.l));
    const DS ty = ds_add(fy, ds_scale(d.g1, sc.h, sc.l));
    const DS tz = ds_add(fz, ds_scale(d.g2, sc.h, sc.l));
    // ---- stage 1: surrogate screen ----
    float part = 0.f;
    float col[SG_RBF];  // this lane's atoms' contributions to the moved atom's row
#pragma unroll
    for (int k = 0; k < SG_RBF; ++k) col[k] = 0.f;
    // a lane per row for slot 0, and for slot 1 when it holds more than 8 atoms
    const int m1 = n - 32;  // atoms in slot 1
    const int full_slots = (APL > 1 && m1 > 8) ? 2 : 1;
#pragma unroll 1
    for (int q = 0; q < full_slots; ++q) {
      const int i = lane + 32 * q;
      if (i < n && i != a) {
        float xi, yi, zi;
        hi_of(q, xi, yi, zi);
        float dx = xi - fx.h, dy = yi - fy.h, dz = zi - fz.h;
        const float ro = sqrtf(dx * dx + dy * dy + dz * dz);
        dx = xi - tx.h; dy = yi - ty.h; dz = zi - tz.h;
        const float rn = sqrtf(dx * dx + dy * dy + dz * dz);
        da_row_update<SG_RBF>(sG, sGf, sGbw, i, 0, ro, rn, l2w, col);
      }
    }
    if (APL > 1 && m1 > 0 && m1 <= 8)  // group-uniform: n is the walker's
      da_slot1_packed<8, APL>(lj, lane, n, a, fx.h, fy.h, fz.h, tx.h, ty.h, tz.h, sG, sGf, sGbw, l2w, col);
    // moved atom's row: lane k takes column k of the contributions
    const float ga = warp_reduce_scatter32(col, lane);
    sGf[a * GW + lane] = ga;
    sGb[a * 2 * BW + lane] = __float2bfloat16_rn(ga);
    __syncwarp();
    forward_rows(sEn);
    for (int q = 0; q < APL; ++q) {
      const int i = lane + 32 * q;
      if (i < n) part += sEn[i] - sE[i];
    }
    const float des = group_sum<32>(part, 0xffffffffu);
    const double e1 = fh.c.E;
    const double e_til = e1 + (double)des;
    if (m.trace && lane == 0 && t > m.trace_t0 && t - m.trace_t0 <= m.trace_cap) {
      // (E before, proposed E: NaN when screened out or impossible) and dS
      const size_t k = (size_t)w * m.trace_cap + (t - m.trace_t0 - 1);
      m.trace[k] = TraceRec{e1, __longlong_as_double(0x7ff8000000000000ll)};
      if (m.trace_ds) m.trace_ds[k] = des;
    }
    const double lnw_cur = fh.lnw_current();
    const double lnw_til = fh.lnw_at(e_til);
    const bool uphill1 = dgt(lnw_til, lnw_cur);
    const bool rej1 = fh.uni(uphill1 && metropolis_reject(lnw_cur - lnw_til, d.u53));
    // a certain stage-1 acceptance consumed no randomness: stage 2 may use the move's own
    // uniform (with a constant surrogate the chain is then the plain chain, bit for bit)
    const uint64_t u_second = uphill1 ? u2 : d.u53;
    bool acc = false;
    if (rej1) {
      ++screened_out;
    } else {
      // ---- stage 2: exact energy ----
      ++exact_evals;
      DS ux, uy, uz;
      float de = 0.f;
      const bool possible = lj.plan(a, d.g0, d.g1, d.g2, sc.h, sc.l, s.radius2, ux, uy, uz, de);
      // Christen-Fox second stage for a state-dependent first stage: accept with
      // min(1, [pi(y) a1(y,x)] / [pi(x) a1(x,y)]), pi = exp(-ln w(E)), where the first stage
      // from x used E~ = E + dS and the reverse one from y would use e2 - dS:
      //   ln a1(x,y) = min(0, ln w(E) - ln w(E~)),  ln a1(y,x) = min(0, ln w(e2) - ln w(e2 - dS)).
      // decide_de accepts with min(1, exp(lnw_first - ln w(e2))), so
      //   lnw_first = ln w(E) - ln a1(x,y) + ln a1(y,x).
      // (A constant surrogate, dS = 0, gives ln w(E): the plain chain.)
      double lnw_first = lnw_cur;
      if (possible && fabsf(de) <= 3.0e38f) {
        const double e2x = fh.c.E + (double)de;
        const double back = fh.lnw_at(e2x) - fh.lnw_at(e2x - (double)des);
        lnw_first = lnw_cur - (uphill1 ? lnw_cur - lnw_til : 0.0) + (back < 0.0 ? back : 0.0);
      }
      if (m.trace && lane == 0 && t > m.trace_t0 && t - m.trace_t0 <= m.trace_cap)
        m.trace[(size_t)w * m.trace_cap + (t - m.trace_t0 - 1)].e2 =
            possible ? e1 + (double)de : __longlong_as_double(0x7ff8000000000000ll);
      acc = fh.decide_de(possible, de, u_second, rs, true, lnw_first);
      if (acc) {
        lj.put(a, tx, ty, tz);
        // every row < n of the proposed buffers was rewritten by this move: they become
        // the current ones
        float* t0 = sG; sG = sGf; sGf = t0;
        float* t1 = sE; sE = sEn; sEn = t1;
      }
    }
    fh.finish_move(acc);
    if (fh.tscale_changed) { fh.tscale_changed = false; sc = ds_from_double(fh.c.tscale); }
    if (resum.tick()) {
      const double e64 = lj.energy64();
      const double dr = fabs(e64 - fh.c.E);
      if (dr > fh.c.drift) fh.c.drift = dr;
      if (dr > m.drift_tol) fh.c.status |= ST_DRIFT;
      fh.set_E(e64);
      fh.grew_front = false;
      if (!fh.prepare(e64)) fh.c.status |= ST_BIN_RANGE;
      else {
        if (fh.grew_front) fh.reindex_after_growth();
        fh.move_cur(fh.gidx(e64));
      }
    }
    if (refresh_every.tick()) refresh();
  }
  lj.store(pw, s.np, true);
  fh.store(m.cores, w);
  if (stats && lane == 0) {
    stats[2 * w] += screened_out;
    stats[2 * w + 1] += exact_evals;
  }
}

}  // namespace dev

cudaError_t launch_lj_da(const MoveLaunch& m, const LjSys& s, const SgWeights& w, int max_atoms,
                         int refresh_interval, uint64_t* stats, cudaStream_t st) {
  if ((s.np != 32 && s.np != 64) || max_atoms < 2 || max_atoms > s.np) return cudaErrorInvalidConfiguration;
  const int R = dev::da_rows(max_atoms);
  // The limit (for R = np) is set once per device and shape.  Host threads launching on
  // one device may race to set it; setting it twice is harmless, and the flags are atomic.
  static std::atomic<bool> attr[64][2] = {};
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return e;
  const int shape = s.np == 32 ? 0 : 1;
  if (device < 0 || device >= 64 || !attr[device][shape].load(std::memory_order_acquire)) {
    const int lim = (int)dev::da_smem_bytes(s.np);
    e = shape == 0 ? cudaFuncSetAttribute(dev::lj_da_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim)
                   : cudaFuncSetAttribute(dev::lj_da_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (e != cudaSuccess) return e;
    if (device >= 0 && device < 64) attr[device][shape].store(true, std::memory_order_release);
  }
  const size_t bytes = dev::da_smem_bytes(R);
  const int blocks = (m.n_walkers + dev::DA_WPB - 1) / dev::DA_WPB;
  if (shape == 0) dev::lj_da_kernel<1><<<blocks, 32 * dev::DA_WPB, bytes, st>>>(m, s, w, R, refresh_interval, stats);
  else dev::lj_da_kernel<2><<<blocks, 32 * dev::DA_WPB, bytes, st>>>(m, s, w, R, refresh_interval, stats);
  return cudaGetLastError();
}

}  // namespace sadmc
