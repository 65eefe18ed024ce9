// LJ cluster in a spherical wall (src/system/lj.rs), many walkers per launch.
//
// Layout: a warp packs 32/LPW walkers; walker atom j lives in lane (j % LPW) of the
// walker's lane group, register slot j / LPW, as a double-single position (hi + lo,
// binary32).  Per move the group computes the reference's
//   e = E + sum_{j != which} [V(|r_j - to|^2) - V(|r_j - from|^2)]      (lj.rs:86-105)
// with binary32 pair terms on the hi parts and a group shuffle reduction, then runs the
// shared flat-histogram bookkeeping.  Every resum_interval moves the energy is replaced
// by an FP64 pair sum over the double-single positions (compute_energy, lj.rs:236-244);
// the largest observed |E_incremental - E_fp64| is kept in WalkerCore::drift.
#include <cuda_runtime.h>

#include "sadmc_common.cuh"
#include "sadmc_fh.cuh"
#include "sadmc_launch.h"
#include "sadmc_rng.cuh"
#include "sadmc_lj_walker.cuh"

namespace sadmc {
namespace dev {

template <int LPW, int APL>
__global__ void __launch_bounds__(128) lj_move_kernel(MoveLaunch m, LjSys s) {
  constexpr int WPW = 32 / LPW;
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (warp * WPW >= m.n_walkers) return;  // whole warp is padding (warp-uniform)
  const int group = lane / LPW, glane = lane % LPW;
  int w = warp * WPW + group;
  const bool wr = w < m.n_walkers;
  if (!wr) w = m.n_walkers - 1;
  const unsigned gmask = group_mask<LPW>(group);

  Fh<LPW> fh;
  fh.load(m.cores, m.P, m.B, w, gmask, glane, wr);
  LjWalker<LPW, APL> lj;
  lj.glane = glane;
  lj.gmask = gmask;
  lj.n = fh.c.n;
  float* pw = s.pos + (size_t)w * 6 * (size_t)s.np;
  lj.load(pw, s.np);

  if (m.descent) {
    // from_params descent (energy.rs:840-851): downhill-only proposals of rms 0.05 on
    // the descent stream until E < max_allowed_energy.
    const DS sc = ds_from_double(0.05);
    bool done = fh.c.pad1 != 0;  // finished in an earlier launch
    uint64_t steps = fh.c.pad2;
    for (uint64_t it = 0; it < m.n_moves; ++it) {
      if (__all_sync(0xffffffffu, done)) break;
      if (!done) {
        ++steps;
        Draws d = draws_continuous(m.seed, (uint32_t)w, steps, (uint32_t)lj.n, 1u);
        DS tx, ty, tz;
        float de;
        bool ok = lj.plan((int)d.which, d.g0, d.g1, d.g2, sc.h, sc.l, s.radius2, tx, ty, tz, de);
        const double e2 = fh.c.E + (double)de;
        if (ok && finite64(e2)) {
          if (e2 < fh.c.E) { lj.put((int)d.which, tx, ty, tz); fh.c.E = e2; }
          if (fh.c.E < m.descent_max) {
            // binary32 increments from overlapping starts drift; decide on the FP64 sum
            fh.c.E = lj.energy64();
            if (fh.c.E < m.descent_max) done = true;
          }
        }
        if (steps >= m.descent_limit) done = true;
      }
    }
    fh.c.pad2 = steps;
    fh.c.pad1 = done ? 1 : 0;
    double e64 = lj.energy64();
    fh.c.E = e64;
    if (!(e64 < m.descent_max)) fh.c.status |= ST_DESCENT_FAILED;
    else fh.c.status &= ~(uint32_t)ST_DESCENT_FAILED;
    lj.store(pw, s.np, wr);
    if (wr && glane == 0) m.cores[w] = fh.c;
    return;
  }

  RecentScale rsb;
  rsb.init();
  DrawCache<LPW, false> dc;
  dc.init();
  DS sc = ds_from_double(fh.c.tscale);
  for (uint64_t it = 0; it < m.n_moves; ++it) {
    const uint64_t t = fh.c.moves + 1;
    double rs, omrs;
    rsb.get(t, lane, rs, omrs);
    fh.begin_move(omrs);
    const Draws d = dc.get(m.seed, (uint32_t)w, t, (uint32_t)lj.n, gmask, glane);
    DS tx, ty, tz;
    float de = 0.0f;
    const bool possible = lj.plan((int)d.which, d.g0, d.g1, d.g2, sc.h, sc.l, s.radius2, tx, ty, tz, de);
    if (m.trace && wr && glane == 0 && t > m.trace_t0 && t - m.trace_t0 <= m.trace_cap) {
      TraceRec r;
      r.e1 = fh.c.E;
      r.e2 = possible ? fh.c.E + (double)de : __longlong_as_double(0x7ff8000000000000ll);
      m.trace[(size_t)w * m.trace_cap + (t - m.trace_t0 - 1)] = r;
    }
    const bool acc = fh.decide_de(possible, de, d.u53, rs);
    if (acc) lj.put((int)d.which, tx, ty, tz);
    fh.finish_move(acc);
    if (fh.tscale_changed) { fh.tscale_changed = false; sc = ds_from_double(fh.c.tscale); }
    if (m.resum_interval > 0 && (t % (uint64_t)m.resum_interval) == 0) {
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
  }
  lj.store(pw, s.np, wr);
  fh.store(m.cores, w);
}

template <int APL>
__global__ void lj_energy_kernel(const WalkerCore* cores, LjSys s, int n_walkers, double* out) {
  const int lane = threadIdx.x & 31;
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (w >= n_walkers) return;
  LjWalker<32, APL> lj;
  lj.glane = lane;
  lj.gmask = 0xffffffffu;
  lj.n = cores[w].n;
  lj.load(s.pos + (size_t)w * 6 * (size_t)s.np, s.np);
  double e = lj.energy64();
  if (lane == 0) out[w] = e;
}

template <int APL>
__global__ void lj_plan_kernel(WalkerCore* cores, LjSys s, int w, int which, float g0, float g1,
                               float g2, double scale, int confirm, double* out) {
  const int lane = threadIdx.x & 31;
  LjWalker<32, APL> lj;
  lj.glane = lane;
  lj.gmask = 0xffffffffu;
  lj.n = cores[w].n;
  float* pw = s.pos + (size_t)w * 6 * (size_t)s.np;
  lj.load(pw, s.np);
  const DS sc = ds_from_double(scale);
  DS tx, ty, tz;
  float de = 0.0f;
  bool ok = lj.plan(which, g0, g1, g2, sc.h, sc.l, s.radius2, tx, ty, tz, de);
  const double e2 = cores[w].E + (double)de;
  if (lane == 0) { out[0] = ok ? e2 : 0.0; out[1] = ok ? 1.0 : 0.0; }
  if (ok && confirm) {
    lj.put(which, tx, ty, tz);
    lj.store(pw, s.np, true);
    if (lane == 0) cores[w].E = e2;
  }
}

}  // namespace dev

#define SADMC_LJ_CASE(L, A)                                                            \
  if (lpw == L && s.np == L * A) {                                                     \
    const int wpb = m.warps_per_block >= 1 && m.warps_per_block <= 4 ? m.warps_per_block : 4; \
    const int warps = (m.n_walkers + (32 / L) - 1) / (32 / L);                         \
    dev::lj_move_kernel<L, A><<<(warps + wpb - 1) / wpb, 32 * wpb, 0, st>>>(m, s);     \
    return cudaGetLastError();                                                         \
  }

cudaError_t launch_lj_move(const MoveLaunch& m, const LjSys& s, int lpw, cudaStream_t st) {
  SADMC_LJ_CASE(32, 1) SADMC_LJ_CASE(16, 2) SADMC_LJ_CASE(8, 4) SADMC_LJ_CASE(4, 8)
  SADMC_LJ_CASE(32, 2) SADMC_LJ_CASE(16, 4) SADMC_LJ_CASE(8, 8)
  SADMC_LJ_CASE(32, 4) SADMC_LJ_CASE(32, 8)
  return cudaErrorInvalidConfiguration;
}

cudaError_t launch_lj_energy(const WalkerCore* cores, const LjSys& s, int n_walkers, double* out,
                             cudaStream_t st) {
  const int blocks = (n_walkers * 32 + 127) / 128;
  switch (s.np) {
    case 32: dev::lj_energy_kernel<1><<<blocks, 128, 0, st>>>(cores, s, n_walkers, out); break;
    case 64: dev::lj_energy_kernel<2><<<blocks, 128, 0, st>>>(cores, s, n_walkers, out); break;
    case 128: dev::lj_energy_kernel<4><<<blocks, 128, 0, st>>>(cores, s, n_walkers, out); break;
    case 256: dev::lj_energy_kernel<8><<<blocks, 128, 0, st>>>(cores, s, n_walkers, out); break;
    default: return cudaErrorInvalidConfiguration;
  }
  return cudaGetLastError();
}

cudaError_t launch_lj_plan(WalkerCore* cores, const LjSys& s, int walker, int which, float g0,
                           float g1, float g2, double scale, int confirm, double* out,
                           cudaStream_t st) {
  switch (s.np) {
    case 32: dev::lj_plan_kernel<1><<<1, 32, 0, st>>>(cores, s, walker, which, g0, g1, g2, scale, confirm, out); break;
    case 64: dev::lj_plan_kernel<2><<<1, 32, 0, st>>>(cores, s, walker, which, g0, g1, g2, scale, confirm, out); break;
    case 128: dev::lj_plan_kernel<4><<<1, 32, 0, st>>>(cores, s, walker, which, g0, g1, g2, scale, confirm, out); break;
    case 256: dev::lj_plan_kernel<8><<<1, 32, 0, st>>>(cores, s, walker, which, g0, g1, g2, scale, confirm, out); break;
    default: return cudaErrorInvalidConfiguration;
  }
  return cudaGetLastError();
}

}  // namespace sadmc
