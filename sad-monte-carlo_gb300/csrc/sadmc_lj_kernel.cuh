// The LJ-cluster move kernel (src/system/lj.rs), many walkers per launch; included by
// the translation units that instantiate it (sadmc_lj.cu: any method; sadmc_lj_sad.cu:
// specialised for SAD).
//
// Layout: a warp packs 32/LPW walkers; walker atom j lives in lane (j % LPW) of the
// walker's lane group, register slot j / LPW, as a double-single position (hi + lo,
// binary32).  Per move the group computes the reference's
//   e = E + sum_{j != which} [V(|r_j - to|^2) - V(|r_j - from|^2)]      (lj.rs:86-105)
// with binary32 pair terms on double-single differences and a group shuffle reduction,
// then runs the shared flat-histogram bookkeeping.  Every resum_interval moves the energy
// is replaced by an FP64 pair sum over the double-single positions (compute_energy,
// lj.rs:236-244); the largest observed |E_incremental - E_fp64| is kept in
// WalkerCore::drift.
#pragma once
#include <cuda_runtime.h>

#include "sadmc_common.cuh"
#include "sadmc_fh.cuh"
#include "sadmc_launch.h"
#include "sadmc_rng.cuh"
#include "sadmc_lj_walker.cuh"

namespace sadmc {
namespace dev {

// DESC: the initial descent (its own instantiation, so that the move kernel's code holds
// only the move loop).
template <int LPW, int APL, int FAM, bool DESC>
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

  Fh<LPW, FAM> fh;
  fh.load(m.cores, m.P, m.B, w, gmask, glane, wr);
  LjWalker<LPW, APL> lj;
  lj.set_radius2(s.radius2);
  lj.glane = glane;
  lj.gmask = gmask;
  lj.n = fh.c.n;
  float* pw = s.pos + (size_t)w * 6 * (size_t)s.np;
  lj.load(pw, s.np);

  if (DESC) {
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
  Every resum;
  resum.init(fh.c.moves, m.resum_interval > 0 ? (uint64_t)m.resum_interval : 0);
  for (uint64_t it = 0; it < m.n_moves; ++it) {
    const uint64_t t = fh.c.moves + 1;
    double rs, omrs;
    rsb.get(t, lane, rs, omrs);
    fh.begin_move(omrs);
    const Draws d = dc.get(m.seed, (uint32_t)w, t, (uint32_t)lj.n, gmask, glane);
    DS tx, ty, tz;
    float de = 0.0f;
    const bool possible = lj.plan((int)d.which, d.g0, d.g1, d.g2, sc.h, sc.l, s.radius2, tx, ty, tz, de);
    if (SADMC_RARE(m.trace && wr && glane == 0 && t > m.trace_t0 && t - m.trace_t0 <= m.trace_cap)) {
      TraceRec r;
      r.e1 = fh.c.E;
      r.e2 = possible ? fh.c.E + (double)de : __longlong_as_double(0x7ff8000000000000ll);
      m.trace[(size_t)w * m.trace_cap + (t - m.trace_t0 - 1)] = r;
    }
    const bool acc = fh.decide_de(possible, de, d.u53, rs);
    if (acc) lj.put((int)d.which, tx, ty, tz);
    fh.finish_move(acc);
    if (SADMC_RARE(fh.tscale_changed)) { fh.tscale_changed = false; sc = ds_from_double(fh.c.tscale); }
    if (SADMC_RARE(resum.tick())) {
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

}  // namespace dev

// Launch lj_move_kernel<LPW, APL, FAM, D> for the (lanes per walker, atoms per lane) shape;
// D true only for the descent launches (method-generic translation unit).
#define SADMC_LJ_CASE(L, A, F, D)                                                      \
  if (lpw == L && s.np == L * A) {                                                     \
    const int wpb = m.warps_per_block >= 1 && m.warps_per_block <= 4 ? m.warps_per_block : 4; \
    const int warps = (m.n_walkers + (32 / L) - 1) / (32 / L);                         \
    if (D) dev::lj_move_kernel<L, A, F, D><<<(warps + wpb - 1) / wpb, 32 * wpb, 0, st>>>(m, s); \
    else dev::lj_move_kernel<L, A, F, false><<<(warps + wpb - 1) / wpb, 32 * wpb, 0, st>>>(m, s); \
    return cudaGetLastError();                                                         \
  }
#define SADMC_LJ_ALL_SHAPES(F, D)                                                      \
  SADMC_LJ_CASE(32, 1, F, D) SADMC_LJ_CASE(16, 2, F, D) SADMC_LJ_CASE(8, 4, F, D)      \
  SADMC_LJ_CASE(4, 8, F, D) SADMC_LJ_CASE(32, 2, F, D) SADMC_LJ_CASE(16, 4, F, D)      \
  SADMC_LJ_CASE(8, 8, F, D) SADMC_LJ_CASE(32, 4, F, D) SADMC_LJ_CASE(32, 8, F, D)

}  // namespace sadmc
