// Grand-canonical LJ cluster with the energy-number method, many walkers per launch:
// EnergyNumberMC::move_once (src/mc/energy_number.rs:540-666) with the GrandSystem moves
// of src/system/lj.rs:291-319 (add at a uniform point of the sphere, remove a uniform
// atom by swap_remove) and translations (lj.rs:86-105, 365-374).
//
// LPW lanes per walker (32 / LPW walkers per warp): atom j in lane j % LPW of the
// walker's group, register slot j / LPW, double-single positions; pair energies in
// binary32 over double-single differences with a group reduction, every decision on the
// FP64 energy E + de as the reference takes it.  The
// (E, N) bins keep the reference's layout parameters (min, num_E, max_N) and its index
// arithmetic, including the quirks that affect results (max_S_index is not remapped
// when the layout grows; Wang-Landau's histogram is a second set of bins).
#include <cuda_runtime.h>

#include "sadmc_common.cuh"
#include "sadmc_fh.cuh"
#include "sadmc_grand.h"
#include "sadmc_grand_book.cuh"
#include "sadmc_lj_walker.cuh"
#include "sadmc_rng.cuh"

namespace sadmc {
namespace dev {

template <int LPW, int APL>
__global__ void __launch_bounds__(128) lj_grand_kernel(GrandLaunch m) {
  constexpr int WPW = 32 / LPW;
  const int lane = threadIdx.x & 31;
  const int group = lane / LPW, glane = lane % LPW;
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * WPW + group;
  // every collective below is over the walker's own group: a group past the last walker
  // leaves without disturbing the others
  if (w >= m.n_walkers) return;
  const unsigned gmask = group_mask<LPW>(group);
  GrandBook<LPW> bk;
  bk.load(m, w, glane, gmask);
  LjWalker<LPW, APL> lj;
  lj.set_radius2(m.radius2);
  lj.glane = glane;
  lj.gmask = gmask;
  lj.n = bk.c.N;
  float* pw = m.pos + (size_t)w * 6 * (size_t)m.np;
  lj.load(pw, m.np);
  const DS sc = ds_from_double(m.translation_scale);

  Every resum;
  resum.init(bk.c.moves, m.resum_interval > 0 ? (uint64_t)m.resum_interval : 0);
  for (uint64_t it = 0; it < m.n_moves; ++it) {
    bk.c.moves += 1;
    const uint64_t t = bk.c.moves;
    const GrandDraws d = draws_grand(m.seed, (uint32_t)w, t);
    const double E1 = bk.c.E;
    const int N1 = bk.c.N;
    int kind_move = -1;  // 0 translate, 1 add, 2 remove; -1 impossible
    int which = 0, N2 = N1;
    DS tx{0.f, 0.f}, ty{0.f, 0.f}, tz{0.f, 0.f};
    float de = 0.0f;
    const bool translation = bk.choose(d);
    if (translation) {
      if (N1 > 0) {  // plan_move (lj.rs:365-374)
        which = (int)mulhi_range(d.pick, (uint32_t)N1);
        if (lj.plan(which, d.g0, d.g1, d.g2, sc.h, sc.l, m.radius2, tx, ty, tz, de)) kind_move = 0;
      }
    } else if (d.add_bit == 0) {
      // plan_add (lj.rs:292-309): a uniform point of the unit ball times the radius
      if (!(m.has_max_N && N1 == m.max_N) && N1 + 1 < m.ncol && N1 < LPW * APL) {
        double ux = 0, uy = 0, uz = 0;
        bool found = false;
        for (int k = 0; k < 64 && !found; ++k) {
          add_candidate(m.seed, (uint32_t)w, t, k, ux, uy, uz);
          found = ux * ux + uy * uy + uz * uz < 1.0;
        }
        if (found) {
          tx = ds_from_double(ux * m.radius);
          ty = ds_from_double(uy * m.radius);
          tz = ds_from_double(uz * m.radius);
          float e = 0.0f;
#pragma unroll
          for (int k = 0; k < APL; ++k) {
            const int j = glane + LPW * k;
            if (j < N1) {
              const float dx = (lj.x[k].h - tx.h) + (lj.x[k].l - tx.l);
              const float dy = (lj.y[k].h - ty.h) + (lj.y[k].l - ty.l);
              const float dz = (lj.z[k].h - tz.h) + (lj.z[k].l - tz.l);
              e += lj_v32(dx * dx + dy * dy + dz * dz);
            }
          }
          de = group_sum<LPW>(e, gmask);
          kind_move = 1;
          N2 = N1 + 1;
        }
      }
    } else if (N1 > 0) {  // plan_remove (lj.rs:310-315)
      which = (int)mulhi_range(d.pick, (uint32_t)N1);
      DS fx, fy, fz;
      lj.fetch(which, fx, fy, fz);
      float e = 0.0f;
#pragma unroll
      for (int k = 0; k < APL; ++k) {
        const int j = glane + LPW * k;
        if (j < N1 && j != which) {
          const float dx = (lj.x[k].h - fx.h) + (lj.x[k].l - fx.l);
          const float dy = (lj.y[k].h - fy.h) + (lj.y[k].l - fy.l);
          const float dz = (lj.z[k].h - fz.h) + (lj.z[k].l - fz.l);
          e += lj_v32(dx * dx + dy * dy + dz * dz);
        }
      }
      de = -group_sum<LPW>(e, gmask);
      kind_move = 2;
      N2 = N1 - 1;
    }
    const bool possible = kind_move >= 0 && fabsf(de) <= 3.0e38f;
    if (m.trace && glane == 0 && t > m.trace_t0 && t - m.trace_t0 <= m.trace_cap) {
      TraceRec r;
      r.e1 = E1;
      r.e2 = possible ? E1 + (double)de : __longlong_as_double(0x7ff8000000000000ll);
      m.trace[(size_t)w * m.trace_cap + (t - m.trace_t0 - 1)] = r;
    }
    if (possible && bk.decide(m, E1, N1, E1 + (double)de, N2, translation, d.u53)) {
      // ConfirmSystem::confirm (lj.rs:339-358)
      if (kind_move == 0) {
        lj.put(which, tx, ty, tz);
      } else if (kind_move == 1) {
        lj.put(N1, tx, ty, tz);
        lj.n = N1 + 1;
      } else {  // swap_remove
        DS lx, ly, lz;
        lj.fetch(N1 - 1, lx, ly, lz);
        lj.put(which, lx, ly, lz);
        lj.n = N1 - 1;
      }
    }
    bk.finish(m, t, E1, N1);
    if (resum.tick()) bk.resummed(m, lj.energy64());
  }
  lj.store(pw, m.np, true);
  bk.store(m.cores, w);
}

// Initial bins of every walker (energy_number.rs:474-533): the reference's one bin
// (E = 0, N = 0) has histogram 1 and round_trips 1, and Wang-Landau's histogram 1.
__global__ void grand_init_kernel(GrandLaunch m) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= m.n_walkers) return;
  const GrandCore& c = m.cores[w];
  const size_t g = (size_t)w * m.rows * m.ncol + (size_t)c.e_base * m.ncol;
  m.B.hist[g] = 1;
  m.B.round_trips[g] = 1;
  m.B.wl_hist[g] = c.kind == 2 ? 1 : 0;
  m.B.visit[g] = 0;  // generation 0, not visited
}

}  // namespace dev

#define SADMC_GRAND_CASE(L, A)                                                          \
  if (m.lanes == L && m.np == L * A) {                                                  \
    const int warps = (m.n_walkers + (32 / L) - 1) / (32 / L);                          \
    dev::lj_grand_kernel<L, A><<<(warps + 3) / 4, 128, 0, st>>>(m);                     \
    return cudaGetLastError();                                                          \
  }

cudaError_t launch_grand_move(const GrandLaunch& m, cudaStream_t st) {
  SADMC_GRAND_CASE(32, 1) SADMC_GRAND_CASE(16, 2) SADMC_GRAND_CASE(8, 4) SADMC_GRAND_CASE(4, 8)
  SADMC_GRAND_CASE(32, 2) SADMC_GRAND_CASE(16, 4) SADMC_GRAND_CASE(8, 8)
  return cudaErrorInvalidConfiguration;
}

cudaError_t launch_grand_init(const GrandLaunch& m, cudaStream_t st) {
  dev::grand_init_kernel<<<(m.n_walkers + 127) / 128, 128, 0, st>>>(m);
  return cudaGetLastError();
}

}  // namespace sadmc
