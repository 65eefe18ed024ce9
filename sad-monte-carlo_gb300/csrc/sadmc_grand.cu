// Grand-canonical LJ cluster with the energy-number method, many walkers per launch:
// EnergyNumberMC::move_once (src/mc/energy_number.rs:540-666) with the GrandSystem moves
// of src/system/lj.rs:291-319 (add at a uniform point of the sphere, remove a uniform
// atom by swap_remove) and translations (lj.rs:86-105, 365-374).
//
// One warp per walker: atom j in lane j % 32, register slot j / 32, double-single
// positions; pair energies in binary32 over double-single differences with a warp
// reduction, every decision on the FP64 energy E + de as the reference takes it.  The
// (E, N) bins keep the reference's layout parameters (min, num_E, max_N) and its index
// arithmetic, including the quirks that affect results (max_S_index is not remapped
// when the layout grows; Wang-Landau's histogram is a second set of bins).
#include <cuda_runtime.h>

#include "sadmc_common.cuh"
#include "sadmc_fh.cuh"
#include "sadmc_grand.h"
#include "sadmc_lj_walker.cuh"
#include "sadmc_rng.cuh"

namespace sadmc {
namespace dev {

// have_visited_since_maxentropy: a bin's own value holds while its generation is current,
// else the value of the last fill of every bin.
__device__ __forceinline__ bool grand_visited(const GrandCore& c, uint64_t v) {
  return (v >> 1) == c.fill_gen ? (v & 1ull) != 0 : c.fill_val != 0;
}

template <int APL>
__global__ void __launch_bounds__(128) lj_grand_kernel(GrandLaunch m) {
  const int lane = threadIdx.x & 31;
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (w >= m.n_walkers) return;
  const unsigned full = 0xffffffffu;
  GrandCore c = m.cores[w];
  LjWalker<32, APL> lj;
  lj.glane = lane;
  lj.gmask = full;
  lj.n = c.N;
  float* pw = m.pos + (size_t)w * 6 * (size_t)m.np;
  lj.load(pw, m.np);
  const size_t base = (size_t)w * (size_t)m.rows * (size_t)m.ncol;
  double* lnw = m.B.lnw + base;
  uint64_t* hist = m.B.hist + base;
  uint64_t* wlh = m.B.wl_hist + base;
  uint64_t* visit = m.B.visit + base;
  uint64_t* rt = m.B.round_trips + base;
  uint64_t* tr_att = m.B.tr_att + (size_t)w * m.ncol;
  uint64_t* tr_acc = m.B.tr_acc + (size_t)w * m.ncol;
  const DS sc = ds_from_double(m.translation_scale);
  const bool wl_method = c.kind == 2;

  // state_to_index (energy_number.rs:227-229) as a plane row, and the reference's index
  auto row_of = [&](double e) -> int {
    const double q = div_by(e - c.min, m.width, m.inv_width);
    const int r = c.e_base + (q > 0.0 ? (q < (double)m.rows ? (int)q : m.rows) : 0);
    return r < m.rows ? r : m.rows - 1;  // energies are prepared first; kept in the planes
  };
  auto plane = [&](int row, int n) -> size_t { return (size_t)row * m.ncol + (size_t)n; };
  auto ref_index = [&](int row, int n) -> uint64_t {
    return (uint64_t)(row - c.e_base) * (uint64_t)(c.max_N_ref + 1) + (uint64_t)n;
  };
  // prepare_for_state (energy_number.rs:249-290) on the fixed planes: grow the layout,
  // mark the bins it gains as not visited; false when the planes cannot hold it
  auto prepare = [&](double e, int n, bool& changed) -> bool {
    changed = false;
    if (!(n > c.max_N_ref || e < c.min || e >= c.min + m.width * (double)c.num_E)) return true;
    if (n >= m.ncol) return false;
    const int old_lo = c.e_base, old_hi = c.e_base + c.num_E, old_n = c.max_N_ref;
    double mn = c.min;
    int num_E = c.num_E, e_base = c.e_base;
    const int max_n = n > c.max_N_ref ? n : c.max_N_ref;
    while (mn > e) {
      if (e_base == 0) return false;
      mn -= m.width;
      num_E += 1;
      e_base -= 1;
    }
    while (mn + m.width * (double)num_E <= e) {
      if (e_base + num_E >= m.rows) return false;
      num_E += 1;
    }
    c.min = mn;
    c.num_E = num_E;
    c.e_base = e_base;
    c.max_N_ref = max_n;
    changed = true;
    const int ncols = max_n + 1;
    const int total = num_E * ncols;
    for (int k = lane; k < total; k += 32) {
      const int r = e_base + k / ncols, q = k % ncols;
      if (r >= old_lo && r < old_hi && q <= old_n) continue;
      visit[plane(r, q)] = c.fill_gen << 1;  // a new bin starts not visited
    }
    __syncwarp(full);
    return true;
  };

  Every resum;
  resum.init(c.moves, m.resum_interval > 0 ? (uint64_t)m.resum_interval : 0);
  for (uint64_t it = 0; it < m.n_moves; ++it) {
    c.moves += 1;
    const uint64_t t = c.moves;
    const GrandDraws d = draws_grand(m.seed, (uint32_t)w, t);
    const double E1 = c.E;
    const int N1 = c.N;
    int kind_move = -1;  // 0 translate, 1 add, 2 remove; -1 impossible
    int which = 0, N2 = N1;
    DS tx{0.f, 0.f}, ty{0.f, 0.f}, tz{0.f, 0.f};
    float de = 0.0f;
    if ((double)d.u_choice53 * (1.0 / 9007199254740992.0) > c.addremove_prob) {
      if (lane == 0) tr_att[N1] += 1;
      if (N1 > 0) {
        which = (int)mulhi_range(d.pick, (uint32_t)N1);
        if (lj.plan(which, d.g0, d.g1, d.g2, sc.h, sc.l, m.radius2, tx, ty, tz, de)) kind_move = 0;
      }
    } else {
      c.ar_attempts += 1;
      if (d.add_bit == 0) {
        if (!(m.has_max_N && N1 == m.max_N) && N1 + 1 < m.ncol && N1 < 32 * APL) {
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
              const int j = lane + 32 * k;
              if (j < N1) {
                const float dx = (lj.x[k].h - tx.h) + (lj.x[k].l - tx.l);
                const float dy = (lj.y[k].h - ty.h) + (lj.y[k].l - ty.l);
                const float dz = (lj.z[k].h - tz.h) + (lj.z[k].l - tz.l);
                e += lj_v32(dx * dx + dy * dy + dz * dz);
              }
            }
            de = group_sum<32>(e, full);
            kind_move = 1;
            N2 = N1 + 1;
          }
        }
      } else if (N1 > 0) {
        which = (int)mulhi_range(d.pick, (uint32_t)N1);
        DS fx, fy, fz;
        lj.fetch(which, fx, fy, fz);
        float e = 0.0f;
#pragma unroll
        for (int k = 0; k < APL; ++k) {
          const int j = lane + 32 * k;
          if (j < N1 && j != which) {
            const float dx = (lj.x[k].h - fx.h) + (lj.x[k].l - fx.l);
            const float dy = (lj.y[k].h - fy.h) + (lj.y[k].l - fy.l);
            const float dz = (lj.z[k].h - fz.h) + (lj.z[k].l - fz.l);
            e += lj_v32(dx * dx + dy * dy + dz * dz);
          }
        }
        de = -group_sum<32>(e, full);
        kind_move = 2;
        N2 = N1 - 1;
      }
    }
    bool possible = kind_move >= 0 && fabsf(de) <= 3.0e38f;
    if (m.trace && lane == 0 && t > m.trace_t0 && t - m.trace_t0 <= m.trace_cap) {
      TraceRec r;
      r.e1 = E1;
      r.e2 = possible ? E1 + (double)de : __longlong_as_double(0x7ff8000000000000ll);
      m.trace[(size_t)w * m.trace_cap + (t - m.trace_t0 - 1)] = r;
    }
    if (possible) {
      const double e2 = E1 + (double)de;
      bool oob = false;
      if (m.has_max_allowed) oob = e2 > m.max_allowed && e2 > E1;
      if (m.has_min_allowed) oob = oob || (e2 < m.min_allowed && e2 < E1);
      if (!oob) {
        bool changed = false;
        if (!prepare(e2, N2, changed)) {
          c.status |= ST_BIN_RANGE;
        } else {
          // reject_move (energy_number.rs:314-355); WL regroups when its bins grew
          if (wl_method && changed && c.gamma != 1.0) {
            c.gamma = 1.0;
            c.lowest = 0;
            c.highest = 0;
            c.total = 0;
          }
          const double lnw1 = lnw[plane(row_of(E1), N1)], lnw2 = lnw[plane(row_of(e2), N2)];
          const bool rejected = lnw2 > lnw1 && metropolis_reject2(lnw1, lnw2, d.u53);
          if (!rejected) {
            c.accepted += 1;
            if (kind_move == 0) {
              if (lane == 0) tr_acc[N1] += 1;
              lj.put(which, tx, ty, tz);
            } else {
              c.ar_accepted += 1;
              if (kind_move == 1) {
                lj.put(N1, tx, ty, tz);
                lj.n = N1 + 1;
              } else {  // swap_remove
                DS lx, ly, lz;
                lj.fetch(N1 - 1, lx, ly, lz);
                lj.put(which, lx, ly, lz);
                lj.n = N1 - 1;
              }
              c.N = N2;
            }
            c.E = e2;
          }
        }
      }
    }
    __syncwarp(full);
    // energy_number.rs:607-664
    const double E = c.E;
    const int N = c.N;
    const int row = row_of(E);
    const size_t g = plane(row, N);
    const uint64_t h0 = hist[g];
    if (h0 == 0) {
      c.num_states += 1;
      c.t_last = t;
    }
    if (m.acc_mode && t % c.t_last == 0) {
      const double acc_ar = (double)c.ar_accepted / (double)c.ar_attempts;
      const double acc_tr = (double)(c.accepted - c.ar_accepted) / (double)(t - c.ar_attempts);
      const double new_p = (m.target_rate - acc_tr) / (acc_ar - acc_tr);
      if (!is_nan64(new_p)) c.addremove_prob = new_p > 0.999 ? 0.999 : new_p;
    }
    const uint64_t h = h0 + 1;
    // update_weights (energy_number.rs:357-413)
    double gam;
    if (wl_method) gam = c.gamma;
    else gam = (double)t > m.t0 ? m.t0 / (double)t : 1.0;
    const double lnw_i = lnw[g] + gam;
    uint64_t wl_i = 0;
    if (wl_method) wl_i = wlh[g] + 1;
    __syncwarp(full);
    if (lane == 0) {
      hist[g] = h;
      lnw[g] = lnw_i;
      if (wl_method) wlh[g] = wl_i;
    }
    __syncwarp(full);
    if (wl_method) {
      const double num_states = (double)c.num_states;
      if (wl_i > c.highest) c.highest = wl_i;
      c.total += 1;
      if (wl_i == c.lowest + 1) {
        const int ncols = c.max_N_ref + 1, total = c.num_E * ncols;
        uint64_t mn = ~0ull;
        for (int k = lane; k < total; k += 32) {
          const size_t q = plane(c.e_base + k / ncols, k % ncols);
          if (hist[q] != 0) {
            const uint64_t v = wlh[q];
            mn = v < mn ? v : mn;
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const uint64_t x = __shfl_xor_sync(full, mn, o);
          mn = x < mn ? x : mn;
        }
        if (mn == c.lowest + 1) {
          c.lowest = wl_i;
          if (total > 1 && (double)c.lowest >= 0.8 * (double)c.total / num_states) {
            c.gamma *= 0.5;
            for (int k = lane; k < total; k += 32) wlh[plane(c.e_base + k / ncols, k % ncols)] = 0;
            c.total = 0;
            c.lowest = 0;
            __syncwarp(full);
          }
        }
      }
    }
    // max_S and round trips (energy_number.rs:651-664), in the reference's index space
    const uint64_t ri = ref_index(row, N);
    if (lnw_i > c.max_S) {
      c.max_S = lnw_i;
      c.max_S_index = ri;
      c.fill_gen += 1;
      c.fill_val = 1;
    } else if (ri == c.max_S_index) {
      if (ref_index(row_of(E1), N1) != ri) {
        c.fill_gen += 1;
        c.fill_val = 0;
      }
    } else if (!grand_visited(c, visit[g])) {
      const uint64_t r0 = rt[g];
      __syncwarp(full);
      if (lane == 0) {
        visit[g] = (c.fill_gen << 1) | 1ull;
        rt[g] = r0 + 1;
      }
    }
    __syncwarp(full);
    if (resum.tick()) {
      const double e64 = lj.energy64();
      const double dr = fabs(e64 - c.E);
      if (dr > c.drift) c.drift = dr;
      if (dr > m.drift_tol) c.status |= ST_DRIFT;
      c.E = e64;
      bool changed = false;  // the re-summed energy may sit across a bin edge
      if (!prepare(e64, c.N, changed)) c.status |= ST_BIN_RANGE;
    }
  }
  lj.store(pw, m.np, true);
  if (lane == 0) m.cores[w] = c;
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

cudaError_t launch_grand_move(const GrandLaunch& m, cudaStream_t st) {
  const int blocks = (m.n_walkers + 3) / 4;
  if (m.np == 32) dev::lj_grand_kernel<1><<<blocks, 128, 0, st>>>(m);
  else if (m.np == 64) dev::lj_grand_kernel<2><<<blocks, 128, 0, st>>>(m);
  else return cudaErrorInvalidConfiguration;
  return cudaGetLastError();
}

cudaError_t launch_grand_init(const GrandLaunch& m, cudaStream_t st) {
  dev::grand_init_kernel<<<(m.n_walkers + 127) / 128, 128, 0, st>>>(m);
  return cudaGetLastError();
}

}  // namespace sadmc
