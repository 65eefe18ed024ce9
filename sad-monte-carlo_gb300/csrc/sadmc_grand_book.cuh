// Energy-number bookkeeping of one walker, run by the LPW lanes of its group (all lanes
// hold the same state; the group's lane 0 stores): EnergyNumberMC's move choice, bounds,
// prepare_for_state, reject_move, histogram, update_weights and max-entropy logic
// (src/mc/energy_number.rs:249-355, 357-413, 540-666) over fixed (E, N) planes that keep
// the reference's own layout parameters.  The system (LJ cluster, WCA fluid) supplies
// the proposals and applies accepted ones.
#pragma once
#include <cstdint>

#include "sadmc_common.cuh"
#include "sadmc_fh.cuh"
#include "sadmc_grand.h"
#include "sadmc_rng.cuh"

namespace sadmc {
namespace dev {

template <int LPW>
struct GrandBook {
  GrandCore c;
  double* lnw;
  uint64_t *hist, *wlh, *visit, *rt, *tr_att, *tr_acc;
  int glane, rows, ncol;
  unsigned gmask;
  double width, inv_width;
  bool wl_method;
  // u_choice53 > ar_thresh  <=>  u_choice53 * 2^-53 > addremove_prob (scaling by a power of
  // two is exact, and u is an integer: u > p 2^53 <=> u > floor(p 2^53))
  int64_t ar_thresh;
  // plane row of c.E in the current layout (cur_row_ok), and the rows of the move's E1
  // and e2 once decide() has looked them up (rows_set; accepted: the move was taken)
  int cur_row, row1, row2;
  bool cur_row_ok, rows_set, accepted;
  // SAMC: gamma(gb_t0 + glane + LPW q) in gb_val[q], four independent divides per lane
  // covering 4 LPW moves
  double gb_val[4];
  uint64_t gb_t0;
  bool gb_valid;

  __device__ void load(const GrandLaunch& m, int w, int glane_, unsigned gmask_) {
    c = m.cores[w];
    glane = glane_;
    gmask = gmask_;
    rows = m.rows;
    ncol = m.ncol;
    width = m.width;
    inv_width = m.inv_width;
    const size_t base = (size_t)w * (size_t)m.rows * (size_t)m.ncol;
    lnw = m.B.lnw + base;
    hist = m.B.hist + base;
    wlh = m.B.wl_hist + base;
    visit = m.B.visit + base;
    rt = m.B.round_trips + base;
    tr_att = m.B.tr_att + (size_t)w * m.ncol;
    tr_acc = m.B.tr_acc + (size_t)w * m.ncol;
    wl_method = c.kind == 2;
    set_threshold();
    cur_row_ok = false;
    rows_set = false;
    accepted = false;
    gb_valid = false;
  }
  __device__ void store(GrandCore* cores, int w) const {
    if (glane == 0) cores[w] = c;
  }
  __device__ void set_threshold() {
    const double p = c.addremove_prob;
    if (is_nan64(p)) ar_thresh = INT64_MAX;  // a comparison with NaN is false: add/remove
    else ar_thresh = p < 0.0 ? -1ll : (p >= 1.0 ? (1ll << 53) : (int64_t)floor(p * 9007199254740992.0));
  }

  // have_visited_since_maxentropy: a bin's own value holds while its generation is
  // current, else the value of the last fill of every bin
  __device__ bool visited(uint64_t v) const {
    return (v >> 1) == c.fill_gen ? (v & 1ull) != 0 : c.fill_val != 0;
  }
  // state_to_index (energy_number.rs:227-229) as a plane row (kept inside the planes),
  // the plane offset, and the reference's own index
  __device__ int row_of(double e) const {
    const double q = div_by(e - c.min, width, inv_width);
    const int r = c.e_base + (q > 0.0 ? (q < (double)rows ? (int)q : rows) : 0);
    return r < rows ? r : rows - 1;
  }
  __device__ size_t plane(int row, int n) const { return (size_t)row * ncol + (size_t)n; }
  __device__ uint64_t ref_index(int row, int n) const {
    return (uint64_t)(row - c.e_base) * (uint64_t)(c.max_N_ref + 1) + (uint64_t)n;
  }

  // prepare_for_state (energy_number.rs:249-290): grow the layout and mark the bins it
  // gains as not visited; false when the planes cannot hold it
  __device__ bool prepare(double e, int n, bool& changed) {
    changed = false;
    if (!(n > c.max_N_ref || e < c.min || e >= c.min + width * (double)c.num_E)) return true;
    if (n >= ncol) return false;
    const int old_lo = c.e_base, old_hi = c.e_base + c.num_E, old_n = c.max_N_ref;
    double mn = c.min;
    int num_E = c.num_E, e_base = c.e_base;
    const int max_n = n > c.max_N_ref ? n : c.max_N_ref;
    while (mn > e) {
      if (e_base == 0) return false;
      mn -= width;
      num_E += 1;
      e_base -= 1;
    }
    while (mn + width * (double)num_E <= e) {
      if (e_base + num_E >= rows) return false;
      num_E += 1;
    }
    c.min = mn;
    c.num_E = num_E;
    c.e_base = e_base;
    c.max_N_ref = max_n;
    changed = true;
    const int ncols = max_n + 1;
    const int total = num_E * ncols;
    for (int k = glane; k < total; k += LPW) {
      const int r = e_base + k / ncols, q = k % ncols;
      if (r >= old_lo && r < old_hi && q <= old_n) continue;
      visit[plane(r, q)] = c.fill_gen << 1;  // a new bin starts not visited
    }
    __syncwarp(gmask);
    cur_row_ok = false;
    return true;
  }

  // Start of move_once: the move counter, and translate-or-add/remove with its attempt
  // counter (energy_number.rs:541-545, 567-568); true = translation.
  __device__ bool choose(const GrandDraws& d) {
    rows_set = false;
    accepted = false;
    if ((int64_t)d.u_choice53 > ar_thresh) {
      if (glane == 0) tr_att[c.N] += 1;
      return true;
    }
    c.ar_attempts += 1;
    return false;
  }

  // Bounds, prepare_for_state and reject_move for a possible proposal (E1, N1) ->
  // (e2, n2); true = accepted (counters and E, N updated; the caller applies the move).
  __device__ bool decide(const GrandLaunch& m, double E1, int N1, double e2, int n2,
                         bool translation, uint64_t u53) {
    bool oob = false;
    if (m.has_max_allowed) oob = e2 > m.max_allowed && e2 > E1;
    if (m.has_min_allowed) oob = oob || (e2 < m.min_allowed && e2 < E1);
    if (oob) return false;
    bool changed = false;
    if (!prepare(e2, n2, changed)) {
      c.status |= ST_BIN_RANGE;
      return false;
    }
    // reject_move (energy_number.rs:314-355); WL regroups when its bins grew
    if (wl_method && changed && c.gamma != 1.0) {
      c.gamma = 1.0;
      c.lowest = 0;
      c.highest = 0;
      c.total = 0;
    }
    row1 = cur_row_ok ? cur_row : row_of(E1);
    row2 = row_of(e2);
    rows_set = true;
    const double lnw1 = lnw[plane(row1, N1)], lnw2 = lnw[plane(row2, n2)];
    const bool rejected = lnw2 > lnw1 && metropolis_reject2(lnw1, lnw2, u53);
    if (rejected) return false;
    c.accepted += 1;
    if (translation) {
      if (glane == 0) tr_acc[N1] += 1;
    } else {
      c.ar_accepted += 1;
    }
    c.E = e2;
    c.N = n2;
    accepted = true;
    return true;
  }

  // End of move_once (energy_number.rs:607-664): histogram, the add/remove probability,
  // update_weights, max-entropy and round trips.
  // SAMC's gamma t0 / t for t > t0 (energy_number.rs:616-619), from the batch
  __device__ double samc_gamma(const GrandLaunch& m, uint64_t t) {
    uint64_t off = t - gb_t0;
    if (!gb_valid || off >= (uint64_t)(4 * LPW)) {
      gb_t0 = t;
      off = 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double td = (double)(t + (uint64_t)(glane + LPW * q));
        gb_val[q] = td > m.t0 ? m.t0 / td : 1.0;
      }
      gb_valid = true;
    }
    const int o = (int)off, q = o / LPW;
    const double v = q == 0 ? gb_val[0] : q == 1 ? gb_val[1] : q == 2 ? gb_val[2] : gb_val[3];
    if (LPW == 1) return v;
    return __shfl_sync(gmask, v, o % LPW, LPW);
  }

  __device__ void finish(const GrandLaunch& m, uint64_t t, double E1, int N1) {
    __syncwarp(gmask);
    const double E = c.E;
    const int N = c.N;
    // the row of E: from decide() when it looked the rows up, else (the state did not
    // change) the row kept from the last move unless the layout changed since
    const int row = rows_set ? (accepted ? row2 : row1) : (cur_row_ok ? cur_row : row_of(E));
    const int row_E1 = rows_set ? row1 : row;
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
      if (!is_nan64(new_p)) {
        c.addremove_prob = new_p > 0.999 ? 0.999 : new_p;
        set_threshold();
      }
    }
    const uint64_t h = h0 + 1;
    double gam;
    if (wl_method) gam = c.gamma;
    else gam = samc_gamma(m, t);
    const double lnw_i = lnw[g] + gam;
    uint64_t wl_i = 0;
    if (wl_method) wl_i = wlh[g] + 1;
    __syncwarp(gmask);
    if (glane == 0) {
      hist[g] = h;
      lnw[g] = lnw_i;
      if (wl_method) wlh[g] = wl_i;
    }
    __syncwarp(gmask);
    if (wl_method) {  // update_weights (energy_number.rs:357-413)
      const double num_states = (double)c.num_states;
      if (wl_i > c.highest) c.highest = wl_i;
      c.total += 1;
      if (wl_i == c.lowest + 1) {
        const int ncols = c.max_N_ref + 1, total = c.num_E * ncols;
        uint64_t mn = ~0ull;
        for (int k = glane; k < total; k += LPW) {
          const size_t q = plane(c.e_base + k / ncols, k % ncols);
          if (hist[q] != 0) {
            const uint64_t v = wlh[q];
            mn = v < mn ? v : mn;
          }
        }
#pragma unroll
        for (int o = LPW / 2; o > 0; o >>= 1) {
          const uint64_t x = __shfl_xor_sync(gmask, mn, o, LPW);
          mn = x < mn ? x : mn;
        }
        if (mn == c.lowest + 1) {
          c.lowest = wl_i;
          if (total > 1 && (double)c.lowest >= 0.8 * (double)c.total / num_states) {
            c.gamma *= 0.5;
            for (int k = glane; k < total; k += LPW) wlh[plane(c.e_base + k / ncols, k % ncols)] = 0;
            c.total = 0;
            c.lowest = 0;
            __syncwarp(gmask);
          }
        }
      }
    }
    const uint64_t ri = ref_index(row, N);
    if (lnw_i > c.max_S) {
      c.max_S = lnw_i;
      c.max_S_index = ri;
      c.fill_gen += 1;
      c.fill_val = 1;
    } else if (ri == c.max_S_index) {
      if (ref_index(row_E1, N1) != ri) {
        c.fill_gen += 1;
        c.fill_val = 0;
      }
    } else if (!visited(visit[g])) {
      const uint64_t r0 = rt[g];
      __syncwarp(gmask);
      if (glane == 0) {
        visit[g] = (c.fill_gen << 1) | 1ull;
        rt[g] = r0 + 1;
      }
    }
    __syncwarp(gmask);
    cur_row = row;
    cur_row_ok = true;
    rows_set = false;
  }

  // After a periodic FP64 re-sum: keep the largest drift, and bins for the new energy.
  __device__ void resummed(const GrandLaunch& m, double e64) {
    const double dr = fabs(e64 - c.E);
    if (dr > c.drift) c.drift = dr;
    if (dr > m.drift_tol) c.status |= ST_DRIFT;
    c.E = e64;
    cur_row_ok = false;
    bool changed = false;  // the re-summed energy may sit across a bin edge
    if (!prepare(e64, c.N, changed)) c.status |= ST_BIN_RANGE;
  }
};

}  // namespace dev
}  // namespace sadmc
