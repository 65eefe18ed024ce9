// ORACLE / TEST INFRASTRUCTURE ONLY.  FP64 C++ restatement of the reference's
// flat-histogram driver EnergyMC (src/mc/energy.rs), single walker, single thread.
// Every function cites the reference lines it follows.  Plugins (report/save/movie)
// and the `extra` per-bin data are not restated; the random source is the Philox
// stream of philox_draws.hpp or a caller-supplied tape.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <functional>
#include <optional>
#include <vector>

#include "philox_draws.hpp"

namespace orc {

enum MethodKind : int32_t { M_SAD = 0, M_SAMC = 1, M_WL = 2, M_INV_T_WL = 3, M_CANONICAL = 4 };

struct MethodParams {
  int32_t kind = M_SAD;
  double min_T = 0.2;          // SAD (energy.rs:46-49, default 0.2 at energy.rs:102-104)
  double t0 = 1e4;             // SAMC
  bool has_min_gamma = false;  // WL
  double min_gamma = 0.0;
  double T = 1.0;              // canonical
};

struct MCParams {
  MethodParams method;
  uint64_t seed = 0;
  bool has_energy_bin = false;
  double energy_bin = 1.0;
  bool has_min_allowed = false, has_max_allowed = false;
  double min_allowed = 0, max_allowed = 0;
  bool acceptance_rate_mode = false;  // MoveParams::AcceptanceRate (energy.rs:73-78)
  double target_rate = 0.5;
  double translation_scale = 0.05;    // energy.rs:109, 884-887
  uint32_t walker = 0;                // Philox key word (one stream per walker)
  bool has_e0 = false;                // replace the energy after the descent (test hook)
  double e0 = 0.0;
};

struct Method {  // energy.rs:212-244
  int32_t kind = M_SAD;
  // SAD
  double min_T = 0, too_lo = 0, too_hi = 0;
  uint64_t tL = 0, tF = 0, num_states = 1, highest_hist = 1;
  double latest_parameter = 0;
  // SAMC
  double t0 = 0;
  // WL
  double gamma = 1.0;
  uint64_t lowest_hist = 1, wl_highest_hist = 1, total_hist = 0;
  double wl_num_states = 1.0;
  std::vector<uint64_t> hist;
  double min_energy = 0;
  bool inv_t = false, has_min_gamma = false;
  double min_gamma = 0;
  // canonical
  double temperature = 1.0;
};

struct Bins {  // energy.rs:145-163
  double min = 0, width = 1;
  std::vector<uint64_t> histogram, t_found;
  std::vector<double> lnw, energy_total, energy_squared_total;
  // the one `extra` datum of the systems here: WCA "pressure" (BinCounts, energy.rs:136-142)
  std::vector<uint64_t> extra_count;
  std::vector<double> extra_total;
};

// System::data_to_collect (src/system/mod.rs:88-90): only the WCA fluid collects data
// (wca.rs:202-218), every N^2 moves.
template <class S>
inline bool collect_extra(const S&, uint64_t, double*) { return false; }

// SadVersion::compute_gamma, energy.rs:22-38
inline double sad_compute_gamma(double latest_parameter, double t, double tF, double num_states) {
  if (latest_parameter * tF * num_states == 0.0) return 0.0;
  return (latest_parameter + t / tF) / (latest_parameter + t / num_states * (t / tF));
}

template <class S>
struct EnergyMC {
  S sys;
  Method method;
  uint64_t moves = 0, accepted_moves = 0;
  bool has_min_allowed = false, has_max_allowed = false;
  double min_allowed = 0, max_allowed = 0;
  bool acceptance_rate_mode = false;
  double target_rate = 0.5;
  double translation_scale = 0.05;
  double acceptance_rate = 0.5;
  Bins bins;
  std::vector<char> have_visited_since_maxentropy;
  std::vector<uint64_t> round_trips;
  double max_S = 0;
  size_t max_S_index = 0;
  // random source and diagnostics.  The move loop takes its draws straight from the
  // Philox stream (seed, walker) of the system kind (no indirect call in the timed loop);
  // `draw`, when set, replaces it (tests that inject their own stream).
  std::function<Draws(uint64_t)> draw;
  bool philox_ising = false;
  uint64_t philox_seed = 0;
  uint32_t philox_walker = 0, philox_n = 0;
  bool philox_set = false;
  Draws next_draws(uint64_t t) const {
    if (philox_set) return philox_ising ? draws_ising(philox_seed, philox_walker, t, philox_n, 0)
                                        : draws_continuous(philox_seed, philox_walker, t, philox_n, 0);
    return draw(t);
  }
  void use_philox(uint64_t seed, uint32_t walker, uint32_t n, bool ising) {
    philox_seed = seed; philox_walker = walker; philox_n = n; philox_ising = ising; philox_set = true;
  }
  uint64_t verify_failures = 0;
  bool nan_gamma = false;
  // Trace replay: when set, move k starts from the caller's energy e1[k] (the GPU's
  // incrementally tracked E, after its periodic FP64 re-sum) and decides with the
  // caller's proposed energy e2[k] (binary32 pair terms); this oracle's own FP64 e2 is
  // only compared against it.  An accepted move leaves E = e2[k], as on the GPU.
  const double* e1_override = nullptr;
  const double* e2_override = nullptr;
  double max_e2_discrepancy = 0.0;
  uint64_t override_base = 0;
  uint64_t override_mismatch = 0;
  double worst[4] = {0, 0, 0, 0};  // move, e2 given, e2 own, gross magnitude at the worst move
  // Delayed-acceptance replay (with the overrides): da_ds[k] is the GPU surrogate's energy
  // change dS of move k and da_u2(t) the second-stage uniform of move t; e2 is NaN when
  // the first stage screened the move out (or it was impossible).
  const float* da_ds = nullptr;
  std::function<double(uint64_t)> da_u2;

  // EnergyMC::from_params, energy.rs:830-898 (descent loop at 840-851 uses the
  // descent stream with scale 0.05; at most `descent_limit` proposals).
  void init(S system, const MCParams& p, std::function<Draws(uint64_t, uint32_t)> src,
            uint64_t descent_limit = 100000000ull) {
    sys = std::move(system);
    double ewidth = p.has_energy_bin ? p.energy_bin : sys.delta_energy().value_or(1.0);
    if (p.has_max_allowed) {
      for (uint64_t k = 0; k < descent_limit; ++k) {
        Draws d = src(k + 1, 1);
        auto newe = sys.plan_move(d, 0.05);
        if (newe) {
          if (*newe < sys.energy()) sys.confirm();
          if (sys.energy() < p.max_allowed) break;
        }
      }
    }
    if (p.has_e0) sys.E = p.e0;
    double E = sys.energy();
    double emin = (std::round(E / ewidth) - 0.5) * ewidth;
    // Method::new, energy.rs:247-313
    const MethodParams& mp = p.method;
    method = Method{};
    method.kind = mp.kind;
    switch (mp.kind) {
      case M_SAD:
        method.min_T = mp.min_T; method.too_lo = E; method.too_hi = E;
        method.tL = 0; method.tF = 0; method.num_states = 1; method.highest_hist = 1;
        method.latest_parameter = 0.0;
        break;
      case M_SAMC: method.t0 = mp.t0; break;
      case M_WL:
      case M_INV_T_WL: {
        bool both = p.has_min_allowed && p.has_max_allowed;
        method.kind = M_WL;
        method.gamma = 1.0;
        method.lowest_hist = both ? 0 : 1;
        method.wl_highest_hist = 1;
        method.total_hist = 0;
        method.wl_num_states = both ? (p.max_allowed - p.min_allowed) / ewidth : 1.0;
        method.hist.clear();
        method.min_energy = E;
        method.inv_t = (mp.kind == M_INV_T_WL);
        method.has_min_gamma = (mp.kind == M_WL) && mp.has_min_gamma;
        method.min_gamma = mp.min_gamma;
        break;
      }
      case M_CANONICAL: method.temperature = mp.T; break;
    }
    moves = 0;
    accepted_moves = 0;
    acceptance_rate = 0.5;
    has_min_allowed = p.has_min_allowed; has_max_allowed = p.has_max_allowed;
    min_allowed = p.min_allowed; max_allowed = p.max_allowed;
    bins = Bins{};
    bins.histogram = {1};
    bins.t_found = {0};
    bins.lnw = {0.0};
    bins.energy_total = {E};
    bins.energy_squared_total = {E * E};
    bins.min = emin;
    bins.width = ewidth;
    have_visited_since_maxentropy = {0};
    round_trips = {1};
    max_S = 0.0;
    max_S_index = 0;
    acceptance_rate_mode = p.acceptance_rate_mode;
    target_rate = p.target_rate;
    translation_scale = p.translation_scale;
    draw = [src](uint64_t t) { return src(t, 0); };
  }

  size_t state_to_index(double E) const { return (size_t)((E - bins.min) / bins.width); }  // 371-373
  double index_to_state(size_t i) const { return bins.min + ((double)i + 0.5) * bins.width; }  // 366-370

  void prepare_for_state(double e) {  // energy.rs:400-434
    while (e < bins.min) {
      bins.histogram.insert(bins.histogram.begin(), 0);
      bins.t_found.insert(bins.t_found.begin(), 0);
      bins.lnw.insert(bins.lnw.begin(), 0.0);
      bins.energy_total.insert(bins.energy_total.begin(), 0.0);
      bins.energy_squared_total.insert(bins.energy_squared_total.begin(), 0.0);
      if (!bins.extra_count.empty()) {
        bins.extra_count.insert(bins.extra_count.begin(), 0);
        bins.extra_total.insert(bins.extra_total.begin(), 0.0);
      }
      have_visited_since_maxentropy.insert(have_visited_since_maxentropy.begin(), 1);
      round_trips.insert(round_trips.begin(), 1);
      bins.min -= bins.width;
    }
    while (e >= bins.min + bins.width * (double)bins.lnw.size()) {
      bins.lnw.push_back(0.0);
      bins.histogram.push_back(0);
      bins.t_found.push_back(0);
      bins.energy_total.push_back(0.0);
      bins.energy_squared_total.push_back(0.0);
      if (!bins.extra_count.empty()) {
        bins.extra_count.push_back(0);
        bins.extra_total.push_back(0.0);
      }
      have_visited_since_maxentropy.push_back(1);
      round_trips.push_back(1);
    }
  }

  double gamma() const {  // energy.rs:799-825
    switch (method.kind) {
      case M_CANONICAL: return 0.0;
      case M_SAD:
        return sad_compute_gamma(method.latest_parameter, (double)moves, (double)method.tF,
                                 (double)method.num_states);
      case M_SAMC: {
        double t = (double)moves;
        return t > method.t0 ? method.t0 / t : 1.0;
      }
      default: return method.gamma;
    }
  }

  // ln w at energy e as the Metropolis test would read it, without growing the bins: the
  // SAD extrapolations outside its window, 0 outside the allocated bins (a new bin's
  // value).  The delayed-acceptance screen of the GPU kernel (Fh::lnw_at).
  double lnw_at(double e) const {
    if (method.kind == M_SAD) {
      const double too_lo = method.too_lo, too_hi = method.too_hi;
      if (e < too_lo) return bins.lnw[state_to_index(too_lo)] + (e - too_lo) / method.min_T;
      if (e > too_hi) return bins.lnw[state_to_index(too_hi)];
    }
    if (e < bins.min || e >= bins.min + bins.width * (double)bins.lnw.size()) return 0.0;
    return bins.lnw[state_to_index(e)];
  }

  // lnw1_given: the Metropolis test uses it in place of ln w(e1) (the second stage of a
  // delayed-acceptance move).
  bool reject_move(double e1, double e2, double u, const double* lnw1_given = nullptr) {  // energy.rs:440-512
    size_t i1 = state_to_index(e1), i2 = state_to_index(e2);
    switch (method.kind) {
      case M_SAD: {
        const double too_lo = method.too_lo, too_hi = method.too_hi, min_T = method.min_T;
        const auto& lnw = bins.lnw;
        double lnw1 = lnw1_given ? *lnw1_given
                      : e1 < too_lo ? lnw[state_to_index(too_lo)] + (e1 - too_lo) / min_T
                      : e1 > too_hi ? lnw[state_to_index(too_hi)] : lnw[i1];
        double lnw2 = e2 < too_lo ? lnw[state_to_index(too_lo)] + (e2 - too_lo) / min_T
                      : e2 > too_hi ? lnw[state_to_index(too_hi)] : lnw[i2];
        bool rejected = lnw2 > lnw1 && u > std::exp(lnw1 - lnw2);
        if (!rejected && bins.histogram[i2] == 0 && e2 < too_hi && e2 > too_lo) {
          method.latest_parameter = (too_hi - too_lo) / min_T;
          method.num_states += 1;
          method.tL = moves;
        }
        return rejected;
      }
      case M_SAMC: {
        double lnw1 = lnw1_given ? *lnw1_given : bins.lnw[i1], lnw2 = bins.lnw[i2];
        return lnw2 > lnw1 && u > std::exp(lnw1 - lnw2);
      }
      case M_WL: {
        double lnw1 = lnw1_given ? *lnw1_given : bins.lnw[i1], lnw2 = bins.lnw[i2];
        bool rejected = lnw2 > lnw1 && u > std::exp(lnw1 - lnw2);
        if (!rejected && bins.histogram[i2] == 0 && method.lowest_hist > 0) method.wl_num_states += 1.0;
        return rejected;
      }
      default: {  // canonical
        if (e1 >= e2) return false;
        return u > std::exp((e1 - e2) / method.temperature);
      }
    }
  }

  void update_weights(double energy) {  // energy.rs:514-761
    size_t i = state_to_index(energy);
    double g = gamma();
    if (std::isnan(g)) nan_gamma = true;
    double old_lnw = bins.lnw[i];
    bins.lnw[i] += g;
    bool switch_to_samc = false;
    double samc_t0 = 0.0;
    Method& m = method;
    switch (m.kind) {
      case M_CANONICAL: break;
      case M_SAD: {
        auto& histogram = bins.histogram;
        if (m.too_lo > m.too_hi || energy < m.too_lo || energy > m.too_hi) bins.lnw[i] = old_lnw;
        if (histogram[i] > m.highest_hist) {
          m.highest_hist = histogram[i];
          if (energy > m.too_hi) {
            size_t ihi = state_to_index(m.too_hi);
            for (size_t j = 0; j < histogram.size(); ++j) {
              double ej = index_to_state(j);
              if (ej > m.too_hi && ej <= energy) {
                if (histogram[j] != 0) { bins.lnw[j] = bins.lnw[ihi]; m.num_states += 1; }
                else bins.lnw[j] = 0.0;
              }
            }
            m.latest_parameter = (energy - m.too_lo) / m.min_T;
            m.tL = moves;
            m.too_hi = index_to_state(state_to_index(energy));
          } else if (energy < m.too_lo) {
            size_t ilo = state_to_index(m.too_lo);
            for (size_t j = 0; j < histogram.size(); ++j) {
              double ej = index_to_state(j);
              if (ej < m.too_lo && ej >= energy) {
                if (histogram[j] != 0) {
                  bins.lnw[j] = bins.lnw[ilo] + (ej - m.too_lo) / m.min_T;
                  if (bins.lnw[j] < 0.0) bins.lnw[j] = 0.0;
                  m.num_states += 1;
                } else {
                  bins.lnw[j] = 0.0;
                }
              }
            }
            m.latest_parameter = (m.too_hi - energy) / m.min_T;
            m.tL = moves;
            m.too_lo = index_to_state(state_to_index(energy));
          }
        }
        if (m.tL == moves) {
          size_t ilo = state_to_index(m.too_lo), ihi = state_to_index(m.too_hi);
          uint64_t old_tF = m.tF;
          uint64_t mx = 0;
          for (size_t j = ilo; j <= ihi; ++j) mx = std::max(mx, bins.t_found[j]);
          m.tF = mx;
          if (old_tF != m.tF && acceptance_rate_mode) {
            double s = acceptance_rate / target_rate;
            s = s < 0.8 ? 0.8 : (s > 1.2 ? 1.2 : s);
            translation_scale *= s;
          }
        }
        break;
      }
      case M_SAMC: break;
      case M_WL: {
        if (m.has_min_gamma && m.gamma < m.min_gamma) {
          m.hist[i] += 1;
          return;
        }
        if (m.hist.size() != bins.lnw.size()) {
          if (m.hist.empty() || (m.gamma != 1.0 && m.lowest_hist > 0)) {
            m.gamma = 1.0;
            m.lowest_hist = 0;
            m.wl_highest_hist = 0;
            m.total_hist = 0;
            m.hist.assign(bins.lnw.size(), 0);
            m.min_energy = bins.min;
          } else {
            while (m.min_energy > bins.min) {
              m.min_energy -= bins.width;
              m.hist.insert(m.hist.begin(), 0);
            }
            while (m.hist.size() < bins.lnw.size()) m.hist.push_back(0);
            m.lowest_hist = *std::min_element(m.hist.begin(), m.hist.end());
          }
        }
        m.hist[i] += 1;
        if (m.hist[i] > m.wl_highest_hist) m.wl_highest_hist = m.hist[i];
        m.total_hist += 1;
        const auto& histogram = bins.histogram;
        double max_energy = m.min_energy + (double)m.hist.size() * bins.width;
        bool cond = m.hist[i] == m.lowest_hist + 1 && m.hist.size() > 1 &&
                    (!has_min_allowed || min_allowed >= m.min_energy) &&
                    (!has_max_allowed || max_allowed <= max_energy);
        if (cond) {
          bool any = false;
          uint64_t mn = 0;
          for (size_t k = 0; k < m.hist.size(); ++k)
            if (histogram[k] != 0) {
              if (!any || m.hist[k] < mn) mn = m.hist[k];
              any = true;
            }
          cond = any && mn == m.lowest_hist + 1;
        }
        if (cond) {
          m.lowest_hist = m.hist[i];
          if ((m.inv_t && m.lowest_hist > 0) ||
              (double)m.lowest_hist >= 0.8 * (double)m.total_hist / m.wl_num_states) {
            m.gamma *= 0.5;
            std::fill(m.hist.begin(), m.hist.end(), 0);
            m.total_hist = 0;
            m.lowest_hist = 0;
            m.wl_highest_hist = 0;
            if (m.has_min_gamma && m.gamma < m.min_gamma) m.gamma = 0.0;
          }
          if (m.inv_t && m.gamma < m.wl_num_states / (double)moves) {
            switch_to_samc = true;
            samc_t0 = m.wl_num_states;
          }
        }
        break;
      }
    }
    if (switch_to_samc) {
      Method nm;
      nm.kind = M_SAMC;
      nm.t0 = samc_t0;
      method = nm;
    }
  }

  void move_once() {  // energy.rs:904-974
    moves += 1;
    uint64_t nb = (uint64_t)bins.histogram.size();
    if (moves % (nb * nb * 1000) == 0 && !sys.verify_energy()) verify_failures += 1;
    if (e1_override) sys.E = e1_override[moves - 1 - override_base];
    double e1 = sys.energy();
    double recent_scale = std::sqrt(1.0 / (double)moves);
    acceptance_rate *= 1. - recent_scale;
    Draws d = next_draws(moves);
    // delayed acceptance (sadmc_da.cu): stage 1 screens with E~ = E + dS
    double lnw_first = 0.0;
    bool use_first = false;
    if (da_ds) {
      const double ds = (double)da_ds[moves - 1 - override_base];
      const double lnw_cur = lnw_at(e1), lnw_til = lnw_at(e1 + ds);
      const bool uphill1 = lnw_til > lnw_cur;
      if (uphill1 && d.u > std::exp(lnw_cur - lnw_til)) {  // screened out: a rejected move
        if (e2_override[moves - 1 - override_base] == e2_override[moves - 1 - override_base])
          ++override_mismatch;  // the GPU evaluated it
        finish_move(e1);
        return;
      }
      // stage 2 (Christen-Fox with the reverse screen from the proposed state); a certain
      // first stage used no randomness, so the second reuses the move's uniform
      const double ge2 = e2_override[moves - 1 - override_base];
      if (ge2 == ge2) {
        const double back = lnw_at(ge2) - lnw_at(ge2 - ds);
        lnw_first = lnw_cur - (uphill1 ? lnw_cur - lnw_til : 0.0) + (back < 0.0 ? back : 0.0);
        use_first = true;
      }
      if (uphill1) d.u = da_u2(moves);
    }
    auto e2o = sys.plan_move(d, translation_scale);
    if (da_ds && e2o && !use_first) ++override_mismatch;  // the GPU screened out or lost a possible move
    if (!e2o && e2_override && e2_override[moves - 1 - override_base] ==
                                   e2_override[moves - 1 - override_base])
      ++override_mismatch;
    if (e2o && e2_override && e2_override[moves - 1 - override_base] !=
                                  e2_override[moves - 1 - override_base])
      e2o.reset();
    if (e2o) {
      double e2 = *e2o;
      if (e2_override) {
        double ge2 = e2_override[moves - 1 - override_base];
        // |e2_gpu - e2| relative to the gross magnitude of the proposal's pair terms
        // (sum of 4 s^6 + 4 s^3), the scale of binary32 rounding in 4 (s^6 - s^3)
        if (ge2 != ge2) ++override_mismatch;  // GPU said impossible, oracle possible
        else {
          const double dd = std::fabs(ge2 - e2) / (1e-3 + sys.last_abs);
          if (dd > max_e2_discrepancy) {
            max_e2_discrepancy = dd;
            worst[0] = (double)moves; worst[1] = ge2; worst[2] = e2; worst[3] = sys.last_abs;
          }
        }
        e2 = ge2;
      }
      bool oob = false;
      if (has_max_allowed) oob = e2 > max_allowed && e2 > e1;
      if (has_min_allowed) oob = oob || (e2 < min_allowed && e2 < e1);
      if (!oob) {
        prepare_for_state(e2);
        if (!reject_move(e1, e2, d.u, use_first ? &lnw_first : nullptr)) {
          accepted_moves += 1;
          acceptance_rate += recent_scale;
          sys.confirm();
          if (e2_override) sys.E = e2;
        }
      }
    }
    finish_move(e1);
  }

  // The end of move_once (energy.rs:936-965): histogram, sums, extra data, update_weights
  // and the max-entropy bookkeeping for the energy the move left.
  void finish_move(double e1) {
    double energy = sys.energy();
    size_t i = state_to_index(energy);
    if (bins.histogram[i] == 0) bins.t_found[i] = moves;
    bins.histogram[i] += 1;
    bins.energy_total[i] += energy;
    bins.energy_squared_total[i] += energy * energy;
    double datum;
    if (collect_extra(sys, moves, &datum)) {  // energy.rs:944-946, accumulate_extra 374-386
      if (bins.extra_count.empty()) {
        bins.extra_count.assign(bins.lnw.size(), 0);
        bins.extra_total.assign(bins.lnw.size(), 0.0);
      }
      bins.extra_count[i] += 1;
      bins.extra_total[i] += datum;
    }
    update_weights(energy);
    if (bins.lnw[i] > max_S) {
      max_S = bins.lnw[i];
      max_S_index = i;
      std::fill(have_visited_since_maxentropy.begin(), have_visited_since_maxentropy.end(), 1);
    } else if (i == max_S_index) {
      if (state_to_index(e1) != i)
        std::fill(have_visited_since_maxentropy.begin(), have_visited_since_maxentropy.end(), 0);
    } else if (!have_visited_since_maxentropy[i]) {
      have_visited_since_maxentropy[i] = 1;
      round_trips[i] += 1;
    }
  }

  double temperature(double energy) const {  // energy.rs:764-795
    size_t i = state_to_index(energy);
    double lnwi = bins.lnw[i];
    double Tlo = 0.0;
    for (size_t j = 0; j < i; ++j) {
      double lnwj = bins.lnw[j];
      if (lnwj > 0.0) {
        double Tj = (energy - index_to_state(j)) / (lnwi - lnwj);
        if (Tj > Tlo) Tlo = Tj;
      }
    }
    double Thi = 1e300;
    for (size_t j = i + 1; j < bins.lnw.size(); ++j) {
      double lnwj = bins.lnw[j];
      if (lnwj > 0.0) {
        double Tj = (energy - index_to_state(j)) / (lnwi - lnwj);
        if (Tj < Thi) Thi = Tj;
      }
    }
    if (Thi > Tlo && Tlo > 0.0) return 0.5 * (Thi + Tlo);
    if (Tlo > 0.0) return Tlo;
    return Thi;
  }
};

// heat_capacity(T, E, S), plotting/final_heat_capacity.py:79-88, in FP64:
// P = exp(b - max b), b = S - E/T; P /= sum P; U = sum E P; C = sum (E-U)^2 P / T^2.
inline void heat_capacity(const double* T, size_t nT, const double* E, const double* S, size_t n,
                          double* C) {
  std::vector<double> P(n);
  for (size_t t = 0; t < nT; ++t) {
    double mx = -INFINITY;
    for (size_t k = 0; k < n; ++k) mx = std::max(mx, S[k] - E[k] / T[t]);
    double Z = 0.0;
    for (size_t k = 0; k < n; ++k) { P[k] = std::exp(S[k] - E[k] / T[t] - mx); Z += P[k]; }
    double U = 0.0;
    for (size_t k = 0; k < n; ++k) { P[k] = P[k] / Z; U += E[k] * P[k]; }
    double c = 0.0;
    for (size_t k = 0; k < n; ++k) { double dE = E[k] - U; c += dE * dE * P[k]; }
    C[t] = c / (T[t] * T[t]);
  }
}

}  // namespace orc
