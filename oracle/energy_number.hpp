// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// FP64 C++ restatement of the energy-number Monte Carlo: grand-canonical add/remove
// moves with flat-histogram weights over (E, N), src/mc/energy_number.rs, for systems
// with the GrandSystem surface (src/system/mod.rs:123-136; Lj lj.rs:291-319).  It
// follows the reference step by step, quirks included:
//  * bins are (E, N) with index (E bin) * (max_N + 1) + N, regrown and remapped on
//    demand (energy_number.rs:225-300); max_S_index is copied, not remapped;
//  * Wang-Landau keeps its histogram in a second set of bins (Method::WL::bins) that
//    grows with the main bins, while ln w and the visited histogram live in the main bins;
//  * the add/remove probability adapts toward the target acceptance rate every t_last
//    moves (energy_number.rs:614-646);
//  * translation scales per N are stored but never adapted.
// The reference's xoroshiro stream is replaced by the Philox draws below (draws_grand,
// add_candidate), shared with the GPU kernel.
#pragma once
#include <cmath>
#include <cstdint>
#include <optional>
#include <vector>

#include "philox_draws.hpp"
#include "systems.hpp"

namespace orc {

// Draws of one energy-number move on Philox stream pair 2 (counter word 2 = 4, 5, 6):
// u_choice (translate iff u_choice > addremove_probability, energy_number.rs:544),
// add_bit (add iff 0, :569), pick (atom to move or remove, mulhi_range(pick, N)), three
// normals (the translation, rng.rs:111-117), u (the Metropolis uniform).
struct GrandDraws {
  double u_choice;
  uint32_t add_bit;
  uint32_t pick;
  float g[3];
  double u;
};
inline GrandDraws draws_grand(uint64_t seed, uint32_t walker, uint64_t t) {
  const uint32_t k0 = walker, k1 = (uint32_t)seed, shi = (uint32_t)(seed >> 32);
  U4 A = philox4x32_10(U4{(uint32_t)t, (uint32_t)(t >> 32), 4u, shi}, k0, k1);
  U4 B = philox4x32_10(U4{(uint32_t)t, (uint32_t)(t >> 32), 5u, shi}, k0, k1);
  U4 C = philox4x32_10(U4{(uint32_t)t, (uint32_t)(t >> 32), 6u, shi}, k0, k1);
  GrandDraws d;
  d.u_choice = u53(A.x, A.y);
  d.add_bit = A.z & 1u;
  d.pick = A.w;
  float z3;
  normal_pair(B.x, B.y, d.g[0], d.g[1]);
  normal_pair(B.z, B.w, d.g[2], z3);
  (void)z3;
  d.u = u53(C.x, C.y);
  return d;
}
// Candidate k of an LJ add: uniform in (-1, 1)^3 (lj.rs:294-302: Uniform::new(-1, 1) per
// component), counter word 2 = 8 + 2k and 9 + 2k.  At most kAddTries candidates; an add
// whose candidates all fall outside the unit ball is impossible (probability ~1e-21).
constexpr int kAddTries = 64;
inline void add_candidate(uint64_t seed, uint32_t walker, uint64_t t, int k, double out[3]) {
  const uint32_t k0 = walker, k1 = (uint32_t)seed, shi = (uint32_t)(seed >> 32);
  U4 D = philox4x32_10(U4{(uint32_t)t, (uint32_t)(t >> 32), 8u + 2u * (uint32_t)k, shi}, k0, k1);
  U4 E = philox4x32_10(U4{(uint32_t)t, (uint32_t)(t >> 32), 9u + 2u * (uint32_t)k, shi}, k0, k1);
  out[0] = -1.0 + 2.0 * u53(D.x, D.y);
  out[1] = -1.0 + 2.0 * u53(D.z, D.w);
  out[2] = -1.0 + 2.0 * u53(E.x, E.y);
}

// A uniform point of the periodic box for a WCA add (wca.rs:309-313: Uniform::new(0, L)
// per axis, then put_in_cell), from the words of add candidate 0.
inline V3 add_point_box(uint64_t seed, uint32_t walker, uint64_t t, const V3& box) {
  const uint32_t k0 = walker, k1 = (uint32_t)seed, shi = (uint32_t)(seed >> 32);
  U4 D = philox4x32_10(U4{(uint32_t)t, (uint32_t)(t >> 32), 8u, shi}, k0, k1);
  U4 E = philox4x32_10(U4{(uint32_t)t, (uint32_t)(t >> 32), 9u, shi}, k0, k1);
  return {box[0] * u53(D.x, D.y), box[1] * u53(D.z, D.w), box[2] * u53(E.x, E.y)};
}

// The system-specific moves of move_once: translation (plan_move), add, remove.
inline std::optional<double> grand_translate(Lj& s, size_t which, const float g[3], double sc) {
  const V3& f = s.pos[which];  // lj.rs:365-374
  return s.move_atom(which, {f[0] + (double)g[0] * sc, f[1] + (double)g[1] * sc, f[2] + (double)g[2] * sc});
}
inline std::optional<double> grand_translate(Wca& s, size_t which, const float g[3], double sc) {
  const V3& f = s.cell.pos[which];  // wca.rs:342-353
  return s.move_atom(which, s.cell.put_in_cell({f[0] + (double)g[0] * sc, f[1] + (double)g[1] * sc,
                                                f[2] + (double)g[2] * sc}));
}
inline std::optional<double> grand_add(Lj& s, uint64_t seed, uint32_t walker, uint64_t t) {
  double c[3];  // lj.rs:292-309
  for (int k = 0; k < kAddTries; ++k) {
    add_candidate(seed, walker, t, k, c);
    if (c[0] * c[0] + c[1] * c[1] + c[2] * c[2] < 1.0) return s.plan_add_at({c[0], c[1], c[2]});
  }
  return std::nullopt;
}
inline std::optional<double> grand_add(Wca& s, uint64_t seed, uint32_t walker, uint64_t t) {
  return s.plan_add_at(s.cell.put_in_cell(add_point_box(seed, walker, t, s.cell.box)));
}

// Bins of energy_number.rs:115-150, 225-300
struct NBins {
  double min = 0, width = 1;
  size_t max_N = 0, num_E = 1;
  std::vector<uint64_t> histogram{1};
  std::vector<double> lnw{0.0};
  std::vector<double> translation_scale{0.05};
  std::vector<uint64_t> num_translation_attempts{0}, num_translation_accepted{0};
  uint64_t num_addremove_attempts = 0, num_addremove_accepted = 0;
  std::vector<uint8_t> visited{0};
  std::vector<uint64_t> round_trips{1};
  double max_S = 0.0;
  size_t max_S_index = 0;
  size_t num_states = 1;
  uint64_t t_last = 1;

  size_t index(double E, size_t N) const {  // state_to_index (energy_number.rs:227-229)
    const double q = (E - min) / width;
    const size_t k = q > 0.0 ? (size_t)q : 0;  // `as usize` saturates at 0
    return k * (max_N + 1) + N;
  }
  double index_E(size_t i) const { return min + ((double)(i / (max_N + 1)) + 0.5) * width; }
  size_t index_N(size_t i) const { return i % (max_N + 1); }
  double emax() const { return min + width * (double)num_E; }
  size_t nbins() const { return num_E * (max_N + 1); }
  bool prepare(double E, size_t N) {  // prepare_for_state (energy_number.rs:249-290)
    if (!(N > max_N || E < min || E >= emax())) return false;
    NBins nb = *this;
    nb.max_N = N > max_N ? N : max_N;
    while (nb.min > E) { nb.min -= width; nb.num_E += 1; }
    while (nb.emax() <= E) nb.num_E += 1;
    const size_t nn = nb.nbins();
    nb.lnw.assign(nn, 0.0);
    nb.histogram.assign(nn, 0);
    nb.translation_scale.assign(nb.max_N + 1, translation_scale[0]);
    nb.num_translation_attempts.assign(nb.max_N + 1, 0);
    nb.num_translation_accepted.assign(nb.max_N + 1, 0);
    nb.visited.assign(nn, 0);
    nb.round_trips.assign(nn, 0);
    for (size_t n = 0; n <= max_N; ++n) {
      nb.translation_scale[n] = translation_scale[n];
      nb.num_translation_attempts[n] = num_translation_attempts[n];
      nb.num_translation_accepted[n] = num_translation_accepted[n];
    }
    for (size_t i = 0; i < lnw.size(); ++i) {
      const size_t j = nb.index(index_E(i), index_N(i));
      nb.lnw[j] = lnw[i];
      nb.histogram[j] = histogram[i];
      nb.visited[j] = visited[i];
      nb.round_trips[j] = round_trips[i];
    }
    *this = nb;
    return true;
  }
};

struct NumberParams {
  int kind = 1;                  // 1 SAMC, 2 WL (MethodParams, energy_number.rs:18-27)
  double t0 = 1e4;
  bool has_energy_bin = false;
  double energy_bin = 1.0;
  bool has_max_N = false;
  size_t max_N = 0;
  bool has_min_allowed = false, has_max_allowed = false;
  double min_allowed = 0, max_allowed = 0;
  bool acc_mode = false;         // MoveParams::AcceptanceRate(target) or _Explicit
  double target_rate = 0.5;
  double translation_scale = 0.05, addremove_probability = 0.05;
};

template <class S>
struct EnergyNumberMC {
  S sys;
  int kind = 1;
  double t0 = 1e4;
  double gamma_wl = 1.0;
  uint64_t lowest_hist = 1, highest_hist = 1, total_hist = 0;
  NBins wl;                      // Method::WL::bins (its histogram)
  uint64_t moves = 0, accepted = 0;
  NBins bins;
  bool acc_mode = false;
  double target_rate = 0.5, addremove_probability = 0.05;
  bool has_max_N = false;
  size_t max_N = 0;
  bool has_min_allowed = false, has_max_allowed = false;
  double min_allowed = 0, max_allowed = 0;
  uint64_t seed = 0;
  uint32_t walker = 0;
  // trace replay (as EnergyMC): energies given per move replace the own ones
  const double* e1_override = nullptr;
  const double* e2_override = nullptr;
  uint64_t override_base = 0;
  uint64_t override_mismatch = 0;
  double max_e2_discrepancy = 0.0;
  double worst[4] = {0, 0, 0, 0};

  // from_params (energy_number.rs:474-533) on an empty system
  void init(S system, const NumberParams& p, uint64_t seed_, uint32_t walker_) {
    sys = std::move(system);
    seed = seed_;
    walker = walker_;
    const double w = p.has_energy_bin ? p.energy_bin : 1.0;
    bins = NBins{};
    bins.min = sys.energy() - w * 0.5;
    bins.width = w;
    bins.translation_scale = {p.acc_mode ? 0.05 : p.translation_scale};
    kind = p.kind;
    t0 = p.t0;
    wl = NBins{};
    wl.min = sys.energy() - w * 0.5;
    wl.width = w;
    wl.visited = {0};
    bins.visited = {0};
    gamma_wl = 1.0;
    lowest_hist = 1;
    highest_hist = 1;
    total_hist = 0;
    acc_mode = p.acc_mode;
    target_rate = p.target_rate;
    addremove_probability = p.acc_mode ? 0.5 : p.addremove_probability;
    has_max_N = p.has_max_N;
    max_N = p.max_N;
    has_min_allowed = p.has_min_allowed;
    has_max_allowed = p.has_max_allowed;
    min_allowed = p.min_allowed;
    max_allowed = p.max_allowed;
  }
  double gamma() const {  // energy_number.rs:436-449
    if (kind == 1) {
      const double t = (double)moves;
      return t > t0 ? t0 / t : 1.0;
    }
    return gamma_wl;
  }
  // reject_move (energy_number.rs:314-355)
  bool reject_move(double E1, size_t N1, double E2, size_t N2, double u) {
    const size_t i1 = bins.index(E1, N1), i2 = bins.index(E2, N2);
    if (kind == 2) {
      if (wl.prepare(E2, N2)) {
        if (gamma_wl != 1.0 || wl.histogram.empty()) {
          gamma_wl = 1.0;
          lowest_hist = 0;
          highest_hist = 0;
          total_hist = 0;
        }
      }
    }
    const double lnw1 = bins.lnw[i1], lnw2 = bins.lnw[i2];
    return lnw2 > lnw1 && u > std::exp(lnw1 - lnw2);
  }
  // update_weights (energy_number.rs:357-413)
  void update_weights(double E, size_t N) {
    const size_t i = bins.index(E, N);
    const double g = gamma();
    bins.lnw[i] += g;
    if (kind != 2) return;
    const double num_states = (double)bins.num_states;
    wl.histogram[i] += 1;
    if (wl.histogram[i] > highest_hist) highest_hist = wl.histogram[i];
    total_hist += 1;
    if (wl.histogram[i] == lowest_hist + 1) {
      bool any = false;
      uint64_t mn = 0;
      for (size_t j = 0; j < wl.histogram.size(); ++j) {
        if (bins.histogram[j] == 0) continue;
        if (!any || wl.histogram[j] < mn) mn = wl.histogram[j];
        any = true;
      }
      if (any && mn == lowest_hist + 1) {
        lowest_hist = wl.histogram[i];
        if (wl.histogram.size() > 1 && (double)lowest_hist >= 0.8 * (double)total_hist / num_states) {
          gamma_wl *= 0.5;
          for (auto& x : wl.histogram) x = 0;
          total_hist = 0;
          lowest_hist = 0;
        }
      }
    }
  }
  bool oob(double e2, double e1) const {
    bool o = false;
    if (has_max_allowed) o = e2 > max_allowed && e2 > e1;
    if (has_min_allowed) o = o || (e2 < min_allowed && e2 < e1);
    return o;
  }
  // e2 of a proposal: the own one, or the given one in trace replay
  double given(double own) {
    if (!e2_override) return own;
    const double ge2 = e2_override[moves - 1 - override_base];
    if (std::isnan(ge2)) { ++override_mismatch; return own; }
    const double dd = std::fabs(ge2 - own) / (1e-3 + sys.last_abs);
    if (dd > max_e2_discrepancy) {
      max_e2_discrepancy = dd;
      worst[0] = (double)moves; worst[1] = ge2; worst[2] = own; worst[3] = sys.last_abs;
    }
    return ge2;
  }
  void impossible() {
    if (e2_override && !std::isnan(e2_override[moves - 1 - override_base])) ++override_mismatch;
  }
  // move_once (energy_number.rs:540-666)
  void move_once() {
    moves += 1;
    if (e1_override) sys.E = e1_override[moves - 1 - override_base];
    const GrandDraws d = draws_grand(seed, walker, moves);
    const double E1 = sys.energy();
    const size_t N1 = sys.num_atoms();
    if (d.u_choice > addremove_probability) {
      bins.num_translation_attempts[N1] += 1;
      std::optional<double> e2;
      if (N1 > 0)
        e2 = grand_translate(sys, mulhi_range(d.pick, (uint32_t)N1), d.g, bins.translation_scale[N1]);
      if (e2) {
        const double E2 = given(*e2);
        if (!oob(E2, E1)) {
          bins.prepare(E2, N1);
          if (!reject_move(E1, N1, E2, N1, d.u)) {
            accepted += 1;
            bins.num_translation_accepted[N1] += 1;
            sys.ch_e = E2;
            sys.confirm();
          }
        }
      } else {
        impossible();
      }
    } else {
      bins.num_addremove_attempts += 1;
      std::optional<double> e2;
      size_t N2 = 0;
      if (d.add_bit == 0) {
        if (!(has_max_N && N1 == max_N)) {
          e2 = grand_add(sys, seed, walker, moves);
          N2 = N1 + 1;
        }
      } else if (N1 > 0) {
        e2 = sys.plan_remove(mulhi_range(d.pick, (uint32_t)N1));
        N2 = N1 - 1;
      }
      if (e2) {
        const double E2 = given(*e2);
        if (!oob(E2, E1)) {
          bins.prepare(E2, N2);
          if (!reject_move(E1, N1, E2, N2, d.u)) {
            accepted += 1;
            bins.num_addremove_accepted += 1;
            sys.ch_e = E2;
            sys.confirm();
          }
        }
      } else {
        impossible();
      }
    }
    const double E = sys.energy();
    const size_t N = sys.num_atoms();
    const size_t i = bins.index(E, N);
    if (bins.histogram[i] == 0) {
      bins.num_states += 1;
      bins.t_last = moves;
    }
    if (moves % bins.t_last == 0 && acc_mode) {  // energy_number.rs:614-646
      const double acc_ar = (double)bins.num_addremove_accepted / (double)bins.num_addremove_attempts;
      const double acc_tr = (double)(accepted - bins.num_addremove_accepted) /
                            (double)(moves - bins.num_addremove_attempts);
      const double new_p = (target_rate - acc_tr) / (acc_ar - acc_tr);
      if (!std::isnan(new_p)) addremove_probability = new_p > 0.999 ? 0.999 : new_p;
    }
    bins.histogram[i] += 1;
    update_weights(E, N);
    if (bins.lnw[i] > bins.max_S) {  // energy_number.rs:651-664
      bins.max_S = bins.lnw[i];
      bins.max_S_index = i;
      for (auto& v : bins.visited) v = 1;
    } else if (i == bins.max_S_index) {
      if (bins.index(E1, N1) != i)
        for (auto& v : bins.visited) v = 0;
    } else if (!bins.visited[i]) {
      bins.visited[i] = 1;
      bins.round_trips[i] += 1;
    }
  }
};

}  // namespace orc
