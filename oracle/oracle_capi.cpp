// ORACLE / TEST INFRASTRUCTURE ONLY.  ctypes-facing C API over the FP64 restatement
// (systems.hpp, energy_mc.hpp).  Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg load this library; the CUDA product never links it.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "energy_mc.hpp"
#include "energy_number.hpp"
#include "systems.hpp"

using namespace orc;

extern "C" {

struct orc_config {
  int32_t system;        // 0 Ising, 1 LJ cluster, 2 WCA, 3 square well / hard core
  int32_t n;             // atoms (or L for Ising)
  double radius;         // LJ spherical wall
  double box[3];         // WCA / square-well periodic box
  double well_width;     // square-well lambda (cell r_cutoff); WCA uses 2^(1/6)
  int32_t method;        // MethodKind
  double min_T, t0;
  int32_t has_min_gamma;
  double min_gamma, T;
  uint64_t seed;
  uint32_t walker;
  int32_t has_energy_bin;
  double energy_bin;
  int32_t has_min_allowed, has_max_allowed;
  double min_allowed, max_allowed;
  int32_t acceptance_rate_mode;
  double target_rate, translation_scale;
  uint64_t descent_limit;
  int32_t has_e0;        // start the flat-histogram run from this energy (after descent)
  double e0;             // e.g. the GPU's FP64 re-sum, summed in a different order
};

}  // extern "C"

namespace {

struct AnyMC {
  int32_t kind;
  uint64_t seed;
  uint32_t walker;
  uint32_t n;
  std::unique_ptr<EnergyMC<Ising>> ising;
  std::unique_ptr<EnergyMC<Lj>> lj;
  std::unique_ptr<EnergyMC<Wca>> wca;
  std::unique_ptr<EnergyMC<SquareWell>> sw;
  template <class F>
  auto visit(F&& f) {
    switch (kind) {
      case 0: return f(*ising);
      case 1: return f(*lj);
      case 2: return f(*wca);
      default: return f(*sw);
    }
  }
};

MCParams to_params(const orc_config* c) {
  MCParams p;
  p.method.kind = c->method;
  p.method.min_T = c->min_T;
  p.method.t0 = c->t0;
  p.method.has_min_gamma = c->has_min_gamma != 0;
  p.method.min_gamma = c->min_gamma;
  p.method.T = c->T;
  p.seed = c->seed;
  p.has_energy_bin = c->has_energy_bin != 0;
  p.energy_bin = c->energy_bin;
  p.has_min_allowed = c->has_min_allowed != 0;
  p.has_max_allowed = c->has_max_allowed != 0;
  p.min_allowed = c->min_allowed;
  p.max_allowed = c->max_allowed;
  p.acceptance_rate_mode = c->acceptance_rate_mode != 0;
  p.target_rate = c->target_rate;
  p.translation_scale = c->translation_scale;
  p.walker = c->walker;
  p.has_e0 = c->has_e0 != 0;
  p.e0 = c->e0;
  return p;
}

Cell make_cell(const double box[3], double rc, const double* pos, int n) {
  Cell cell;
  cell.box = {box[0], box[1], box[2]};
  cell.r_cutoff = rc;
  cell.pos.clear();
  cell.update_caches();
  for (int k = 0; k < n; ++k) cell.add_atom_at({pos[3 * k], pos[3 * k + 1], pos[3 * k + 2]});
  return cell;
}

}  // namespace

extern "C" {

void* orc_create(const orc_config* c, const double* state) {
  auto* h = new AnyMC();
  h->kind = c->system;
  h->seed = c->seed;
  h->walker = c->walker;
  h->n = (uint32_t)c->n;
  MCParams p = to_params(c);
  uint64_t seed = c->seed;
  uint32_t walker = c->walker;
  uint64_t dl = c->descent_limit ? c->descent_limit : 100000000ull;
  if (c->system == 0) {
    Ising s;
    s.L = c->n;
    s.S.resize((size_t)c->n * c->n);
    for (size_t k = 0; k < s.S.size(); ++k) s.S[k] = (int8_t)(state[k] > 0 ? 1 : -1);
    s.E = s.compute_energy();
    uint32_t L = (uint32_t)c->n;
    h->ising.reset(new EnergyMC<Ising>());
    h->ising->init(std::move(s), p, [seed, walker, L](uint64_t t, uint32_t stream) {
      return draws_ising(seed, walker, t, L, stream);
    }, dl);
    h->ising->use_philox(seed, walker, L, true);
  } else {
    uint32_t n = (uint32_t)c->n;
    auto src = [seed, walker, n](uint64_t t, uint32_t stream) {
      return draws_continuous(seed, walker, t, n, stream);
    };
    if (c->system == 1) {
      Lj s;
      s.pos.resize(n);
      for (uint32_t k = 0; k < n; ++k) s.pos[k] = {state[3 * k], state[3 * k + 1], state[3 * k + 2]};
      s.max_radius_squared = c->radius * c->radius;
      s.max_radius = c->radius;
      s.E = s.compute_energy();
      h->lj.reset(new EnergyMC<Lj>());
      h->lj->init(std::move(s), p, src, dl);
      h->lj->use_philox(seed, walker, n, false);
    } else if (c->system == 2) {
      Wca s;
      s.cell = make_cell(c->box, wca_r_cutoff(), state, c->n);
      s.E = s.compute_energy();
      h->wca.reset(new EnergyMC<Wca>());
      h->wca->init(std::move(s), p, src, dl);
      h->wca->use_philox(seed, walker, n, false);
    } else {
      SquareWell s;
      s.cell = make_cell(c->box, c->well_width, state, c->n);
      s.E = s.compute_energy();
      h->sw.reset(new EnergyMC<SquareWell>());
      h->sw->init(std::move(s), p, src, dl);
      h->sw->use_philox(seed, walker, n, false);
    }
  }
  return h;
}

void orc_destroy(void* h) { delete (AnyMC*)h; }

void orc_run(void* hv, uint64_t nmoves) {
  auto* h = (AnyMC*)hv;
  h->visit([&](auto& mc) { for (uint64_t k = 0; k < nmoves; ++k) mc.move_once(); return 0; });
}

// Replay of a GPU trace: e1[k] (energy at move start) and e2[k] (proposed energy,
// NaN when impossible) belong to move (moves_at_call + k + 1).  Returns the largest
// |e2_gpu - e2_oracle| / (1e-3 + sum |pair terms|); *mismatch counts moves whose
// possibility differed.
double orc_run_override(void* hv, uint64_t nmoves, const double* e1, const double* e2,
                        uint64_t* mismatch) {
  auto* h = (AnyMC*)hv;
  return h->visit([&](auto& mc) {
    mc.e1_override = e1;
    mc.e2_override = e2;
    mc.override_base = mc.moves;
    mc.max_e2_discrepancy = 0.0;
    mc.override_mismatch = 0;
    for (uint64_t k = 0; k < nmoves; ++k) mc.move_once();
    mc.e1_override = nullptr;
    mc.e2_override = nullptr;
    if (mismatch) *mismatch = mc.override_mismatch;
    return mc.max_e2_discrepancy;
  });
}

// Replay of a traced delayed-acceptance run (sadmc_da.cu): as orc_run_override, with the
// GPU surrogate's energy change ds[k] of each move; e2[k] is NaN for moves the first stage
// screened out.  The oracle takes both stages' decisions itself from its own FP64 ln w.
double orc_run_override_da(void* hv, uint64_t nmoves, const double* e1, const double* e2,
                           const float* ds, uint64_t* mismatch) {
  auto* h = (AnyMC*)hv;
  const uint64_t seed = h->seed;
  const uint32_t walker = h->walker;
  return h->visit([&](auto& mc) {
    mc.e1_override = e1;
    mc.e2_override = e2;
    mc.da_ds = ds;
    mc.da_u2 = [seed, walker](uint64_t t) {  // counter word 2 = 4 of the move's counter
      U4 U = philox4x32_10(U4{(uint32_t)t, (uint32_t)(t >> 32), 4u, (uint32_t)(seed >> 32)}, walker,
                           (uint32_t)seed);
      return u53(U.x, U.y);
    };
    mc.override_base = mc.moves;
    mc.max_e2_discrepancy = 0.0;
    mc.override_mismatch = 0;
    for (uint64_t k = 0; k < nmoves; ++k) mc.move_once();
    mc.e1_override = nullptr;
    mc.e2_override = nullptr;
    mc.da_ds = nullptr;
    if (mismatch) *mismatch = mc.override_mismatch;
    return mc.max_e2_discrepancy;
  });
}

// The "pressure" BinCounts of the bins (empty unless the system collects it).
int64_t orc_extra(void* hv, uint64_t* count, double* total) {
  return ((AnyMC*)hv)->visit([&](auto& mc) {
    const size_t n = mc.bins.extra_count.size();
    for (size_t k = 0; k < n; ++k) {
      if (count) count[k] = mc.bins.extra_count[k];
      if (total) total[k] = mc.bins.extra_total[k];
    }
    return (int64_t)n;
  });
}

void orc_override_worst(void* hv, double* out4) {
  ((AnyMC*)hv)->visit([&](auto& mc) { for (int k = 0; k < 4; ++k) out4[k] = mc.worst[k]; return 0; });
}

double orc_energy(void* hv) { return ((AnyMC*)hv)->visit([](auto& mc) { return mc.sys.energy(); }); }
double orc_compute_energy(void* hv) {
  return ((AnyMC*)hv)->visit([](auto& mc) { return mc.sys.compute_energy(); });
}
int orc_verify_energy(void* hv) {
  return ((AnyMC*)hv)->visit([](auto& mc) { return mc.sys.verify_energy() ? 1 : 0; });
}

void orc_get_state(void* hv, double* out) {
  auto* h = (AnyMC*)hv;
  if (h->kind == 0) {
    auto& S = h->ising->sys.S;
    for (size_t k = 0; k < S.size(); ++k) out[k] = S[k];
    return;
  }
  const std::vector<V3>* pos = h->kind == 1 ? &h->lj->sys.pos
                               : h->kind == 2 ? &h->wca->sys.cell.pos
                                              : &h->sw->sys.cell.pos;
  for (size_t k = 0; k < pos->size(); ++k)
    for (int a = 0; a < 3; ++a) out[3 * k + a] = (*pos)[k][a];
}

// plan_move with an injected proposal (the parity hook that mirrors plan_move).
int orc_plan_move(void* hv, uint32_t which, uint32_t j, double g0, double g1, double g2,
                  double scale, double* e_out) {
  auto* h = (AnyMC*)hv;
  Draws d;
  d.which = which;
  d.j = j;
  d.g[0] = (float)g0;
  d.g[1] = (float)g1;
  d.g[2] = (float)g2;
  d.u = 0.0;
  return h->visit([&](auto& mc) {
    auto e = mc.sys.plan_move(d, scale);
    if (!e) return 0;
    *e_out = *e;
    return 1;
  });
}
void orc_confirm(void* hv) { ((AnyMC*)hv)->visit([](auto& mc) { mc.sys.confirm(); return 0; }); }

int64_t orc_nbins(void* hv) {
  return ((AnyMC*)hv)->visit([](auto& mc) { return (int64_t)mc.bins.lnw.size(); });
}
void orc_get_bins(void* hv, double* lnw, uint64_t* hist, uint64_t* tfound, double* sumE,
                  double* sumE2, uint64_t* round_trips, uint8_t* visited, double* min_width) {
  ((AnyMC*)hv)->visit([&](auto& mc) {
    size_t n = mc.bins.lnw.size();
    for (size_t k = 0; k < n; ++k) {
      lnw[k] = mc.bins.lnw[k];
      hist[k] = mc.bins.histogram[k];
      tfound[k] = mc.bins.t_found[k];
      sumE[k] = mc.bins.energy_total[k];
      sumE2[k] = mc.bins.energy_squared_total[k];
      round_trips[k] = mc.round_trips[k];
      visited[k] = (uint8_t)mc.have_visited_since_maxentropy[k];
    }
    min_width[0] = mc.bins.min;
    min_width[1] = mc.bins.width;
    return 0;
  });
}
int64_t orc_wl_hist(void* hv, uint64_t* out, double* min_energy) {
  return ((AnyMC*)hv)->visit([&](auto& mc) {
    if (out)
      for (size_t k = 0; k < mc.method.hist.size(); ++k) out[k] = mc.method.hist[k];
    if (min_energy) *min_energy = mc.method.min_energy;
    return (int64_t)mc.method.hist.size();
  });
}

// Scalar state, in a fixed order (see ORC_SCALARS in tests/oracle.py).
void orc_get_scalars(void* hv, double* o) {
  ((AnyMC*)hv)->visit([&](auto& mc) {
    const Method& m = mc.method;
    double v[] = {(double)mc.moves, (double)mc.accepted_moves, mc.acceptance_rate,
                  mc.translation_scale, (double)m.kind, m.too_lo, m.too_hi, (double)m.tL,
                  (double)m.tF, (double)m.num_states, (double)m.highest_hist,
                  m.latest_parameter, m.gamma, (double)m.lowest_hist,
                  (double)m.wl_highest_hist, (double)m.total_hist, m.wl_num_states,
                  m.min_energy, m.t0, mc.max_S, (double)mc.max_S_index,
                  (double)mc.verify_failures, mc.nan_gamma ? 1.0 : 0.0, mc.sys.energy()};
    std::memcpy(o, v, sizeof(v));
    return 0;
  });
}

double orc_temperature(void* hv, double e) {
  return ((AnyMC*)hv)->visit([&](auto& mc) { return mc.temperature(e); });
}

double orc_pressure(void* hv) {
  auto* h = (AnyMC*)hv;
  return h->kind == 2 ? h->wca->sys.pressure() : 0.0;
}

// ---- RNG and math helpers for cross-checking the GPU implementation ----
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  U4 r = philox4x32_10(U4{ctr[0], ctr[1], ctr[2], ctr[3]}, key[0], key[1]);
  out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
}
void orc_draws(int32_t system, uint32_t n, uint64_t seed, uint32_t walker, uint64_t t,
               uint32_t stream_pair, uint32_t* idx2, float* g3, double* u) {
  Draws d = system == 0 ? draws_ising(seed, walker, t, n)
                        : draws_continuous(seed, walker, t, n, stream_pair);
  idx2[0] = d.which;
  idx2[1] = d.j;
  g3[0] = d.g[0]; g3[1] = d.g[1]; g3[2] = d.g[2];
  *u = d.u;
}
void orc_normal_pairs(const uint32_t* a, const uint32_t* b, size_t n, float* z0, float* z1) {
  for (size_t k = 0; k < n; ++k) normal_pair(a[k], b[k], z0[k], z1[k]);
}
void orc_heat_capacity(const double* T, size_t nT, const double* E, const double* S, size_t n,
                       double* C) {
  heat_capacity(T, nT, E, S, n, C);
}
uint64_t orc_max_balls_within(double d) { return max_balls_within(d); }
double orc_lj_potential(double r2) { return lj_potential(r2); }
double orc_wca_potential(double r2) { return wca_potential(r2); }

// ---- The reference's own invariant tests, run on this restatement ----
// ising.rs:125-147: after every planned+confirmed flip, energy() == compute_energy().
int64_t orc_selftest_ising(int32_t L, uint64_t flips, uint64_t seed) {
  Ising s;
  s.L = L;
  s.S.resize((size_t)L * L);
  for (size_t k = 0; k < s.S.size(); ++k) {
    U4 r = philox4x32_10(U4{(uint32_t)k, 0, 7, 0}, 10137u, (uint32_t)seed);
    s.S[k] = (int8_t)((r.x & 1) * 2 - 1);
  }
  s.E = s.compute_energy();
  int64_t bad = s.E == s.compute_energy() ? 0 : 1;
  for (uint64_t t = 1; t <= flips; ++t) {
    Draws d = draws_ising(seed, 0, t, (uint32_t)L);
    s.plan_move(d, 0.0);
    s.confirm();
    if (s.energy() != s.compute_energy()) ++bad;
  }
  return bad;
}

// Reference-style initial configurations, restated with the Philox stream.
// Lj::from (lj.rs:126-204): uniform in the ball, centred, retried until E < 0, then relaxed.
int orc_init_lj(int32_t n, double radius, uint64_t seed, double* out) {
  Lj lj;
  lj.max_radius_squared = radius * radius;
  uint64_t ctr = 0;
  auto unif = [&](uint32_t stream) {
    U4 r = philox4x32_10(U4{(uint32_t)ctr, (uint32_t)(ctr >> 32), stream, 0}, 0xC1u, (uint32_t)seed);
    ++ctr;
    return -1.0 + 2.0 * u53(r.x, r.y);
  };
  double best = 1e80;
  std::vector<V3> best_pos;
  for (int attempt = 0; attempt < 100000; ++attempt) {
    std::vector<V3> pos;
    for (int k = 0; k < n; ++k) {
      V3 r;
      do { r = {unif(3), unif(3), unif(3)}; } while (!(norm2(r) < 1.0));
      pos.push_back({r[0] * radius, r[1] * radius, r[2] * radius});
    }
    V3 cm = pos[0];
    for (int k = 1; k < n; ++k) cm = {cm[0] + pos[k][0], cm[1] + pos[k][1], cm[2] + pos[k][2]};
    cm = {cm[0] / n, cm[1] / n, cm[2] / n};
    bool outside = false;
    for (auto& x : pos) {
      x = sub(x, cm);
      if (norm2(x) > radius * radius) outside = true;
    }
    if (outside) continue;
    lj.pos = pos;
    lj.E = lj.compute_energy();
    if (lj.E < best) { best = lj.E; best_pos = lj.pos; }
    if (lj.E < 0.0) break;
  }
  lj.pos = best_pos;
  lj.E = best;
  for (uint64_t t = 1; t <= 100000000ull && lj.E >= 0.0; ++t) {
    Draws d = draws_continuous(seed, 0xFFFFu, t, (uint32_t)n, 1);
    auto e = lj.plan_move(d, 0.03);
    if (e && *e < lj.E) lj.confirm();
  }
  for (int k = 0; k < n; ++k)
    for (int a = 0; a < 3; ++a) out[3 * k + a] = lj.pos[k][a];
  return lj.E < 0.0 ? 1 : 0;
}

// SquareWell::from(SquareWellNParams) (optsquare.rs:357-435): random FCC spots, no jitter.
int orc_init_sw_fcc(int32_t n, double filling_fraction, double well_width, uint64_t seed,
                    double* box_out, double* out) {
  const double PI = 3.141592653589793;
  double vol = (double)n * (PI * 1.0 * 1.0 * 1.0 / 6.0) / filling_fraction;
  double w = std::cbrt(vol);
  double box[3] = {w, w, w};
  double min_cell_width = 2.0 * std::sqrt(2.0) * 0.5;
  size_t cells[3];
  double cw[3];
  for (int a = 0; a < 3; ++a) {
    cells[a] = (size_t)(box[a] / min_cell_width);
    cw[a] = box[a] / (double)cells[a];
  }
  size_t total = 4 * cells[0] * cells[1] * cells[1];
  if (total < (size_t)n) return 0;
  V3 off[4] = {{0, 0, 0}, {0, cw[1] / 2.0, cw[2] / 2.0}, {cw[0] / 2.0, 0, cw[2] / 2.0},
               {cw[0] / 2.0, cw[1] / 2.0, 0}};
  std::vector<char> reserved(cells[0] * cells[1] * cells[2] * 4, 0);
  uint64_t ctr = 0;
  auto pick = [&](size_t m) {
    U4 r = philox4x32_10(U4{(uint32_t)ctr, (uint32_t)(ctr >> 32), 5, 0}, 0x5Au, (uint32_t)seed);
    ++ctr;
    return (size_t)mulhi_range(r.x, (uint32_t)m);
  };
  SquareWell sw;
  sw.cell.box = {box[0], box[1], box[2]};
  sw.cell.r_cutoff = well_width;
  sw.cell.update_caches();
  for (int k = 0; k < n; ++k) {
    for (;;) {
      size_t i = pick(cells[0]), j = pick(cells[1]), kk = pick(cells[2]), l = pick(4);
      size_t id = ((i * cells[1] + j) * cells[2] + kk) * 4 + l;
      if (!reserved[id]) {
        reserved[id] = 1;
        V3 r = {(double)i * cw[0] + off[l][0], (double)j * cw[1] + off[l][1],
                (double)kk * cw[2] + off[l][2]};
        if (!sw.add_atom_at(r)) return 0;
        break;
      }
    }
  }
  for (int a = 0; a < 3; ++a) box_out[a] = box[a];
  for (int k = 0; k < n; ++k)
    for (int a = 0; a < 3; ++a) out[3 * k + a] = sw.cell.pos[k][a];
  return 1;
}

// lj.rs:381-427 / wca.rs:647-694 / optsquare.rs:585-618: after each planned move that is
// confirmed, the incremental energy passes verify_energy (exact for the square well).
int64_t orc_selftest_moves(void* hv, uint64_t nmoves, double scale, double maxe_per_atom,
                           uint64_t seed) {
  auto* h = (AnyMC*)hv;
  int64_t bad = 0;
  h->visit([&](auto& mc) {
    double maxe = (double)h->n * maxe_per_atom;
    double old_e = mc.sys.energy();
    uint64_t done = 0;
    for (uint64_t t = 1; done < nmoves && t < 100 * nmoves; ++t) {
      Draws d = draws_continuous(seed, 0xABCDu, t, h->n, 0);
      auto e = mc.sys.plan_move(d, scale);
      if (!e) continue;
      if (h->kind == 3 || *e < maxe || *e < old_e) {
        mc.sys.confirm();
        if (!mc.sys.verify_energy()) ++bad;
        old_e = *e;
        ++done;
      }
    }
    return 0;
  });
  return bad;
}

// optcell tests (wca.rs:500-583, optsquare.rs:438-521): the three minimum-image
// variants agree bit for bit, and every candidate image equals the minimum image.
int64_t orc_selftest_cell(void* hv) {
  auto* h = (AnyMC*)hv;
  const Cell* cell = h->kind == 2 ? &h->wca->sys.cell : h->kind == 3 ? &h->sw->sys.cell : nullptr;
  if (!cell) return -1;
  int64_t bad = 0;
  for (const V3& r1 : cell->pos)
    for (const V3& r2 : cell->pos) {
      double a = cell->closest_distance2(r1, r2);
      if (a != cell->unsafe_closest_distance2(r1, r2)) ++bad;
      if (a != cell->sloppy_closest_distance2(r1, r2)) ++bad;
    }
  for (size_t w = 0; w < cell->pos.size(); ++w) {
    const V3 r1 = cell->pos[w];
    cell->for_each_candidate(r1, w, [&](const V3& r2) {
      double a = cell->closest_distance2(r1, r2);
      if (a != norm2(sub(r1, r2))) ++bad;
      if (a != cell->unsafe_closest_distance2(r1, r2)) ++bad;
      return true;
    });
  }
  return bad;
}

// ---- CPU baseline: W walkers x K moves on `threads` host threads ----
double orc_bench(const orc_config* cfgs, const double* const* states, int32_t nwalkers,
                 uint64_t moves, int32_t threads, uint64_t* total_moves, uint64_t* total_accepted) {
  std::vector<void*> hs(nwalkers);
  for (int w = 0; w < nwalkers; ++w) hs[w] = orc_create(&cfgs[w], states[w]);
  std::atomic<int> next{0};
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&]() {
      for (int w; (w = next.fetch_add(1)) < nwalkers;) orc_run(hs[w], moves);
    });
  for (auto& th : pool) th.join();
  auto t1 = std::chrono::steady_clock::now();
  uint64_t tm = 0, ta = 0;
  for (int w = 0; w < nwalkers; ++w) {
    double s[24];
    orc_get_scalars(hs[w], s);
    tm += (uint64_t)s[0];
    ta += (uint64_t)s[1];
    orc_destroy(hs[w]);
  }
  *total_moves = tm;
  *total_accepted = ta;
  return std::chrono::duration<double>(t1 - t0).count();
}


// ---- energy-number MC (grand-canonical LJ cluster / WCA fluid), src/mc/energy_number.rs
typedef struct orc_grand_config {
  int32_t kind;            // 1 SAMC, 2 WL
  int32_t has_energy_bin;
  double t0;
  double energy_bin;
  int32_t has_max_N, max_N;
  int32_t has_min_allowed, has_max_allowed;
  double min_allowed, max_allowed;
  int32_t acc_mode, system;  // system: 1 LJ cluster, 2 WCA fluid
  double target_rate, translation_scale, addremove_probability;
  double radius;           // LJ
  double box[3];           // WCA
  uint64_t seed;
  uint32_t walker, pad2;
} orc_grand_config;

}  // extern "C"

namespace {
inline const std::vector<V3>& grand_positions(const Lj& s) { return s.pos; }
inline const std::vector<V3>& grand_positions(const Wca& s) { return s.cell.pos; }
struct AnyGrand {
  int system = 1;
  std::unique_ptr<EnergyNumberMC<Lj>> lj;
  std::unique_ptr<EnergyNumberMC<Wca>> wca;
  template <class F>
  auto visit(F&& f) { return system == 1 ? f(*lj) : f(*wca); }
};
}  // namespace

extern "C" {

void* orc_grand_create(const orc_grand_config* c) {
  NumberParams p;
  p.kind = c->kind;
  p.t0 = c->t0;
  p.has_energy_bin = c->has_energy_bin != 0;
  p.energy_bin = c->energy_bin;
  p.has_max_N = c->has_max_N != 0;
  p.max_N = (size_t)c->max_N;
  p.has_min_allowed = c->has_min_allowed != 0;
  p.has_max_allowed = c->has_max_allowed != 0;
  p.min_allowed = c->min_allowed;
  p.max_allowed = c->max_allowed;
  p.acc_mode = c->acc_mode != 0;
  p.target_rate = c->target_rate;
  p.translation_scale = c->translation_scale;
  p.addremove_probability = c->addremove_probability;
  auto* h = new AnyGrand();
  h->system = c->system == 2 ? 2 : 1;
  if (h->system == 1) {
    Lj s;
    s.max_radius_squared = c->radius * c->radius;
    s.max_radius = c->radius;
    s.E = 0.0;
    h->lj.reset(new EnergyNumberMC<Lj>());
    h->lj->init(std::move(s), p, c->seed, c->walker);
  } else {
    Wca s;  // wca.rs:368-390 on an empty box
    s.cell.box = {c->box[0], c->box[1], c->box[2]};
    s.cell.r_cutoff = wca_r_cutoff();
    s.cell.update_caches();
    s.E = 0.0;
    h->wca.reset(new EnergyNumberMC<Wca>());
    h->wca->init(std::move(s), p, c->seed, c->walker);
  }
  return h;
}
void orc_grand_destroy(void* h) { delete (AnyGrand*)h; }
void orc_grand_run(void* h, uint64_t n) {
  ((AnyGrand*)h)->visit([&](auto& mc) {
    for (uint64_t k = 0; k < n; ++k) mc.move_once();
    return 0;
  });
}
double orc_grand_run_override(void* h, uint64_t n, const double* e1, const double* e2,
                              uint64_t* mismatch) {
  return ((AnyGrand*)h)->visit([&](auto& mc) {
    mc.e1_override = e1;
    mc.e2_override = e2;
    mc.override_base = mc.moves;
    for (uint64_t k = 0; k < n; ++k) mc.move_once();
    mc.e1_override = mc.e2_override = nullptr;
    if (mismatch) *mismatch = mc.override_mismatch;
    return mc.max_e2_discrepancy;
  });
}
void orc_grand_worst(void* h, double* out4) {
  ((AnyGrand*)h)->visit([&](auto& mc) {
    for (int k = 0; k < 4; ++k) out4[k] = mc.worst[k];
    return 0;
  });
}
int64_t orc_grand_state(void* h, double* pos) {
  return ((AnyGrand*)h)->visit([&](auto& mc) {
    const auto& P = grand_positions(mc.sys);
    if (pos)
      for (size_t i = 0; i < P.size(); ++i)
        for (int a = 0; a < 3; ++a) pos[3 * i + a] = P[i][a];
    return (int64_t)P.size();
  });
}
double orc_grand_compute_energy(void* h) {
  return ((AnyGrand*)h)->visit([&](auto& mc) { return mc.sys.compute_energy(); });
}
// moves, accepted, addremove_probability, N, E, num_states, t_last, gamma (WL), lowest,
// highest, total (WL), max_S, max_S_index, bins.min, width, max_N, num_E, add/remove
// attempts, add/remove accepted
void orc_grand_scalars(void* h, double* o) {
  ((AnyGrand*)h)->visit([&](auto& mc) {
    const NBins& b = mc.bins;
    const double v[19] = {(double)mc.moves, (double)mc.accepted, mc.addremove_probability,
                          (double)mc.sys.num_atoms(), mc.sys.E, (double)b.num_states,
                          (double)b.t_last, mc.gamma_wl, (double)mc.lowest_hist,
                          (double)mc.highest_hist, (double)mc.total_hist, b.max_S,
                          (double)b.max_S_index, b.min, b.width, (double)b.max_N,
                          (double)b.num_E, (double)b.num_addremove_attempts,
                          (double)b.num_addremove_accepted};
    for (int k = 0; k < 19; ++k) o[k] = v[k];
    return 0;
  });
}
// The bins in the reference's layout (index E bin * (max_N + 1) + N); returns their count.
int64_t orc_grand_bins(void* h, double* lnw, uint64_t* hist, uint64_t* wl_hist, uint8_t* visited,
                       uint64_t* round_trips) {
  return ((AnyGrand*)h)->visit([&](auto& mc) {
    const NBins& b = mc.bins;
    const size_t n = b.lnw.size();
    for (size_t i = 0; i < n; ++i) {
      if (lnw) lnw[i] = b.lnw[i];
      if (hist) hist[i] = b.histogram[i];
      if (wl_hist) wl_hist[i] = mc.kind == 2 && i < mc.wl.histogram.size() ? mc.wl.histogram[i] : 0;
      if (visited) visited[i] = b.visited[i];
      if (round_trips) round_trips[i] = b.round_trips[i];
    }
    return (int64_t)n;
  });
}
// Subcell lists of a WCA grand walker against a rebuild from its positions (as
// multisets of (index, image offset)); returns the number of differing subcells.
int64_t orc_grand_check_cells(void* hv) {
  auto* h = (AnyGrand*)hv;
  if (h->system != 2) return 0;
  const Cell& c = h->wca->sys.cell;
  Cell fresh = c;
  fresh.update_caches();
  int64_t bad = 0;
  for (size_t k = 0; k < c.subcells.size(); ++k) {
    auto key = [](const Neighbor& n) {
      return ((uint64_t)n.index << 24) | ((uint64_t)(uint8_t)n.off[0] << 16) |
             ((uint64_t)(uint8_t)n.off[1] << 8) | (uint64_t)(uint8_t)n.off[2];
    };
    std::vector<uint64_t> a, b;
    for (const auto& n : c.subcells[k]) a.push_back(key(n));
    for (const auto& n : fresh.subcells[k]) b.push_back(key(n));
    std::sort(a.begin(), a.end());
    std::sort(b.begin(), b.end());
    if (a != b) ++bad;
  }
  return bad;
}
// Translation attempts and acceptances per N (max_N + 1 entries).
void orc_grand_translation(void* h, uint64_t* attempts, uint64_t* accepted) {
  ((AnyGrand*)h)->visit([&](auto& mc) {
    for (size_t n = 0; n <= mc.bins.max_N; ++n) {
      attempts[n] = mc.bins.num_translation_attempts[n];
      accepted[n] = mc.bins.num_translation_accepted[n];
    }
    return 0;
  });
}
void orc_grand_draws(uint64_t seed, uint32_t walker, uint64_t t, double* dbl3, uint32_t* u2,
                     float* g3, double* cand) {
  const GrandDraws d = draws_grand(seed, walker, t);
  dbl3[0] = d.u_choice; dbl3[1] = d.u;
  u2[0] = d.add_bit; u2[1] = d.pick;
  for (int a = 0; a < 3; ++a) g3[a] = d.g[a];
  if (cand) add_candidate(seed, walker, t, 0, cand);
}

}  // extern "C"

