// ORACLE / TEST INFRASTRUCTURE ONLY.  FP64 C++ restatement of the reference's systems,
// the FP64 statement the CUDA kernels are compared with and as the timed CPU baseline.
// Parity is pinned by the reference's own invariant tests (energy == compute_energy
// after every move, minimum-image agreement), re-run on this restatement in
// tests/test_oracle.py; the reference ships no golden numeric vectors.
//
// Arithmetic follows the reference expression by expression, with no FMA contraction
// (built with -ffp-contract=off): vector3d's norm2 is x*x + y*y + z*z left to right,
// and Rust's powi(6)/powi(3) are expanded as x2=x*x, x6=(x2*x2)*x2, x3=x*x2.
#pragma once
#include <array>
#include <cmath>
#include <cstdint>
#include <optional>
#include <vector>

#include "philox_draws.hpp"

namespace orc {

using V3 = std::array<double, 3>;
inline V3 sub(const V3& a, const V3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
inline double norm2(const V3& a) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]; }

inline double powi6(double x) { double x2 = x * x; double x4 = x2 * x2; return x4 * x2; }
inline double powi3(double x) { double x2 = x * x; return x * x2; }

// ---------------------------------------------------------------------------------
// Ising: src/system/ising.rs:20-123
struct Ising {
  int L = 0;
  double E = 0;
  double last_abs = 0;
  std::vector<int8_t> S;       // index i + j*L (ising.rs:64)
  bool have_change = false;
  size_t change_site = 0;
  double change_e = 0;

  double compute_energy() const {  // ising.rs:59-75
    double e = 0.0;
    for (int i1 = 0; i1 < L; ++i1)
      for (int j1 = 0; j1 < L; ++j1) {
        int j2 = (j1 + 1) % L;
        int nt = S[i1 + j2 * L];
        int i2 = (i1 + 1) % L;
        nt += S[i2 + j1 * L];
        e += (double)nt * (double)S[i1 + j1 * L];
      }
    return e;
  }
  double energy() const { return E; }
  std::optional<double> delta_energy() const { return 4.0; }  // ising.rs:76-78
  // ising.rs:104-119
  std::optional<double> plan_move_at(uint32_t i, uint32_t j) {
    int j2 = (j + 1) % L;
    int nt = S[i + j2 * L];
    j2 = (j + L - 1) % L;
    nt += S[i + j2 * L];
    int i2 = (i + 1) % L;
    nt += S[i2 + j * L];
    i2 = (i + L - 1) % L;
    nt += S[i2 + j * L];
    double e = E - (double)nt * (double)S[i + j * L] * 2.0;
    have_change = true;
    change_site = i + (size_t)j * L;
    change_e = e;
    return e;
  }
  std::optional<double> plan_move(const Draws& d, double) { return plan_move_at(d.which, d.j); }
  void confirm() {  // ising.rs:95-100
    if (have_change) { S[change_site] = (int8_t)(-S[change_site]); E = change_e; }
  }
  bool verify_energy() const { return E == compute_energy(); }
};

// ---------------------------------------------------------------------------------
// LJ cluster in a spherical wall: src/system/lj.rs:32-124, 219-261, 339-374
inline double lj_potential(double r2) {  // lj.rs:78-81
  double s = 1.0 / r2;
  return 4.0 * (powi6(s) - powi3(s));
}

// 4 s^6 + 4 s^3: the magnitude of the two parts of a pair term that cancel in
// 4 (s^6 - s^3) near r = sigma, which sets the scale of a binary32 evaluation's error.
inline double lj_gross(double r2) {
  double s = 1.0 / r2;
  return 4.0 * (powi6(s) + powi3(s));
}

struct Lj {
  double E = 0, error = 0;
  std::vector<V3> pos;
  double max_radius_squared = 0;
  double max_radius = 0;
  double last_abs = 0;  // sum of lj_gross over the pair terms of the last plan
  bool have_change = false;
  int ch_kind = 0;  // Change::Move / Add / Remove (lj.rs:56-74)
  size_t ch_which = 0;
  V3 ch_to{};
  double ch_e = 0;

  size_t n() const { return pos.size(); }
  size_t num_atoms() const { return pos.size(); }
  double compute_energy() const {  // lj.rs:236-244
    double e = 0.0;
    for (size_t w = 0; w < pos.size(); ++w)
      for (size_t k = 0; k < w; ++k) e += lj_potential(norm2(sub(pos[w], pos[k])));
    return e;
  }
  double energy() const { return E; }
  std::optional<double> delta_energy() const { return std::nullopt; }
  std::optional<double> move_atom(size_t which, const V3& r) {  // lj.rs:86-105
    double prev = norm2(pos[which]);
    if (norm2(r) > max_radius_squared && norm2(r) > prev) return std::nullopt;
    double e = E;
    V3 from = pos[which];
    last_abs = 0.0;
    for (size_t k = 0; k < pos.size(); ++k) {
      if (k == which) continue;
      const double rn = norm2(sub(pos[k], r)), ro = norm2(sub(pos[k], from));
      e += lj_potential(rn) - lj_potential(ro);
      last_abs += lj_gross(rn) + lj_gross(ro);
    }
    have_change = true;
    ch_kind = 0;
    ch_which = which;
    ch_to = r;
    ch_e = e;
    return e;
  }
  // compute_one_atom_energy (lj.rs:220-230) for an atom at r2 with index i (skipped)
  double one_atom_energy(const V3& r2, size_t i) {
    double e = 0.0;
    last_abs = 0.0;
    for (size_t j = 0; j < pos.size(); ++j) {
      if (j == i) continue;
      const double q = norm2(sub(pos[j], r2));
      e += lj_potential(q);
      last_abs += lj_gross(q);
    }
    return e;
  }
  // GrandSystem::plan_add (lj.rs:292-309) with the accepted point of the unit ball
  double plan_add_at(const V3& unit) {
    const double R = max_radius;  // r * self.max_radius (lj.rs:303)
    const V3 to = {unit[0] * R, unit[1] * R, unit[2] * R};
    const double e = E + one_atom_energy(to, pos.size());
    have_change = true;
    ch_kind = 1;
    ch_to = to;
    ch_e = e;
    return e;
  }
  // GrandSystem::plan_remove (lj.rs:310-315)
  double plan_remove(size_t which) {
    const double e = E - one_atom_energy(pos[which], which);
    have_change = true;
    ch_kind = 2;
    ch_which = which;
    ch_e = e;
    return e;
  }
  double expected_accuracy(double newe) const {  // lj.rs:106-108
    double nn = (double)pos.size();
    return std::fabs(newe) * 1e-14 * nn * nn;
  }
  void set_energy(double new_e) {  // lj.rs:110-123
    double nn = (double)pos.size();
    double new_error = std::fabs(new_e) > std::fabs(E) ? std::fabs(new_e) * 1e-15 * nn
                                                       : std::fabs(E) * 1e-15 * nn;
    error = new_error + error;
    if (error > expected_accuracy(new_e)) {
      error *= 0.0;
      E = compute_energy();
    } else {
      E = new_e;
    }
  }
  std::optional<double> plan_move(const Draws& d, double scale) {  // lj.rs:365-374
    if (pos.empty()) return std::nullopt;
    size_t which = d.which;
    const V3& f = pos[which];
    V3 to = {f[0] + (double)d.g[0] * scale, f[1] + (double)d.g[1] * scale,
             f[2] + (double)d.g[2] * scale};
    return move_atom(which, to);
  }
  void confirm() {  // lj.rs:339-358
    if (!have_change) return;
    if (ch_kind == 0) pos[ch_which] = ch_to;
    else if (ch_kind == 1) pos.push_back(ch_to);
    else { pos[ch_which] = pos.back(); pos.pop_back(); }  // swap_remove
    have_change = false;
    set_energy(ch_e);
  }
  bool verify_energy() const {  // lj.rs:249-261
    double egood = compute_energy();
    return !(std::fabs(egood - E) > expected_accuracy(E));
  }
};

// ---------------------------------------------------------------------------------
// Periodic cell with 27-fold neighbour registration: src/system/optcell.rs:27-346
struct Neighbor { uint32_t index; int8_t off[3]; };

static const int NEIGHBORS[27][3] = {  // optcell.rs:373-405 (same order)
    {0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},   {0, -1, 0},  {0, 0, 1},   {0, 0, -1},
    {0, 1, 1},  {0, 1, -1},  {0, -1, 1}, {0, -1, -1}, {1, 0, 1},   {1, 0, -1},  {-1, 0, 1},
    {-1, 0, -1}, {1, 1, 0},  {1, -1, 0}, {-1, 1, 0},  {-1, -1, 0}, {1, 1, 1},   {-1, 1, 1},
    {1, -1, 1}, {1, 1, -1},  {1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};

struct Cell {
  V3 box{};
  double r_cutoff = 0;
  std::vector<V3> pos;
  int nsc[3] = {0, 0, 0};
  std::vector<std::vector<Neighbor>> subcells;

  void update_caches() {  // optcell.rs:63-73
    for (int a = 0; a < 3; ++a) nsc[a] = (int)std::floor(box[a] / r_cutoff);
    subcells.assign((size_t)nsc[0] * nsc[1] * nsc[2], {});
    for (size_t i = 0; i < pos.size(); ++i) add_to_subcells((uint32_t)i, pos[i]);
  }
  void get_subcell(const V3& r, long sc[3]) const {  // optcell.rs:112-124
    for (int a = 0; a < 3; ++a) sc[a] = (long)std::floor(r[a] / box[a] * (double)nsc[a]);
  }
  static long modulus(long i, long sz) { return (i + sz) % sz; }  // optcell.rs:343-346
  size_t index(const long s[3]) const {  // optcell.rs:349-359
    long ix = modulus(s[0], nsc[0]), iy = modulus(s[1], nsc[1]), iz = modulus(s[2], nsc[2]);
    return (size_t)(ix * (nsc[1] * nsc[2]) + iy * nsc[2] + iz);
  }
  void add_to_subcells(uint32_t index_, const V3& r) {  // optcell.rs:131-160
    long sc[3];
    get_subcell(r, sc);
    for (int k = 0; k < 27; ++k) {
      long scp[3];
      Neighbor nb;
      nb.index = index_;
      for (int a = 0; a < 3; ++a) {
        scp[a] = sc[a] + NEIGHBORS[k][a];
        nb.off[a] = (int8_t)(scp[a] < 0 ? -1 : (scp[a] == nsc[a] ? 1 : 0));
      }
      subcells[index(scp)].push_back(nb);
    }
  }
  void add_atom_at(const V3& r) {  // optcell.rs:126-130
    uint32_t idx = (uint32_t)pos.size();
    pos.push_back(r);
    add_to_subcells(idx, r);
  }
  void remove_atom(size_t which) {  // optcell.rs:177-193 (swap_remove, then rename)
    const V3 r = pos[which];
    pos[which] = pos.back();
    pos.pop_back();
    long sc[3];
    get_subcell(r, sc);
    for (int k = 0; k < 27; ++k) {
      long q[3] = {sc[0] + NEIGHBORS[k][0], sc[1] + NEIGHBORS[k][1], sc[2] + NEIGHBORS[k][2]};
      remove_if_index(subcells[index(q)], (uint32_t)which);
    }
    if (pos.size() != which) {
      const uint32_t oldindex = (uint32_t)pos.size();
      long s2[3];
      get_subcell(pos[which], s2);
      for (int k = 0; k < 27; ++k) {
        long q[3] = {s2[0] + NEIGHBORS[k][0], s2[1] + NEIGHBORS[k][1], s2[2] + NEIGHBORS[k][2]};
        for (Neighbor& nb : subcells[index(q)])  // rename_neighbor (optcell.rs:419-426)
          if (nb.index == oldindex) { nb.index = (uint32_t)which; break; }
      }
    }
  }
  static void remove_if_index(std::vector<Neighbor>& v, uint32_t idx) {  // optcell.rs:407-418
    for (size_t i = 0; i < v.size(); ++i)
      if (v[i].index == idx) { v[i] = v.back(); v.pop_back(); return; }
  }
  void move_atom(size_t which, const V3& r) {  // optcell.rs:162-175
    V3 old = pos[which];
    pos[which] = r;
    long sc[3], osc[3];
    get_subcell(r, sc);
    get_subcell(old, osc);
    if (sc[0] != osc[0] || sc[1] != osc[1] || sc[2] != osc[2]) {
      for (int k = 0; k < 27; ++k) {
        long s[3] = {osc[0] + NEIGHBORS[k][0], osc[1] + NEIGHBORS[k][1], osc[2] + NEIGHBORS[k][2]};
        remove_if_index(subcells[index(s)], (uint32_t)which);
      }
      add_to_subcells((uint32_t)which, r);
    }
  }
  // Calls f(image_position) for each candidate of maybe_interacting_atoms_excluding
  // (optcell.rs:93-110); which == SIZE_MAX excludes nothing (optcell.rs:75-90).
  template <class F>
  void for_each_candidate(const V3& r, size_t which, F&& f) const {
    long sc[3];
    get_subcell(r, sc);
    for (const Neighbor& nb : subcells[index(sc)]) {
      if (nb.index == (uint32_t)which) continue;
      const V3& p = pos[nb.index];
      V3 img = {p[0] - (double)nb.off[0] * box[0], p[1] - (double)nb.off[1] * box[1],
                p[2] - (double)nb.off[2] * box[2]};
      if (!f(img)) return;
    }
  }
  V3 put_in_cell(V3 r) const {  // optcell.rs:277-309
    for (int a = 0; a < 3; ++a) {
      if (r[a] < 0.0) {
        do { r[a] += box[a]; } while (r[a] < 0.0);
      } else {
        while (r[a] >= box[a]) r[a] -= box[a];
      }
    }
    return r;
  }
  double closest_distance2(const V3& r1, const V3& r2) const {  // optcell.rs:199-232
    V3 dr = sub(r2, r1);
    for (int a = 0; a < 3; ++a) {
      if (dr[a] < -0.5 * box[a]) {
        do { dr[a] += box[a]; } while (dr[a] < -0.5 * box[a]);
      } else {
        while (dr[a] > 0.5 * box[a]) dr[a] -= box[a];
      }
    }
    return norm2(dr);
  }
  double sloppy_closest_distance2(const V3& r1, const V3& r2) const {  // optcell.rs:234-255
    V3 dr = sub(r2, r1);
    for (int a = 0; a < 3; ++a) {
      while (dr[a] < -0.5 * box[a]) dr[a] += box[a];
      while (dr[a] > 0.5 * box[a]) dr[a] -= box[a];
    }
    return norm2(dr);
  }
  double unsafe_closest_distance2(const V3& r1, const V3& r2) const {  // optcell.rs:257-275
    V3 dr = sub(r2, r1);
    for (int a = 0; a < 3; ++a) {
      if (dr[a] < -0.5 * box[a]) dr[a] += box[a];
      else if (dr[a] > 0.5 * box[a]) dr[a] -= box[a];
    }
    return norm2(dr);
  }
  double volume() const { return box[0] * box[1] * box[2]; }
};

// ---------------------------------------------------------------------------------
// WCA fluid: src/system/wca.rs:23-181, 219-250, 342-353
inline double wca_r_cutoff() { return std::pow(2.0, 1.0 / 6.0); }  // wca.rs:61-63
inline double wca_potential(double r2) {  // wca.rs:66-76
  double rc = wca_r_cutoff();
  if (r2 < rc * rc) {
    double s = 1.0 / r2;
    return 4.0 * (powi6(s) - powi3(s)) + 1.0;
  }
  return 0.0;
}
inline double wca_potential_pressure(double r2) {  // wca.rs:79-92
  double rc = wca_r_cutoff();
  if (r2 < rc * rc) {
    double s = 1.0 / r2;
    return 4.0 * 3.0 * (2.0 * powi6(s) - powi3(s));
  }
  return 0.0;
}

struct Wca {
  double E = 0, error = 0;
  double last_abs = 0;
  Cell cell;
  bool have_change = false;
  int ch_kind = 0;  // Change::Move / Add / Remove (wca.rs:34-55)
  size_t ch_which = 0;
  V3 ch_to{};
  double ch_e = 0, ch_dabse = 0;

  size_t num_atoms() const { return cell.pos.size(); }
  double compute_energy() const {  // wca.rs:222-230
    double e = 0.0;
    for (size_t w = 0; w < cell.pos.size(); ++w) {
      const V3 r1 = cell.pos[w];
      cell.for_each_candidate(r1, w, [&](const V3& r2) {
        e += wca_potential(norm2(sub(r1, r2)));
        return true;
      });
    }
    return e * 0.5;
  }
  double pressure() const {  // wca.rs:202-218 (the "pressure" extra datum)
    double p = 0.0;
    for (size_t w = 0; w < cell.pos.size(); ++w) {
      const V3 r1 = cell.pos[w];
      cell.for_each_candidate(r1, w, [&](const V3& r2) {
        p += wca_potential_pressure(norm2(sub(r1, r2)));
        return true;
      });
    }
    return p / (3.0 * cell.volume());
  }
  double energy() const { return E; }
  std::optional<double> delta_energy() const { return std::nullopt; }
  double expected_accuracy(double newe) const {  // wca.rs:178-180
    double nn = (double)num_atoms();
    return std::fabs(newe) * 1e-13 * nn * nn;
  }
  void set_energy(double new_e, double dabse) {  // wca.rs:164-177
    double nn = (double)num_atoms();
    double single = dabse > std::fabs(new_e) ? 1e-14 * dabse * nn : 1e-14 * std::fabs(new_e) * nn;
    error += single * nn;
    if (error > expected_accuracy(new_e)) {
      E = compute_energy();
      error = 1e-15 * E * nn;
    } else {
      E = new_e;
    }
  }
  std::optional<double> move_atom(size_t which, const V3& r) {  // wca.rs:119-140
    double e = E, dabse = 0.0;
    V3 from = cell.pos[which];
    double gross = 0.0;
    const double rc2 = wca_r_cutoff() * wca_r_cutoff();
    cell.for_each_candidate(r, which, [&](const V3& r1) {
      const double r2 = norm2(sub(r1, r));
      double de = wca_potential(r2);
      e += de;
      dabse += de;
      if (r2 < rc2) gross += lj_gross(r2) + 1.0;
      return true;
    });
    cell.for_each_candidate(from, which, [&](const V3& r1) {
      const double r2 = norm2(sub(r1, from));
      double de = wca_potential(r2);
      e -= de;
      dabse += de;
      if (r2 < rc2) gross += lj_gross(r2) + 1.0;
      return true;
    });
    last_abs = gross;
    have_change = true;
    ch_kind = 0;
    ch_which = which;
    ch_to = r;
    ch_e = e;
    ch_dabse = dabse;
    return e;
  }
  // GrandSystem (wca.rs:307-323): add_atom_at (wca.rs:105-116), remove_atom_number
  // (wca.rs:151-163)
  double plan_add_at(const V3& r) {
    double dabse = 0.0, gross = 0.0;
    const double rc2 = wca_r_cutoff() * wca_r_cutoff();
    cell.for_each_candidate(r, SIZE_MAX, [&](const V3& r1) {
      const double q = norm2(sub(r1, r));
      dabse += wca_potential(q);
      if (q < rc2) gross += lj_gross(q) + 1.0;
      return true;
    });
    last_abs = gross;
    have_change = true;
    ch_kind = 1;
    ch_to = r;
    ch_e = E + dabse;
    ch_dabse = dabse;
    return ch_e;
  }
  double plan_remove(size_t which) {
    const V3 r = cell.pos[which];
    double dabse = 0.0, gross = 0.0;
    const double rc2 = wca_r_cutoff() * wca_r_cutoff();
    cell.for_each_candidate(r, which, [&](const V3& r1) {
      const double q = norm2(sub(r1, r));
      dabse += wca_potential(q);
      if (q < rc2) gross += lj_gross(q) + 1.0;
      return true;
    });
    last_abs = gross;
    have_change = true;
    ch_kind = 2;
    ch_which = which;
    ch_e = E - dabse;
    ch_dabse = dabse;
    return ch_e;
  }
  std::optional<double> plan_move(const Draws& d, double scale) {  // wca.rs:342-353
    if (cell.pos.empty()) return std::nullopt;
    const V3& f = cell.pos[d.which];
    V3 to = cell.put_in_cell({f[0] + (double)d.g[0] * scale, f[1] + (double)d.g[1] * scale,
                              f[2] + (double)d.g[2] * scale});
    return move_atom(d.which, to);
  }
  void confirm() {  // wca.rs:276-301
    if (!have_change) return;
    if (ch_kind == 0) cell.move_atom(ch_which, ch_to);
    else if (ch_kind == 1) cell.add_atom_at(ch_to);
    else cell.remove_atom(ch_which);
    set_energy(ch_e, ch_dabse);
    have_change = false;
  }
  bool verify_energy() const {  // wca.rs:237-250
    double egood = compute_energy();
    return !(std::fabs(egood - E) > expected_accuracy(E));
  }
};

// System::data_to_collect (src/system/mod.rs:88-90); the primary template (no datum)
// lives with the bins in energy_mc.hpp.
template <class S>
inline bool collect_extra(const S&, uint64_t, double*);
// wca.rs:202-218: the pressure datum every N^2 moves
template <>
inline bool collect_extra<Wca>(const Wca& s, uint64_t iter, double* out) {
  const uint64_t n = (uint64_t)s.num_atoms();
  if (n == 0 || iter % (n * n) != 0) return false;
  *out = s.pressure();
  return true;
}

// ---------------------------------------------------------------------------------
// Square well with a hard core (the "hard sphere with contact-count bins" system):
// src/system/optsquare.rs:24-322
inline uint64_t max_balls_within(double distance) {  // optsquare.rs:290-322
  distance += 1e-10;
  double a = std::sqrt(2.0);
  long c = (long)std::ceil(distance / a) + 1;
  long num = -1;
  double d2 = distance * distance;
  for (long n = -c; n < c + 1; ++n)
    for (long m = -c; m < c + 1; ++m)
      for (long l = -c; l < c + 1; ++l) {
        double x0 = (double)(m + l) * a, y0 = (double)(n + l) * a, z0 = (double)(m + n) * a;
        if (x0 * x0 + y0 * y0 + z0 * z0 <= d2) num += 1;
        if ((x0 + 0.5 * a) * (x0 + 0.5 * a) + (y0 + 0.5 * a) * (y0 + 0.5 * a) + z0 * z0 <= d2) num += 1;
        if ((x0 + 0.5 * a) * (x0 + 0.5 * a) + y0 * y0 + (z0 + 0.5 * a) * (z0 + 0.5 * a) <= d2) num += 1;
        if (x0 * x0 + (y0 + 0.5 * a) * (y0 + 0.5 * a) + (z0 + 0.5 * a) * (z0 + 0.5 * a) <= d2) num += 1;
      }
  return (uint64_t)num;
}

struct SquareWell {
  double E = 0;
  double last_abs = 0;
  Cell cell;
  bool have_change = false;
  size_t ch_which = 0;
  V3 ch_to{};
  double ch_e = 0;

  size_t num_atoms() const { return cell.pos.size(); }
  double energy() const { return E; }
  std::optional<double> delta_energy() const { return 1.0; }  // optsquare.rs:190-192
  double compute_energy() const {  // optsquare.rs:176-186
    double e = 0.0, rc2 = cell.r_cutoff * cell.r_cutoff;
    for (size_t w = 0; w < cell.pos.size(); ++w) {
      const V3 r1 = cell.pos[w];
      cell.for_each_candidate(r1, w, [&](const V3& r2) {
        if (norm2(sub(r1, r2)) < rc2) e -= 1.0;
        return true;
      });
    }
    return e * 0.5;
  }
  double compute_energy_slowly() const {  // optsquare.rs:108-152
    double e = 0.0;
    const V3& L = cell.box;
    double rc2 = cell.r_cutoff * cell.r_cutoff;
    for (const V3& r1 : cell.pos)
      for (const V3& r2 : cell.pos) {
        V3 r12 = sub(r1, r2);
        for (int a = 0; a < 3; ++a) {
          while (r12[a] > L[a] / 2.0) r12[a] -= L[a];
        }
        for (int a = 0; a < 3; ++a) {
          while (r12[a] < -L[a] / 2.0) r12[a] += L[a];
        }
        for (int i = -1; i < 2; ++i)
          for (int j = -1; j < 2; ++j)
            for (int k = -1; k < 2; ++k) {
              V3 r = {r12[0] + L[0] * (double)i, r12[1] + L[1] * (double)j, r12[2] + L[2] * (double)k};
              double d2 = norm2(r);
              if (d2 < rc2 && d2 > 0.0) e -= 1.0;
            }
      }
    return e * 0.5;
  }
  std::optional<double> add_atom_at(const V3& r) {  // optsquare.rs:58-71
    double e = E, rc2 = cell.r_cutoff * cell.r_cutoff;
    bool overlap = false;
    cell.for_each_candidate(r, SIZE_MAX, [&](const V3& r1) {
      double d2 = norm2(sub(r1, r));
      if (d2 < 1.0) { overlap = true; return false; }
      if (d2 < rc2) e -= 1.0;
      return true;
    });
    if (overlap) { have_change = false; return std::nullopt; }
    cell.add_atom_at(r);
    E = e;
    return e;
  }
  std::optional<double> move_atom(size_t which, const V3& r) {  // optsquare.rs:74-95
    double e = E, wsqr = cell.r_cutoff * cell.r_cutoff;
    V3 from = cell.pos[which];
    bool overlap = false;
    cell.for_each_candidate(r, which, [&](const V3& r1) {
      double d2 = norm2(sub(r1, r));
      if (d2 < 1.0) { overlap = true; return false; }
      if (d2 < wsqr) e -= 1.0;
      return true;
    });
    if (overlap) { have_change = false; return std::nullopt; }
    cell.for_each_candidate(from, which, [&](const V3& r1) {
      if (norm2(sub(r1, from)) < wsqr) e += 1.0;
      return true;
    });
    have_change = true;
    ch_which = which;
    ch_to = r;
    ch_e = e;
    return e;
  }
  std::optional<double> plan_move(const Draws& d, double scale) {  // optsquare.rs:273-284
    if (cell.pos.empty()) return std::nullopt;
    const V3& f = cell.pos[d.which];
    V3 to = cell.put_in_cell({f[0] + (double)d.g[0] * scale, f[1] + (double)d.g[1] * scale,
                              f[2] + (double)d.g[2] * scale});
    return move_atom(d.which, to);
  }
  void confirm() {  // optsquare.rs:213-234 (Move arm)
    if (!have_change) return;
    cell.move_atom(ch_which, ch_to);
    E = ch_e;
    have_change = false;
  }
  bool verify_energy() const { return E == compute_energy_slowly(); }  // optsquare.rs:199-201
  double lowest_possible_energy() const {  // optsquare.rs:196-198
    return -(double)num_atoms() * (double)max_balls_within(cell.r_cutoff);
  }
};

}  // namespace orc
