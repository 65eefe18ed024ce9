// Flat-histogram bookkeeping of one walker, executed by the LPW lanes of the walker's
// lane group.  All lanes of a group hold identical copies of the scalar state, run the
// same FP64 instructions and issue the same stores, so one warp instruction serves
// every walker packed into the warp (on GB300 an FP64 warp instruction costs the same
// with one active lane as with 32) and every lane reads back its own writes.
//
// Restates EnergyMC::move_once / reject_move / update_weights / gamma
// (src/mc/energy.rs:904-974, 440-512, 514-761, 799-825) over preallocated bin planes:
//  * prepare_for_state (energy.rs:400-434) grows the allocated range [b_lo, b_hi] with
//    the reference's own bins.min arithmetic (cur_min -= width);
//  * SAD's t_F = max(t_found[ilo..=ihi]) (energy.rs:585-592) is kept incrementally:
//    t_found entries are written once and the window [too_lo, too_hi] only widens;
//  * the SAD refill loops (energy.rs:542-583) visit only bins whose centre can meet the
//    loop condition, each still tested with the reference's FP64 expression;
//  * have_visited_since_maxentropy fills (energy.rs:950-965) are O(1) generation stamps;
//  * gamma (SAD, SAMC) is evaluated for 4*LPW consecutive moves at once;
//  * the proposed bin's fields are fetched in one memory round trip and adopted when the
//    move is accepted; the current bin lives in registers.
#pragma once
#include <cstdint>

#include "sadmc_types.h"

namespace sadmc {
namespace dev {

__device__ __forceinline__ double u53_to_double(uint64_t v) {
  return (double)v * (1.0 / 9007199254740992.0);
}

// rejected = (u > exp(d)) with u = u53 * 2^-53 and d <= 0 (energy.rs:465, 489, 498, 508).
// Decided in FP32 when the FP32 estimate is outside its error margin; otherwise the
// reference's FP64 comparison is evaluated.
__device__ __forceinline__ float f32_trunc(double x);
__device__ __forceinline__ bool metropolis_reject(double d, uint64_t u53) {
  float df = f32_trunc(d);
  if (df < -80.0f) return u53 != 0;  // exp(d) < 2e-35 < 2^-53: only u == 0 is accepted
  float e32 = __expf(df);
  float m = 4.0e-6f + fabsf(df) * 4.0e-7f;
  float uf = (float)(u53 >> 29) * (1.0f / 16777216.0f);  // u in [uf, uf + 2^-24)
  if (uf > e32 * (1.0f + m)) return true;
  if (uf + (1.0f / 16777216.0f) < e32 * (1.0f - m)) return false;
  return u53_to_double(u53) > exp(d);
}


// binary32 value of a finite double by truncating its mantissa (relative error < 2^-23),
// with integer instructions only; |x| < 2^-126 gives +-0, |x| >= 2^128 gives +-inf.
__device__ __forceinline__ float f32_trunc(double x) {
  const long long b = __double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32);
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023;
  if (e < -126) return __uint_as_float(sign);
  if (e > 127) return __uint_as_float(sign | 0x7f800000u);
  const unsigned m = (unsigned)((b >> 29) & 0x7fffffll);
  return __uint_as_float(sign | ((unsigned)(e + 127) << 23) | m);
}
// x < y for finite doubles, by integer instructions (IEEE order: a double's bit pattern
// read as a signed integer orders the non-negative values; flipping the magnitude bits of
// the negative ones orders them below, and +0 and -0 compare equal).  It keeps dgt off
// the FP64 pipe.  Measured on the LJ move kernel: replacing every FP64 comparison of the
// decision path this way took a third of the kernel's FP64 instructions away (they are
// issued ahead of their branches) and still ran 1-5 % slower, its integer sequence being
// longer than a comparison on the kernel's dependent chain; so the decision path keeps
// its FP64 comparisons.
__device__ __forceinline__ bool dlt(double x, double y) {
  long long a = __double_as_longlong(x), b = __double_as_longlong(y);
  if (((a | b) << 1) == 0) return false;  // both zero
  a = a < 0 ? (a ^ 0x7FFFFFFFFFFFFFFFll) : a;
  b = b < 0 ? (b ^ 0x7FFFFFFFFFFFFFFFll) : b;
  return a < b;
}
// x > y for finite doubles (integer instructions, as dlt).
__device__ __forceinline__ bool dgt(double x, double y) {
  const long long a = __double_as_longlong(x), b = __double_as_longlong(y);
  if ((a | b) >= 0) return a > b;
  return dlt(y, x);
}
// x is NaN, by integer instructions
__device__ __forceinline__ bool is_nan64(double x) {
  return (unsigned long long)(__double_as_longlong(x) & 0x7fffffffffffffffll) > 0x7ff0000000000000ull;
}
// (double)f for a binary32 value, by integer instructions for zero and normal numbers
__device__ __forceinline__ double f2d(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  if (e == 0u && (b & 0x7fffffffu) == 0u) return __longlong_as_double((long long)(b & 0x80000000u) << 32);
  if (e == 0u || e == 255u) return (double)f;
  const unsigned long long d = ((unsigned long long)(b >> 31) << 63) |
                               ((unsigned long long)(e + (1023u - 127u)) << 52) |
                               ((unsigned long long)(b & 0x7fffffu) << 29);
  return __longlong_as_double((long long)d);
}
// (double)x for an integer x < 2^53 (exact), by integer instructions: the FP64 pipe, the
// scarce one on GB300, also runs the integer-to-double conversion.
__device__ __forceinline__ double u2d(uint64_t x) {
  if (x == 0) return 0.0;
  const int e = 63 - __clzll((long long)x);  // x in [2^e, 2^(e+1)), e <= 52
  const uint64_t m = x << (52 - e);           // leading 1 at bit 52
  return __longlong_as_double((long long)(((uint64_t)(e + 1023) << 52) | (m & 0xFFFFFFFFFFFFFull)));
}
// a / b, correctly rounded, for a divisor b whose correctly rounded reciprocal y = 1/b is
// known: q = a y, r = a - b q (exact, one FMA), a / b = RN(q + r y) (P. Markstein,
// IBM J. Res. Dev. 34(1), 1990).  Finite normal operands and quotient.
__device__ __forceinline__ double div_by(double a, double b, double y) {
  const double q = __dmul_rn(a, y);
  const double r = __fma_rn(-b, q, a);
  return __fma_rn(r, y, q);
}
// The translation-scale factor clamp(acceptance_rate / target_rate, 0.8, 1.2)
// (energy.rs:600-609), the quotient taken by div_by with y = 1/target_rate.  The clamped
// value equals the reference's: where the quotient lies in [0.8, 1.2] the rate (at most 1)
// and target are normal numbers and div_by is correctly rounded; below 0.8 (the rate
// tiny or zero included) div_by's value stays below 0.8, and both clamp to 0.8.
__device__ __forceinline__ double rate_factor(double rate, double target, double y) {
  const double s = div_by(rate, target, y);
  return s < 0.8 ? 0.8 : (s > 1.2 ? 1.2 : s);
}
// rejected = (u > exp(lnw1 - lnw2)) for lnw1 - lnw2 <= 0, taken on the binary32 copies
// of the two weights when far enough from the threshold; otherwise the FP64 difference
// goes through metropolis_reject.
__device__ __forceinline__ bool metropolis_reject2(double lnw1, double lnw2, uint64_t u53) {
  const float a = f32_trunc(lnw1), b = f32_trunc(lnw2);
  const float df = a - b;
  // |df - (lnw1 - lnw2)| <= (|a| + |b|) 2^-23 + |df| 2^-24; exp's relative error is that
  const float dd = (fabsf(a) + fabsf(b)) * 1.2e-7f + fabsf(df) * 6.0e-8f + 1e-30f;
  if (df + dd < -80.0f) return u53 != 0;
  if (df - dd > -80.0f && dd < 0.25f) {
    const float e32 = __expf(df);
    const float m = 4.0e-6f + fabsf(df) * 4.0e-7f + 2.0f * dd;
    const float uf = (float)(u53 >> 29) * (1.0f / 16777216.0f);
    if (uf > e32 * (1.0f + m)) return true;
    if (uf + (1.0f / 16777216.0f) < e32 * (1.0f - m)) return false;
  }
  return metropolis_reject(lnw1 - lnw2, u53);
}

// SadVersion::compute_gamma (energy.rs:22-38) for move count t and parameters (p, tF, ns),
// with the same operations as Fh::gamma_at (reciprocals, Markstein divisions), so that a
// lane filling a table computes the bits the walker's own lane would.
__device__ __forceinline__ double sad_gamma_value(double p, uint64_t tF, uint64_t ns, uint64_t t) {
  const double tF_d = u2d(tF), ns_d = u2d(ns);
  if (p * tF_d * ns_d == 0.0) return 0.0;
  const double td = u2d(t);
  const double t_tF = div_by(td, tF_d, 1.0 / tF_d);
  return (p + t_tF) / (p + div_by(td, ns_d, 1.0 / ns_d) * t_tF);
}

// FAM: the method a kernel is specialised for (M_SAD, ...), or FAM_ANY for the kind held
// in each walker's state (WL and 1/t-WL, whose walkers switch to SAMC at run time).
constexpr int FAM_ANY = -1;

// SPLIT: the bookkeeping that no decision reads -- the acceptance rate and translation
// scale, the energy sums, and the max-entropy / round-trip stamps -- is left to another
// warp, which replays it from a per-move record (out_li, out_i1l, tsc_event and the
// state after the move); this object then holds neither those fields nor their planes.
template <int LPW, int FAM = FAM_ANY, bool SPLIT = false>
struct Fh {
  static_assert(!SPLIT || (LPW == 1 && FAM == M_SAD), "the split bookkeeping is SAD on one lane");
  WalkerCore c;
  // launch constants
  double width, inv_width, min_allowed, max_allowed, target_rate, inv_target;
  int nbins;
  bool has_min_allowed, has_max_allowed, acc_mode;
  // this walker's planes
  double *lnw, *sE, *sE2;
  uint64_t *hist, *tf, *rt, *wlh, *stamp;
  // lane group
  unsigned gmask;
  int glane;
  bool wr;  // stores enabled (false for padding groups past the last walker)
  // cached current bin (global index cur)
  int cur;
  double k_lnw, k_sE, k_sE2;
  uint64_t k_hist, k_tf, k_stamp;
  // the proposed bin's fields, fetched together in decide() (one memory round trip)
  double p_lnw, p_sE, p_sE2;
  uint64_t p_hist, p_tf, p_stamp;
  double cur_max;      // upper edge of the allocated range
  double E2;           // c.E * c.E, formed when E changes (energy_squared_total term)
  int win_lo, win_hi;  // SAD window as bin indices
  // gamma batch (see gamma())
  double gb_val[4];
  uint32_t gb_base;  // low 32 bits of the move count the batch starts at
  uint32_t gb_ok;    // bit q: gb_val[q] holds gamma for the current parameters
  // per-move scratch
  double e1;
  int i2;
  uint64_t hist2;
  bool grew_front;
  bool tscale_changed;  // set when the SAD discovery adapted translation_scale
  // binary32 copies for the FP32-first comparisons of decide_de (refreshed on change)
  float Ef, cminf, cmaxf, maxf, minf, inv_wf;
  // correctly rounded reciprocals for div_by: 1/min_T, and 1/tF, 1/num_states for the
  // tF and num_states they were taken for
  double inv_minT, inv_tF, inv_ns;
  uint64_t inv_tF_of, inv_ns_of;
  double tF_d, ns_d;    // (double) tF and num_states for the values above
  bool g_zero;          // latest_param * tF * num_states == 0 (SAD gamma is 0), per refresh
  // A table of gamma for the moves [xg_t0, xg_t0 + 32), filled by a whole warp for a
  // walker that one lane runs (the single-walker chain kernel); valid while xg_ok, that
  // is until the method's parameters change.  Null for the other kernels.
  const double* xg;
  uint64_t xg_t0;
  bool xg_ok;
  uint32_t pgen;  // count of parameter changes (tables computed ahead carry the count they saw)
  // SPLIT: the last move's local bin index, the local index of the bin it started from
  // (energy.rs:950-965), and whether tF changed with the acceptance-rate mode on
  // (energy.rs:600-609)
  int out_li, out_i1l;
  bool tsc_event;
  __device__ void invalidate_gamma() { gb_ok = 0; xg_ok = false; ++pgen; }
  bool inverted;        // too_lo > too_hi (never true for SAD; kept exact)

  // ---- index helpers ---------------------------------------------------------------
  __device__ int gidx_exact(double e) const { return (int)((e - c.cur_min) / width) + c.b_lo; }
  // state_to_index (energy.rs:371-373).  The FP64 quotient is evaluated only when the
  // FP32 estimate lies within its error bound of an integer.
  __device__ int gidx(double e) const {
    double d = e - c.cur_min;
    float q = __fmul_rn((float)d, (float)inv_width);
    int qi = __float2int_rz(q);
    float fr = q - (float)qi;
    float m = q * 4.0e-7f + 1.0e-6f;
    if (fr > m && fr < 1.0f - m) return qi + c.b_lo;
    return (int)(d / width) + c.b_lo;
  }
  __device__ double center(int g) const {  // index_to_state (energy.rs:366-370)
    return c.cur_min + ((double)(g - c.b_lo) + 0.5) * width;
  }

  // cached-bin aware accessors
  __device__ double ld_lnw(int g) const { return g == cur ? k_lnw : lnw[g]; }
  __device__ uint64_t ld_hist(int g) const { return g == cur ? k_hist : hist[g]; }
  __device__ uint64_t ld_tf(int g) const { return g == cur ? k_tf : tf[g]; }
  __device__ void st_lnw(int g, double v) {
    if (g == cur) k_lnw = v;
    else if (wr) lnw[g] = v;
  }
  __device__ void flush_cur() {
    if (wr) {
      lnw[cur] = k_lnw; hist[cur] = k_hist; tf[cur] = k_tf;
      if (!SPLIT) { sE[cur] = k_sE; sE2[cur] = k_sE2; }
    }
  }
  __device__ void load_cur(int g) {
    g = g < 0 ? 0 : (g >= nbins ? nbins - 1 : g);
    cur = g;
    k_lnw = lnw[g]; k_hist = hist[g]; k_tf = tf[g];
    if (!SPLIT) { k_sE = sE[g]; k_sE2 = sE2[g]; k_stamp = stamp[g]; }
  }
  __device__ void fetch_pending(int g) {
    if (g == cur) {
      p_lnw = k_lnw; p_hist = k_hist; p_tf = k_tf; p_sE = k_sE; p_sE2 = k_sE2; p_stamp = k_stamp;
    } else {
      p_lnw = lnw[g]; p_hist = hist[g]; p_tf = tf[g];
      if (!SPLIT) { p_sE = sE[g]; p_sE2 = sE2[g]; p_stamp = stamp[g]; }
    }
  }
  // adopt the prefetched fields of bin g (== i2) as the current bin
  __device__ void adopt_pending(int g) {
    if (g == cur) return;
    flush_cur();
    cur = g;
    k_lnw = p_lnw; k_hist = p_hist; k_tf = p_tf;
    if (!SPLIT) { k_sE = p_sE; k_sE2 = p_sE2; k_stamp = p_stamp; }
  }
  __device__ void move_cur(int g) {
    if (g != cur) { flush_cur(); load_cur(g); }
  }
  __device__ void sync() {
    if (LPW > 1) __syncwarp(gmask);
  }
  // Lane 0's value of a predicate for the whole lane group.  Every branch that leads to a
  // group collective (__syncwarp, shuffles) takes its predicate through here, so the
  // lanes of a group always reach the same collectives.
  // the method: a compile-time constant in a specialised kernel (dead paths vanish)
  __device__ int kind() const { return FAM >= 0 ? FAM : (int)c.kind; }
  __device__ bool uni(bool x) const {
    if (LPW == 1) return x;
    return __shfl_sync(gmask, (int)x, 0, LPW) != 0;
  }
  __device__ uint64_t group_min(uint64_t v) const {
#pragma unroll
    for (int o = LPW / 2; o > 0; o >>= 1) {
      uint64_t x = __shfl_xor_sync(gmask, v, o, LPW);
      v = x < v ? x : v;
    }
    return v;
  }

  // ---- load / store ------------------------------------------------------------------
  __device__ void load(const WalkerCore* cores, const FhParams& P, const BinPlanes& B, int w,
                       unsigned gmask_, int glane_, bool wr_) {
    c = cores[w];
    width = P.width; inv_width = P.inv_width; nbins = P.nbins;
    has_min_allowed = P.has_min_allowed != 0; has_max_allowed = P.has_max_allowed != 0;
    acc_mode = P.acc_mode != 0;
    min_allowed = P.min_allowed; max_allowed = P.max_allowed; target_rate = P.target_rate;
    inv_target = P.inv_target;
    size_t off = (size_t)w * (size_t)P.nbins;
    lnw = B.lnw + off; sE = B.sumE + off; sE2 = B.sumE2 + off;
    hist = B.hist + off; tf = B.t_found + off; rt = B.round_trips + off;
    wlh = B.wl_hist + off; stamp = B.visit_stamp + off;
    gmask = gmask_; glane = glane_; wr = wr_;
    cur_max = c.cur_min + width * (double)(c.b_hi - c.b_lo + 1);
    if (c.kind != M_DESCENT) {
      load_cur(gidx_exact(c.E));
      if (kind() == M_SAD) { win_lo = gidx_exact(c.too_lo); win_hi = gidx_exact(c.too_hi); }
    } else {
      cur = -1;
    }
    inverted = c.too_lo > c.too_hi;
    gb_ok = 0;
    gb_base = ~0u;
    grew_front = false;
    tscale_changed = false;
    // binary32 shadows of decide_de (each within |x| 2^-23 of its FP64 value)
    Ef = f32_trunc(c.E);
    E2 = c.E * c.E;
    cminf = f32_trunc(c.cur_min);
    cmaxf = f32_trunc(cur_max);
    maxf = f32_trunc(max_allowed);
    minf = f32_trunc(min_allowed);
    inv_wf = (float)inv_width;
    inv_minT = 1.0 / c.min_T;
    inv_tF_of = 0; inv_ns_of = 0; inv_tF = inv_ns = 0.0;
    tF_d = ns_d = 0.0;
    g_zero = true;
    xg = nullptr;
    xg_t0 = 0;
    xg_ok = false;
    pgen = 0;
  }
  __device__ void store(WalkerCore* cores, int w) {
    if (c.kind != M_DESCENT) flush_cur();
    if (!(wr && glane == 0)) return;
    if (FAM == M_SAD) {
      // the fields a SAD move can change; the other methods' fields keep the values the
      // launch loaded, so a SAD kernel need not hold them in registers for the whole loop
      // (SPLIT: nor those of the other warp's bookkeeping, which stores them itself)
      WalkerCore* o = &cores[w];
      o->E = c.E; o->cur_min = c.cur_min;
      o->too_lo = c.too_lo; o->too_hi = c.too_hi; o->latest_param = c.latest_param;
      o->drift = c.drift; o->win_tmax = c.win_tmax; o->moves = c.moves;
      o->accepted = c.accepted; o->tL = c.tL; o->tF = c.tF; o->num_states = c.num_states;
      o->highest_hist = c.highest_hist; o->b_lo = c.b_lo; o->b_hi = c.b_hi;
      o->status = c.status; o->pad1 = c.pad1; o->pad2 = c.pad2;
      if (!SPLIT) {
        o->acc_rate = c.acc_rate; o->tscale = c.tscale; o->max_S = c.max_S;
        o->max_S_local = c.max_S_local; o->fill_val = c.fill_val; o->fill_gen = c.fill_gen;
      }
    } else {
      cores[w] = c;
    }
  }

  // ---- gamma (energy.rs:799-825; SadVersion::compute_gamma energy.rs:22-38) -----------
  __device__ double gamma_at(uint64_t t) const {
    switch (kind()) {
      case M_SAD: {
        // tF_d, ns_d, their reciprocals and g_zero are refreshed by gamma() for the
        // current parameters; the expression is compute_gamma's
        if (g_zero) return 0.0;
        const double p = c.latest_param, td = u2d(t);
        const double t_tF = div_by(td, tF_d, inv_tF);
        return (p + t_tF) / (p + div_by(td, ns_d, inv_ns) * t_tF);
      }
      case M_SAMC: {
        const double td = u2d(t);
        return td > c.t0 ? c.t0 / td : 1.0;
      }
      case M_WL:
      case M_INV_T_WL: return c.gamma;
      default: return 0.0;
    }
  }
  // gamma(base + glane + LPW*q) sits in gb_val[q], base = the move count rounded down to a
  // multiple of 4*LPW: four independent divide chains per lane hide the FP64 divide
  // latency and cover 4*LPW moves.  The walkers of a launch share the move count, so the
  // lane groups of a warp take their full refreshes at the same moves (one instruction
  // stream).  A change of the SAD parameters mid-batch (gb_ok = 0) refreshes only the
  // slot of the current move, one chain per lane for the next LPW moves, where other
  // walkers share the warp.  (The low 32
  // bits of the count suffice: a batch is replaced at least every 4*LPW moves.)
  // tF_d, ns_d, their reciprocals and g_zero for the current SAD parameters
  __device__ void refresh_sad_params() {
    if (c.tF != inv_tF_of) { tF_d = u2d(c.tF); inv_tF = 1.0 / tF_d; inv_tF_of = c.tF; }
    if (c.num_states != inv_ns_of) { ns_d = u2d(c.num_states); inv_ns = 1.0 / ns_d; inv_ns_of = c.num_states; }
    g_zero = c.latest_param * tF_d * ns_d == 0.0;
  }
  __device__ double gamma() {
    if (kind() != M_SAD && kind() != M_SAMC) return gamma_at(c.moves);
    if (xg) {  // the warp's table, or this lane alone after a parameter change
      const uint64_t k = c.moves - xg_t0;
      if (xg_ok && k < 32) return xg[k];
      if (kind() == M_SAD) refresh_sad_params();
      return gamma_at(c.moves);
    }
    constexpr uint32_t SPAN = 4 * LPW;
    const uint32_t m32 = (uint32_t)c.moves;
    const uint32_t base = m32 & ~(SPAN - 1);
    const int off = (int)(m32 - base);
    const int qc = off / LPW;
    if (base != gb_base) {
      gb_base = base;
      gb_ok = 0;
    }
    if (SADMC_RARE(!((gb_ok >> qc) & 1u))) {
      if (kind() == M_SAD) refresh_sad_params();
      const uint64_t t0 = c.moves - (uint64_t)off;
      if (off == 0 || LPW == 32) {
        // the batch boundary, or a warp that holds one walker (its chains run in parallel,
        // so the remaining slots cost no more latency than one): every slot still ahead
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (q >= qc) gb_val[q] = gamma_at(t0 + (uint64_t)(glane + LPW * q));
        gb_ok = 0xfu;
      } else {
        const double v = gamma_at(t0 + (uint64_t)(glane + LPW * qc));
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (q == qc) gb_val[q] = v;
        gb_ok |= 1u << qc;
      }
    }
    const int q = off / LPW;
    double v = q == 0 ? gb_val[0] : q == 1 ? gb_val[1] : q == 2 ? gb_val[2] : gb_val[3];
    if (LPW == 1) return v;
    return __shfl_sync(gmask, v, off % LPW, LPW);
  }

  // ---- have_visited_since_maxentropy as generation stamps ------------------------------
  __device__ bool visited_cur() const { return k_stamp == c.fill_gen ? true : (c.fill_val != 0); }
  __device__ void fill_visited(bool v) { c.fill_gen += 1; c.fill_val = v ? 1 : 0; }

  // ---- prepare_for_state (energy.rs:400-434); false: outside the preallocated planes ---
  __device__ bool prepare(double e) {
    while (e < c.cur_min) {
      if (c.b_lo == 0) return false;
      c.b_lo -= 1;
      if (!SPLIT) {
        if (wr) stamp[c.b_lo] = c.fill_gen;  // inserted as visited, round_trips already 1
        if (c.b_lo == cur) k_stamp = c.fill_gen;
      }
      c.cur_min -= width;
      grew_front = true;
    }
    if (grew_front) cur_max = c.cur_min + width * (double)(c.b_hi - c.b_lo + 1);
    while (e >= cur_max) {
      if (c.b_hi >= nbins - 1) return false;
      c.b_hi += 1;
      if (!SPLIT) {
        if (wr) stamp[c.b_hi] = c.fill_gen;
        if (c.b_hi == cur) k_stamp = c.fill_gen;
      }
      cur_max = c.cur_min + width * (double)(c.b_hi - c.b_lo + 1);
    }
    cminf = f32_trunc(c.cur_min);
    cmaxf = f32_trunc(cur_max);
    return true;
  }
  // After the front grew the reference recomputes every local index with the new
  // bins.min; refresh the cached indices the same way.
  __device__ void reindex_after_growth() {
    move_cur(gidx_exact(c.E));
    if (kind() == M_SAD) { win_lo = gidx_exact(c.too_lo); win_hi = gidx_exact(c.too_hi); }
  }

  // e < too_lo and e > too_hi from the bin index g of e: the index is monotone in e, so
  // only e in the window's edge bin needs the FP64 comparison.
  __device__ bool below(double e, int g) const {
    return g < win_lo ? true : (g > win_lo ? false : e < c.too_lo);
  }
  __device__ bool above(double e, int g) const {
    return g > win_hi ? true : (g < win_hi ? false : e > c.too_hi);
  }
  __device__ double sad_lnw(double e, int g) const {  // energy.rs:451-464
    if (below(e, g)) return ld_lnw(win_lo) + div_by(e - c.too_lo, c.min_T, inv_minT);
    if (above(e, g)) return ld_lnw(win_hi);
    return ld_lnw(g);
  }

  __device__ void set_E(double e) {
    c.E = e;
    E2 = e * e;
    Ef = f32_trunc(e);
  }

  // ln w the Metropolis test would use at energy e (no bin growth; energies outside the
  // allocated bins read 0, the value a newly allocated bin starts with, or the SAD
  // extrapolation).  Used for the surrogate stage of delayed-acceptance moves.
  __device__ double lnw_at(double e) const {
    int g;
    if (e < c.cur_min) g = c.b_lo - 1;
    else if (e >= cur_max) g = c.b_hi + 1;
    else g = gidx(e);  // the FP32-estimate index, identical to gidx_exact's
    if (kind() == M_SAD) {
      if (e < c.too_lo) return ld_lnw(win_lo) + div_by(e - c.too_lo, c.min_T, inv_minT);
      if (e > c.too_hi) return ld_lnw(win_hi);
    }
    if (g < c.b_lo || g > c.b_hi) return 0.0;
    return ld_lnw(g);
  }
  __device__ double lnw_current() const {
    return kind() == M_SAD ? sad_lnw(c.E, cur) : k_lnw;
  }

  // ---- one move ----------------------------------------------------------------------
  __device__ void begin_move(double one_minus_rs) {
    c.moves += 1;                  // energy.rs:905
    if (!SPLIT) c.acc_rate *= one_minus_rs;    // energy.rs:913-914
    e1 = c.E;
    grew_front = false;
  }

  // Bounds test, prepare_for_state and reject_move (energy.rs:915-931) for
  // e2 = E + (double)de with de in binary32; true = accept.  Each
  // comparison of the reference on e2 is first taken on the binary32 estimate
  // e2f = Ef + de, whose error is below tol (|E - Ef| < |E| 2^-23, one binary32 rounding,
  // one binary64 rounding); inside the bound, or wherever the exact value enters
  // arithmetic (SAD extrapolation, window edges, discoveries, the accepted energy), the
  // FP64 e2 is formed and the reference's comparison is evaluated on it.
  // has_first: the Metropolis test uses lnw_first in place of ln w(E) -- the second stage
  // of a delayed-acceptance move, which accepts with min(1, exp(ln w(E~) - ln w(e2))) for
  // the surrogate-predicted energy E~.
  // The group takes lane 0's decision (all lanes hold the same state, so they agree).
  __device__ bool decide_de(bool possible, float de, uint64_t u53, double rs,
                            bool has_first = false, double lnw_first = 0.0) {
    double e2 = 0.0;
    bool have = false;
    const bool accepted = uni(!rejects(possible, de, u53, has_first, lnw_first, e2, have));
    if (accepted) {
      if (c.kind != M_DESCENT) { c.accepted += 1; if (!SPLIT) c.acc_rate += rs; }
      set_E(have ? e2 : c.E + f2d(de));
    }
    return accepted;
  }
  __device__ bool rejects(bool possible, float de, uint64_t u53, bool has_first,
                          double lnw_first, double& e2, bool& have) {
    if (!possible || !(fabsf(de) <= 3.0e38f)) return true;
    const float e2f = Ef + de;
    const float tol = (fabsf(Ef) + fabsf(e2f)) * 2.5e-7f + 1e-30f;
    // The FP64 e2 is formed here, once and by every walker of the warp alike: taken at
    // each place that needs it, the walkers' different places each cost the warp an FP64
    // instruction of their own.
    e2 = c.E + f2d(de);
    have = true;
    auto exact = [&]() -> double { return e2; };
    // e2 > T (T's binary32 copy Tf within |T| 2^-23)
    auto gt = [&](float Tf, double T) -> bool {
      const float m = tol + fabsf(Tf) * 2.5e-7f;
      const float d = e2f - Tf;
      if (d > m) return true;
      if (d < -m) return false;
      return exact() > T;
    };
    auto lt = [&](float Tf, double T) -> bool {
      const float m = tol + fabsf(Tf) * 2.5e-7f;
      const float d = e2f - Tf;
      if (d < -m) return true;
      if (d > m) return false;
      return exact() < T;
    };
    // e2 > E (resp. e2 < E): the sign of de unless de is within rounding of E
    const float tiny = fabsf(Ef) * 1e-15f + 1e-37f;
    auto gtE = [&]() -> bool { return de > tiny ? true : (de <= 0.0f ? false : exact() > c.E); };
    auto ltE = [&]() -> bool { return de < -tiny ? true : (de >= 0.0f ? false : exact() < c.E); };
    bool oob = false;
    if (has_max_allowed) oob = gt(maxf, max_allowed) && gtE();
    if (has_min_allowed) oob = oob || (lt(minf, min_allowed) && ltE());
    if (oob) return true;
    if (c.kind == M_DESCENT) return !ltE();
    // prepare_for_state: only when e2 may lie outside [cur_min, cur_max)
    if (SADMC_RARE(lt(cminf, c.cur_min) || !lt(cmaxf, cur_max))) {
      if (!prepare(exact())) { c.status |= ST_BIN_RANGE; return true; }
      if (grew_front) reindex_after_growth();
    }
    // state_to_index, from the binary32 estimate unless it lies within its error bound
    // of a bin edge
    {
      const float q = (e2f - cminf) * inv_wf;
      const int qi = __float2int_rd(q);
      const float fr = q - (float)qi;
      const float m = (tol + fabsf(cminf) * 2.5e-7f) * inv_wf + fabsf(q) * 2.5e-7f + 1e-6f;
      i2 = (fr > m && fr < 1.0f - m) ? qi + c.b_lo : gidx(e2);
    }
    if (SADMC_RARE(i2 < c.b_lo || i2 > c.b_hi)) {
      c.status |= ST_BIN_RANGE;
      return true;
    }
    fetch_pending(i2);
    const double lnw2_raw = p_lnw;
    hist2 = p_hist;
    bool rejected;
    switch (kind()) {
      case M_SAD: {
        const double lnw1 = has_first ? lnw_first : sad_lnw(c.E, cur);
        if (i2 <= win_lo || i2 >= win_hi) exact();  // extrapolation / edge comparisons
        const double lnw2 = sad_lnw(e2, i2);
        rejected = dgt(lnw2, lnw1) && metropolis_reject2(lnw1, lnw2, u53);
        if (SADMC_RARE(!rejected && hist2 == 0)) {  // energy.rs:466-483
          exact();
          if (e2 < c.too_hi && e2 > c.too_lo) {
            c.latest_param = div_by(c.too_hi - c.too_lo, c.min_T, inv_minT);
            c.num_states += 1;
            c.tL = c.moves;
            invalidate_gamma();
          }
        }
        break;
      }
      case M_SAMC: {
        const double lnw1 = has_first ? lnw_first : k_lnw;
        rejected = dgt(lnw2_raw, lnw1) && metropolis_reject2(lnw1, lnw2_raw, u53);
        break;
      }
      case M_WL:
      case M_INV_T_WL: {
        const double lnw1 = has_first ? lnw_first : k_lnw;
        rejected = dgt(lnw2_raw, lnw1) && metropolis_reject2(lnw1, lnw2_raw, u53);
        if (!rejected && hist2 == 0 && c.lowest_hist > 0) c.wl_num_states += 1.0;
        break;
      }
      default: {  // canonical (energy.rs:504-510)
        rejected = gtE() ? metropolis_reject((c.E - exact()) / c.temperature, u53) : false;
        break;
      }
    }
    return rejected;
  }

  // Histogram, energy sums, update_weights and max-entropy bookkeeping
  // (energy.rs:934-965).  Call after the system confirmed (c.E updated) or not.
  __device__ void finish_move(bool accepted) {
    if (c.kind == M_DESCENT) return;
    int old_cur = cur;
    if (accepted) adopt_pending(i2);
    const double E = c.E;
    if (SADMC_RARE(k_hist == 0)) {  // energy.rs:938-940
      k_tf = c.moves;
      if (kind() == M_SAD && cur >= win_lo && cur <= win_hi && c.moves > c.win_tmax) c.win_tmax = c.moves;
    }
    k_hist += 1;
    if (!SPLIT) {
      k_sE += E;
      k_sE2 += E2;  // E2 == E * E (set_E)
    }
    if (SPLIT) tsc_event = false;
    update_weights(E);
    const int li = cur - c.b_lo;
    if (SPLIT) {
      out_li = li;
      out_i1l = (grew_front ? gidx_exact(e1) : old_cur) - c.b_lo;
      return;
    }
    if (dgt(k_lnw, c.max_S)) {
      c.max_S = k_lnw;
      c.max_S_local = li;
      fill_visited(true);
    } else if (li == c.max_S_local) {
      int i1 = grew_front ? gidx_exact(e1) : old_cur;
      if (i1 - c.b_lo != li) fill_visited(false);
    } else if (!visited_cur()) {
      k_stamp = c.fill_gen;
      if (wr) { stamp[cur] = c.fill_gen; rt[cur] = rt[cur] + 1; }
    }
  }

  // energy.rs:514-761
  __device__ void update_weights(double energy) {
    double g = gamma();
    if (SADMC_RARE(is_nan64(g))) c.status |= ST_NAN_GAMMA;
    double old = k_lnw;
    k_lnw += g;
    if (kind() == M_SAD) sad_update(energy, old);
    else if (kind() == M_WL || kind() == M_INV_T_WL) wl_update();
  }

  __device__ void sad_update(double energy, double old_lnw) {  // energy.rs:523-636
    const bool e_below = below(energy, cur), e_above = above(energy, cur);
    if (inverted || e_below || e_above) k_lnw = old_lnw;
    if (SADMC_RARE(k_hist > c.highest_hist)) {
      c.highest_hist = k_hist;
      if (e_above) {
        const double base = ld_lnw(win_hi);
        const int jlo = win_hi > c.b_lo ? win_hi : c.b_lo;
        const int jhi = cur < c.b_hi ? cur : c.b_hi;
        for (int j = jlo; j <= jhi; ++j) {
          double ej = center(j);
          if (ej > c.too_hi && ej <= energy) {
            if (ld_hist(j) != 0) { st_lnw(j, base); c.num_states += 1; }
            else st_lnw(j, 0.0);
          }
        }
        c.latest_param = div_by(energy - c.too_lo, c.min_T, inv_minT);
        c.tL = c.moves;
        c.too_hi = center(cur);
        inverted = c.too_lo > c.too_hi;
        const int nhi = gidx_exact(c.too_hi);
        for (int j = win_hi + 1; j <= nhi; ++j) {
          uint64_t t = ld_tf(j);
          if (t > c.win_tmax) c.win_tmax = t;
        }
        win_hi = nhi;
        invalidate_gamma();
      } else if (e_below) {
        const double base = ld_lnw(win_lo);
        const int jlo = cur > c.b_lo ? cur : c.b_lo;
        const int jhi = win_lo < c.b_hi ? win_lo : c.b_hi;
        for (int j = jlo; j <= jhi; ++j) {
          double ej = center(j);
          if (ej < c.too_lo && ej >= energy) {
            if (ld_hist(j) != 0) {
              double v = base + (ej - c.too_lo) / c.min_T;
              if (v < 0.0) v = 0.0;
              st_lnw(j, v);
              c.num_states += 1;
            } else {
              st_lnw(j, 0.0);
            }
          }
        }
        c.latest_param = div_by(c.too_hi - energy, c.min_T, inv_minT);
        c.tL = c.moves;
        c.too_lo = center(cur);
        inverted = c.too_lo > c.too_hi;
        const int nlo = gidx_exact(c.too_lo);
        for (int j = nlo; j < win_lo; ++j) {
          uint64_t t = ld_tf(j);
          if (t > c.win_tmax) c.win_tmax = t;
        }
        win_lo = nlo;
        invalidate_gamma();
      }
    }
    if (SADMC_RARE(c.tL == c.moves)) {
      uint64_t old_tF = c.tF;
      c.tF = c.win_tmax;
      invalidate_gamma();
      if (SPLIT) {
        tsc_event = old_tF != c.tF && acc_mode;
      } else if (old_tF != c.tF && acc_mode) {  // energy.rs:600-609
        c.tscale *= rate_factor(c.acc_rate, target_rate, inv_target);
        tscale_changed = true;
      }
    }
  }

  __device__ void wl_zero_range(int lo, int hi) {
    for (int j = lo + glane; j <= hi; j += LPW)
      if (wr) wlh[j] = 0;
    sync();
  }

  __device__ void wl_update() {  // energy.rs:638-752
    const bool inv_t = kind() == M_INV_T_WL;
    if (uni(c.has_min_gamma && c.gamma < c.min_gamma)) {  // production run
      int k = c.wl_lo + (cur - c.b_lo);
      if (k >= c.wl_lo && k <= c.wl_hi) { if (wr) wlh[k] = wlh[k] + 1; }
      else c.status |= ST_BIN_RANGE;
      return;
    }
    const int len_b = c.b_hi - c.b_lo + 1;
    int len_w = c.wl_hi >= c.wl_lo ? c.wl_hi - c.wl_lo + 1 : 0;
    if (uni(len_w != len_b)) {
      if (uni(len_w == 0 || (c.gamma != 1.0 && c.lowest_hist > 0))) {
        c.gamma = 1.0;
        c.lowest_hist = 0;
        c.wl_highest_hist = 0;
        c.total_hist = 0;
        c.wl_lo = c.b_lo;
        c.wl_hi = c.b_hi;
        wl_zero_range(c.wl_lo, c.wl_hi);
        c.min_energy = c.cur_min;
      } else {
        for (int guard = 0; c.min_energy > c.cur_min; ++guard) {
          if (guard > nbins || c.wl_lo <= 0) { c.status |= ST_BIN_RANGE; break; }
          c.min_energy -= width;
          c.wl_lo -= 1;
          if (wr) wlh[c.wl_lo] = 0;
          ++len_w;  // hist.insert(0, 0) lengthens hist (energy.rs:678-681)
        }
        while (len_w < len_b) {
          c.wl_hi += 1;
          if (wr && c.wl_hi < nbins) wlh[c.wl_hi] = 0;
          ++len_w;
        }
        sync();
        uint64_t mn = ~0ull;
        for (int j = c.wl_lo + glane; j <= c.wl_hi; j += LPW) {
          uint64_t h = wlh[j];
          mn = h < mn ? h : mn;
        }
        c.lowest_hist = group_min(mn);
      }
      len_w = c.wl_hi - c.wl_lo + 1;
    }
    const int k = c.wl_lo + (cur - c.b_lo);
    const uint64_t h = wlh[k] + 1;
    if (wr) wlh[k] = h;
    if (h > c.wl_highest_hist) c.wl_highest_hist = h;
    c.total_hist += 1;
    const double max_energy = c.min_energy + (double)len_w * width;
    bool cond = h == c.lowest_hist + 1 && len_w > 1 &&
                (!has_min_allowed || min_allowed >= c.min_energy) &&
                (!has_max_allowed || max_allowed <= max_energy);
    if (uni(cond)) {
      sync();
      uint64_t mn = ~0ull;
      for (int j = glane; j < len_w; j += LPW) {
        if (ld_hist(c.b_lo + j) != 0) {
          uint64_t v = wlh[c.wl_lo + j];
          mn = v < mn ? v : mn;
        }
      }
      mn = group_min(mn);
      cond = mn == c.lowest_hist + 1;
    }
    if (uni(cond)) {
      c.lowest_hist = h;
      if ((inv_t && c.lowest_hist > 0) ||
          (double)c.lowest_hist >= 0.8 * (double)c.total_hist / c.wl_num_states) {
        c.gamma *= 0.5;
        wl_zero_range(c.wl_lo, c.wl_hi);
        c.total_hist = 0;
        c.lowest_hist = 0;
        c.wl_highest_hist = 0;
        if (c.has_min_gamma && c.gamma < c.min_gamma) c.gamma = 0.0;
      }
      if (inv_t && c.gamma < c.wl_num_states / (double)c.moves) {  // energy.rs:747-750
        c.kind = M_SAMC;
        c.t0 = c.wl_num_states;
        invalidate_gamma();
      }
    }
  }
};

// sqrt(1/t) and 1 - sqrt(1/t) (energy.rs:913) for 32 consecutive t, one per lane.
struct RecentScale {
  uint32_t off;  // calls since the batch was taken (32: take the next batch)
  double rs, omrs;
  __device__ void init() { off = 32; }
  // called once per move with consecutive t
  __device__ void get(uint64_t t, int lane, double& r, double& om) {
    if (SADMC_RARE(off >= 32)) {
      off = 0;
      double v = sqrt(1.0 / (double)(t + (uint64_t)lane));
      rs = v;
      omrs = 1. - v;
    }
    const int src = (int)off++;
    r = __shfl_sync(0xffffffffu, rs, src);
    om = __shfl_sync(0xffffffffu, omrs, src);
  }
};

}  // namespace dev
}  // namespace sadmc
