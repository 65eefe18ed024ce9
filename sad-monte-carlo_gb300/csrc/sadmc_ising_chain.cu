// One Ising walker as a serial chain (src/system/ising.rs with the bookkeeping of
// src/mc/energy.rs), the shape of a single-walker run.
//
// A lone walker's Markov chain is sequential: each move's decision reads the weights the
// previous move updated.  Two kernels run it with the walker's bin planes and spins in
// shared memory:
//  * ising_chain_kernel (Wang-Landau, 1/t-WL, SAMC, canonical): lane 0 runs the chain;
//    what does not depend on it is computed ahead by the whole warp, 32 moves at a time,
//    into shared-memory tables: the Philox draws of each move, the acceptance-rate factor
//    sqrt(1/t) and the SAMC gamma;
//  * ising_sad_pipe_kernel (SAD): three warps, one deciding, one filling the next
//    batch's tables, one replaying the bookkeeping no decision reads (below).
// A parameter change inside a batch (a SAD discovery, a window edge, a new tF)
// invalidates the gamma table, and the deciding lane computes gamma itself until the next
// valid table, so every value is the one the reference's arithmetic gives.
#include <cuda_runtime.h>

#include <atomic>

#include "sadmc_common.cuh"
#include "sadmc_fh.cuh"
#include "sadmc_launch.h"
#include "sadmc_rng.cuh"

namespace sadmc {
namespace dev {

struct ChainTables {
  uint16_t i[32], j[32];
  uint64_t u53[32];
  double rs[32], omrs[32];  // sqrt(1/t) and 1 - sqrt(1/t) (energy.rs:913)
  double gamma[32];
};

// Bytes of shared memory: 8 planes of 8 B per bin, the spins, the tables.
__host__ __device__ inline size_t ising_chain_bytes(int nbins, int L) {
  return (size_t)nbins * 64 + (((size_t)L * (size_t)L + 15) & ~(size_t)15) + sizeof(ChainTables);
}

template <int FAM>
__global__ void __launch_bounds__(32, 1) ising_chain_kernel(MoveLaunch m, IsingSys s) {
  extern __shared__ __align__(16) unsigned char stage[];
  const int lane = threadIdx.x;
  const int w = blockIdx.x;  // one walker per block of one warp
  Fh<1, FAM> fh;
  fh.load(m.cores, m.P, m.B, w, 1u << lane, 0, lane == 0);
  const int L = s.L;
  const int nb = m.P.nbins;
  int8_t* gS = s.spins + (size_t)w * (size_t)L * (size_t)L;
  double* gp[3] = {fh.lnw, fh.sE, fh.sE2};
  uint64_t* gq[5] = {fh.hist, fh.tf, fh.rt, fh.wlh, fh.stamp};
  double* sd = reinterpret_cast<double*>(stage);
  uint64_t* sq = reinterpret_cast<uint64_t*>(sd + 3 * (size_t)nb);
  int8_t* S = reinterpret_cast<int8_t*>(sq + 5 * (size_t)nb);
  ChainTables* tb = reinterpret_cast<ChainTables*>(S + (((size_t)L * (size_t)L + 15) & ~(size_t)15));
  for (int a = 0; a < 3; ++a)
    for (int k = lane; k < nb; k += 32) sd[(size_t)a * nb + k] = gp[a][k];
  for (int a = 0; a < 5; ++a)
    for (int k = lane; k < nb; k += 32) sq[(size_t)a * nb + k] = gq[a][k];
  for (int k = lane; k < L * L; k += 32) S[k] = gS[k];
  __syncwarp();
  fh.lnw = sd; fh.sE = sd + nb; fh.sE2 = sd + 2 * (size_t)nb;
  fh.hist = sq; fh.tf = sq + nb; fh.rt = sq + 2 * (size_t)nb; fh.wlh = sq + 3 * (size_t)nb;
  fh.stamp = sq + 4 * (size_t)nb;
  fh.xg = tb->gamma;

  for (uint64_t base = 0; base < m.n_moves; base += 32) {
    const int cnt = (int)(m.n_moves - base < 32 ? m.n_moves - base : 32);
    // ---- the warp fills the next batch's tables from lane 0's current state ----------
    const uint64_t moves0 = __shfl_sync(0xffffffffu, fh.c.moves, 0);
    const int kind = __shfl_sync(0xffffffffu, fh.kind(), 0);
    const double p = __shfl_sync(0xffffffffu, fh.c.latest_param, 0);
    const uint64_t tF = __shfl_sync(0xffffffffu, fh.c.tF, 0);
    const uint64_t ns = __shfl_sync(0xffffffffu, fh.c.num_states, 0);
    const double t0 = __shfl_sync(0xffffffffu, fh.c.t0, 0);
    if (lane < cnt) {
      const uint64_t t = moves0 + 1 + (uint64_t)lane;
      const Draws d = draws_ising(m.seed, (uint32_t)w, t, (uint32_t)L);
      tb->i[lane] = (uint16_t)d.which;
      tb->j[lane] = (uint16_t)d.j;
      tb->u53[lane] = d.u53;
      const double v = sqrt(1.0 / (double)t);  // RecentScale's expression
      tb->rs[lane] = v;
      tb->omrs[lane] = 1. - v;
      double g = 0.0;
      if (kind == M_SAD) g = sad_gamma_value(p, tF, ns, t);
      else if (kind == M_SAMC) { const double td = u2d(t); g = td > t0 ? t0 / td : 1.0; }
      tb->gamma[lane] = g;
    }
    __syncwarp();
    // ---- lane 0 runs the chain --------------------------------------------------------
    if (lane == 0) {
      fh.xg_t0 = moves0 + 1;
      fh.xg_ok = true;
      for (int k = 0; k < cnt; ++k) {
        const uint64_t t = fh.c.moves + 1;
        fh.begin_move(tb->omrs[k]);
        const int i = tb->i[k], j = tb->j[k];
        const int jp = j + 1 == L ? 0 : j + 1, jm = j == 0 ? L - 1 : j - 1;
        const int ip = i + 1 == L ? 0 : i + 1, im = i == 0 ? L - 1 : i - 1;
        const int site = i + j * L;
        const int sij = S[site];
        const int nt = S[i + jp * L] + S[i + jm * L] + S[ip + j * L] + S[im + j * L];
        const float de = (float)(-(nt * sij * 2));  // exact: |de| <= 8
        if (SADMC_RARE(m.trace && t > m.trace_t0 && t - m.trace_t0 <= m.trace_cap)) {
          TraceRec r;
          r.e1 = fh.c.E;
          r.e2 = fh.c.E + (double)de;
          m.trace[(size_t)w * m.trace_cap + (t - m.trace_t0 - 1)] = r;
        }
        const bool acc = fh.decide_de(true, de, tb->u53[k], tb->rs[k]);
        if (acc) S[site] = (int8_t)(-sij);
        fh.finish_move(acc);
      }
    }
    __syncwarp();
  }
  fh.store(m.cores, w);
  __syncwarp();
  for (int a = 0; a < 3; ++a)
    for (int k = lane; k < nb; k += 32) gp[a][k] = sd[(size_t)a * nb + k];
  for (int a = 0; a < 5; ++a)
    for (int k = lane; k < nb; k += 32) gq[a][k] = sq[(size_t)a * nb + k];
  for (int k = lane; k < L * L; k += 32) gS[k] = S[k];
}

// ---- SAD: the chain pipelined over three warps, with an integer fast path ---------------
//
// Warp 0's lane 0 runs the decisions and the state they read: the energy, the bins' ln w,
// histogram and t_found, the SAD window and parameters.  It records each move (bin,
// acceptance, energy, ln w after the update; the local indices and allocated bins of a
// generic move) in a log.  Warp 2's lane 0 replays
// the log of the previous batch for the bookkeeping no decision reads: the acceptance
// rate and translation scale (energy.rs:600-621, 913-914), the energy sums (energy.rs:
// 941-942) and the max-entropy / round-trip stamps (energy.rs:950-965).  Warp 1 fills the
// tables of the next batch of 32 moves: draws, the site and its four neighbours,
// sqrt(1/t), and gamma for the SAD parameters at the start of the current batch (a table
// whose parameters changed since is not used).  A batch boundary is one block barrier;
// the three warps' dependent chains overlap instead of adding up.
//
// Ising energies, bin edges and (for power-of-two bin widths) the SAD window edges are
// integers or half-integers, so the comparisons the reference makes on e2 = E + dE
// (bounds, bin range, state_to_index, window) are integer comparisons against thresholds
// derived exactly once per change (x < T <=> x < ceil(T) for an integer x).  The common
// move -- its proposed bin already visited, no window or bin growth possible, gamma from
// the table -- runs on those integers and the FP64 ln w; every other move (a possible
// discovery, growth of the window or of the bins, a parameter change, a trace) takes the
// generic bookkeeping.
//
// Per move the deciding lane reads one 32-byte table record (two 128-bit loads) and
// writes one 16-byte log record; measured on the single-walker workload, loading the next
// move's spins ahead of the flip (with a reload on conflicts) was slower than loading them
// when needed.
//
// Table record of one move, as eight 32-bit words: site | n0 << 16, n1 | n2 << 16, n3,
// bits of the binary32 lower and upper bounds of ln u for the Metropolis uniform u,
// unused, and gamma (low word, high word).
struct alignas(16) PipeTables {
  uint4 mv[32][2];
  uint64_t u53[32];
  double gamma[32];         // gamma again, as the generic bookkeeping's table
  double rs[32], omrs[32];  // sqrt(1/t) and 1 - sqrt(1/t) (energy.rs:913)
  uint32_t gen;             // Fh::pgen the gamma values were computed for
  uint32_t nan_gamma;       // some gamma of the batch is NaN (the generic path reports it)
  uint32_t pad[2];
};
struct PipeSnap {  // the walker's SAD parameters at a batch boundary
  double p;
  uint64_t tF, ns;
  uint32_t gen;
};
// One move as the bookkeeping warp needs it: ln w of the bin after the update (written
// one move late), and a record of the energy after the move (low 32 bits; Ising energies
// are integers), the bin after the move (bits 32-47; the shared-memory planes of this
// kernel hold at most 3200 bins) and flags (bits 48-63): 1 accepted, 2 tF changed with the acceptance-rate mode on,
// 4 a generic move, whose PipeExt holds its local indices and allocated bins.  After a
// fast-path move the local indices are the bins after and before it minus b_lo, and the
// allocated bins are unchanged.
struct PipeLog {
  double lnw;
  uint64_t rec;
};
struct PipeExt {
  int16_t li, i1l;     // local indices of the bin after and before the move
  int16_t b_lo, b_hi;  // allocated bins after the move (prepare_for_state)
};
struct PipeBook {  // the bookkeeping warp's fields, handed back at the end of a launch
  double acc_rate, tscale, max_S;
  int32_t max_S_local, fill_val;
  uint64_t fill_gen;
};

__host__ __device__ inline size_t ising_pipe_bytes(int nbins, int L) {
  return (size_t)nbins * 64 + (((size_t)L * (size_t)L + 15) & ~(size_t)15) + 3 * sizeof(PipeTables) +
         2 * 32 * (sizeof(PipeLog) + sizeof(PipeExt)) + 2 * sizeof(PipeSnap) + 2 * sizeof(uint64_t);
}

using FhSplit = Fh<1, M_SAD, true>;

// Integer view of a SAD walker: energy, bin range, window and bounds (see above).
struct LeanSad {
  bool ok;
  int ws;            // log2 of the bin width, or -1 when it is not a power of two
  int Ei, cmin, cmax, tlo, thi, mx, mn;
  int cls;           // -1 / 0 / +1: E below / inside / above the window [too_lo, too_hi]
  double lnw1c;      // ln w at E when cls != 0 (energy.rs:451-464)
};

__device__ __forceinline__ int clamp_floor(double x) {
  const double c = 1073741824.0;  // 2^30
  return x >= c ? (int)c : (x <= -c ? -(int)c : (int)floor(x));
}
__device__ __forceinline__ int clamp_ceil(double x) {
  const double c = 1073741824.0;
  return x >= c ? (int)c : (x <= -c ? -(int)c : (int)ceil(x));
}

// Re-derive the integer view from the walker state after a generic move or at a batch
// start; z.ok = false keeps the walker on the generic bookkeeping.
__device__ void lean_sync(const FhSplit& fh, LeanSad& z, bool traced) {
  z.ok = false;
  if (z.ws < 0 || traced || !fh.xg_ok || fh.inverted || fh.k_hist == 0 || fh.c.kind != M_SAD) return;
  const double E = fh.c.E, cm = fh.c.cur_min, lim = 536870912.0;  // 2^29
  if (!(E == floor(E) && fabs(E) < lim && cm == floor(cm) && fabs(cm) < lim)) return;
  const double span = (double)(fh.c.b_hi - fh.c.b_lo + 1) * fh.width;
  if (!(fabs(cm + span) < lim)) return;
  if (fh.c.highest_hist >= 0x7fffffffull) return;  // the fast path counts in 32 bits
  if (is_nan64(fh.c.too_lo) || is_nan64(fh.c.too_hi) || is_nan64(fh.max_allowed) || is_nan64(fh.min_allowed))
    return;
  z.Ei = (int)E;
  z.cmin = (int)cm;
  z.cmax = (int)(cm + span);  // cur_max, exact
  z.tlo = clamp_ceil(fh.c.too_lo);   // e < too_lo  <=> e < tlo
  z.thi = clamp_floor(fh.c.too_hi);  // e > too_hi  <=> e > thi
  z.mx = fh.has_max_allowed ? clamp_floor(fh.max_allowed) : (1 << 30);
  z.mn = fh.has_min_allowed ? clamp_ceil(fh.min_allowed) : -(1 << 30);
  z.cls = z.Ei < z.tlo ? -1 : (z.Ei > z.thi ? 1 : 0);
  z.lnw1c = z.cls != 0 ? fh.sad_lnw(E, fh.cur) : 0.0;
  z.ok = true;
}

// One common move on the integer view: bounds, reject_move and the decision-side
// bookkeeping of move_once (energy.rs:904-974) for a move whose proposed bin was visited
// before and which can neither grow the window nor the bins.  Returns 0 (rejected) or 1
// (accepted), or 2 without changing anything when the move needs the generic path.  The
// move and acceptance counts and the FP64 energy are the caller's to bring up to date
// (from z.Ei) when the fast path is left.  The common path is straight-line code: the
// loads are issued together and the outcomes merged by selection, so that the compiler
// can overlap its independent parts.
__device__ __forceinline__ int lean_move(FhSplit& fh, LeanSad& z, int de, const uint64_t* u53, float lo,
                                         float hi, double g) {
  const int e2 = z.Ei + de;
  const bool oob = (e2 > z.mx && de > 0) || (e2 < z.mn && de < 0);
  // the proposed bin, clamped into the allocated range so that every load stays inside
  // it; a proposal outside the range is a generic move
  const int i2r = fh.c.b_lo + ((e2 - z.cmin) >> z.ws);
  const int i2 = min(max(i2r, fh.c.b_lo), fh.c.b_hi);
  const double l2m = fh.lnw[i2], lhm = fh.lnw[fh.win_hi];
  const uint64_t h2m = fh.hist[i2];
  const bool same = i2 == fh.cur;
  const uint32_t hist2 = (uint32_t)(same ? fh.k_hist : h2m);
  const int cls2 = e2 < z.tlo ? -1 : (e2 > z.thi ? 1 : 0);
  const uint32_t top = (uint32_t)fh.c.highest_hist;
  // a bin growth (prepare_for_state), a first visit (energy.rs:466-483, 938-940) or a
  // window edge (energy.rs:530-580)
  const bool rare_prop =
      !oob && (e2 < z.cmin || e2 >= z.cmax || hist2 == 0 || (cls2 != 0 && hist2 >= top));
  if (rare_prop || (z.cls != 0 && (uint32_t)fh.k_hist >= top)) return 2;
  const double lnw1 = z.cls == 0 ? fh.k_lnw : z.lnw1c;
  const double l2raw = same ? fh.k_lnw : l2m;
  double lnw2 = cls2 == 0 ? l2raw : (fh.win_hi == fh.cur ? fh.k_lnw : lhm);
  if (cls2 < 0)  // below the window: the linear extrapolation at min_T (energy.rs:461-462)
    lnw2 = fh.ld_lnw(fh.win_lo) + div_by((double)e2 - fh.c.too_lo, fh.c.min_T, fh.inv_minT);
  // rejected = lnw2 > lnw1 && u > exp(lnw1 - lnw2) (energy.rs:461-465): the binary32
  // truncations a, b order the weights unless equal (truncation is monotone), and the
  // test u > exp(d) <=> ln u > d is taken against the bounds [lo, hi] of ln u and the
  // error bound dd of a - b; the FP64 test where those cannot tell
  const float a = f32_trunc(lnw1), b = f32_trunc(lnw2);
  const float df = a - b;
  // |df - (lnw1 - lnw2)| <= (|a| + |b|) 2^-23 + |df| 2^-24; 1e-12 covers exp's FP64 rounding
  const float dd = (fabsf(a) + fabsf(b)) * 1.2e-7f + fabsf(df) * 6.0e-8f + 1e-12f;
  const bool acc_sure = b < a || hi < df - dd;
  const bool rej_sure = b > a && lo > df + dd;
  bool rejected;
  if (SADMC_RARE(!oob && !acc_sure && !rej_sure))
    rejected = dgt(lnw2, lnw1) && u53_to_double(*u53) > exp(lnw1 - lnw2);
  else
    rejected = oob || rej_sure;
  const bool acc = !rejected, moved = acc && !same;
  if (moved) {  // the cached bin moves: write back, take the new one's fields
    fh.lnw[fh.cur] = fh.k_lnw;
    fh.hist[fh.cur] = fh.k_hist;
    fh.tf[fh.cur] = fh.k_tf;
    fh.k_tf = fh.tf[i2];
  }
  fh.cur = moved ? i2 : fh.cur;
  fh.k_lnw = moved ? l2m : fh.k_lnw;
  const uint32_t kh = (uint32_t)(moved ? h2m : fh.k_hist) + 1u;
  fh.k_hist = kh;
  z.Ei = acc ? e2 : z.Ei;
  z.cls = acc ? cls2 : z.cls;
  z.lnw1c = acc ? lnw2 : z.lnw1c;  // ln w at the new E when it lies outside the window
  // SAD updates ln w inside the window only (energy.rs:523-529)
  const bool inw = z.cls == 0;
  const double up = fh.k_lnw + g;
  fh.k_lnw = inw ? up : fh.k_lnw;
  fh.c.highest_hist = inw && kh > top ? kh : top;
  return acc ? 1 : 0;
}

// The bookkeeping warp's replay of one logged move (energy.rs:913-914, 600-609, 941-942,
// 950-965), in the order move_once applies it.
struct Book {
  PipeBook s;
  double target_rate, inv_target;
  int kb_lo, kb_hi;  // allocated bins as last seen
  int kprev;         // bin after the previous move
  int kcur;          // bin whose sums are held in ksE, ksE2
  double ksE, ksE2;
  double *sE, *sE2;
  uint64_t *stamp, *rt;
  __device__ void replay(const PipeLog& e, const PipeExt& x, double rs, double omrs) {
    const int Ei = (int)(uint32_t)e.rec;
    const int cur = (int)((e.rec >> 32) & 0xffffu);
    const unsigned flags = (unsigned)(e.rec >> 48);
    int li, i1l;
    if (flags & 4u) {
      li = x.li;
      i1l = x.i1l;
      while (kb_lo > x.b_lo) stamp[--kb_lo] = s.fill_gen;  // inserted as visited
      while (kb_hi < x.b_hi) stamp[++kb_hi] = s.fill_gen;
    } else {
      li = cur - kb_lo;
      i1l = kprev - kb_lo;
    }
    kprev = cur;
    s.acc_rate *= omrs;
    if (flags & 1u) s.acc_rate += rs;
    if (SADMC_RARE(flags & 2u)) {
      // the guarded quotient: rate_factor gives the same value, but this form keeps the
      // kernel's register allocation, and with it the deciding lane's schedule, as measured
      // (rate_factor here made the single-walker chain 9 % slower)
      double f = (s.acc_rate >= 0x1p-1000 && s.acc_rate <= 0x1p+1000 && target_rate >= 0x1p-1000 &&
                  target_rate <= 0x1p+1000)
                     ? div_by(s.acc_rate, target_rate, inv_target)
                     : s.acc_rate / target_rate;
      f = f < 0.8 ? 0.8 : (f > 1.2 ? 1.2 : f);
      s.tscale *= f;
    }
    if (cur != kcur) {
      if (kcur >= 0) { sE[kcur] = ksE; sE2[kcur] = ksE2; }
      kcur = cur;
      ksE = sE[kcur];
      ksE2 = sE2[kcur];
    }
    const double E = (double)Ei;
    ksE += E;
    ksE2 += E * E;
    if (dgt(e.lnw, s.max_S)) {
      s.max_S = e.lnw;
      s.max_S_local = li;
      s.fill_gen += 1;
      s.fill_val = 1;
    } else if (li == s.max_S_local) {
      if (i1l != li) { s.fill_gen += 1; s.fill_val = 0; }
    } else if (!(stamp[cur] == s.fill_gen || s.fill_val != 0)) {
      stamp[cur] = s.fill_gen;
      rt[cur] = rt[cur] + 1;
    }
  }
};

__global__ void __launch_bounds__(96, 1) ising_sad_pipe_kernel(MoveLaunch m, IsingSys s) {
  extern __shared__ __align__(16) unsigned char stage[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int w = blockIdx.x;  // one walker per block of three warps
  const int L = s.L;
  const int nb = m.P.nbins;
  int8_t* gS = s.spins + (size_t)w * (size_t)L * (size_t)L;
  const size_t off = (size_t)w * (size_t)nb;
  double* gp[3] = {m.B.lnw + off, m.B.sumE + off, m.B.sumE2 + off};
  uint64_t* gq[5] = {m.B.hist + off, m.B.t_found + off, m.B.round_trips + off, m.B.wl_hist + off,
                     m.B.visit_stamp + off};
  double* sd = reinterpret_cast<double*>(stage);
  uint64_t* sq = reinterpret_cast<uint64_t*>(sd + 3 * (size_t)nb);
  int8_t* S = reinterpret_cast<int8_t*>(sq + 5 * (size_t)nb);
  PipeTables* tbs = reinterpret_cast<PipeTables*>(S + (((size_t)L * (size_t)L + 15) & ~(size_t)15));
  PipeLog* logs = reinterpret_cast<PipeLog*>(tbs + 3);
  PipeExt* exts = reinterpret_cast<PipeExt*>(logs + 64);
  PipeSnap* snap = reinterpret_cast<PipeSnap*>(exts + 64);
  uint64_t* t_launch = reinterpret_cast<uint64_t*>(snap + 2);  // move count, first bin
  for (int a = 0; a < 3; ++a)
    for (int k = tid; k < nb; k += 96) sd[(size_t)a * nb + k] = gp[a][k];
  for (int a = 0; a < 5; ++a)
    for (int k = tid; k < nb; k += 96) sq[(size_t)a * nb + k] = gq[a][k];
  for (int k = tid; k < L * L; k += 96) S[k] = gS[k];
  __syncthreads();

  FhSplit fh;
  LeanSad z;
  Book bk;
  if (tid == 0) {
    fh.load(m.cores, m.P, m.B, w, 1u, 0, true);
    fh.lnw = sd; fh.sE = sd + nb; fh.sE2 = sd + 2 * (size_t)nb;
    fh.hist = sq; fh.tf = sq + nb; fh.rt = sq + 2 * (size_t)nb; fh.wlh = sq + 3 * (size_t)nb;
    fh.stamp = sq + 4 * (size_t)nb;
    fh.cur = -1;  // the cached bin is re-read from the staged planes
    fh.load_cur(fh.gidx_exact(fh.c.E));
    z.ws = -1;
    for (int k = 0; k <= 20; ++k)
      if (fh.width == (double)(1 << k)) z.ws = k;
    snap[0] = PipeSnap{fh.c.latest_param, fh.c.tF, fh.c.num_states, fh.pgen};
    t_launch[0] = fh.c.moves;
    t_launch[1] = (uint64_t)fh.cur;
  } else if (tid == 64) {
    const WalkerCore& c = m.cores[w];
    bk.s = PipeBook{c.acc_rate, c.tscale, c.max_S, c.max_S_local, c.fill_val, c.fill_gen};
    bk.target_rate = m.P.target_rate;
    bk.inv_target = m.P.inv_target;
    bk.kb_lo = c.b_lo;
    bk.kb_hi = c.b_hi;
    bk.kcur = -1;
    bk.ksE = bk.ksE2 = 0.0;
    bk.sE = sd + nb; bk.sE2 = sd + 2 * (size_t)nb;
    bk.stamp = sq + 4 * (size_t)nb; bk.rt = sq + 2 * (size_t)nb;
  }
  __syncthreads();
  const uint64_t t0 = t_launch[0];
  if (tid == 64) bk.kprev = (int)t_launch[1];
  const uint64_t n = m.n_moves;
  const uint64_t nbatch = (n + 31) / 32;
  // warp 1: the tables of batch c from the parameters in snap[q]
  auto fill = [&](uint64_t c, int q) {
    PipeTables* T = &tbs[c % 3];
    const PipeSnap P = snap[q];
    const uint64_t t = t0 + 32 * c + 1 + (uint64_t)lane;
    const Draws d = draws_ising(m.seed, (uint32_t)w, t, (uint32_t)L);
    const int i = (int)d.which, j = (int)d.j;
    const int jp = j + 1 == L ? 0 : j + 1, jm = j == 0 ? L - 1 : j - 1;
    const int ip = i + 1 == L ? 0 : i + 1, im = i == 0 ? L - 1 : i - 1;
    const unsigned site = (unsigned)(i + j * L);
    const unsigned n0 = (unsigned)(i + jp * L), n1 = (unsigned)(i + jm * L), n2 = (unsigned)(ip + j * L),
                   n3 = (unsigned)(im + j * L);
    T->u53[lane] = d.u53;
    // u lies in [top, top + 1) 2^-24; logf is within 1 ulp, widened by 2^-20
    const uint32_t top = (uint32_t)(d.u53 >> 29);
    const float uf = (float)top * (1.0f / 16777216.0f), uh = (float)(top + 1u) * (1.0f / 16777216.0f);
    const float lo = top == 0u ? -INFINITY : logf(uf) * (1.0f + 9.6e-7f);
    const float hi = logf(uh) * (1.0f - 9.6e-7f);
    const double v = sqrt(1.0 / (double)t);  // RecentScale's expression
    T->rs[lane] = v;
    T->omrs[lane] = 1. - v;
    const double gm = sad_gamma_value(P.p, P.tF, P.ns, t);
    T->gamma[lane] = gm;
    T->mv[lane][0] = make_uint4(site | (n0 << 16), n1 | (n2 << 16), n3, __float_as_uint(lo));
    T->mv[lane][1] = make_uint4(__float_as_uint(hi), 0u, (unsigned)__double2loint(gm), (unsigned)__double2hiint(gm));
    const unsigned nan_any = __ballot_sync(0xffffffffu, is_nan64(gm));
    if (lane == 0) { T->gen = P.gen; T->nan_gamma = nan_any != 0u ? 1u : 0u; }
  };
  if (warp == 1 && nbatch > 0) fill(0, 0);
  __syncthreads();
  const bool traced = m.trace != nullptr;
  for (uint64_t b = 0; b <= nbatch; ++b) {
    if (warp == 1) {
      if (b + 1 < nbatch) fill(b + 1, (int)(b & 1));
    } else if (warp == 2) {
      if (lane == 0 && b > 0) {  // replay the previous batch
        const PipeTables* T = &tbs[(b - 1) % 3];
        const PipeLog* lg = &logs[((b - 1) & 1) * 32];
        const PipeExt* xs = &exts[((b - 1) & 1) * 32];
        const int cnt = (int)(n - 32 * (b - 1) < 32 ? n - 32 * (b - 1) : 32);
        for (int k = 0; k < cnt; ++k) bk.replay(lg[k], xs[k], T->rs[k], T->omrs[k]);
      }
    } else if (lane == 0 && b < nbatch) {
      const PipeTables* T = &tbs[b % 3];
      PipeLog* lg = &logs[(b & 1) * 32];
      PipeExt* xs = &exts[(b & 1) * 32];
      const int cnt = (int)(n - 32 * b < 32 ? n - 32 * b : 32);
      fh.xg = T->gamma;
      fh.xg_t0 = fh.c.moves + 1;
      fh.xg_ok = T->gen == fh.pgen && T->nan_gamma == 0u;
      lean_sync(fh, z, traced);
      const uint64_t mbase = fh.c.moves;  // fast-path moves leave the counts to this loop
      unsigned lacc = 0;                  // fast-path acceptances not yet counted
      double pend_lnw = 0.0;  // the previous move's ln w, logged one move late
      uint4 nx0 = T->mv[0][0], nx1 = T->mv[0][1];  // the next move's table record
      for (int k = 0; k < cnt; ++k) {
        const uint4 qa = nx0, qb = nx1;
        if (k + 1 < cnt) { nx0 = T->mv[k + 1][0]; nx1 = T->mv[k + 1][1]; }
        const int site = (int)(qa.x & 0xffffu);
        const int sc = S[site];
        const int nt = S[qa.x >> 16] + S[qa.y & 0xffffu] + S[qa.y >> 16] + S[qa.z];
        const int de = -(nt * sc * 2);  // exact: |de| <= 8
        const double g = __hiloint2double((int)qb.w, (int)qb.z);
        int r = z.ok ? lean_move(fh, z, de, &T->u53[k], __uint_as_float(qa.w), __uint_as_float(qb.x), g) : 2;
        unsigned flags = 0u;
        int Elog = z.Ei;
        if (SADMC_RARE(r == 2)) {  // the generic bookkeeping
          fh.c.moves = mbase + (uint64_t)k;
          fh.c.accepted += lacc;
          lacc = 0;
          if (z.ok) fh.c.E = (double)z.Ei;
          const uint64_t t = fh.c.moves + 1;
          fh.Ef = f32_trunc(fh.c.E);
          fh.begin_move(T->omrs[k]);
          if (SADMC_RARE(traced && t > m.trace_t0 && t - m.trace_t0 <= m.trace_cap)) {
            TraceRec rec;
            rec.e1 = fh.c.E;
            rec.e2 = fh.c.E + (double)de;
            m.trace[(size_t)w * m.trace_cap + (t - m.trace_t0 - 1)] = rec;
          }
          r = fh.decide_de(true, (float)de, T->u53[k], T->rs[k]) ? 1 : 0;
          fh.finish_move(r == 1);
          lean_sync(fh, z, traced);
          xs[k] = PipeExt{(int16_t)fh.out_li, (int16_t)fh.out_i1l, (int16_t)fh.c.b_lo, (int16_t)fh.c.b_hi};
          flags = 4u | (fh.tsc_event ? 2u : 0u);
          Elog = (int)fh.c.E;
        } else {
          lacc += (unsigned)r;
        }
        if (k > 0) lg[k - 1].lnw = pend_lnw;
        pend_lnw = fh.k_lnw;
        lg[k].rec = (uint64_t)(uint32_t)Elog | ((uint64_t)(uint32_t)fh.cur << 32) |
                    ((uint64_t)(flags | (unsigned)r) << 48);
        if (r == 1) S[site] = (int8_t)(-sc);
      }
      if (cnt > 0) lg[cnt - 1].lnw = pend_lnw;
      fh.c.moves = mbase + (uint64_t)cnt;
      fh.c.accepted += lacc;
      if (z.ok) fh.c.E = (double)z.Ei;
      snap[(b + 1) & 1] = PipeSnap{fh.c.latest_param, fh.c.tF, fh.c.num_states, fh.pgen};
    }
    __syncthreads();
  }
  if (tid == 0) {
    fh.store(m.cores, w);
  } else if (tid == 64) {
    if (bk.kcur >= 0) { bk.sE[bk.kcur] = bk.ksE; bk.sE2[bk.kcur] = bk.ksE2; }
    WalkerCore* o = &m.cores[w];
    o->acc_rate = bk.s.acc_rate; o->tscale = bk.s.tscale; o->max_S = bk.s.max_S;
    o->max_S_local = bk.s.max_S_local; o->fill_val = bk.s.fill_val; o->fill_gen = bk.s.fill_gen;
  }
  __syncthreads();
  for (int a = 0; a < 3; ++a)
    for (int k = tid; k < nb; k += 96) gp[a][k] = sd[(size_t)a * nb + k];
  for (int a = 0; a < 5; ++a)
    for (int k = tid; k < nb; k += 96) gq[a][k] = sq[(size_t)a * nb + k];
  for (int k = tid; k < L * L; k += 96) gS[k] = S[k];
}


template <int FAM>
cudaError_t launch_chain(const MoveLaunch& m, const IsingSys& s, size_t bytes, size_t max_bytes,
                         cudaStream_t st) {
  static std::atomic<bool> attr[64] = {};  // the limit is raised once per device
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return e;
  if (device < 0 || device >= 64 || !attr[device].load(std::memory_order_acquire)) {
    e = cudaFuncSetAttribute(ising_chain_kernel<FAM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_bytes);
    if (e != cudaSuccess) return e;
    if (device >= 0 && device < 64) attr[device].store(true, std::memory_order_release);
  }
  ising_chain_kernel<FAM><<<m.n_walkers, 32, bytes, st>>>(m, s);
  return cudaGetLastError();
}

}  // namespace dev

// the larger of the two chain kernels' needs
size_t ising_chain_bytes(int nbins, int L) {
  const size_t a = dev::ising_chain_bytes(nbins, L), b = dev::ising_pipe_bytes(nbins, L);
  return a > b ? a : b;
}

cudaError_t launch_ising_chain(const MoveLaunch& m, const IsingSys& s, size_t max_bytes, cudaStream_t st) {
  if (m.descent) return cudaErrorInvalidConfiguration;
  if (m.method == M_SAD) {
    const size_t bytes = dev::ising_pipe_bytes(m.P.nbins, s.L);
    if (bytes > max_bytes) return cudaErrorInvalidConfiguration;
    static std::atomic<bool> attr[64] = {};  // the limit is raised once per device
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return e;
    if (device < 0 || device >= 64 || !attr[device].load(std::memory_order_acquire)) {
      e = cudaFuncSetAttribute(dev::ising_sad_pipe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)max_bytes);
      if (e != cudaSuccess) return e;
      if (device >= 0 && device < 64) attr[device].store(true, std::memory_order_release);
    }
    dev::ising_sad_pipe_kernel<<<m.n_walkers, 96, bytes, st>>>(m, s);
    return cudaGetLastError();
  }
  const size_t bytes = dev::ising_chain_bytes(m.P.nbins, s.L);
  if (bytes > max_bytes) return cudaErrorInvalidConfiguration;
  return dev::launch_chain<dev::FAM_ANY>(m, s, bytes, max_bytes, st);
}

}  // namespace sadmc
