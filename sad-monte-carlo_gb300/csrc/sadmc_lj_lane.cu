// The LJ-cluster move kernel with one or two lanes per walker (src/system/lj.rs): 32 or 16
// walkers per warp, their positions in shared memory.
//
// Why: the flat-histogram bookkeeping is FP64 and an FP64 warp instruction costs the same
// whether one lane or 32 use it; with a lane per walker each such instruction serves 32
// walkers (8 with the register kernel's 4-lane groups of 8), and the move needs no group
// shuffles at all.  The pair work, 2 (N-1) binary32 terms, runs in the walker's own lane
// (or two), at full FP32 rate.
//
// Layout: each warp holds its walkers' double-single positions (hi, lo as a float2) in
// shared memory as [coordinate][atom slot][walker of the warp][lane of the walker], atom
// j = lane + LPW * slot, so that the 32 lanes of a warp reading "their" atom of one slot
// touch 32 consecutive 8-byte words (two wavefronts of 16 lanes, no bank conflict; with
// the lanes of a walker 16 walkers apart instead, a wavefront's two halves met the same
// banks).
// Global memory keeps the register kernel's [walker][6][np] planes, so the two kernels
// continue each other's runs.
#include <cuda_runtime.h>

#include <atomic>

#include "sadmc_common.cuh"
#include "sadmc_fh.cuh"
#include "sadmc_launch.h"
#include "sadmc_lj_walker.cuh"
#include "sadmc_rng.cuh"

namespace sadmc {
namespace dev {

// 4 (s^6 - s^3), s = 1/r^2 (lj.rs:78-81) in binary32 with fused steps (the kernels'
// pair terms carry a stated tolerance; the FP64 re-sum and the oracle replay bound it).
__device__ __forceinline__ float lj_v32_fused(float dx, float dy, float dz) {
  const float r2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
  const float s = __fdividef(1.0f, r2);
  const float s3 = __fmul_rn(__fmul_rn(s, s), s);
  return __fmul_rn(4.0f, __fmaf_rn(s3, s3, -s3));
}

template <int LPW, int NP>
struct LjLaneWalker {
  static constexpr int WPW = 32 / LPW;   // walkers per warp
  static constexpr int APL = NP / LPW;   // atom slots per lane
  float2* sp;                            // this warp's [3][APL][WPW][LPW] (hi, lo)
  int slot;                              // this lane's walker within the warp
  int glane;
  unsigned gmask;
  int n;
  float wall_r2f;  // binary32 R^2 of the wall, set once per launch

  __device__ float2& at(int c, int j) const {
    return sp[((c * APL + j / LPW) * WPW + slot) * LPW + j % LPW];
  }
  __device__ void load(const float* p) {
#pragma unroll
    for (int k = 0; k < APL; ++k) {
      const int j = glane + LPW * k;
#pragma unroll
      for (int c = 0; c < 3; ++c) at(c, j) = make_float2(p[c * NP + j], p[(3 + c) * NP + j]);
    }
  }
  __device__ void store(float* p, bool wr) const {
    if (!wr) return;
#pragma unroll
    for (int k = 0; k < APL; ++k) {
      const int j = glane + LPW * k;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float2 v = at(c, j);
        p[c * NP + j] = v.x;
        p[(3 + c) * NP + j] = v.y;
      }
    }
  }
  __device__ void put(int which, DS tx, DS ty, DS tz) {
    if (glane == which % LPW) {
      at(0, which) = make_float2(tx.h, tx.l);
      at(1, which) = make_float2(ty.h, ty.l);
      at(2, which) = make_float2(tz.h, tz.l);
    }
    if (LPW > 1) __syncwarp(gmask);  // the other lane reads the moved atom next move
  }

  // plan_move of lj.rs:365-374 and move_atom of lj.rs:86-105 for a given displacement:
  // possible, and the energy change summed in binary32 over the walker's lanes.
  __device__ bool plan(int which, float g0, float g1, float g2, float sh, float sl, double radius2,
                       DS& tx, DS& ty, DS& tz, float& de_out) const {
    const float2 a = at(0, which), b = at(1, which), c = at(2, which);
    const DS fx{a.x, a.y}, fy{b.x, b.y}, fz{c.x, c.y};
    tx = ds_add(fx, ds_scale(g0, sh, sl));
    ty = ds_add(fy, ds_scale(g1, sh, sl));
    tz = ds_add(fz, ds_scale(g2, sh, sl));
    // wall: impossible iff |to|^2 > R^2 and |to|^2 > |from|^2 (lj.rs:87-90)
    const float r2t = tx.h * tx.h + ty.h * ty.h + tz.h * tz.h;
    const float r2f = fx.h * fx.h + fy.h * fy.h + fz.h * fz.h;
    const float R2 = wall_r2f;
    bool impossible;
    if (r2t < R2 * (1.0f - 1e-5f)) {
      impossible = false;
    } else if (r2t > R2 * (1.0f + 1e-5f) && r2t > r2f * (1.0f + 1e-5f)) {
      impossible = true;
    } else {
      const double x = ds_to_double(tx), y = ds_to_double(ty), z = ds_to_double(tz);
      const double p = ds_to_double(fx), q = ds_to_double(fy), r = ds_to_double(fz);
      const double nt = x * x + y * y + z * z, nf = p * p + q * q + r * r;
      impossible = nt > radius2 && nt > nf;
    }
    if (impossible) return false;
    float dn = 0.0f, dold = 0.0f;
#pragma unroll
    for (int k = 0; k < APL; ++k) {
      const int j = glane + LPW * k;
      if (j < n && j != which) {
        const float2 xj = at(0, j), yj = at(1, j), zj = at(2, j);
        // double-single differences: the high parts of nearby atoms subtract exactly
        dn += lj_v32_fused((xj.x - tx.h) + (xj.y - tx.l), (yj.x - ty.h) + (yj.y - ty.l),
                           (zj.x - tz.h) + (zj.y - tz.l));
        dold += lj_v32_fused((xj.x - fx.h) + (xj.y - fx.l), (yj.x - fy.h) + (yj.y - fy.l),
                             (zj.x - fz.h) + (zj.y - fz.l));
      }
    }
    de_out = group_sum<LPW>(dn - dold, gmask);
    return true;
  }

  // FP64 pair sum over the double-single positions (compute_energy, lj.rs:236-244).
  __device__ double energy64() const {
    double e = 0.0;
#pragma unroll 1
    for (int j = 0; j < n; ++j) {
      const float2 a = at(0, j), b = at(1, j), c = at(2, j);
      const double xj = (double)a.x + (double)a.y, yj = (double)b.x + (double)b.y,
                   zj = (double)c.x + (double)c.y;
#pragma unroll 4
      for (int k = 0; k < APL; ++k) {
        const int i = glane + LPW * k;
        if (i < n && i > j) {
          const float2 p = at(0, i), q = at(1, i), r = at(2, i);
          const double dx = ((double)p.x + (double)p.y) - xj, dy = ((double)q.x + (double)q.y) - yj,
                       dz = ((double)r.x + (double)r.y) - zj;
          const double s = 1.0 / (dx * dx + dy * dy + dz * dz);
          e += 4.0 * (powi6(s) - powi3(s));
        }
      }
    }
    return group_sum<LPW>(e, gmask);
  }
};

template <int LPW, int NP, int FAM>
__global__ void __launch_bounds__(128) lj_lane_kernel(MoveLaunch m, LjSys s) {
  constexpr int WPW = 32 / LPW;
  extern __shared__ float2 lane_smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;  // warp in block
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (warp * WPW >= m.n_walkers) return;  // whole warp is padding (warp-uniform)
  const int group = lane / LPW, glane = lane % LPW;
  int w = warp * WPW + group;
  const bool wr = w < m.n_walkers;
  if (!wr) w = m.n_walkers - 1;
  const unsigned gmask = group_mask<LPW>(group);

  Fh<LPW, FAM> fh;
  fh.load(m.cores, m.P, m.B, w, gmask, glane, wr);
  LjLaneWalker<LPW, NP> lj;
  lj.sp = lane_smem + (size_t)wib * 3 * NP * WPW;
  lj.slot = group;
  lj.glane = glane;
  lj.gmask = gmask;
  lj.n = fh.c.n;
  lj.wall_r2f = __double2float_rn(s.radius2);
  float* pw = s.pos + (size_t)w * 6 * (size_t)NP;
  lj.load(pw);
  if (LPW > 1) __syncwarp();

  RecentScale rsb;
  rsb.init();
  DS sc = ds_from_double(fh.c.tscale);
  Every resum;
  resum.init(fh.c.moves, m.resum_interval > 0 ? (uint64_t)m.resum_interval : 0);
  // the draws of the next move are taken a move ahead, off the state's critical path
  DrawCache<LPW, false> dc;
  dc.init();
  Draws nxt = dc.get(m.seed, (uint32_t)w, fh.c.moves + 1, (uint32_t)lj.n, gmask, glane);
  for (uint64_t it = 0; it < m.n_moves; ++it) {
    const uint64_t t = fh.c.moves + 1;
    const Draws d = nxt;
    if (it + 1 < m.n_moves) nxt = dc.get(m.seed, (uint32_t)w, t + 1, (uint32_t)lj.n, gmask, glane);
    double rs, omrs;
    rsb.get(t, lane, rs, omrs);
    fh.begin_move(omrs);
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
  lj.store(pw, wr);
  fh.store(m.cores, w);
}

template <int LPW, int NP, int FAM>
cudaError_t launch_lane(const MoveLaunch& m, const LjSys& s, cudaStream_t st) {
  constexpr int WPW = 32 / LPW;
  const int wpb = m.warps_per_block >= 1 && m.warps_per_block <= 4 ? m.warps_per_block : 1;
  const size_t bytes = (size_t)wpb * 3 * NP * WPW * sizeof(float2);
  // Larger than the default 48 KB for 64-atom walkers: the limit is raised once per device
  // (host threads may race to set it; setting it twice is harmless).
  static std::atomic<bool> attr[64] = {};
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return e;
  if (device < 0 || device >= 64 || !attr[device].load(std::memory_order_acquire)) {
    e = cudaFuncSetAttribute(lj_lane_kernel<LPW, NP, FAM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(4 * 3 * NP * WPW * sizeof(float2)));
    if (e != cudaSuccess) return e;
    if (device >= 0 && device < 64) attr[device].store(true, std::memory_order_release);
  }
  const int warps = (m.n_walkers + WPW - 1) / WPW;
  lj_lane_kernel<LPW, NP, FAM><<<(warps + wpb - 1) / wpb, 32 * wpb, bytes, st>>>(m, s);
  return cudaGetLastError();
}

}  // namespace dev

bool lj_lane_shape(int lpw, int np) { return (lpw == 1 || lpw == 2) && (np == 32 || np == 64); }

cudaError_t launch_lj_lane(const MoveLaunch& m, const LjSys& s, int lpw, cudaStream_t st) {
  const bool sad = m.method == M_SAD;
#define SADMC_LANE_CASE(L, N)                                                                  \
  if (lpw == L && s.np == N)                                                                   \
    return sad ? dev::launch_lane<L, N, M_SAD>(m, s, st) : dev::launch_lane<L, N, dev::FAM_ANY>(m, s, st);
  SADMC_LANE_CASE(1, 32)
  SADMC_LANE_CASE(2, 32)
  SADMC_LANE_CASE(1, 64)
  SADMC_LANE_CASE(2, 64)
#undef SADMC_LANE_CASE
  return cudaErrorInvalidConfiguration;
}

}  // namespace sadmc
