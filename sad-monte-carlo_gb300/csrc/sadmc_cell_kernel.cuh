// Periodic fluids with subcell lists: the square well with a hard core
// (src/system/optsquare.rs, the hard-sphere contact-count system) and the WCA fluid
// (src/system/wca.rs), many walkers of uneven N and box per launch.
//
// Cell list: the reference registers every atom in the 27 subcells around its own
// (optcell.rs:131-160) and a query reads one list.  Here each atom sits in one bucket of
// its own subcell and a query walks the 27 buckets around the query point; for each
// neighbour bucket the periodic image shift is the one the reference stores with the
// registration (offset -1 / +1 when the unwrapped neighbour index is below 0 / at n_c),
// so the candidate set and every candidate image position are identical whenever
// n_c >= 3 (geometries with fewer subcells are rejected: the reference double-counts
// there, optcell.rs:343-346).
//
// Square well: overlap (r^2 < sigma^2) and contact (r^2 < lambda^2) decisions are those
// of optsquare.rs:74-95 on the FP64 expression (p_j - off*L) - r, x*x + y*y + z*z.  They
// are taken from binary32 copies when the binary32 r^2 lies outside a proven error
// margin of both thresholds, else from the FP64 expression itself.  Energies are
// integers and exact.  WCA: binary32 pair energies (wca.rs:66-76) on differences of
// double-single positions (close pairs keep their relative precision), FP64 re-sum
// every resum_interval moves.
#pragma once
#include <cuda_runtime.h>

#include "sadmc_common.cuh"
#include "sadmc_fh.cuh"
#include "sadmc_grand_book.cuh"
#include "sadmc_launch.h"
#include "sadmc_rng.cuh"

namespace sadmc {
namespace dev {

__device__ __forceinline__ float wca_v32(float r2, float rc2) {
  if (!(r2 < rc2)) return 0.0f;
  float s = __fdividef(1.0f, r2);
  float s3 = s * s * s;
  return 4.0f * s3 * (s3 - 1.0f) + 1.0f;
}
__device__ __forceinline__ double wca_v64(double r2, double rc2) {
  if (!(r2 < rc2)) return 0.0;
  double s = 1.0 / r2;
  return 4.0 * (powi6(s) - powi3(s)) + 1.0;
}

// floor(x / L * n) of optcell.rs:112-124 with an FP32 pre-filter.
__device__ __forceinline__ int subcell_axis(double x, double L, int n) {
  float q = __fmul_rn(__fdiv_rn((float)x, (float)L), (float)n);
  int qi = __float2int_rd(q);
  float fr = q - (float)qi;
  if (fr > 2e-5f && fr < 1.0f - 2e-5f) return qi;
  int e = (int)floor(x / L * (double)n);
  // x / L * n rounds up to n only for x within an ulp of L; keep the index in the grid
  return e < 0 ? 0 : (e >= n ? n - 1 : e);
}

// put_in_cell (optcell.rs:277-309) for one coordinate; bounded loop (a step of more
// than 64 boxes is reported through *bad).
__device__ __forceinline__ double wrap_axis(double r, double L, bool* bad) {
  int guard = 0;
  if (r < 0.0) {
    do { r += L; } while (r < 0.0 && ++guard < 64);
  } else {
    while (r >= L && ++guard < 64) r -= L;
  }
  if (guard >= 64) *bad = true;
  return r;
}

struct CellWalker {
  double* p;       // [3][np] FP64 planes of this walker
  float4* p32;     // binary32 copy, 2 np float4: WCA (x, y, z) high and low parts of
                   // atom j at 2j and 2j + 1; square well high parts at j
  int* cell_of;    // [np]
  int* cnt;        // [cells]
  int* atoms;      // [cells][bucket]
  double L[3];
  float L32[3], Ll32[3];  // the box as double-single binary32
  int nc[3];
  int np, bucket;
  __device__ int cell_index(int x, int y, int z) const { return (x * nc[1] + y) * nc[2] + z; }
  // FP64 sum of f(|q - r_j|^2) over the candidates j != skip in the 27 subcells around
  // subcell (cx, cy, cz), with the reference's periodic image offsets (the
  // maybe_interacting_atoms_excluding loops of wca.rs:202-218 and 222-230); neighbour
  // subcells k0 = k_first, k_first + k_step, ... (a lane's share).
  template <class F>
  __device__ double near_sum64(double qx, double qy, double qz, int cx, int cy, int cz, int skip,
                               F f, int k_first, int k_step) const {
    double e = 0.0;
    for (int k0 = k_first; k0 < 27; k0 += k_step) {
      const int dx = k0 / 9 - 1, dy = (k0 / 3) % 3 - 1, dz = k0 % 3 - 1;
      int ux = cx + dx, uy = cy + dy, uz = cz + dz, ox = 0, oy = 0, oz = 0;
      if (ux < 0) { ux += nc[0]; ox = 1; } else if (ux >= nc[0]) { ux -= nc[0]; ox = -1; }
      if (uy < 0) { uy += nc[1]; oy = 1; } else if (uy >= nc[1]) { uy -= nc[1]; oy = -1; }
      if (uz < 0) { uz += nc[2]; oz = 1; } else if (uz >= nc[2]) { uz -= nc[2]; oz = -1; }
      const int c = cell_index(ux, uy, uz);
      const int mm = min(cnt[c], bucket);  // counts never exceed the bucket
      for (int q = 0; q < mm; ++q) {
        const int j = atoms[(size_t)c * bucket + q];
        if (j == skip) continue;
        const double bx = (p[j] - (double)ox * L[0]) - qx;
        const double by = (p[np + j] - (double)oy * L[1]) - qy;
        const double bz = (p[2 * np + j] - (double)oz * L[2]) - qz;
        e += f(bx * bx + by * by + bz * bz);
      }
    }
    return e;
  }
  // The same sum for atom i over all 27 subcells around its own.
  template <class F>
  __device__ double pair_sum64(int i, F f) const {
    const int ci = cell_of[i];
    return near_sum64(p[i], p[np + i], p[2 * np + i], ci / (nc[1] * nc[2]), (ci / nc[2]) % nc[1],
                      ci % nc[2], i, f, 0, 1);
  }
};

// potential_pressure (wca.rs:79-92): -r dV/dr / 2 for r < 2^(1/6), sigma = epsilon = 1.
__device__ __forceinline__ double wca_pressure64(double r2, double rc2) {
  if (!(r2 < rc2)) return 0.0;
  double s = 1.0 / r2;
  return 4.0 * 3.0 * (2.0 * powi6(s) - powi3(s));
}

// A query point: its FP64 coordinates and their double-single binary32 copy.
struct Query {
  double x, y, z;
  float hx, hy, hz, lx, ly, lz;
};
// WITH_LO: the low parts too (the WCA pair terms use them; the square well does not).
template <bool WITH_LO>
__device__ __forceinline__ Query make_query(double x, double y, double z) {
  Query q;
  q.x = x; q.y = y; q.z = z;
  q.hx = (float)x; q.hy = (float)y; q.hz = (float)z;
  q.lx = q.ly = q.lz = 0.0f;
  if (WITH_LO) {
    q.lx = (float)(x - (double)q.hx); q.ly = (float)(y - (double)q.hy); q.lz = (float)(z - (double)q.hz);
  }
  return q;
}
template <bool WITH_LO>
__device__ __forceinline__ Query query_of(const CellWalker& cw, int a) {
  const float4 h = cw.p32[WITH_LO ? 2 * a : a];
  const float4 l = WITH_LO ? cw.p32[2 * a + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
  Query q;
  q.x = cw.p[a]; q.y = cw.p[cw.np + a]; q.z = cw.p[2 * cw.np + a];
  q.hx = h.x; q.hy = h.y; q.hz = h.z; q.lx = l.x; q.ly = l.y; q.lz = l.z;
  return q;
}
// The binary32 copy of atom j: WITH_LO (WCA) high and low parts side by side at 2j and
// 2j + 1, so a refined pair reads one 32-byte sector; else (square well) the high parts
// alone at j, densely packed for the screen.
template <bool WITH_LO>
__device__ __forceinline__ void put_ds(float4* p32, int j, double x, double y, double z) {
  const float hx = (float)x, hy = (float)y, hz = (float)z;
  if (WITH_LO) {
    p32[2 * j] = make_float4(hx, hy, hz, 0.0f);
    p32[2 * j + 1] = make_float4((float)(x - (double)hx), (float)(y - (double)hy),
                                 (float)(z - (double)hz), 0.0f);
  } else {
    p32[j] = make_float4(hx, hy, hz, 0.0f);
  }
}
// (p - off L) - q on one axis, p = ph + pl, q = qh + ql, L = Lh + Ll (off in -1, 0, 1).
// ph - qh is split exactly into a + e (two-sum); for a pair within reach of the cutoff
// a - off Lh is exact (the two are within a factor of 2 because the box holds at least
// 3 subcells of the cutoff), so the difference keeps its relative precision however
// small it is.
__device__ __forceinline__ float ds_image_diff(float ph, float pl, float qh, float ql, float off,
                                               float Lh, float Ll) {
  const float a = __fsub_rn(ph, qh);
  const float bb = __fsub_rn(a, ph);
  const float e = __fadd_rn(__fsub_rn(ph, __fsub_rn(a, bb)), __fsub_rn(-qh, bb));
  const float b = __fsub_rn(a, off * Lh);
  const float lo = __fadd_rn(e, __fsub_rn(__fsub_rn(pl, ql), off * Ll));
  return __fadd_rn(b, lo);
}

// The neighbour buckets of a lane group's queries, in shared memory: subcell, image
// offset and the prefix of the bucket counts.  With the prefix every lane takes
// candidates glane, glane + LPW, ... wherever they lie, so no lane waits for the fullest
// bucket of its group.
struct BucketScan {
  int cell[54];
  int pref[55];
  signed char off[54][3];
};

template <int LPW, int KIND>
struct CellOps {
  // Neighbour subcell k0 (0..26) of subcell (cx, cy, cz) and the reference's image
  // offset: image = p - off * L.
  __device__ static int bucket(const CellWalker& cw, int k0, int cx, int cy, int cz, int& ox,
                               int& oy, int& oz) {
    const int dx = k0 / 9 - 1, dy = (k0 / 3) % 3 - 1, dz = k0 % 3 - 1;
    int ux = cx + dx, uy = cy + dy, uz = cz + dz;
    ox = 0; oy = 0; oz = 0;
    if (ux < 0) { ux += cw.nc[0]; ox = 1; } else if (ux >= cw.nc[0]) { ux -= cw.nc[0]; ox = -1; }
    if (uy < 0) { uy += cw.nc[1]; oy = 1; } else if (uy >= cw.nc[1]) { uy -= cw.nc[1]; oy = -1; }
    if (uz < 0) { uz += cw.nc[2]; oz = 1; } else if (uz >= cw.nc[2]) { uz -= cw.nc[2]; oz = -1; }
    return cw.cell_index(ux, uy, uz);
  }

  // One candidate j seen from query q through image offset (ox, oy, oz).  SW: counts a
  // contact or sets *overlap (new position); WCA: binary32 pair energy into e32.
  __device__ static void pair(const CellWalker& cw, int j, int ox, int oy, int oz, const Query& q,
                              double wsqr, float wsqr32, bool newq, int& contacts, bool& overlap,
                              float& e32) {
    const float fx = (float)ox, fy = (float)oy, fz = (float)oz;
    const float4 pj = cw.p32[KIND == SYS_WCA ? 2 * j : j];
    const float ax = (pj.x - fx * cw.L32[0]) - q.hx, ay = (pj.y - fy * cw.L32[1]) - q.hy,
                az = (pj.z - fz * cw.L32[2]) - q.hz;
    const float d2 = ax * ax + ay * ay + az * az;
    if (KIND == SYS_SW) {
      bool near = fabsf(d2 - 1.0f) < 2e-4f || fabsf(d2 - wsqr32) < 2e-4f;
      if (!near) {
        if (d2 < 1.0f) { if (newq) overlap = true; else ++contacts; }
        else if (d2 < wsqr32) ++contacts;
      } else {
        // the reference's FP64 expression (optsquare.rs:78-86)
        const double bx = (cw.p[j] - (double)ox * cw.L[0]) - q.x;
        const double by = (cw.p[cw.np + j] - (double)oy * cw.L[1]) - q.y;
        const double bz = (cw.p[2 * cw.np + j] - (double)oz * cw.L[2]) - q.z;
        const double e2 = bx * bx + by * by + bz * bz;
        if (e2 < 1.0) { if (newq) overlap = true; else ++contacts; }
        else if (e2 < wsqr) ++contacts;
      }
    } else if (d2 < wsqr32 + 1e-3f) {
      // WCA: pairs whose high-part r^2 may lie inside the cutoff (the high parts are
      // within 2^-24 |L| of each coordinate) are refined on the double-single positions
      const float4 pl = cw.p32[2 * j + 1];
      const float rx = ds_image_diff(pj.x, pl.x, q.hx, q.lx, fx, cw.L32[0], cw.Ll32[0]);
      const float ry = ds_image_diff(pj.y, pl.y, q.hy, q.ly, fy, cw.L32[1], cw.Ll32[1]);
      const float rz = ds_image_diff(pj.z, pl.z, q.hz, q.lz, fz, cw.L32[2], cw.Ll32[2]);
      e32 += wca_v32(rx * rx + ry * ry + rz * rz, wsqr32);
    }
  }

  // Sum over the candidates of one bucket k0 (0..26) around cell (cx,cy,cz) of query q
  // (excluding atom `skip`); one lane per bucket.
  __device__ static void scan(const CellWalker& cw, int k0, int cx, int cy, int cz, const Query& q,
                              int skip, double wsqr, float wsqr32, bool newq, int& contacts,
                              bool& overlap, float& e32) {
    int ox, oy, oz;
    const int c = bucket(cw, k0, cx, cy, cz, ox, oy, oz);
    const int m = min(cw.cnt[c], cw.bucket);
    const int* list = cw.atoms + (size_t)c * cw.bucket;
    for (int k = 0; k < m; ++k) {
      const int j = list[k];
      if (j != skip) pair(cw, j, ox, oy, oz, q, wsqr, wsqr32, newq, contacts, overlap, e32);
    }
  }

  // The candidates of nq queries (1 or 2), 27 buckets each, spread evenly over the group:
  // query 0's buckets around (c0x, c0y, c0z) are entries 0..26 of bs, query 1's around
  // (c1x, c1y, c1z) entries 27..53.  Results go to each query's accumulators (SW:
  // contacts and the overlap flag; WCA: energy).
  __device__ static void scan_group(const CellWalker& cw, BucketScan& bs, int nq, int c0x, int c0y,
                                    int c0z, int c1x, int c1y, int c1z, const Query& q0,
                                    const Query& q1, bool new0, bool new1, int skip, double wsqr,
                                    float wsqr32, int glane, unsigned gmask, int& cont0,
                                    int& cont1, bool& overlap, float& e0, float& e1) {
    const int nb = 27 * nq;
    for (int k = glane; k < nb; k += LPW) {
      const bool second = k >= 27;
      int ox, oy, oz;
      const int c = bucket(cw, second ? k - 27 : k, second ? c1x : c0x, second ? c1y : c0y,
                           second ? c1z : c0z, ox, oy, oz);
      bs.cell[k] = c;
      bs.off[k][0] = (signed char)ox; bs.off[k][1] = (signed char)oy; bs.off[k][2] = (signed char)oz;
      bs.pref[k + 1] = min(cw.cnt[c], cw.bucket);
    }
    if (LPW > 1) __syncwarp(gmask);
    // prefix of the counts: each lane sums a contiguous chunk, then a scan over the group
    constexpr int kMaxChunk = (54 + LPW - 1) / LPW;
    const int chunk = (nb + LPW - 1) / LPW, e0i = glane * chunk;
    int mine = 0;
#pragma unroll
    for (int i = 0; i < kMaxChunk; ++i)
      if (i < chunk && e0i + i < nb) mine += bs.pref[e0i + i + 1];
    int incl = mine;
#pragma unroll
    for (int o = 1; o < LPW; o <<= 1) {
      const int y = __shfl_up_sync(gmask, incl, o, LPW);
      if (glane >= o) incl += y;
    }
    const int total = LPW > 1 ? __shfl_sync(gmask, incl, LPW - 1, LPW) : incl;
    int run = incl - mine;
#pragma unroll
    for (int i = 0; i < kMaxChunk; ++i)
      if (i < chunk && e0i + i < nb) {
        run += bs.pref[e0i + i + 1];
        bs.pref[e0i + i + 1] = run;
      }
    if (glane == 0) bs.pref[0] = 0;
    if (LPW > 1) __syncwarp(gmask);
    // each candidate is an atom index then that atom's position, two dependent loads.  For
    // WCA the next candidate's index is loaded while this one's pair is evaluated (same
    // order; C3 5 % faster); the square-well scan measured 1 % slower that way and loads
    // each index when it needs it
    if (KIND != SYS_WCA) {
      int k = 0;
      for (int cnd = glane; cnd < total; cnd += LPW) {
        while (bs.pref[k + 1] <= cnd) ++k;
        const int j = cw.atoms[(size_t)bs.cell[k] * cw.bucket + (cnd - bs.pref[k])];
        if (j == skip) continue;
        const bool second = k >= 27;
        int dc = 0;
        float de = 0.0f;
        pair(cw, j, bs.off[k][0], bs.off[k][1], bs.off[k][2], second ? q1 : q0, wsqr, wsqr32,
             second ? new1 : new0, dc, overlap, de);
        if (second) { cont1 += dc; e1 += de; } else { cont0 += dc; e0 += de; }
      }
      if (LPW > 1) __syncwarp(gmask);  // the group may reuse bs next
      return;
    }
    int k = 0, kn = 0, jn = 0;
    if (glane < total) {
      while (bs.pref[k + 1] <= glane) ++k;
      kn = k;
      jn = cw.atoms[(size_t)bs.cell[k] * cw.bucket + (glane - bs.pref[k])];
    }
    for (int cnd = glane; cnd < total; cnd += LPW) {
      const int j = jn, kc = kn;
      const int cn = cnd + LPW;
      if (cn < total) {
        while (bs.pref[k + 1] <= cn) ++k;
        kn = k;
        jn = cw.atoms[(size_t)bs.cell[k] * cw.bucket + (cn - bs.pref[k])];
      }
      if (j == skip) continue;
      const bool second = kc >= 27;
      int dc = 0;
      float de = 0.0f;
      pair(cw, j, bs.off[kc][0], bs.off[kc][1], bs.off[kc][2], second ? q1 : q0, wsqr, wsqr32,
           second ? new1 : new0, dc, overlap, de);
      if (second) { cont1 += dc; e1 += de; } else { cont0 += dc; e0 += de; }
    }
    if (LPW > 1) __syncwarp(gmask);  // the group may reuse bs next
  }
};

// FAM: the method the kernel is specialised for, or FAM_ANY (the method each walker holds).
template <int LPW, int KIND, int FAM>
__global__ void __launch_bounds__(128, 1) cell_move_kernel(MoveLaunch m, CellSys s) {
  constexpr int WPW = 32 / LPW;
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (warp * WPW >= m.n_walkers) return;
  const int group = lane / LPW, glane = lane % LPW;
  int w = warp * WPW + group;
  const bool wr = w < m.n_walkers;
  if (!wr) w = m.n_walkers - 1;
  const unsigned gmask = group_mask<LPW>(group);

  __shared__ BucketScan sbs[128 / LPW];
  Fh<LPW, FAM> fh;
  fh.load(m.cores, m.P, m.B, w, gmask, glane, wr);
  CellWalker cw;
  cw.np = s.np;
  cw.bucket = s.bucket;
  cw.p = s.pos + (size_t)w * 3 * s.np;
  cw.p32 = reinterpret_cast<float4*>(s.pos32) + (size_t)w * 2 * s.np;
  cw.cell_of = s.cell_of + (size_t)w * s.np;
  cw.cnt = s.cell_count + (size_t)w * s.cell_cap;
  cw.atoms = s.cell_atoms + (size_t)w * s.cell_cap * s.bucket;
  for (int a = 0; a < 3; ++a) {
    cw.L[a] = s.box[3 * w + a];
    cw.L32[a] = (float)cw.L[a];
    cw.Ll32[a] = (float)(cw.L[a] - (double)cw.L32[a]);
    cw.nc[a] = s.ncell[3 * w + a];
  }
  const int n = fh.c.n;
  const double rc = s.r_cut;
  const double wsqr = rc * rc;
  const float wsqr32 = (float)wsqr;

  // plan_move: put_in_cell(from + g * scale) (optsquare.rs:273-284, wca.rs:342-353) and the
  // energy change over the 27 subcells around the old and the new position.
  struct Prop {
    int a, old_c, new_c, new_count;
    double fx, fy, fz, tx, ty, tz;
    float de;
    bool possible;
  };
  auto plan = [&](int a, float g0, float g1, float g2, double sc) {
    Prop p;
    p.a = a;
    p.fx = cw.p[a]; p.fy = cw.p[s.np + a]; p.fz = cw.p[2 * s.np + a];
    bool bad = false;
    p.tx = wrap_axis(p.fx + (double)g0 * sc, cw.L[0], &bad);
    p.ty = wrap_axis(p.fy + (double)g1 * sc, cw.L[1], &bad);
    p.tz = wrap_axis(p.fz + (double)g2 * sc, cw.L[2], &bad);
    const int nx = subcell_axis(p.tx, cw.L[0], cw.nc[0]);
    const int ny = subcell_axis(p.ty, cw.L[1], cw.nc[1]);
    const int nz = subcell_axis(p.tz, cw.L[2], cw.nc[2]);
    p.old_c = cw.cell_of[a];
    const int ocx = p.old_c / (cw.nc[1] * cw.nc[2]), ocy = (p.old_c / cw.nc[2]) % cw.nc[1],
              ocz = p.old_c % cw.nc[2];
    const Query qt = make_query<KIND == SYS_WCA>(p.tx, p.ty, p.tz);
    const Query qf = query_of<KIND == SYS_WCA>(cw, a);
    int cn = 0, co = 0;
    float en = 0.0f, eo = 0.0f;
    bool overlap = false;
    BucketScan& bs = sbs[threadIdx.x / LPW];
    if (KIND == SYS_SW) {
      // the new position first: a hard-core overlap makes the move impossible, and then
      // the old position's contacts are not needed
      CellOps<LPW, KIND>::scan_group(cw, bs, 1, nx, ny, nz, 0, 0, 0, qt, qt, true, true, a, wsqr,
                                     wsqr32, glane, gmask, cn, cn, overlap, en, en);
      if (!__any_sync(gmask, overlap))
        CellOps<LPW, KIND>::scan_group(cw, bs, 1, ocx, ocy, ocz, 0, 0, 0, qf, qf, false, false, a,
                                       wsqr, wsqr32, glane, gmask, co, co, overlap, eo, eo);
    } else {
      CellOps<LPW, KIND>::scan_group(cw, bs, 2, nx, ny, nz, ocx, ocy, ocz, qt, qf, true, false, a,
                                     wsqr, wsqr32, glane, gmask, cn, co, overlap, en, eo);
    }
    p.new_c = cw.cell_index(nx, ny, nz);
    if (KIND == SYS_SW) {
      // e = E - (contacts at the new position) + (contacts at the old position); the
      // FP64 sequence of unit steps of optsquare.rs:75-92 is exact on integers, and so
      // is the binary32 difference of the two counts
      const int newc = group_sum<LPW>(cn, gmask);
      const int oldc = group_sum<LPW>(co, gmask);
      p.possible = !__any_sync(gmask, overlap);
      p.de = (float)(oldc - newc);
    } else {
      p.de = group_sum<LPW>(en - eo, gmask);
      p.possible = true;
    }
    p.possible = p.possible && !bad && fabsf(p.de) <= 3.0e38f;
    p.new_count = cw.cnt[p.new_c];
    if (p.possible && p.new_c != p.old_c && p.new_count >= cw.bucket) {
      p.possible = false;
      fh.c.status |= ST_CELL_OVERFLOW;
    }
    return p;
  };
  // ConfirmSystem::confirm -> Cell::move_atom (optcell.rs:162-175)
  auto apply = [&](const Prop& p) {
    const int a = p.a;
    if (p.new_c != p.old_c) {
      int* lo = cw.atoms + (size_t)p.old_c * cw.bucket;
      const int mo = min(cw.cnt[p.old_c], cw.bucket);
      int pos = -1;
      for (int k = glane; k < mo; k += LPW)
        if (lo[k] == a) pos = k;
      for (int o = LPW / 2; o > 0; o >>= 1) {
        int x = __shfl_xor_sync(gmask, pos, o, LPW);
        pos = x > pos ? x : pos;
      }
      __syncwarp(gmask);
      if (wr && pos >= 0) {
        lo[pos] = lo[mo - 1];
        cw.cnt[p.old_c] = mo - 1;
        cw.atoms[(size_t)p.new_c * cw.bucket + p.new_count] = a;
        cw.cnt[p.new_c] = p.new_count + 1;
        cw.cell_of[a] = p.new_c;
      }
    }
    if (wr) {
      cw.p[a] = p.tx; cw.p[s.np + a] = p.ty; cw.p[2 * s.np + a] = p.tz;
      put_ds<KIND == SYS_WCA>(cw.p32, a, p.tx, p.ty, p.tz);
    }
    __syncwarp(gmask);
  };

  if (m.descent) {
    // from_params descent (energy.rs:840-851): proposals of rms 0.05 on the descent stream,
    // confirmed when downhill; after every possible proposal the energy is tested against
    // max_allowed_energy (so at least one proposal is made).  WCA energy changes are the
    // FP64 one-atom sums here; square-well changes are exact integers.
    bool done = fh.c.pad1 != 0;
    uint64_t steps = fh.c.pad2;
    for (uint64_t it = 0; it < m.n_moves; ++it) {
      if (__all_sync(0xffffffffu, done)) break;
      if (!done) {
        ++steps;
        const Draws d = draws_continuous(m.seed, (uint32_t)w, steps, (uint32_t)n, 1u);
        const Prop p = plan((int)d.which, d.g0, d.g1, d.g2, 0.05);
        if (p.possible) {
          double de = (double)p.de;
          if (KIND == SYS_WCA) {
            const int ci = p.new_c;
            const int nx = ci / (cw.nc[1] * cw.nc[2]), ny = (ci / cw.nc[2]) % cw.nc[1], nz = ci % cw.nc[2];
            const int oc = p.old_c;
            const int ox = oc / (cw.nc[1] * cw.nc[2]), oy = (oc / cw.nc[2]) % cw.nc[1], oz = oc % cw.nc[2];
            auto v64 = [&](double r2) { return wca_v64(r2, wsqr); };
            double part = cw.near_sum64(p.tx, p.ty, p.tz, nx, ny, nz, p.a, v64, glane, LPW) -
                          cw.near_sum64(p.fx, p.fy, p.fz, ox, oy, oz, p.a, v64, glane, LPW);
            de = group_sum<LPW>(part, gmask);
          }
          const double e2 = fh.c.E + de;
          if (fh.uni(e2 < fh.c.E)) {
            apply(p);
            fh.c.E = e2;
          }
          if (fh.c.E < m.descent_max) done = true;
        }
        if (steps >= m.descent_limit) done = true;
        done = fh.uni(done);
      }
    }
    fh.c.pad2 = steps;
    fh.c.pad1 = done ? 1 : 0;
    if (wr && glane == 0) m.cores[w] = fh.c;  // the host re-sums E in FP64 afterwards
    return;
  }

  RecentScale rsb;
  rsb.init();
  DrawCache<LPW, false> dc;
  dc.init();
  Every resum, datum;
  resum.init(fh.c.moves, KIND == SYS_WCA && m.resum_interval > 0 ? (uint64_t)m.resum_interval : 0);
  datum.init(fh.c.moves, KIND == SYS_WCA && m.B.ex_count ? (uint64_t)n * (uint64_t)n : 0);
  for (uint64_t it = 0; it < m.n_moves; ++it) {
    const uint64_t t = fh.c.moves + 1;
    double rs, omrs;
    rsb.get(t, lane, rs, omrs);
    fh.begin_move(omrs);
    const Draws d = dc.get(m.seed, (uint32_t)w, t, (uint32_t)n, gmask, glane);
    const Prop p = plan((int)d.which, d.g0, d.g1, d.g2, fh.c.tscale);
    if (m.trace && wr && glane == 0 && t > m.trace_t0 && t - m.trace_t0 <= m.trace_cap) {
      TraceRec r;
      r.e1 = fh.c.E;
      r.e2 = p.possible ? fh.c.E + (double)p.de : __longlong_as_double(0x7ff8000000000000ll);
      m.trace[(size_t)w * m.trace_cap + (t - m.trace_t0 - 1)] = r;
    }
    const bool acc = fh.decide_de(p.possible, p.de, d.u53, rs);
    if (acc) apply(p);
    fh.finish_move(acc);
    if (datum.tick()) {
      // the "pressure" datum every N^2 moves into the current bin (wca.rs:202-218,
      // collected and binned as in energy.rs:944-946 and 374-386)
      double pv = 0.0;
      for (int i = glane; i < n; i += LPW)
        pv += cw.pair_sum64(i, [&](double r2) { return wca_pressure64(r2, wsqr); });
      pv = group_sum<LPW>(pv, gmask);
      if (wr && glane == 0) {
        const size_t k = (size_t)w * fh.nbins + fh.cur;
        m.B.ex_count[k] += 1;
        m.B.ex_total[k] += pv / (3.0 * (cw.L[0] * cw.L[1] * cw.L[2]));
      }
    }
    if (resum.tick()) {
      // FP64 re-sum (wca.rs:222-230)
      double e = 0.0;
      for (int i = glane; i < n; i += LPW)
        e += cw.pair_sum64(i, [&](double r2) { return wca_v64(r2, wsqr); });
      const double e64 = group_sum<LPW>(e, gmask) * 0.5;
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
  fh.store(m.cores, w);
}

}  // namespace dev

// Launch cell_move_kernel<LPW, KIND, FAM> for the lanes per walker and the system.
#define SADMC_CELL_CASE(L, K, F)                                                        \
  if (lpw == L && s.kind == K) {                                                        \
    const int warps = (m.n_walkers + (32 / L) - 1) / (32 / L);                          \
    const int wpb = m.warps_per_block >= 1 && m.warps_per_block <= 4 ? m.warps_per_block : 4; \
    dev::cell_move_kernel<L, K, F><<<(warps + wpb - 1) / wpb, 32 * wpb, 0, st>>>(m, s); \
    return cudaGetLastError();                                                          \
  }
#define SADMC_CELL_ALL_SHAPES(F)                                                        \
  SADMC_CELL_CASE(32, SYS_SW, F) SADMC_CELL_CASE(16, SYS_SW, F)                         \
  SADMC_CELL_CASE(8, SYS_SW, F) SADMC_CELL_CASE(4, SYS_SW, F)                           \
  SADMC_CELL_CASE(32, SYS_WCA, F) SADMC_CELL_CASE(16, SYS_WCA, F)                       \
  SADMC_CELL_CASE(8, SYS_WCA, F) SADMC_CELL_CASE(4, SYS_WCA, F)

}  // namespace sadmc
