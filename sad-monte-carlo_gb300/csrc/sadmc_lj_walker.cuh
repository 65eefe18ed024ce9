// Register-resident LJ cluster walker: atom j in lane j % LPW of the walker's group, slot
// j / LPW, double-single positions (src/system/lj.rs).
#pragma once
#include "sadmc_common.cuh"

namespace sadmc {
namespace dev {

__device__ __forceinline__ float lj_v32(float r2) {  // 4 (s^6 - s^3), s = 1/r^2 (lj.rs:78-81)
  float s = __fdividef(1.0f, r2);
  float s3 = s * s * s;
  return 4.0f * s3 * (s3 - 1.0f);
}

template <int LPW, int APL>
struct LjWalker {
  DS x[APL], y[APL], z[APL];
  int n;
  int glane;
  unsigned gmask;
  float wall_r2f;  // binary32 R^2 of the wall, set once per launch (set_radius2)
  __device__ void set_radius2(double r2) { wall_r2f = __double2float_rn(r2); }

  __device__ void load(const float* p, int np) {
#pragma unroll
    for (int k = 0; k < APL; ++k) {
      int j = glane + LPW * k;
      x[k] = DS{p[j], p[3 * np + j]};
      y[k] = DS{p[np + j], p[4 * np + j]};
      z[k] = DS{p[2 * np + j], p[5 * np + j]};
    }
  }
  __device__ void store(float* p, int np, bool wr) const {
    if (!wr) return;
#pragma unroll
    for (int k = 0; k < APL; ++k) {
      int j = glane + LPW * k;
      p[j] = x[k].h; p[np + j] = y[k].h; p[2 * np + j] = z[k].h;
      p[3 * np + j] = x[k].l; p[4 * np + j] = y[k].l; p[5 * np + j] = z[k].l;
    }
  }
  // Position of atom `which`, broadcast to the whole group.
  __device__ void fetch(int which, DS& fx, DS& fy, DS& fz) const {
    const int owner = which % LPW, slot = which / LPW;
    float a = 0.f, b = 0.f, c = 0.f, d = 0.f, e = 0.f, f = 0.f;
#pragma unroll
    for (int k = 0; k < APL; ++k)
      if (k == slot) { a = x[k].h; b = y[k].h; c = z[k].h; d = x[k].l; e = y[k].l; f = z[k].l; }
    if (LPW > 1) {
      a = __shfl_sync(gmask, a, owner, LPW); b = __shfl_sync(gmask, b, owner, LPW);
      c = __shfl_sync(gmask, c, owner, LPW); d = __shfl_sync(gmask, d, owner, LPW);
      e = __shfl_sync(gmask, e, owner, LPW); f = __shfl_sync(gmask, f, owner, LPW);
    }
    fx = DS{a, d}; fy = DS{b, e}; fz = DS{c, f};
  }
  __device__ void put(int which, DS tx, DS ty, DS tz) {
    const int owner = which % LPW, slot = which / LPW;
    if (glane != owner) return;
#pragma unroll
    for (int k = 0; k < APL; ++k)
      if (k == slot) { x[k] = tx; y[k] = ty; z[k] = tz; }
  }

  // plan_move of lj.rs:365-374 and move_atom of lj.rs:86-105 for a given displacement.
  // Returns possible; de = the energy change summed in binary32 over the group.
  __device__ bool plan(int which, float g0, float g1, float g2, float sh, float sl,
                       double radius2, DS& tx, DS& ty, DS& tz, float& de_out) const {
    DS fx, fy, fz;
    fetch(which, fx, fy, fz);
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
      double a = ds_to_double(tx), b = ds_to_double(ty), c = ds_to_double(tz);
      double p = ds_to_double(fx), q = ds_to_double(fy), r = ds_to_double(fz);
      double nt = a * a + b * b + c * c, nf = p * p + q * q + r * r;
      impossible = nt > radius2 && nt > nf;
    }
    if (impossible) return false;
    float de = 0.0f;
    // Differences of double-single positions: the high parts of two nearby atoms subtract
    // exactly (Sterbenz), so close pairs keep their full relative precision in r^2.
#pragma unroll
    for (int k = 0; k < APL; ++k) {
      const int j = glane + LPW * k;
      if (j < n && j != which) {
        float dx = (x[k].h - tx.h) + (x[k].l - tx.l);
        float dy = (y[k].h - ty.h) + (y[k].l - ty.l);
        float dz = (z[k].h - tz.h) + (z[k].l - tz.l);
        float vn = lj_v32(dx * dx + dy * dy + dz * dz);
        dx = (x[k].h - fx.h) + (x[k].l - fx.l);
        dy = (y[k].h - fy.h) + (y[k].l - fy.l);
        dz = (z[k].h - fz.h) + (z[k].l - fz.l);
        float vo = lj_v32(dx * dx + dy * dy + dz * dz);
        de += vn - vo;
      }
    }
    de_out = group_sum<LPW>(de, gmask);
    return true;
  }

  // FP64 pair sum over the double-single positions (compute_energy, lj.rs:236-244).
  __device__ double energy64() const {
    double xd[APL], yd[APL], zd[APL];
#pragma unroll
    for (int k = 0; k < APL; ++k) { xd[k] = ds_to_double(x[k]); yd[k] = ds_to_double(y[k]); zd[k] = ds_to_double(z[k]); }
    double e = 0.0;
    for (int j = 0; j < n; ++j) {
      DS a, b, c;
      fetch(j, a, b, c);
      const double xj = ds_to_double(a), yj = ds_to_double(b), zj = ds_to_double(c);
#pragma unroll
      for (int k = 0; k < APL; ++k) {
        const int i = glane + LPW * k;
        if (i < n && i > j) {
          double dx = xd[k] - xj, dy = yd[k] - yj, dz = zd[k] - zj;
          double s = 1.0 / (dx * dx + dy * dy + dz * dz);
          e += 4.0 * (powi6(s) - powi3(s));
        }
      }
    }
    return group_sum<LPW>(e, gmask);
  }
};

}  // namespace dev
}  // namespace sadmc
