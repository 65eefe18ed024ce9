// LJ cluster in a spherical wall (src/system/lj.rs): the move kernel for any method,
// the FP64 energy and the injected-proposal kernels, and the launchers.
#include <cuda_runtime.h>

#include "sadmc_lj_kernel.cuh"

namespace sadmc {
cudaError_t launch_lj_move_sad(const MoveLaunch& m, const LjSys& s, int lpw, cudaStream_t st);
namespace dev {

template <int APL>
__global__ void lj_energy_kernel(const WalkerCore* cores, LjSys s, int n_walkers, double* out) {
  const int lane = threadIdx.x & 31;
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (w >= n_walkers) return;
  LjWalker<32, APL> lj;
  lj.set_radius2(s.radius2);
  lj.glane = lane;
  lj.gmask = 0xffffffffu;
  lj.n = cores[w].n;
  lj.load(s.pos + (size_t)w * 6 * (size_t)s.np, s.np);
  double e = lj.energy64();
  if (lane == 0) out[w] = e;
}

template <int APL>
__global__ void lj_plan_kernel(WalkerCore* cores, LjSys s, int w, int which, float g0, float g1,
                               float g2, double scale, int confirm, double* out) {
  const int lane = threadIdx.x & 31;
  LjWalker<32, APL> lj;
  lj.set_radius2(s.radius2);
  lj.glane = lane;
  lj.gmask = 0xffffffffu;
  lj.n = cores[w].n;
  float* pw = s.pos + (size_t)w * 6 * (size_t)s.np;
  lj.load(pw, s.np);
  const DS sc = ds_from_double(scale);
  DS tx, ty, tz;
  float de = 0.0f;
  bool ok = lj.plan(which, g0, g1, g2, sc.h, sc.l, s.radius2, tx, ty, tz, de);
  const double e2 = cores[w].E + (double)de;
  if (lane == 0) { out[0] = ok ? e2 : 0.0; out[1] = ok ? 1.0 : 0.0; }
  if (ok && confirm) {
    lj.put(which, tx, ty, tz);
    lj.store(pw, s.np, true);
    if (lane == 0) cores[w].E = e2;
  }
}

}  // namespace dev

cudaError_t launch_lj_move(const MoveLaunch& m, const LjSys& s, int lpw, cudaStream_t st) {
  if (m.method == M_SAD && !m.descent) return launch_lj_move_sad(m, s, lpw, st);
  if (m.descent) {
    SADMC_LJ_ALL_SHAPES(dev::FAM_ANY, true)
  } else {
    SADMC_LJ_ALL_SHAPES(dev::FAM_ANY, false)
  }
  return cudaErrorInvalidConfiguration;
}

cudaError_t launch_lj_energy(const WalkerCore* cores, const LjSys& s, int n_walkers, double* out,
                             cudaStream_t st) {
  const int blocks = (n_walkers * 32 + 127) / 128;
  switch (s.np) {
    case 32: dev::lj_energy_kernel<1><<<blocks, 128, 0, st>>>(cores, s, n_walkers, out); break;
    case 64: dev::lj_energy_kernel<2><<<blocks, 128, 0, st>>>(cores, s, n_walkers, out); break;
    case 128: dev::lj_energy_kernel<4><<<blocks, 128, 0, st>>>(cores, s, n_walkers, out); break;
    case 256: dev::lj_energy_kernel<8><<<blocks, 128, 0, st>>>(cores, s, n_walkers, out); break;
    default: return cudaErrorInvalidConfiguration;
  }
  return cudaGetLastError();
}

cudaError_t launch_lj_plan(WalkerCore* cores, const LjSys& s, int walker, int which, float g0,
                           float g1, float g2, double scale, int confirm, double* out,
                           cudaStream_t st) {
  switch (s.np) {
    case 32: dev::lj_plan_kernel<1><<<1, 32, 0, st>>>(cores, s, walker, which, g0, g1, g2, scale, confirm, out); break;
    case 64: dev::lj_plan_kernel<2><<<1, 32, 0, st>>>(cores, s, walker, which, g0, g1, g2, scale, confirm, out); break;
    case 128: dev::lj_plan_kernel<4><<<1, 32, 0, st>>>(cores, s, walker, which, g0, g1, g2, scale, confirm, out); break;
    case 256: dev::lj_plan_kernel<8><<<1, 32, 0, st>>>(cores, s, walker, which, g0, g1, g2, scale, confirm, out); break;
    default: return cudaErrorInvalidConfiguration;
  }
  return cudaGetLastError();
}

}  // namespace sadmc
