// Plane initialisation and the FP64 heat-capacity reconstruction.
#include <cuda_runtime.h>

#include "sadmc_fh.cuh"
#include "sadmc_launch.h"
#include "sadmc_rng.cuh"

namespace sadmc {
namespace dev {

// Bins of a new EnergyMC (energy.rs:868-882): the starting bin holds one count and the
// starting energy; round_trips start at 1 everywhere (energy.rs:880, 418, 432).
__global__ void init_planes_kernel(const WalkerCore* cores, BinPlanes B, int nbins, int n_walkers) {
  const size_t total = (size_t)nbins * (size_t)n_walkers;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
       k += (size_t)gridDim.x * blockDim.x) {
    const int w = (int)(k / (size_t)nbins), g = (int)(k % (size_t)nbins);
    const WalkerCore& c = cores[w];
    B.lnw[k] = 0.0;
    B.t_found[k] = 0;
    B.round_trips[k] = 1;
    B.visit_stamp[k] = 0;
    B.wl_hist[k] = 0;
    if (B.ex_count) { B.ex_count[k] = 0; B.ex_total[k] = 0.0; }
    if (g == c.b_lo) {
      B.hist[k] = 1;
      B.sumE[k] = c.E;
      B.sumE2[k] = c.E * c.E;
    } else {
      B.hist[k] = 0;
      B.sumE[k] = 0.0;
      B.sumE2[k] = 0.0;
    }
  }
}

// heat_capacity(T, E, S) of plotting/final_heat_capacity.py:79-88 in FP64:
// b = S - E/T; P = exp(b - max b); P /= sum P; U = sum E P; C = sum (E-U)^2 P / T^2.
__global__ void heat_capacity_kernel(const double* T, const double* E, const double* S, int n,
                                     double* C) {
  __shared__ double red[256];
  const double t = T[blockIdx.x];
  double mx = -1.0 / 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) mx = fmax(mx, S[k] - E[k] / t);
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  mx = red[0];
  __syncthreads();
  double z = 0.0, ez = 0.0, e2z = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double p = exp(S[k] - E[k] / t - mx);
    z += p;
    ez += E[k] * p;
    e2z += E[k] * E[k] * p;
  }
  // U = <E>; C = (<E^2> - U^2)/T^2 evaluated as sum (E-U)^2 P in a second pass
  red[threadIdx.x] = z;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  z = red[0];
  __syncthreads();
  red[threadIdx.x] = ez;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  const double U = red[0] / z;
  __syncthreads();
  (void)e2z;
  double c = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const double p = exp(S[k] - E[k] / t - mx) / z;
    const double de = E[k] - U;
    c += de * de * p;
  }
  red[threadIdx.x] = c;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) C[blockIdx.x] = red[0] / (t * t);
}

}  // namespace dev

cudaError_t launch_init_planes(const WalkerCore* cores, BinPlanes B, int nbins, int n_walkers,
                               cudaStream_t st) {
  dev::init_planes_kernel<<<4 * 152, 256, 0, st>>>(cores, B, nbins, n_walkers);
  return cudaGetLastError();
}

cudaError_t launch_heat_capacity(const double* T, int nT, const double* E, const double* S,
                                 int n, double* C, cudaStream_t st) {
  if (nT <= 0) return cudaSuccess;
  dev::heat_capacity_kernel<<<nT, 256, 0, st>>>(T, E, S, n, C);
  return cudaGetLastError();
}

}  // namespace sadmc

namespace sadmc {
namespace dev {
__global__ void draws_kernel(int system, uint32_t n, uint64_t seed, uint32_t walker, uint64_t t0,
                             int count, uint32_t stream_pair, uint32_t* idx2, float* g3, double* u) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const uint64_t t = t0 + (uint64_t)k;
  Draws d = system == SYS_ISING ? draws_ising(seed, walker, t, n)
                                : draws_continuous(seed, walker, t, n, stream_pair);
  idx2[2 * k] = d.which;
  idx2[2 * k + 1] = d.j;
  g3[3 * k] = d.g0; g3[3 * k + 1] = d.g1; g3[3 * k + 2] = d.g2;
  u[k] = u53_to_double(d.u53);
}
}  // namespace dev

cudaError_t launch_draws(int system, uint32_t n, uint64_t seed, uint32_t walker, uint64_t t0,
                         int count, uint32_t stream_pair, uint32_t* idx2, float* g3, double* u,
                         cudaStream_t st) {
  dev::draws_kernel<<<(count + 127) / 128, 128, 0, st>>>(system, n, seed, walker, t0, count,
                                                         stream_pair, idx2, g3, u);
  return cudaGetLastError();
}
}  // namespace sadmc
