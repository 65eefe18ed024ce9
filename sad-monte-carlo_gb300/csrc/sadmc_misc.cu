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


// Block-wide reductions of walker_cv_kernel (256 threads).
__device__ __forceinline__ double block_max(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}
__device__ __forceinline__ double block_sum(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

// Entropy estimate of bin g of one walker, the treatment of plotting/parse-binning.py:
// 136-160 (restated in export.excess_entropy): ln w inside SAD's [too_lo, too_hi]; below
// it ln w(too_lo) + (E - too_lo)/min_T + ln(hist / mean hist over the window), above it
// ln w(too_hi) + ln(hist / mean hist); a Wang-Landau production run adds ln of its
// production histogram.  -inf for a bin never visited.
struct WalkerEntropy {
  const WalkerCore* c;
  const double* lnw;
  const uint64_t* hist;
  const uint64_t* wlh;
  double width;
  int i_lo, i_hi;
  double mean_hist;
  bool sad, wl_prod;
  __device__ double E(int g) const { return c->cur_min + ((double)(g - c->b_lo) + 0.5) * width; }
  __device__ double S(int g) const {
    const uint64_t h = hist[g];
    if (h == 0) return -1.0 / 0.0;
    const double e = E(g);
    if (sad) {
      if (e < c->too_lo) return lnw[i_lo] + (e - c->too_lo) / c->min_T + log((double)h / mean_hist);
      if (e > c->too_hi) return lnw[i_hi] + log((double)h / mean_hist);
      return lnw[g];
    }
    if (wl_prod) {
      const int k = c->wl_lo + (g - c->b_lo);
      const uint64_t p = (k >= c->wl_lo && k <= c->wl_hi) ? wlh[k] : 0;
      return p > 0 ? lnw[g] + log((double)p) : lnw[g];
    }
    return lnw[g];
  }
};

// C[w][t] = heat_capacity(T[t], E, S) of walker w (plotting/final_heat_capacity.py:79-88)
// over its allocated bins, FP64, one block per walker.
__global__ void walker_cv_kernel(const WalkerCore* cores, BinPlanes B, int nbins, double width,
                                 const double* T, int nT, double* C) {
  __shared__ double red[256];
  const int w = blockIdx.x;
  const WalkerCore* c = &cores[w];
  const size_t off = (size_t)w * (size_t)nbins;
  WalkerEntropy we;
  we.c = c;
  we.lnw = B.lnw + off;
  we.hist = B.hist + off;
  we.wlh = B.wl_hist + off;
  we.width = width;
  we.sad = c->kind == M_SAD;
  we.wl_prod = (c->kind == M_WL || c->kind == M_INV_T_WL) && c->has_min_gamma && c->gamma == 0.0;
  we.i_lo = we.i_hi = c->b_lo;
  we.mean_hist = 1.0;
  if (we.sad) {
    // the window edges are bin centres: the nearest bin of each
    int lo = c->b_lo + (int)floor((c->too_lo - c->cur_min) / width);
    int hi = c->b_lo + (int)floor((c->too_hi - c->cur_min) / width);
    lo = max(c->b_lo, min(c->b_hi, lo));
    hi = max(c->b_lo, min(c->b_hi, hi));
    we.i_lo = lo;
    we.i_hi = hi;
    double hs = 0.0;
    for (int g = lo + threadIdx.x; g <= hi; g += blockDim.x) hs += (double)we.hist[g];
    we.mean_hist = block_sum(hs, red) / (double)(hi - lo + 1);
  }
  for (int t = 0; t < nT; ++t) {
    const double tt = T[t];
    double mx = -1.0 / 0.0;
    for (int g = c->b_lo + threadIdx.x; g <= c->b_hi; g += blockDim.x) mx = fmax(mx, we.S(g) - we.E(g) / tt);
    mx = block_max(mx, red);
    double z = 0.0, ez = 0.0;
    for (int g = c->b_lo + threadIdx.x; g <= c->b_hi; g += blockDim.x) {
      const double p = exp(we.S(g) - we.E(g) / tt - mx);
      z += p;
      ez += we.E(g) * p;
    }
    z = block_sum(z, red);
    const double U = block_sum(ez, red) / z;
    double cc = 0.0;
    for (int g = c->b_lo + threadIdx.x; g <= c->b_hi; g += blockDim.x) {
      const double de = we.E(g) - U;
      cc += de * de * exp(we.S(g) - we.E(g) / tt - mx) / z;
    }
    cc = block_sum(cc, red);
    if (threadIdx.x == 0) C[(size_t)w * nT + t] = cc / (tt * tt);
  }
}

}  // namespace dev

cudaError_t launch_walker_cv(const WalkerCore* cores, const BinPlanes& B, int nbins, double width,
                             int n_walkers, const double* T, int nT, double* C, cudaStream_t st) {
  if (nT <= 0 || n_walkers <= 0) return cudaSuccess;
  dev::walker_cv_kernel<<<n_walkers, 256, 0, st>>>(cores, B, nbins, width, T, nT, C);
  return cudaGetLastError();
}

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

// ---- self-check of the exact rewrites of the decision path --------------------------
namespace sadmc {
namespace dev {

__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__device__ __forceinline__ double rnd_double(uint64_t r, int emin, int emax) {
  const uint64_t span = (uint64_t)(emax - emin + 1);
  const int e = emin + (int)((r >> 52) % span);
  const uint64_t mant = mix64(r) & 0xFFFFFFFFFFFFFull;
  return __longlong_as_double((long long)(((uint64_t)(e + 1023) << 52) | mant));
}

// out[0]: div_by(a, b, 1/b) != a / b; out[1]: f2d(f) != (double)f over the 2^32 bit
// patterns visited; out[2]: metropolis_reject2 != metropolis_reject; out[3]: dlt(x, y) !=
// (x < y) on finite doubles (signed zeros, equal values, neighbours one ulp apart and
// mixed signs among them); out[4]: u2d(k) != (double)k on integers below 2^53.  first:
// the first division mismatch (a, b).
__global__ void numerics_check_kernel(uint64_t n, uint64_t seed, unsigned long long* out, double* first) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r = mix64(seed ^ (i * 0x2545F4914F6CDD1Dull));
    const uint64_t r2 = mix64(r);
    double a, b;
    switch (i & 3) {
      case 0:  // wide exponents, both signs of a
        a = rnd_double(r, -60, 60) * ((r2 & 1) ? -1.0 : 1.0);
        b = rnd_double(r2, -60, 60);
        break;
      case 1:  // integer move counters over integer tF / num_states
        a = (double)(1 + (r >> 24));
        b = (double)(1 + (r2 >> (24 + (r & 15))));
        break;
      case 2:  // SAD extrapolation: (e - too_lo) / min_T
        a = -300.0 * (double)(r >> 11) * (1.0 / 9007199254740992.0);
        b = 0.01 + 2.0 * (double)(r2 >> 11) * (1.0 / 9007199254740992.0);
        break;
      default: {  // divisors with near-all-ones or near-zero mantissas
        const uint64_t m = (r2 & 1) ? (0xFFFFFFFFFFFFFull ^ (r2 >> 40)) : (r2 >> 40);
        b = __longlong_as_double((long long)(((uint64_t)(1023 + (int)(r2 >> 58) - 32) << 52) | m));
        a = rnd_double(r, -40, 40);
        break;
      }
    }
    const double q = div_by(a, b, 1.0 / b), want = a / b;
    if (__double_as_longlong(q) != __double_as_longlong(want)) {
      if (atomicAdd(&out[0], 1ull) == 0ull) { first[0] = a; first[1] = b; }
    }
    const float f = __uint_as_float((unsigned)i ^ (unsigned)(seed >> 32));
    const double fd = f2d(f), fw = (double)f;
    if (!(f != f) && __double_as_longlong(fd) != __double_as_longlong(fw)) atomicAdd(&out[1], 1ull);
    // Metropolis on two weights of SAD-like magnitude (up to 2^20) and close differences
    const double l1 = (double)(r >> 44) + (double)(r2 >> 11) * (1.0 / 9007199254740992.0);
    const double l2 = l1 + (double)((r2 >> 3) & 0xFFFF) * (1.0 / 4096.0) * ((r & 2) ? 1.0 : 1e-6);
    const uint64_t u53 = mix64(r ^ r2) >> 11;
    if (metropolis_reject2(l1, l2, u53) != metropolis_reject(l1 - l2, u53)) atomicAdd(&out[2], 1ull);
    // ordered comparison by integer instructions
    double x = rnd_double(r2 ^ 0x5DEECE66Dull, -1022, 1023) * ((r & 4) ? -1.0 : 1.0);
    double y;
    switch ((r >> 3) & 7) {
      case 0: y = x; break;                                                      // equal
      case 1: y = __longlong_as_double(__double_as_longlong(x) + 1); break;      // next ulp
      case 2: y = __longlong_as_double(__double_as_longlong(x) - 1); break;      // previous ulp
      case 3: y = -x; break;                                                     // sign flip
      case 4: x = (r & 8) ? -0.0 : 0.0; y = (r & 16) ? -0.0 : 0.0; break;        // signed zeros
      case 5: y = (r & 16) ? -0.0 : 0.0; break;                                  // against zero
      default: y = rnd_double(mix64(r2), -1022, 1023) * ((r & 32) ? -1.0 : 1.0); break;
    }
    if (isfinite(x) && isfinite(y) && (dlt(x, y) != (x < y) || dgt(x, y) != (x > y))) atomicAdd(&out[3], 1ull);
    // integer-to-double conversion below 2^53, all magnitudes
    const uint64_t k = (r ^ r2) >> (11 + (int)((r >> 40) % 53));
    if (__double_as_longlong(u2d(k)) != __double_as_longlong((double)k)) atomicAdd(&out[4], 1ull);
  }
}

}  // namespace dev

cudaError_t launch_numerics_check(uint64_t n, uint64_t seed, unsigned long long* out, double* first,
                                  cudaStream_t st) {
  dev::numerics_check_kernel<<<152 * 8, 256, 0, st>>>(n, seed, out, first);
  return cudaGetLastError();
}

}  // namespace sadmc

