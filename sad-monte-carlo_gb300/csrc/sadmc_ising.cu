// 2D Ising model (src/system/ising.rs), many walkers per launch.
//
// Spins are int8 in global memory, index i + j*L (ising.rs:64).  A single-spin flip
// changes E by -2 s_ij (sum of 4 periodic neighbours) (ising.rs:104-119); energies are
// integers held in FP64, so the whole chain is bit-exact.  With LPW == 1 each lane is a
// walker; with LPW == 32 one walker occupies a warp: its moves run as a serial chain on
// one lane (sadmc_ising_chain.cu) when its planes fit in shared memory, here otherwise,
// and its initial descent here.
#include <cuda_runtime.h>

#include "sadmc_common.cuh"
#include "sadmc_fh.cuh"
#include "sadmc_launch.h"
#include "sadmc_rng.cuh"

namespace sadmc {
namespace dev {

template <int LPW>
__global__ void __launch_bounds__(128) ising_move_kernel(MoveLaunch m, IsingSys s) {
  constexpr int WPW = 32 / LPW;
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (warp * WPW >= m.n_walkers) return;
  const int group = lane / LPW, glane = lane % LPW;
  int w = warp * WPW + group;
  const bool wr = w < m.n_walkers;
  if (!wr) w = m.n_walkers - 1;
  const unsigned gmask = group_mask<LPW>(group);
  Fh<LPW> fh;
  fh.load(m.cores, m.P, m.B, w, gmask, glane, wr);
  const int L = s.L;
  int8_t* S = s.spins + (size_t)w * (size_t)L * (size_t)L;
  if (m.descent) {
    // from_params descent (energy.rs:840-851): flips on the descent stream, confirmed when
    // downhill, the energy tested against max_allowed_energy after each (so at least one
    // proposal is made); energies are exact integers.
    bool done = fh.c.pad1 != 0;
    uint64_t steps = fh.c.pad2;
    for (uint64_t it = 0; it < m.n_moves; ++it) {
      if (__all_sync(0xffffffffu, done)) break;
      if (!done) {
        ++steps;
        const Draws d = draws_ising(m.seed, (uint32_t)w, steps, (uint32_t)L, 1u);
        const int i = (int)d.which, j = (int)d.j;
        const int jp = j + 1 == L ? 0 : j + 1, jm = j == 0 ? L - 1 : j - 1;
        const int ip = i + 1 == L ? 0 : i + 1, im = i == 0 ? L - 1 : i - 1;
        const int nt = S[i + jp * L] + S[i + jm * L] + S[ip + j * L] + S[im + j * L];
        const int sij = S[i + j * L];
        const double e2 = fh.c.E - (double)(nt * sij * 2);
        if (fh.uni(e2 < fh.c.E)) {
          if (wr) S[i + j * L] = (int8_t)(-sij);
          if (LPW > 1) __syncwarp(gmask);
          fh.c.E = e2;
        }
        if (fh.c.E < m.descent_max) done = true;
        if (steps >= m.descent_limit) done = true;
        done = fh.uni(done);
      }
    }
    fh.c.pad2 = steps;
    fh.c.pad1 = done ? 1 : 0;
    if (wr && glane == 0) m.cores[w] = fh.c;
    return;
  }
  RecentScale rsb;
  rsb.init();
  DrawCache<LPW, true> dc;
  dc.init();
  for (uint64_t it = 0; it < m.n_moves; ++it) {
    const uint64_t t = fh.c.moves + 1;
    double rs, omrs;
    rsb.get(t, lane, rs, omrs);
    fh.begin_move(omrs);
    const Draws d = dc.get(m.seed, (uint32_t)w, t, (uint32_t)L, gmask, glane);
    const int i = (int)d.which, j = (int)d.j;
    int jp = j + 1 == L ? 0 : j + 1, jm = j == 0 ? L - 1 : j - 1;
    int ip = i + 1 == L ? 0 : i + 1, im = i == 0 ? L - 1 : i - 1;
    const int site = i + j * L;
    const int nt = S[i + jp * L] + S[i + jm * L] + S[ip + j * L] + S[im + j * L];
    const int sij = S[site];
    const float de = (float)(-(nt * sij * 2));  // exact: |de| <= 8
    if (m.trace && wr && glane == 0 && t > m.trace_t0 && t - m.trace_t0 <= m.trace_cap) {
      TraceRec r;
      r.e1 = fh.c.E;
      r.e2 = fh.c.E + (double)de;
      m.trace[(size_t)w * m.trace_cap + (t - m.trace_t0 - 1)] = r;
    }
    const bool acc = fh.decide_de(true, de, d.u53, rs);
    if (acc) {
      if (wr) S[site] = (int8_t)(-sij);  // all lanes of the group store the same value
      if (LPW > 1) __syncwarp(gmask);
    }
    fh.finish_move(acc);
  }
  fh.store(m.cores, w);
}

// compute_energy (ising.rs:59-75): sum over sites of s * (s_down + s_right), exact.
__global__ void ising_energy_kernel(IsingSys s, int n_walkers, double* out) {
  const int lane = threadIdx.x & 31;
  const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (w >= n_walkers) return;
  const int L = s.L;
  const int8_t* S = s.spins + (size_t)w * (size_t)L * (size_t)L;
  long long e = 0;
  for (int k = lane; k < L * L; k += 32) {
    const int i1 = k % L, j1 = k / L;
    const int j2 = (j1 + 1) % L, i2 = (i1 + 1) % L;
    e += (long long)((S[i1 + j2 * L] + S[i2 + j1 * L]) * S[i1 + j1 * L]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if (lane == 0) out[w] = (double)e;
}

}  // namespace dev

// Largest single-walker chain (bins, spins, tables): 200 KB of the 227 KB a block may hold.
constexpr size_t kIsingStageMax = 200 * 1024;

cudaError_t launch_ising_move(const MoveLaunch& m, const IsingSys& s, int lpw, cudaStream_t st) {
  const int wpw = 32 / lpw;
  const int warps = (m.n_walkers + wpw - 1) / wpw;
  const int wpb = m.warps_per_block >= 1 && m.warps_per_block <= 4 ? m.warps_per_block : 4;
  const int blocks = (warps + wpb - 1) / wpb;
  if (lpw == 1) {
    dev::ising_move_kernel<1><<<blocks, 32 * wpb, 0, st>>>(m, s);
  } else if (lpw == 32) {
    // a lone walker per warp: its moves as a serial chain on one lane when its planes and
    // spins fit in shared memory
    if (!m.descent && ising_chain_bytes(m.P.nbins, s.L) <= kIsingStageMax)
      return launch_ising_chain(m, s, kIsingStageMax, st);
    dev::ising_move_kernel<32><<<blocks, 32 * wpb, 0, st>>>(m, s);
  } else {
    return cudaErrorInvalidConfiguration;
  }
  return cudaGetLastError();
}

cudaError_t launch_ising_energy(const IsingSys& s, int n_walkers, double* out, cudaStream_t st) {
  dev::ising_energy_kernel<<<(n_walkers * 32 + 127) / 128, 128, 0, st>>>(s, n_walkers, out);
  return cudaGetLastError();
}

}  // namespace sadmc
