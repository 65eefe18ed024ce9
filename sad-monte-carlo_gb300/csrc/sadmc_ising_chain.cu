// One Ising walker as a serial chain on one lane (src/system/ising.rs with the bookkeeping
// of src/mc/energy.rs), the shape of a single-walker run.
//
// A lone walker's Markov chain is sequential: each move's decision reads the weights the
// previous move updated.  Lane 0 runs that chain with the walker's bin planes and spins
// in shared memory.  What does not depend on the chain is computed ahead by the whole
// warp, 32 moves at a time, into shared-memory tables: the Philox draws of each move
// (site and uniform), the acceptance-rate factor sqrt(1/t), and the SAD (or SAMC) gamma
// for the walker's parameters at the start of the batch.  A parameter change inside a
// batch (a SAD discovery, a window edge, a new tF) invalidates the gamma table, and lane 0
// computes the remaining moves' gamma itself, so every value is the one the reference's
// arithmetic gives.
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

size_t ising_chain_bytes(int nbins, int L) { return dev::ising_chain_bytes(nbins, L); }

cudaError_t launch_ising_chain(const MoveLaunch& m, const IsingSys& s, size_t max_bytes, cudaStream_t st) {
  const size_t bytes = dev::ising_chain_bytes(m.P.nbins, s.L);
  if (bytes > max_bytes || m.descent) return cudaErrorInvalidConfiguration;
  return m.method == M_SAD ? dev::launch_chain<M_SAD>(m, s, bytes, max_bytes, st)
                           : dev::launch_chain<dev::FAM_ANY>(m, s, bytes, max_bytes, st);
}

}  // namespace sadmc
