// Host-side launch entry points of the CUDA kernels (one translation unit per system).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "sadmc_types.h"

namespace sadmc {

struct MoveLaunch {
  WalkerCore* cores;
  FhParams P;
  BinPlanes B;
  int n_walkers;
  uint64_t n_moves;        // moves per walker in this launch
  uint64_t seed;
  TraceRec* trace;         // nullptr unless tracing
  uint64_t trace_cap;      // records per walker
  uint64_t trace_t0;       // move counter before the first traced move
  float* trace_ds;         // with trace: the surrogate change dS of delayed-acceptance moves
  int resum_interval;      // FP64 re-sum period in moves (continuous systems), 0 = never
  double drift_tol;        // ST_DRIFT when |E_incremental - E_fp64| exceeds this
  int descent;             // 1: run the initial descent (energy.rs:840-851) instead
  uint64_t descent_limit;  // maximum descent proposals per walker
  double descent_max;      // max_allowed_energy the descent aims below
  int warps_per_block;     // 1, 2 or 4 (kernels are bounded to 128 threads)
  int method;              // the configured method (selects a specialised kernel)
};

// LJ cluster in a spherical wall.  pos: [walker][6][np] binary32 planes
// (x_hi, y_hi, z_hi, x_lo, y_lo, z_lo), atom j at column j.
struct LjSys {
  float* pos;
  int np;
  double radius2;
};
cudaError_t launch_lj_move(const MoveLaunch& m, const LjSys& s, int lpw, cudaStream_t st);
// The shared-memory LJ move kernel with one or two lanes per walker (sadmc_lj_lane.cu),
// for 32- and 64-atom planes; it runs moves only (no descent).
bool lj_lane_shape(int lpw, int np);
cudaError_t launch_lj_lane(const MoveLaunch& m, const LjSys& s, int lpw, cudaStream_t st);
cudaError_t launch_lj_energy(const WalkerCore* cores, const LjSys& s, int n_walkers, double* out,
                             cudaStream_t st);
// Injected proposal for one walker (the plan_move parity hook): out[0] = e2 (FP64 sum of
// the FP32 pair terms added to E), out[1] = possible; when confirm != 0 an accepted
// plan is applied (position and E) without touching the bins.
cudaError_t launch_lj_plan(WalkerCore* cores, const LjSys& s, int walker, int which, float g0,
                           float g1, float g2, double scale, int confirm, double* out,
                           cudaStream_t st);

// Delayed-acceptance LJ moves screened by the surrogate (sadmc_da.cu); stats gets per
// walker (stage-1 rejections, exact evaluations) added.  One warp per walker; max_atoms is
// the largest cluster of the batch (it sizes each walker's shared-memory descriptors).
struct SgWeights;
cudaError_t launch_lj_da(const MoveLaunch& m, const LjSys& s, const SgWeights& w, int max_atoms,
                         int refresh_interval, uint64_t* stats, cudaStream_t st);

// 2D Ising.  spins: [walker][L*L] int8, index i + j*L.
struct IsingSys {
  int8_t* spins;
  int L;
};
// One Ising walker per block as a serial chain on one lane, planes and spins in shared
// memory (sadmc_ising_chain.cu); moves only, up to max_bytes of shared memory.
size_t ising_chain_bytes(int nbins, int L);
cudaError_t launch_ising_chain(const MoveLaunch& m, const IsingSys& s, size_t max_bytes, cudaStream_t st);
cudaError_t launch_ising_move(const MoveLaunch& m, const IsingSys& s, int lpw, cudaStream_t st);
cudaError_t launch_ising_energy(const IsingSys& s, int n_walkers, double* out, cudaStream_t st);

// Periodic cell systems (square well / hard core and WCA): FP64 positions plus a
// one-bucket-per-atom subcell grid.
struct CellSys {
  double* pos;        // [walker][3][np] FP64 planes
  float* pos32;       // [walker][2 np] float4: WCA high/low parts of atom j at 2j, 2j + 1;
                      // square well high parts at j
  int np;
  double* box;        // [walker][3]
  int* ncell;         // [walker][3] subcells per axis (>= 3)
  int* cell_of;       // [walker][np] subcell index of each atom
  int* cell_count;    // [walker][cell_cap]
  int* cell_atoms;    // [walker][cell_cap][bucket]
  int cell_cap;       // max subcells per walker
  int bucket;         // atom slots per subcell
  double r_cut;       // well width (square well) or 2^(1/6) (WCA)
  int kind;           // SYS_SW or SYS_WCA
  int* build_status;  // [walker] status of the last cell build
};
cudaError_t launch_cell_build(const WalkerCore* cores, const CellSys& s, int n_walkers,
                              cudaStream_t st);
cudaError_t launch_cell_move(const MoveLaunch& m, const CellSys& s, int lpw, cudaStream_t st);
cudaError_t launch_cell_energy(const WalkerCore* cores, const CellSys& s, int n_walkers,
                               double* out, cudaStream_t st);

// Plane initialisation (round_trips = 1, initial bin) for walkers [0, n).
cudaError_t launch_init_planes(const WalkerCore* cores, BinPlanes B, int nbins, int n_walkers,
                               cudaStream_t st);

// Heat capacity C(T) = (<E^2> - <E>^2)/T^2 from (E_k, S_k) with max-shifted weights,
// FP64 (plotting/final_heat_capacity.py:79-88).  One block per temperature.
// Per-walker heat capacity C[w][t] from the bin planes (FP64).
cudaError_t launch_walker_cv(const WalkerCore* cores, const BinPlanes& B, int nbins, double width,
                             int n_walkers, const double* T, int nT, double* C, cudaStream_t st);
cudaError_t launch_heat_capacity(const double* T, int nT, const double* E, const double* S,
                                 int n, double* C, cudaStream_t st);

// The per-move draws of walker `walker` for moves t0 .. t0+count-1 (device pointers).
// Self-check of the exact FP64 rewrites of the decision path (diagnostic).
cudaError_t launch_numerics_check(uint64_t n, uint64_t seed, unsigned long long* out, double* first,
                                  cudaStream_t st);
cudaError_t launch_draws(int system, uint32_t n, uint64_t seed, uint32_t walker, uint64_t t0,
                         int count, uint32_t stream_pair, uint32_t* idx2, float* g3, double* u,
                         cudaStream_t st);

}  // namespace sadmc
