// Grand-canonical LJ cluster with the energy-number method (src/mc/energy_number.rs,
// GrandSystem of src/system/lj.rs:291-319): device state and launch parameters.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "sadmc_types.h"

namespace sadmc {

// One walker's EnergyNumberMC state (energy_number.rs:115-205).  The reference's bins
// (index = E row * (max_N + 1) + N over rows [0, num_E)) live in fixed planes
// [row][N_cap + 1]: the reference's row 0 is plane row e_base.
struct GrandCore {
  double E;
  double addremove_prob;
  double min;            // bins.min, with the reference's own `min -= width` arithmetic
  double max_S;
  double gamma;          // Method::WL::gamma
  double drift;          // largest |E_incremental - E_fp64| at the periodic re-sums
  uint64_t moves, accepted;
  uint64_t ar_attempts, ar_accepted;
  uint64_t num_states, t_last;
  uint64_t max_S_index;  // a reference-layout index, not remapped on growth (as there)
  uint64_t lowest, highest, total;  // Method::WL histogram counters
  uint64_t fill_gen;     // have_visited_since_maxentropy generation (see visit plane)
  int32_t N, max_N_ref, num_E, e_base;
  int32_t kind;          // 1 SAMC, 2 WL
  uint32_t status;
  int32_t fill_val, pad;
};

struct GrandPlanes {      // each [walker][rows][N_cap + 1]
  double* lnw;
  uint64_t* hist;
  uint64_t* wl_hist;     // Method::WL::bins.histogram
  uint64_t* visit;       // (generation << 1) | value; value holds when generation is current
  uint64_t* round_trips;
  uint64_t* tr_att;      // [walker][N_cap + 1] num_translation_attempts
  uint64_t* tr_acc;      // [walker][N_cap + 1] num_translation_accepted
};

struct GrandLaunch {
  GrandCore* cores;
  GrandPlanes B;
  float* pos;            // [walker][6][np] double-single positions
  int np, rows, ncol;    // ncol = N_cap + 1
  int n_walkers;
  int lanes;             // lanes per walker (LJ: 32, 16, 8 or 4, np / lanes atoms a lane;
                         // WCA: 32, 16 or 8)
  uint64_t n_moves, seed;
  double width, inv_width, radius, radius2, t0, target_rate, translation_scale;
  double min_allowed, max_allowed;
  int has_min_allowed, has_max_allowed, has_max_N, max_N, acc_mode;
  TraceRec* trace;
  uint64_t trace_cap, trace_t0;
  int resum_interval;
  double drift_tol;
  // WCA fluid (system 2): FP64 positions [walker][3][np], double-single binary32 copies
  // [walker][2 np] (float4 high and low parts of atom j at 2j and 2j + 1),
  // subcell of each atom, bucket counts [walker][cells], buckets [walker][cells][bucket]
  int system;            // 1 LJ cluster, 2 WCA fluid
  double* pos64;
  float* pos32;
  int* cell_of;
  int* cell_count;
  int* cell_atoms;
  int cell_cap, bucket;
  double box[3];
  int nc[3];
  double r_cut;
};

cudaError_t launch_grand_move(const GrandLaunch& m, cudaStream_t st);
cudaError_t launch_wca_grand_move(const GrandLaunch& m, cudaStream_t st);
cudaError_t launch_grand_init(const GrandLaunch& m, cudaStream_t st);

}  // namespace sadmc
