// Layouts shared by the host library (sadmc_api.cpp) and the CUDA kernels.
#pragma once
#include <cstdint>

// A branch the per-move loops rarely take: its block is laid out away from the hot path.
#define SADMC_RARE(x) __builtin_expect(!!(x), 0)

namespace sadmc {

enum SystemKind : int32_t { SYS_ISING = 0, SYS_LJ = 1, SYS_WCA = 2, SYS_SW = 3 };
enum MethodKind : int32_t { M_SAD = 0, M_SAMC = 1, M_WL = 2, M_INV_T_WL = 3, M_CANONICAL = 4,
                            M_DESCENT = 5 };

// Per-walker status bits (device status words, never traps).
enum StatusBits : uint32_t {
  ST_BIN_RANGE = 1u << 0,      // a proposal fell outside the preallocated bin range
  ST_NAN_GAMMA = 1u << 1,      // gamma evaluated to NaN (energy.rs:30-33 asserts)
  ST_DRIFT = 1u << 2,          // incremental energy drifted beyond the stated bound
  ST_CELL_OVERFLOW = 1u << 3,  // a cell-list bucket overflowed its capacity
  ST_TIMEOUT = 1u << 4,        // a bounded device wait gave up
  ST_DESCENT_FAILED = 1u << 5, // the initial descent did not reach max_allowed_energy
  ST_BAD_INPUT = 1u << 6,      // walker geometry rejected (e.g. fewer than 3 subcells)
};

// Flat-histogram state of one walker: the scalar part of the reference's EnergyMC
// (src/mc/energy.rs:166-210) and Method (energy.rs:212-244).  Bin arrays live in
// separate [walker][nbins] planes; bin indices here are global plane indices, the
// reference's local index being (global - b_lo).
struct alignas(16) WalkerCore {
  double E;            // current energy (EnergyMC::system.energy())
  double acc_rate;     // acceptance_rate (energy.rs:913-914)
  double tscale;       // translation_scale
  double cur_min;      // bins.min of the reference (shifted by prepare_for_state)
  double too_lo, too_hi, latest_param, min_T;   // SAD
  double gamma, wl_num_states, min_energy;      // WL
  double t0;                                    // SAMC (also set by the 1/t-WL switch)
  double max_S;
  double drift;        // accumulated FP32 rounding bound since the last FP64 re-sum
  double temperature;  // canonical
  uint64_t win_tmax;   // max t_found over the SAD window (incrementally maintained t_F)
  uint64_t moves, accepted, tL, tF, num_states, highest_hist;
  uint64_t lowest_hist, wl_highest_hist, total_hist;
  int32_t kind;        // MethodKind of this walker (1/t-WL switches itself to SAMC)
  int32_t b_lo, b_hi;  // allocated bin range (inclusive, global indices)
  int32_t wl_lo, wl_hi;// WL hist range (wl_hi < wl_lo: empty)
  int32_t max_S_local; // max_S_index, in the reference's local indexing
  int32_t fill_val;    // have_visited_since_maxentropy: value of the last fill
  uint32_t status;
  int32_t n;           // atoms of this walker (L for Ising)
  int32_t has_min_gamma;
  int32_t pad1;
  double min_gamma;
  uint64_t fill_gen;   // generation of the last have_visited fill
  uint64_t pad2;
};
static_assert(sizeof(WalkerCore) % 16 == 0, "WalkerCore alignment");

// Launch-wide constants of the flat-histogram driver.
struct FhParams {
  double width;        // bins.width
  double inv_width;    // 1/width for the FP32 bin-index pre-filter
  int32_t nbins;       // plane width (preallocated bins per walker)
  int32_t has_min_allowed, has_max_allowed;
  int32_t acc_mode;    // MoveParams::AcceptanceRate
  double min_allowed, max_allowed;
  double target_rate;
  double inv_target;   // 1/target_rate, correctly rounded (the translation-scale update)
};

// Bin planes, each [n_walkers][nbins].
struct BinPlanes {
  double* lnw;
  uint64_t* hist;
  uint64_t* t_found;
  double* sumE;
  double* sumE2;
  uint64_t* round_trips;
  uint64_t* visit_stamp;  // generation at which a bin was last set visited
  uint64_t* wl_hist;
  // the binned "pressure" datum of the WCA fluid (BinCounts count/total); null for the
  // systems that collect no data
  uint64_t* ex_count;
  double* ex_total;
};

// Per-move record for parity replay (trace mode only).
struct TraceRec {
  double e1;           // system energy at the start of the move (after any FP64 re-sum)
  double e2;           // proposed energy (NaN: plan_move returned None)
};

}  // namespace sadmc
