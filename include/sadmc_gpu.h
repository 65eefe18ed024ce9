/*
 * sadmc_gpu.h - C ABI of the GB300 flat-histogram Monte Carlo hot path.
 *
 * One handle owns a batch of independent walkers of one system kind and one method, all
 * resident on the current CUDA device.  The entry points replace, for a whole batch at
 * once, the per-walker Rust surface of the reference (droundy/sad-monte-carlo):
 *
 *   trait System / ConfirmSystem / MovableSystem      src/system/mod.rs:54-120
 *   trait MonteCarlo, EnergyMC<S>                      src/mc/mod.rs:37-144,
 *                                                      src/mc/energy.rs:166-210, 827-990
 *
 * Conventions.  Every function returns 0 (SADMC_OK) or a negative SADMC_ERR_* code and
 * never aborts; sadmc_last_error() describes the last failure of the calling thread.
 * The library owns all device memory; callers own the host arrays they pass.  Calls are
 * synchronous unless named *_async.  One handle per host thread (like EnergyMC's
 * &mut self); the library starts no threads.  Energies are in units of epsilon, lengths
 * in sigma (src/system/units.rs).
 */
#ifndef SADMC_GPU_H
#define SADMC_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SADMC_OK 0
#define SADMC_ERR_INVALID (-1)   /* bad argument or configuration */
#define SADMC_ERR_CUDA (-2)      /* CUDA runtime error (device missing, launch failure) */
#define SADMC_ERR_STATE (-3)     /* call out of order (e.g. run before initialize) */
#define SADMC_ERR_NOMEM (-4)     /* device allocation failed */

/* System kinds: src/system/{ising,lj,wca,optsquare}.rs */
#define SADMC_ISING 0
#define SADMC_LJ 1
#define SADMC_WCA 2
#define SADMC_SW 3 /* square well with a hard core (optsquare::SquareWell) */

/* Methods: MethodParams, src/mc/energy.rs:42-69 */
#define SADMC_SAD 0
#define SADMC_SAMC 1
#define SADMC_WL 2
#define SADMC_INV_T_WL 3
#define SADMC_CANONICAL 4

/* Per-walker status bits (device status words; the reference panics instead). */
#define SADMC_ST_BIN_RANGE 1u       /* proposal outside the preallocated bins: rejected */
#define SADMC_ST_NAN_GAMMA 2u       /* gamma was NaN (energy.rs:30-33) */
#define SADMC_ST_DRIFT 4u           /* incremental E drifted beyond drift_tol (verify_energy) */
#define SADMC_ST_CELL_OVERFLOW 8u   /* a subcell bucket overflowed */
#define SADMC_ST_TIMEOUT 16u        /* a bounded device wait gave up */
#define SADMC_ST_DESCENT_FAILED 32u /* initial descent did not reach max_allowed_energy */
#define SADMC_ST_BAD_INPUT 64u      /* geometry rejected (fewer than 3 subcells per axis) */

/* Configuration: EnergyMCParams (energy.rs:81-97) plus the batch and system parameters
 * (LjParams lj.rs:14-19, WcaNParams wca.rs:371-380, SquareWellNParams optsquare.rs:336-345,
 * IsingParams ising.rs:12-15). */
typedef struct sadmc_config {
  int32_t system;            /* SADMC_ISING .. SADMC_SW */
  int32_t method;            /* SADMC_SAD .. SADMC_CANONICAL */
  int32_t n_walkers;
  int32_t max_atoms;         /* largest N over the walkers (Ising: the lattice width L) */
  double min_T;              /* SAD minimum temperature (default 0.2, energy.rs:102-104) */
  double t0;                 /* SAMC t0 */
  int32_t has_min_gamma;     /* WL: begin a production run below min_gamma */
  int32_t pad0;
  double min_gamma;
  double T;                  /* canonical temperature */
  int32_t has_energy_bin;    /* energy_bin; default System::delta_energy() or 1.0 */
  int32_t pad1;
  double energy_bin;
  int32_t has_min_allowed, has_max_allowed;
  double min_allowed, max_allowed;
  double e_lo, e_hi;         /* energies the preallocated bins must cover */
  int32_t acceptance_rate_mode; /* MoveParams::AcceptanceRate(target_rate) */
  int32_t pad2;
  double target_rate;        /* in acceptance-rate mode a positive number (else refused) */
  double translation_scale;  /* initial rms step (MoveParams::TranslationScale, 0.05) */
  double well_width;         /* square-well lambda (optsquare default 1.3) */
  uint64_t seed;             /* Philox key; walker w draws from stream (seed, w) */
  uint64_t descent_limit;    /* initial descent proposals per walker (energy.rs:841: 1e8) */
  int32_t lanes_per_walker;  /* lanes cooperating on one walker; 0 = autotuned default */
  int32_t resum_interval;    /* moves between FP64 energy re-sums (LJ, WCA); 0 = 2048 */
  double drift_tol;          /* SADMC_ST_DRIFT threshold on |E - E_fp64| (0 = 1e-2) */
} sadmc_config;

/* Per-walker geometry (walkers of one handle may differ in N and box). */
typedef struct sadmc_geometry {
  int32_t n;                 /* atoms (Ising: L, must equal max_atoms) */
  int32_t pad;
  double radius;             /* LJ spherical wall radius (Lj::max_radius) */
  double box[3];             /* WCA / square-well periodic box (Cell::box_diagonal) */
} sadmc_geometry;

/* An injected proposal (the parity hook for MovableSystem::plan_move): atom `which`
 * displaced by scale * g (Ising: the site (i, j)). */
typedef struct sadmc_proposal {
  int32_t which;
  int32_t j;
  double g[3];
  double scale;
} sadmc_proposal;

typedef struct sadmc_handle sadmc_handle;

int32_t sadmc_version(void);
const char* sadmc_last_error(void);

/* Allocate a batch (EnergyMC::from_params without the initial state).  geom has
 * cfg->n_walkers entries. */
int32_t sadmc_create(const sadmc_config* cfg, const sadmc_geometry* geom, sadmc_handle** out);
int32_t sadmc_destroy(sadmc_handle* h);

/* Upload configurations for walkers [walker_begin, walker_begin + count): positions as
 * packed x,y,z doubles (walker after walker, geom[w].n atoms each), Ising spins as +-1
 * values (L*L per walker, index i + j*L).  Periodic positions must lie in [0, box). */
int32_t sadmc_upload_state(sadmc_handle* h, int32_t walker_begin, int32_t count,
                           const double* state);
int32_t sadmc_read_state(sadmc_handle* h, int32_t walker_begin, int32_t count, double* state);

/* EnergyMC::from_params (energy.rs:830-898): FP64 energies, the downhill descent below
 * max_allowed_energy when set, and bins anchored at (round(E/w) - 0.5) w. */
int32_t sadmc_initialize(sadmc_handle* h);

/* `moves` calls of MonteCarlo::move_once (energy.rs:904-974) on every walker. */
int32_t sadmc_run(sadmc_handle* h, uint64_t moves);
int32_t sadmc_run_async(sadmc_handle* h, uint64_t moves, void* cuda_stream);
int32_t sadmc_synchronize(sadmc_handle* h);

/* System::energy (cached) and System::compute_energy (FP64 full re-sum), per walker. */
int32_t sadmc_energy(sadmc_handle* h, double* E);
int32_t sadmc_compute_energy(sadmc_handle* h, double* E);

/* MovableSystem::plan_move with an injected proposal and ConfirmSystem::confirm.
 * Bins and counters are not touched. */
int32_t sadmc_plan_move_injected(sadmc_handle* h, int32_t walker, const sadmc_proposal* p,
                                 double* e_out, int32_t* possible);
int32_t sadmc_confirm(sadmc_handle* h, int32_t walker);

/* Bins of one walker in the reference's layout (energy.rs:145-163, 202-205): nbins
 * entries starting at bins_min. */
int32_t sadmc_nbins(sadmc_handle* h, int32_t walker, int64_t* nbins, double* bins_min,
                    double* width);
int32_t sadmc_read_bins(sadmc_handle* h, int32_t walker, double* lnw, uint64_t* histogram,
                        uint64_t* t_found, double* energy_total, double* energy_squared_total,
                        uint64_t* round_trips, uint8_t* visited_since_maxentropy);
/* Whole-batch readback of the ln w and histogram planes (the result of a run):
 * lnw and histogram receive n_walkers * plane_bins values, walker-major; range receives
 * per walker (first, last) plane index of the allocated bins and bins_min its bins.min.
 * plane_bins is reported by sadmc_plane_bins. */
int32_t sadmc_plane_bins(sadmc_handle* h, int64_t* plane_bins);
int32_t sadmc_read_planes(sadmc_handle* h, double* lnw, uint64_t* histogram, int32_t* range,
                          double* bins_min);
/* Wang-Landau per-stage histogram (Method::WL::hist), *n entries from *min_energy. */
int32_t sadmc_read_wl_hist(sadmc_handle* h, int32_t walker, uint64_t* hist, int64_t* n,
                           double* min_energy);
/* The binned "pressure" datum of the WCA fluid, collected every N^2 moves
 * (Bins::extra["pressure"], a BinCounts; src/system/wca.rs:202-218 collected at
 * src/mc/energy.rs:944-946): count and total per allocated bin, the same n entries as
 * sadmc_read_bins.  SADMC_ERR_INVALID for the systems that collect no data. */
int32_t sadmc_read_extra(sadmc_handle* h, int32_t walker, uint64_t* count, double* total);

/* Scalar state of one walker, SADMC_N_SCALARS doubles in this order: moves, accepted,
 * acceptance_rate, translation_scale, method, too_lo, too_hi, tL, tF, num_states,
 * highest_hist, latest_parameter, gamma, lowest_hist, wl_highest_hist, total_hist,
 * wl_num_states, min_energy, t0, max_S, max_S_index, drift, status, energy. */
#define SADMC_N_SCALARS 24
int32_t sadmc_read_scalars(sadmc_handle* h, int32_t walker, double* out);
/* MonteCarlo::num_moves / num_accepted_moves summed over walkers. */
int32_t sadmc_counters(sadmc_handle* h, uint64_t* moves, uint64_t* accepted);
int32_t sadmc_status(sadmc_handle* h, uint32_t* per_walker_flags);

/* Record (E at move start, proposed E) for the next `capacity` moves of every walker;
 * 0 disables.  Used to replay a GPU trajectory through the FP64 oracle. */
int32_t sadmc_set_trace(sadmc_handle* h, uint64_t capacity);
int32_t sadmc_read_trace(sadmc_handle* h, int32_t walker, double* e1, double* e2,
                         uint64_t* count);
/* The surrogate energy change dS of each traced delayed-acceptance move (0 for plain
 * moves); the proposed E of a move the first stage screened out is NaN.  No reference
 * counterpart: replays sadmc_run_da's two-stage decisions through the FP64 oracle. */
int32_t sadmc_read_trace_ds(sadmc_handle* h, int32_t walker, float* ds, uint64_t* count);

/* Lanes per walker in use; sadmc_autotune times the candidates on a snapshot of the
 * batch (`moves` moves each), keeps the fastest and restores the snapshot. */
int32_t sadmc_lanes_per_walker(sadmc_handle* h);
int32_t sadmc_autotune(sadmc_handle* h, uint64_t moves, int32_t* best_lpw, double* best_ms);

/* Checkpoint / resume of the whole batch (MonteCarlo::checkpoint, src/mc/mod.rs:111-121;
 * resume by re-entry, mc/mod.rs:55-108).  The file holds the configuration, geometry,
 * every walker's flat-histogram state, bin planes and system state; it is written to a
 * temporary name and renamed, so a crash never leaves a partial file (atomicfile.rs:20-76).
 * Runs continue bit for bit: the random stream is indexed by the move counter. */
int32_t sadmc_checkpoint(sadmc_handle* h, const char* path);
int32_t sadmc_resume(const char* path, sadmc_handle** out);
/* The configuration and per-walker geometry of a handle (geom: n_walkers entries). */
int32_t sadmc_get_config(sadmc_handle* h, sadmc_config* cfg, sadmc_geometry* geom);

/* Learned surrogate for delayed-acceptance LJ moves (no counterpart in the reference):
 * a 32-RBF descriptor per atom -> 64 -> 64 -> 1 SiLU MLP, bf16 tensor-core forward with
 * FP32 accumulation, FP32 backward, Adam.  SADMC_SG_NPARAM FP32 parameters in the order
 * W1[32][64], b1[64], W2[64][64], b2[64], w3[64], b3. */
#define SADMC_SG_NPARAM 6337
/* Allocate the surrogate of an LJ handle: random weights from `seed`, a ring buffer of
 * `ring_capacity` training configurations. */
int32_t sadmc_surrogate_init(sadmc_handle* h, uint64_t seed, int32_t ring_capacity);
int32_t sadmc_surrogate_get_params(sadmc_handle* h, float* params);
int32_t sadmc_surrogate_set_params(sadmc_handle* h, const float* params);
/* Append every walker's current configuration and exact energy to the training ring. */
int32_t sadmc_surrogate_collect(sadmc_handle* h, int32_t* ring_count);
/* `steps` Adam steps on minibatches of `batch` ring configurations drawn with `seed`;
 * *loss receives the last minibatch loss (mean squared configuration-energy error). */
int32_t sadmc_surrogate_train(sadmc_handle* h, int32_t steps, int32_t batch, float lr,
                              uint64_t seed, double* loss);
/* Loss and gradients on caller configurations (positions [configs][N][3], host arrays),
 * without updating the weights (for gradient checks). */
int32_t sadmc_surrogate_loss_grads(sadmc_handle* h, const float* pos, const float* target,
                                   int32_t configs, double* loss, float* grads);
/* No counterpart in the reference.  sadmc_surrogate_loss_grads for callers that cannot
 * call cudaMalloc: a host program whose device memory is all owned by its own pool
 * allocator (a training framework), or code on a latency-critical stream where an
 * allocation's implicit device synchronisation would stall the other streams.  Device
 * pointers in and out, stream-ordered on `stream` (null: the handle's stream), returns
 * without synchronising.  Allocates nothing: the scratch is a file-scope static device
 * array of SADMC_SG_NOALLOC_MAX_ROWS rows (configs x atoms); larger requests fail with
 * SADMC_ERR_INVALID.  *loss is zeroed before it accumulates; grads (SADMC_SG_NPARAM)
 * are overwritten.  The first call on a device resolves the scratch's address (set-up)
 * and should come before any stream capture.  Calls overlapping in time on one device
 * share the scratch and race: serialise them. */
#define SADMC_SG_NOALLOC_MAX_ROWS 4096
int32_t sadmc_surrogate_loss_grads_noalloc(sadmc_handle* h, const float* pos,
                                           const float* target, int32_t configs,
                                           double* loss, float* grads, void* stream);
/* `moves` delayed-acceptance moves of every walker (SAD, SAMC or WL; LJ): the surrogate
 * screens each proposal, the exact pair energy decides (Christen & Fox 2005).  Descriptors
 * are rebuilt from scratch every refresh_interval moves (0: never).  stats (optional) gets
 * per walker the running totals (stage-1 rejections, exact evaluations). */
int32_t sadmc_run_da(sadmc_handle* h, uint64_t moves, int32_t refresh_interval, uint64_t* stats);

/* Online training schedule of sadmc_run_online (no counterpart in the reference). */
typedef struct sadmc_online {
  uint64_t collect_interval;  /* moves between appends of every walker to the ring (0: never) */
  uint64_t retrain_interval;  /* moves between training rounds (0: never) */
  int32_t train_steps;        /* Adam steps per round */
  int32_t batch;              /* ring configurations per step */
  float lr;
  int32_t pad;
  uint64_t seed;              /* minibatch draws (hashed with the move count) */
} sadmc_online;
/* `moves` moves of every walker, plain (delayed = 0, as sadmc_run) or delayed-acceptance
 * (delayed = 1, as sadmc_run_da), while the surrogate is trained online: every
 * collect_interval moves each walker's configuration and exact energy join the training
 * ring, every retrain_interval moves train_steps Adam steps run on minibatches drawn from
 * it.  The schedule counts the handle's moves since sadmc_initialize, so consecutive calls
 * continue it.  Everything runs on the device, stream-ordered, without host round trips;
 * the call synchronises once at the end.  stats as for sadmc_run_da (delayed only).
 * No counterpart in the reference (the learned part is this library's). */
int32_t sadmc_run_online(sadmc_handle* h, uint64_t moves, int32_t delayed, int32_t refresh_interval,
                         const sadmc_online* o, uint64_t* stats);

/* Surrogate energies of caller configurations (host arrays). */
int32_t sadmc_surrogate_predict(sadmc_handle* h, const float* pos, int32_t configs,
                                float* energies);

/* Self-check of the exact FP64 rewrites the decision path uses in place of FP64
 * instructions (a diagnostic with no counterpart in the reference): over n seeded cases,
 * mismatches[0] counts divisions by a known reciprocal that differ from a / b,
 * mismatches[1] integer float-to-double conversions that differ from the cast (n bit
 * patterns), mismatches[2] binary32-first Metropolis tests that differ from the FP64 one,
 * mismatches[3] integer-instruction comparisons of finite doubles that differ from < or >,
 * mismatches[4] integer-instruction conversions of integers below 2^53 that differ from the
 * cast (5 entries); first (optional) gets the first division mismatch (a, b). */
int32_t sadmc_check_numerics(uint64_t n, uint64_t seed, uint64_t* mismatches, double* first);

/* The counter-based draws the kernels consume for moves t0 .. t0+count-1 of one walker
 * (Philox4x32-10 keyed by (walker, seed); stream_pair 0 moves, 1 descent): idx2 gets
 * (atom or i, j) pairs, g3 the three normals, u the Metropolis uniform.  Host arrays.
 * A diagnostic with no counterpart in the reference, whose xoroshiro stream it replaces. */
int32_t sadmc_draws(int32_t system, uint32_t n, uint64_t seed, uint32_t walker, uint64_t t0,
                    int32_t count, uint32_t stream_pair, uint32_t* idx2, float* g3, double* u);

/* Heat capacity C(T) = (<E^2> - <E>^2) / T^2 with P ~ exp(S - E/T - max), FP64 on the
 * device (plotting/final_heat_capacity.py:79-88).  Host arrays. */
int32_t sadmc_heat_capacity(const double* T, int32_t nT, const double* E, const double* S,
                            int32_t n, double* C);

/* Heat capacity of every walker from its own bins, FP64 on the device: C[w * nT + t] =
 * heat_capacity(T[t], E, S) (plotting/final_heat_capacity.py:79-88) over the walker's
 * visited bins, with S the entropy estimate plotting/parse-binning.py:136-160 forms from
 * ln w (SAD: extended below too_lo with slope 1/min_T and above too_hi flat, both
 * corrected by ln(hist / mean hist over the window); Wang-Landau production: plus ln of
 * the production histogram).  Host arrays; C has n_walkers * nT entries. */
int32_t sadmc_walker_heat_capacity(sadmc_handle* h, const double* T, int32_t nT, double* C);

/* ---- Grand-canonical systems with the energy-number method ------------------------
 * EnergyNumberMC<S> (src/mc/energy_number.rs) for the LJ cluster (GrandSystem of
 * src/system/lj.rs:291-319: adds at a uniform point of the sphere) or the WCA fluid
 * (wca.rs:307-323: adds at a uniform point of the periodic box, subcell lists):
 * translations, adds and removals of a uniform atom, weighted by ln w(E, N) (SAMC or
 * Wang-Landau).  Every walker starts empty (E = 0, N = 0), as GrandLjParams / WcaParams
 * do.  The bins are returned in the reference's layout: index = E row * (max_N + 1) + N,
 * rows from bins.min. */
typedef struct sadmc_grand sadmc_grand;
typedef struct sadmc_grand_config {
  int32_t method;            /* SADMC_SAMC or SADMC_WL (energy_number.rs:18-27) */
  int32_t n_walkers;
  int32_t max_N;             /* EnergyNumberMCParams::max_N, required here (LJ 1..63, WCA 1..1024) */
  int32_t acceptance_rate_mode; /* MoveParams::AcceptanceRate(target_rate), else _Explicit */
  double t0;                 /* SAMC t0 */
  double energy_bin;         /* bin width (default 1.0) */
  double radius;             /* LJ: spherical wall radius (GrandLjParams::radius) */
  int32_t has_min_allowed, has_max_allowed;
  double min_allowed, max_allowed;
  double target_rate;
  double translation_scale;  /* _Explicit translation scale (0.05 in acceptance-rate mode) */
  double addremove_probability; /* _Explicit add/remove probability (0.5 initially otherwise) */
  double e_lo, e_hi;         /* energies the preallocated bins must cover (e_lo < 0 < e_hi) */
  uint64_t seed;
  int32_t resum_interval;    /* moves between FP64 energy re-sums; 0 = 2048 */
  int32_t system;            /* SADMC_LJ or SADMC_WCA */
  double drift_tol;          /* 0 = 1e-2 */
  double box[3];             /* WCA: periodic box (at least 3 subcells of 2^(1/6) per axis) */
  int32_t lanes_per_walker;  /* lanes of a warp per walker.  LJ: 32/16/8/4 (at least 8 when
                                max_N >= 32), 0 = 8.  WCA: 32/16/8, 0 = 32. */
} sadmc_grand_config;
int32_t sadmc_grand_create(const sadmc_grand_config* cfg, sadmc_grand** out);
int32_t sadmc_grand_destroy(sadmc_grand* h);
/* `moves` calls of EnergyNumberMC::move_once (energy_number.rs:540-666) per walker. */
int32_t sadmc_grand_run(sadmc_grand* h, uint64_t moves);
/* Record (E before, proposed E or NaN when impossible) for the next `capacity` moves. */
int32_t sadmc_grand_set_trace(sadmc_grand* h, uint64_t capacity);
int32_t sadmc_grand_read_trace(sadmc_grand* h, int32_t walker, double* e1, double* e2, uint64_t* n);
/* Positions (x,y,z per atom, *n atoms) of one walker. */
int32_t sadmc_grand_read_state(sadmc_grand* h, int32_t walker, double* pos, int32_t* n);
/* SADMC_GRAND_N_SCALARS doubles: moves, accepted, addremove_probability, N, E,
 * num_states, t_last, gamma (WL), lowest, highest, total (WL), max_S, max_S_index,
 * bins.min, width, max_N (of the bins), num_E, add/remove attempts, add/remove accepted,
 * drift, status. */
#define SADMC_GRAND_N_SCALARS 21
int32_t sadmc_grand_read_scalars(sadmc_grand* h, int32_t walker, double* out);
/* Bins in the reference's layout: *n_e rows by *n_n columns (N = 0..max_N). */
int32_t sadmc_grand_read_bins(sadmc_grand* h, int32_t walker, double* lnw, uint64_t* histogram,
                              uint64_t* wl_histogram, uint8_t* visited, uint64_t* round_trips,
                              int64_t* n_e, int64_t* n_n);
/* num_translation_attempts / num_translation_accepted per N (n_n entries). */
int32_t sadmc_grand_translation_counts(sadmc_grand* h, int32_t walker, uint64_t* attempts,
                                       uint64_t* accepted);

#ifdef __cplusplus
}
#endif

#endif /* SADMC_GPU_H */
