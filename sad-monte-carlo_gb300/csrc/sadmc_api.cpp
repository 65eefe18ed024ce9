// Host implementation of the C ABI in include/sadmc_gpu.h.
#include "../../include/sadmc_gpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sadmc_grand.h"
#include "sadmc_launch.h"
#include "sadmc_surrogate.h"
#include "sadmc_types.h"

using namespace sadmc;

namespace {

thread_local std::string g_last_error;

int32_t fail(int32_t code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define CUDA_TRY(expr)                                                                  \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(SADMC_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));  \
  } while (0)

template <class T>
cudaError_t dalloc(T** p, size_t n) {
  return cudaMalloc((void**)p, n * sizeof(T) + 16);
}

int pad_atoms(int n) {
  for (int p : {32, 64, 128, 256})
    if (n <= p) return p;
  return -1;
}

bool valid_lpw_lj(int lpw, int np) {
  switch (np) {
    case 32: return lpw == 32 || lpw == 16 || lpw == 8 || lpw == 4 || lpw == 2 || lpw == 1;
    case 64: return lpw == 32 || lpw == 16 || lpw == 8 || lpw == 2 || lpw == 1;
    default: return lpw == 32;
  }
}

}  // namespace

struct sadmc_handle {
  sadmc_config cfg{};
  std::vector<sadmc_geometry> geom;
  int W = 0, nb = 0, np = 0, L = 0, lpw = 0;
  double width = 1.0;
  bool uploaded = false, initialized = false;
  cudaStream_t stream = nullptr;
  WalkerCore* d_cores = nullptr;
  BinPlanes planes{};
  void* plane_mem = nullptr;
  int n_planes = 8;  // 10 with the WCA pressure planes
  float* d_pos = nullptr;      // LJ: [W][6][np]
  int8_t* d_spins = nullptr;   // Ising: [W][L*L]
  // periodic cell systems (square well, WCA)
  double* d_pos64 = nullptr;   // [W][3][np]
  float* d_pos32 = nullptr;    // [W][np] float4
  double* d_box = nullptr;     // [W][3]
  int* d_ncell = nullptr;      // [W][3]
  int* d_cell_of = nullptr;    // [W][np]
  int* d_cnt = nullptr;        // [W][cell_cap]
  int* d_atoms = nullptr;      // [W][cell_cap][bucket]
  int* d_build_status = nullptr;
  int cell_cap = 0, bucket = 16;
  double r_cut = 0.0;
  CellSys cell_sys() const {
    CellSys c{};
    c.pos = d_pos64; c.pos32 = d_pos32; c.np = np; c.box = d_box; c.ncell = d_ncell;
    c.cell_of = d_cell_of; c.cell_count = d_cnt; c.cell_atoms = d_atoms; c.cell_cap = cell_cap;
    c.bucket = bucket; c.r_cut = r_cut; c.kind = cfg.system; c.build_status = d_build_status;
    return c;
  }
  double* d_tmp = nullptr;     // [W] + 2 scratch doubles
  TraceRec* d_trace = nullptr;
  float* d_trace_ds = nullptr;  // dS of traced delayed-acceptance moves (0 for plain moves)
  uint64_t trace_cap = 0, trace_t0 = 0;
  uint64_t moves_done = 0;
  int pend_walker = -1;
  sadmc_proposal pend{};
  std::vector<WalkerCore> h_cores;
  int wpb = 0;                                  // warps per block (0: the kernel's own default)
  // learned surrogate (LJ)
  float* sg_master = nullptr;                   // FP32 parameters
  float* sg_grad = nullptr;
  float* sg_m = nullptr;
  float* sg_v = nullptr;
  __nv_bfloat16* sg_w1t = nullptr;              // bf16 copies for the tensor cores
  __nv_bfloat16* sg_w2t = nullptr;
  __nv_bfloat16* sg_wc = nullptr;               // the same in tcgen05 shared-memory order
  float* sg_ring_pos = nullptr;                 // [cap][N][3] binary32
  float* sg_ring_e = nullptr;
  int sg_cap = 0, sg_head = 0, sg_count = 0, sg_step = 0;
  void* sg_scratch = nullptr;                   // per-row activations of a training step
  size_t sg_scratch_rows = 0;
  float* sg_batch_pos = nullptr;                // gathered minibatch
  float* sg_batch_e = nullptr;
  int sg_batch_cap = 0;
  double* sg_loss = nullptr;
  unsigned int* sg_flag = nullptr;              // the timeout flag, read and cleared
  uint64_t* sg_stats = nullptr;                 // [W][2] delayed-acceptance counters
  SgWeights sg_weights() const { return SgWeights::from(sg_master, sg_w1t, sg_w2t, sg_wc); }
  SgAdam sg_adam(int step, float lr) const { return SgAdam{sg_master, sg_m, sg_v, step, lr}; }
  void free_surrogate() {
    cudaFree(sg_master); cudaFree(sg_grad); cudaFree(sg_m); cudaFree(sg_v); cudaFree(sg_w1t);
    cudaFree(sg_w2t); cudaFree(sg_wc); cudaFree(sg_ring_pos); cudaFree(sg_ring_e); cudaFree(sg_scratch);
    cudaFree(sg_batch_pos); cudaFree(sg_batch_e); cudaFree(sg_loss); cudaFree(sg_flag); cudaFree(sg_stats);
    sg_stats = nullptr;
    sg_master = sg_grad = sg_m = sg_v = sg_ring_pos = sg_ring_e = sg_batch_pos = sg_batch_e = nullptr;
    sg_w1t = sg_w2t = sg_wc = nullptr; sg_scratch = nullptr; sg_loss = nullptr; sg_flag = nullptr;
  }
  // scratch for `rows` rows and a gathered batch of `configs` configurations
  cudaError_t sg_reserve(size_t rows, int configs) {
    cudaError_t e = cudaSuccess;
    if (rows > sg_scratch_rows) {
      cudaFree(sg_scratch);
      sg_scratch = nullptr;
      e = cudaMalloc(&sg_scratch, SgScratch::bytes(rows));
      sg_scratch_rows = e == cudaSuccess ? rows : 0;
    }
    if (e == cudaSuccess && configs > sg_batch_cap) {
      cudaFree(sg_batch_pos); cudaFree(sg_batch_e);
      sg_batch_pos = nullptr; sg_batch_e = nullptr;
      e = cudaMalloc(&sg_batch_pos, sizeof(float) * 3 * (size_t)configs * geom[0].n);
      if (e == cudaSuccess) e = cudaMalloc(&sg_batch_e, sizeof(float) * configs);
      sg_batch_cap = e == cudaSuccess ? configs : 0;
    }
    return e;
  }
  std::map<uint64_t, cudaGraphExec_t> graphs;   // captured run(moves) sequences
  void drop_graphs() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
  }

  FhParams fh_params() const {
    FhParams P{};
    P.width = width;
    P.inv_width = 1.0 / width;
    P.nbins = nb;
    P.has_min_allowed = cfg.has_min_allowed;
    P.has_max_allowed = cfg.has_max_allowed;
    P.acc_mode = cfg.acceptance_rate_mode;
    P.min_allowed = cfg.min_allowed;
    P.max_allowed = cfg.max_allowed;
    P.target_rate = cfg.target_rate;
    P.inv_target = 1.0 / cfg.target_rate;
    return P;
  }
  int resum() const { return cfg.resum_interval > 0 ? cfg.resum_interval : 2048; }
  double drift_tol() const {
    return cfg.drift_tol > 0 ? cfg.drift_tol : 1e-2;
  }
  int32_t pull_cores() {
    h_cores.resize(W);
    CUDA_TRY(cudaMemcpyAsync(h_cores.data(), d_cores, sizeof(WalkerCore) * W,
                             cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    return SADMC_OK;
  }
  int32_t push_cores() {
    CUDA_TRY(cudaMemcpyAsync(d_cores, h_cores.data(), sizeof(WalkerCore) * W,
                             cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    return SADMC_OK;
  }
  cudaError_t launch_move(const MoveLaunch& m) {
    switch (cfg.system) {
      case SADMC_LJ:
        // one or two lanes per walker: the shared-memory kernel for moves; the initial
        // descent runs on the register kernel (8 lanes per walker) either way
        if (lj_lane_shape(lpw, np))
          return m.descent ? launch_lj_move(m, LjSys{d_pos, np, 0.0 + radius2()}, 8, stream)
                           : launch_lj_lane(m, LjSys{d_pos, np, 0.0 + radius2()}, lpw, stream);
        return launch_lj_move(m, LjSys{d_pos, np, 0.0 + radius2()}, lpw, stream);
      case SADMC_ISING: return launch_ising_move(m, IsingSys{d_spins, L}, lpw, stream);
      case SADMC_SW:
      case SADMC_WCA: return launch_cell_move(m, cell_sys(), lpw, stream);
      default: return cudaErrorNotSupported;
    }
  }
  // Before sadmc_initialize the cores only carry each walker's N (and E when planned).
  int32_t prep_cores() {
    if (initialized) return SADMC_OK;
    if ((int)h_cores.size() != W) {
      h_cores.assign(W, WalkerCore{});
      for (int w = 0; w < W; ++w) { h_cores[w].n = geom[w].n; h_cores[w].kind = M_DESCENT; }
      return push_cores();
    }
    return SADMC_OK;
  }
  double radius2() const { return geom.empty() ? 0.0 : geom[0].radius * geom[0].radius; }
  cudaError_t launch_energy(double* out) {
    switch (cfg.system) {
      case SADMC_LJ: return launch_lj_energy(d_cores, LjSys{d_pos, np, radius2()}, W, out, stream);
      case SADMC_ISING: return launch_ising_energy(IsingSys{d_spins, L}, W, out, stream);
      case SADMC_SW:
      case SADMC_WCA: return launch_cell_energy(d_cores, cell_sys(), W, out, stream);
      default: return cudaErrorNotSupported;
    }
  }
  MoveLaunch base_launch() const {
    MoveLaunch m{};
    m.cores = d_cores;
    m.method = cfg.method;
    m.P = fh_params();
    m.B = planes;
    m.n_walkers = W;
    m.seed = cfg.seed;
    m.trace = d_trace;
    m.trace_cap = trace_cap;
    m.trace_t0 = trace_t0;
    m.trace_ds = d_trace_ds;
    m.resum_interval = resum();
    m.drift_tol = drift_tol();
    m.warps_per_block = wpb;
    return m;
  }
};

namespace {

struct DevBuf {
  void* ptr;
  size_t bytes;
};

std::vector<DevBuf> state_buffers(sadmc_handle* h) {
  const size_t W = h->W, nb = h->nb, np = h->np;
  std::vector<DevBuf> v = {{h->d_cores, sizeof(WalkerCore) * W}, {h->plane_mem, W * nb * 8 * (size_t)h->n_planes}};
  switch (h->cfg.system) {
    case SADMC_ISING: v.push_back({h->d_spins, W * (size_t)h->L * h->L}); break;
    case SADMC_LJ: v.push_back({h->d_pos, W * 6 * np * sizeof(float)}); break;
    default:
      v.push_back({h->d_pos64, W * 3 * np * sizeof(double)});
      v.push_back({h->d_pos32, W * 8 * np * sizeof(float)});
      v.push_back({h->d_ncell, W * 3 * sizeof(int)});
      v.push_back({h->d_cell_of, W * np * sizeof(int)});
      v.push_back({h->d_cnt, W * (size_t)h->cell_cap * sizeof(int)});
      v.push_back({h->d_atoms, W * (size_t)h->cell_cap * h->bucket * sizeof(int)});
      break;
  }
  return v;
}

const char kMagic[8] = {'S', 'A', 'D', 'M', 'C', 'G', 'B', '1'};

}  // namespace

namespace {

const uint64_t kChunk = 8192;  // moves per launch (keeps each launch to tens of ms)

cudaError_t launch_chunks(sadmc_handle* h, uint64_t moves, cudaStream_t st) {
  MoveLaunch m = h->base_launch();
  cudaStream_t keep = h->stream;
  h->stream = st;
  cudaError_t e = cudaSuccess;
  for (uint64_t left = moves; left > 0 && e == cudaSuccess;) {
    m.n_moves = std::min(left, kChunk);
    e = h->launch_move(m);
    left -= m.n_moves;
  }
  h->stream = keep;
  return e;
}

std::string tune_cache_path() {
  if (const char* p = std::getenv("SADMC_TUNE_CACHE")) return p;
  const char* home = std::getenv("HOME");
  return std::string(home ? home : "/tmp") + "/.cache/sadmc_gb300_tune.txt";
}

std::string tune_key(const sadmc_handle* h) {
  std::ostringstream k;
  k << "sys" << h->cfg.system << "_np" << (h->cfg.system == SADMC_ISING ? h->L : h->np) << "_W"
    << h->W << "_m" << h->cfg.method;
  return k.str();
}

std::vector<int> lpw_candidates(const sadmc_handle* h) {
  switch (h->cfg.system) {
    case SADMC_ISING: return {1, 32};
    case SADMC_LJ:
      if (h->np == 32) return {1, 2, 4, 8, 16, 32};
      if (h->np == 64) return {1, 2, 8, 16, 32};
      return {32};
    default: return {4, 8, 16, 32};
  }
}

}  // namespace

struct sadmc_grand {
  sadmc_grand_config cfg{};
  int W = 0, np = 0, rows = 0, ncol = 0, lanes = 8;
  GrandCore* d_cores = nullptr;
  void* plane_mem = nullptr;
  GrandPlanes planes{};
  float* d_pos = nullptr;
  // WCA fluid: FP64 positions, binary32 copies, subcell of each atom, bucket lists
  double* d_pos64 = nullptr;
  float* d_pos32 = nullptr;
  int *d_cell_of = nullptr, *d_cnt = nullptr, *d_atoms = nullptr;
  int nc[3] = {0, 0, 0}, cell_cap = 0, bucket = 32;
  TraceRec* d_trace = nullptr;
  uint64_t trace_cap = 0, trace_t0 = 0, moves_done = 0;
  cudaStream_t stream = nullptr;
  bool wca() const { return cfg.system == SADMC_WCA; }
  GrandLaunch launch() const {
    GrandLaunch m{};
    m.cores = d_cores; m.B = planes; m.pos = d_pos; m.np = np; m.rows = rows; m.ncol = ncol;
    m.n_walkers = W; m.seed = cfg.seed; m.lanes = lanes;
    m.width = cfg.energy_bin > 0 ? cfg.energy_bin : 1.0; m.inv_width = 1.0 / m.width;
    m.radius = cfg.radius; m.radius2 = cfg.radius * cfg.radius; m.t0 = cfg.t0;
    m.target_rate = cfg.target_rate;
    m.translation_scale = cfg.acceptance_rate_mode ? 0.05 : cfg.translation_scale;
    m.min_allowed = cfg.min_allowed; m.max_allowed = cfg.max_allowed;
    m.has_min_allowed = cfg.has_min_allowed; m.has_max_allowed = cfg.has_max_allowed;
    m.has_max_N = 1; m.max_N = cfg.max_N; m.acc_mode = cfg.acceptance_rate_mode;
    m.trace = d_trace; m.trace_cap = trace_cap; m.trace_t0 = trace_t0;
    m.resum_interval = cfg.resum_interval > 0 ? cfg.resum_interval : 2048;
    m.drift_tol = cfg.drift_tol > 0 ? cfg.drift_tol : 1e-2;
    m.system = wca() ? 2 : 1;
    m.pos64 = d_pos64; m.pos32 = d_pos32; m.cell_of = d_cell_of; m.cell_count = d_cnt;
    m.cell_atoms = d_atoms; m.cell_cap = cell_cap; m.bucket = bucket;
    for (int a = 0; a < 3; ++a) { m.box[a] = cfg.box[a]; m.nc[a] = nc[a]; }
    m.r_cut = std::pow(2.0, 1.0 / 6.0);
    return m;
  }
};

extern "C" {

int32_t sadmc_version(void) { return 1; }
const char* sadmc_last_error(void) { return g_last_error.c_str(); }

int32_t sadmc_create(const sadmc_config* cfg, const sadmc_geometry* geom, sadmc_handle** out) {
  if (!cfg || !geom || !out) return fail(SADMC_ERR_INVALID, "null argument");
  *out = nullptr;
  const sadmc_config& c = *cfg;
  if (c.n_walkers <= 0) return fail(SADMC_ERR_INVALID, "n_walkers must be positive");
  if (c.system < SADMC_ISING || c.system > SADMC_SW) return fail(SADMC_ERR_INVALID, "unknown system");
  if (c.method < SADMC_SAD || c.method > SADMC_CANONICAL) return fail(SADMC_ERR_INVALID, "unknown method");
  if (!(c.e_hi > c.e_lo)) return fail(SADMC_ERR_INVALID, "e_hi must exceed e_lo");
  // the translation-scale update divides by target_rate through its reciprocal
  if (c.acceptance_rate_mode && !(c.target_rate >= 0x1p-1000 && c.target_rate <= 0x1p+1000))
    return fail(SADMC_ERR_INVALID, "target_rate must be a positive number");
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    return fail(SADMC_ERR_CUDA, "no CUDA device");
  auto* h = new sadmc_handle();
  h->cfg = c;
  h->W = c.n_walkers;
  h->geom.assign(geom, geom + c.n_walkers);
  // bin width: energy_bin, else System::delta_energy() (Ising 4, square well 1), else 1
  // (energy.rs:831-833)
  h->width = c.has_energy_bin ? c.energy_bin : (c.system == SADMC_ISING ? 4.0 : 1.0);
  if (!(h->width > 0)) { delete h; return fail(SADMC_ERR_INVALID, "energy_bin must be positive"); }
  double nbd = std::ceil((c.e_hi - c.e_lo) / h->width) + 4.0;
  if (nbd > (double)(1 << 24)) { delete h; return fail(SADMC_ERR_INVALID, "too many bins"); }
  h->nb = (int)nbd;
  if (c.system == SADMC_ISING) {
    h->L = c.max_atoms;
    if (h->L < 2) { delete h; return fail(SADMC_ERR_INVALID, "Ising needs L > 1 (ising.rs:39)"); }
    for (int w = 0; w < h->W; ++w)
      if (geom[w].n != h->L) { delete h; return fail(SADMC_ERR_INVALID, "Ising walkers must share L"); }
    h->lpw = c.lanes_per_walker ? c.lanes_per_walker : (h->W == 1 ? 32 : 1);
    if (h->lpw != 1 && h->lpw != 32) { delete h; return fail(SADMC_ERR_INVALID, "Ising lanes_per_walker must be 1 or 32"); }
  } else if (c.system == SADMC_SW || c.system == SADMC_WCA) {
    h->r_cut = c.system == SADMC_SW ? c.well_width : std::pow(2.0, 1.0 / 6.0);
    if (!(h->r_cut > 0)) { delete h; return fail(SADMC_ERR_INVALID, "well_width must be positive"); }
    int mx = 0, cap = 0;
    for (int w = 0; w < h->W; ++w) {
      if (geom[w].n < 2 || geom[w].n > 4096) { delete h; return fail(SADMC_ERR_INVALID, "2..4096 atoms per periodic walker"); }
      mx = std::max(mx, (int)geom[w].n);
      int cells = 1;
      for (int a = 0; a < 3; ++a) {
        const int nc = (int)std::floor(geom[w].box[a] / h->r_cut);  // optcell.rs:64-66
        if (nc < 3) {
          delete h;
          return fail(SADMC_ERR_INVALID, "walker " + std::to_string(w) +
                      ": fewer than 3 subcells per axis (the reference double counts there)");
        }
        cells *= nc;
      }
      cap = std::max(cap, cells);
    }
    h->np = (mx + 31) / 32 * 32;
    h->cell_cap = cap;
    h->lpw = c.lanes_per_walker ? c.lanes_per_walker : 8;
    if (h->lpw != 32 && h->lpw != 16 && h->lpw != 8 && h->lpw != 4) { delete h; return fail(SADMC_ERR_INVALID, "unsupported lanes_per_walker"); }
  } else {
    int mx = 0;
    for (int w = 0; w < h->W; ++w) {
      if (geom[w].n < 2) { delete h; return fail(SADMC_ERR_INVALID, "walkers need at least 2 atoms"); }
      mx = std::max(mx, (int)geom[w].n);
      if (geom[w].radius != geom[0].radius) { delete h; return fail(SADMC_ERR_INVALID, "LJ walkers must share the wall radius"); }
    }
    h->np = pad_atoms(mx);
    if (h->np < 0) { delete h; return fail(SADMC_ERR_INVALID, "at most 256 atoms per LJ walker"); }
    h->lpw = c.lanes_per_walker ? c.lanes_per_walker : (h->np <= 64 ? 8 : 32);
    if (!valid_lpw_lj(h->lpw, h->np)) { delete h; return fail(SADMC_ERR_INVALID, "unsupported lanes_per_walker"); }
  }
  if (c.lanes_per_walker == 0) {  // a recorded autotuning result for this shape wins
    std::ifstream in(tune_cache_path());
    const std::string key = tune_key(h);
    for (std::string line; std::getline(in, line);) {
      std::istringstream ls(line);
      std::string k;
      int lpw = 0, wpb = 0;
      if (ls >> k >> lpw >> wpb && k == key) {
        const auto cand = lpw_candidates(h);
        if (std::find(cand.begin(), cand.end(), lpw) != cand.end() && wpb >= 1 && wpb <= 4) {
          h->lpw = lpw;
          h->wpb = wpb;
        }
      }
    }
  }
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete h; return fail(SADMC_ERR_CUDA, cudaGetErrorString(e)); }
  const size_t plane = (size_t)h->W * (size_t)h->nb;
  h->n_planes = c.system == SADMC_WCA ? 10 : 8;
  bool ok = dalloc(&h->d_cores, h->W) == cudaSuccess && dalloc(&h->d_tmp, h->W + 2) == cudaSuccess &&
            cudaMalloc(&h->plane_mem, plane * 8 * (size_t)h->n_planes) == cudaSuccess;
  if (ok) {
    char* b = (char*)h->plane_mem;
    h->planes.lnw = (double*)(b + 0 * plane * 8);
    h->planes.hist = (uint64_t*)(b + 1 * plane * 8);
    h->planes.t_found = (uint64_t*)(b + 2 * plane * 8);
    h->planes.sumE = (double*)(b + 3 * plane * 8);
    h->planes.sumE2 = (double*)(b + 4 * plane * 8);
    h->planes.round_trips = (uint64_t*)(b + 5 * plane * 8);
    h->planes.visit_stamp = (uint64_t*)(b + 6 * plane * 8);
    h->planes.wl_hist = (uint64_t*)(b + 7 * plane * 8);
    if (h->n_planes == 10) {
      h->planes.ex_count = (uint64_t*)(b + 8 * plane * 8);
      h->planes.ex_total = (double*)(b + 9 * plane * 8);
    }
    if (c.system == SADMC_ISING) ok = dalloc(&h->d_spins, (size_t)h->W * h->L * h->L) == cudaSuccess;
    else if (c.system == SADMC_LJ) ok = dalloc(&h->d_pos, (size_t)h->W * 6 * h->np) == cudaSuccess;
    else {
      const size_t W = h->W, np = h->np, cap = h->cell_cap;
      ok = dalloc(&h->d_pos64, W * 3 * np) == cudaSuccess && dalloc(&h->d_pos32, W * 8 * np) == cudaSuccess &&
           dalloc(&h->d_box, W * 3) == cudaSuccess && dalloc(&h->d_ncell, W * 3) == cudaSuccess &&
           dalloc(&h->d_cell_of, W * np) == cudaSuccess && dalloc(&h->d_cnt, W * cap) == cudaSuccess &&
           dalloc(&h->d_atoms, W * cap * h->bucket) == cudaSuccess &&
           dalloc(&h->d_build_status, W) == cudaSuccess;
      if (ok) {
        std::vector<double> box(W * 3);
        for (size_t w = 0; w < W; ++w)
          for (int a = 0; a < 3; ++a) box[3 * w + a] = geom[w].box[a];
        ok = cudaMemcpy(h->d_box, box.data(), box.size() * 8, cudaMemcpyHostToDevice) == cudaSuccess;
      }
    }
  }
  if (!ok) {
    sadmc_destroy(h);
    return fail(SADMC_ERR_NOMEM, "device allocation failed");
  }
  if (h->d_pos) cudaMemsetAsync(h->d_pos, 0, sizeof(float) * (size_t)h->W * 6 * h->np, h->stream);
  *out = h;
  return SADMC_OK;
}

int32_t sadmc_destroy(sadmc_handle* h) {
  if (!h) return SADMC_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  h->drop_graphs();
  h->free_surrogate();
  cudaFree(h->d_cores);
  cudaFree(h->d_tmp);
  cudaFree(h->plane_mem);
  cudaFree(h->d_pos);
  cudaFree(h->d_spins);
  cudaFree(h->d_trace);
  cudaFree(h->d_trace_ds);
  cudaFree(h->d_pos64); cudaFree(h->d_pos32); cudaFree(h->d_box); cudaFree(h->d_ncell);
  cudaFree(h->d_cell_of); cudaFree(h->d_cnt); cudaFree(h->d_atoms); cudaFree(h->d_build_status);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return SADMC_OK;
}

int32_t sadmc_upload_state(sadmc_handle* h, int32_t begin, int32_t count, const double* state) {
  if (!h || !state || begin < 0 || count < 0 || begin + count > h->W)
    return fail(SADMC_ERR_INVALID, "bad walker range");
  if (h->cfg.system == SADMC_ISING) {
    const size_t n = (size_t)h->L * h->L;
    std::vector<int8_t> s(n * count);
    for (size_t k = 0; k < s.size(); ++k) s[k] = (int8_t)(state[k] > 0 ? 1 : -1);
    CUDA_TRY(cudaMemcpyAsync(h->d_spins + (size_t)begin * n, s.data(), s.size(), cudaMemcpyHostToDevice, h->stream));
  } else if (h->cfg.system == SADMC_SW || h->cfg.system == SADMC_WCA) {
    const int np = h->np;
    std::vector<double> p((size_t)count * 3 * np, 0.0);
    size_t off = 0;
    for (int w = 0; w < count; ++w) {
      const int n = h->geom[begin + w].n;
      double* q = p.data() + (size_t)w * 3 * np;
      for (int j = 0; j < n; ++j)
        for (int a = 0; a < 3; ++a) q[a * np + j] = state[off + 3 * j + a];
      off += 3 * (size_t)n;
    }
    CUDA_TRY(cudaMemcpyAsync(h->d_pos64 + (size_t)begin * 3 * np, p.data(), p.size() * sizeof(double),
                             cudaMemcpyHostToDevice, h->stream));
    h->h_cores.clear();
    int32_t r = h->prep_cores();
    if (r) return r;
    CUDA_TRY(launch_cell_build(h->d_cores, h->cell_sys(), h->W, h->stream));
    std::vector<int> st(h->W);
    CUDA_TRY(cudaMemcpyAsync(st.data(), h->d_build_status, sizeof(int) * h->W, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    for (int w = 0; w < h->W; ++w)
      if (st[w]) return fail(SADMC_ERR_INVALID, "walker " + std::to_string(w) +
                             (st[w] == ST_CELL_OVERFLOW ? ": subcell bucket overflow" : ": position outside [0, box)"));
  } else {
    const int np = h->np;
    std::vector<float> p((size_t)count * 6 * np, 0.0f);
    size_t off = 0;
    for (int w = 0; w < count; ++w) {
      const int n = h->geom[begin + w].n;
      float* q = p.data() + (size_t)w * 6 * np;
      for (int j = 0; j < n; ++j)
        for (int a = 0; a < 3; ++a) {
          const double x = state[off + 3 * j + a];
          const float hi = (float)x;
          q[a * np + j] = hi;
          q[(3 + a) * np + j] = (float)(x - (double)hi);
        }
      off += 3 * (size_t)n;
    }
    CUDA_TRY(cudaMemcpyAsync(h->d_pos + (size_t)begin * 6 * np, p.data(), p.size() * sizeof(float),
                             cudaMemcpyHostToDevice, h->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->uploaded = true;
  h->initialized = false;
  h->h_cores.clear();
  return SADMC_OK;
}

int32_t sadmc_read_state(sadmc_handle* h, int32_t begin, int32_t count, double* state) {
  if (!h || !state || begin < 0 || count < 0 || begin + count > h->W)
    return fail(SADMC_ERR_INVALID, "bad walker range");
  if (h->cfg.system == SADMC_ISING) {
    const size_t n = (size_t)h->L * h->L;
    std::vector<int8_t> s(n * count);
    CUDA_TRY(cudaMemcpyAsync(s.data(), h->d_spins + (size_t)begin * n, s.size(), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    for (size_t k = 0; k < s.size(); ++k) state[k] = s[k];
  } else if (h->cfg.system == SADMC_SW || h->cfg.system == SADMC_WCA) {
    const int np = h->np;
    std::vector<double> p((size_t)count * 3 * np);
    CUDA_TRY(cudaMemcpyAsync(p.data(), h->d_pos64 + (size_t)begin * 3 * np, p.size() * sizeof(double),
                             cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    size_t off = 0;
    for (int w = 0; w < count; ++w) {
      const int n = h->geom[begin + w].n;
      const double* q = p.data() + (size_t)w * 3 * np;
      for (int j = 0; j < n; ++j)
        for (int a = 0; a < 3; ++a) state[off + 3 * j + a] = q[a * np + j];
      off += 3 * (size_t)n;
    }
  } else {
    const int np = h->np;
    std::vector<float> p((size_t)count * 6 * np);
    CUDA_TRY(cudaMemcpyAsync(p.data(), h->d_pos + (size_t)begin * 6 * np, p.size() * sizeof(float),
                             cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    size_t off = 0;
    for (int w = 0; w < count; ++w) {
      const int n = h->geom[begin + w].n;
      const float* q = p.data() + (size_t)w * 6 * np;
      for (int j = 0; j < n; ++j)
        for (int a = 0; a < 3; ++a)
          state[off + 3 * j + a] = (double)q[a * np + j] + (double)q[(3 + a) * np + j];
      off += 3 * (size_t)n;
    }
  }
  return SADMC_OK;
}

int32_t sadmc_initialize(sadmc_handle* h) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  if (!h->uploaded) return fail(SADMC_ERR_STATE, "upload a state first");
  const sadmc_config& c = h->cfg;
  h->h_cores.assign(h->W, WalkerCore{});
  for (int w = 0; w < h->W; ++w) {
    h->h_cores[w].n = h->geom[w].n;
    h->h_cores[w].kind = M_DESCENT;
  }
  int32_t r = h->push_cores();
  if (r) return r;
  CUDA_TRY(h->launch_energy(h->d_tmp));
  std::vector<double> E(h->W);
  CUDA_TRY(cudaMemcpyAsync(E.data(), h->d_tmp, sizeof(double) * h->W, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  for (int w = 0; w < h->W; ++w) h->h_cores[w].E = E[w];
  if (c.has_max_allowed) {
    // from_params descent (energy.rs:840-851)
    r = h->push_cores();
    if (r) return r;
    MoveLaunch m = h->base_launch();
    m.trace = nullptr;
    m.descent = 1;
    m.descent_limit = c.descent_limit ? c.descent_limit : 100000000ull;
    m.descent_max = c.max_allowed;
    uint64_t left = m.descent_limit;
    while (left > 0) {
      m.n_moves = std::min<uint64_t>(left, 1ull << 16);
      CUDA_TRY(h->launch_move(m));
      r = h->pull_cores();
      if (r) return r;
      bool all = true;
      for (int w = 0; w < h->W; ++w)
        if (!(h->h_cores[w].E < c.max_allowed) && h->h_cores[w].pad2 < m.descent_limit) all = false;
      if (all) break;
      left -= m.n_moves;
    }
    if (c.system != SADMC_LJ) {
      // the descent accumulated energy changes; start from the FP64 energy of the result
      // (the LJ kernel re-sums itself)
      CUDA_TRY(h->launch_energy(h->d_tmp));
      CUDA_TRY(cudaMemcpyAsync(E.data(), h->d_tmp, sizeof(double) * h->W, cudaMemcpyDeviceToHost, h->stream));
      CUDA_TRY(cudaStreamSynchronize(h->stream));
      for (int w = 0; w < h->W; ++w) {
        h->h_cores[w].E = E[w];
        if (!(E[w] < c.max_allowed)) h->h_cores[w].status |= ST_DESCENT_FAILED;
      }
    }
  }
  // EnergyMC fields (energy.rs:852-898) and Method::new (energy.rs:247-313)
  const double wdt = h->width;
  const bool both = c.has_min_allowed && c.has_max_allowed;
  for (int w = 0; w < h->W; ++w) {
    WalkerCore k{};
    const WalkerCore& o = h->h_cores[w];
    const double e0 = o.E;
    const double emin = (std::round(e0 / wdt) - 0.5) * wdt;
    const double g0d = std::floor((emin - c.e_lo) / wdt) + 2.0;
    if (!(g0d >= 0.0 && g0d < (double)h->nb))
      return fail(SADMC_ERR_INVALID, "walker " + std::to_string(w) + " starts at E=" +
                                         std::to_string(e0) + ", outside [e_lo, e_hi]");
    k.E = e0;
    k.acc_rate = 0.5;
    k.tscale = c.translation_scale;
    k.cur_min = emin;
    k.too_lo = e0; k.too_hi = e0; k.latest_param = 0.0; k.min_T = c.min_T;
    k.gamma = 1.0;
    k.wl_num_states = both ? (c.max_allowed - c.min_allowed) / wdt : 1.0;
    k.min_energy = e0;
    k.t0 = c.t0;
    k.max_S = 0.0;
    k.drift = 0.0;
    k.temperature = c.T;
    k.win_tmax = 0;
    k.moves = 0; k.accepted = 0; k.tL = 0; k.tF = 0; k.num_states = 1; k.highest_hist = 1;
    k.lowest_hist = both ? 0 : 1; k.wl_highest_hist = 1; k.total_hist = 0;
    k.kind = c.method;
    k.b_lo = k.b_hi = (int)g0d;
    k.wl_lo = 0; k.wl_hi = -1;
    k.max_S_local = 0;
    k.fill_val = 0;
    k.fill_gen = 1;
    k.status = o.status & ST_DESCENT_FAILED;
    k.n = h->geom[w].n;
    k.has_min_gamma = (c.method == SADMC_WL) ? c.has_min_gamma : 0;
    k.min_gamma = c.min_gamma;
    k.pad2 = o.pad2;
    h->h_cores[w] = k;
  }
  r = h->push_cores();
  if (r) return r;
  CUDA_TRY(launch_init_planes(h->d_cores, h->planes, h->nb, h->W, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->moves_done = 0;
  h->initialized = true;
  return SADMC_OK;
}

// The chunk launches of run(moves) are captured once per distinct `moves` into a CUDA
// graph and replayed (the kernels read all walker state from device memory, so a replay
// continues the chain); tracing runs launch directly.
int32_t sadmc_run_async(sadmc_handle* h, uint64_t moves, void* stream) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  if (!h->initialized) return fail(SADMC_ERR_STATE, "initialize first");
  if (moves == 0) return SADMC_OK;
  cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
  if (h->d_trace || std::getenv("SADMC_NO_GRAPHS")) {
    CUDA_TRY(launch_chunks(h, moves, st));
  } else {
    auto it = h->graphs.find(moves);
    if (it == h->graphs.end()) {
      cudaGraph_t g = nullptr;
      cudaGraphExec_t ge = nullptr;
      CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      cudaError_t e = launch_chunks(h, moves, st);
      cudaError_t e2 = cudaStreamEndCapture(st, &g);
      if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(SADMC_ERR_CUDA, std::string("graph capture: ") +
                                        cudaGetErrorString(e != cudaSuccess ? e : e2));
      }
      e = cudaGraphInstantiate(&ge, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess)
        return fail(SADMC_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
      it = h->graphs.emplace(moves, ge).first;
    }
    CUDA_TRY(cudaGraphLaunch(it->second, st));
  }
  h->moves_done += moves;
  return SADMC_OK;
}

int32_t sadmc_run(sadmc_handle* h, uint64_t moves) {
  int32_t r = sadmc_run_async(h, moves, nullptr);
  if (r) return r;
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return SADMC_OK;
}

int32_t sadmc_synchronize(sadmc_handle* h) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return SADMC_OK;
}

int32_t sadmc_energy(sadmc_handle* h, double* E) {
  if (!h || !E) return fail(SADMC_ERR_INVALID, "null argument");
  int32_t r = h->pull_cores();
  if (r) return r;
  for (int w = 0; w < h->W; ++w) E[w] = h->h_cores[w].E;
  return SADMC_OK;
}

int32_t sadmc_compute_energy(sadmc_handle* h, double* E) {
  if (!h || !E) return fail(SADMC_ERR_INVALID, "null argument");
  if (!h->uploaded) return fail(SADMC_ERR_STATE, "upload a state first");
  int32_t r = h->prep_cores();
  if (r) return r;
  CUDA_TRY(h->launch_energy(h->d_tmp));
  CUDA_TRY(cudaMemcpyAsync(E, h->d_tmp, sizeof(double) * h->W, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return SADMC_OK;
}

int32_t sadmc_plan_move_injected(sadmc_handle* h, int32_t walker, const sadmc_proposal* p,
                                 double* e_out, int32_t* possible) {
  if (!h || !p || !e_out || !possible || walker < 0 || walker >= h->W)
    return fail(SADMC_ERR_INVALID, "bad argument");
  if (h->cfg.system != SADMC_LJ) return fail(SADMC_ERR_INVALID, "injected plans support the LJ cluster");
  if (p->which < 0 || p->which >= h->geom[walker].n) return fail(SADMC_ERR_INVALID, "bad atom index");
  if (!h->uploaded) return fail(SADMC_ERR_STATE, "upload a state first");
  int32_t r = h->prep_cores();
  if (r) return r;
  if (!h->initialized) {  // plan against System::energy() of the uploaded state
    CUDA_TRY(h->launch_energy(h->d_tmp));
    std::vector<double> E(h->W);
    CUDA_TRY(cudaMemcpyAsync(E.data(), h->d_tmp, sizeof(double) * h->W, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    for (int w = 0; w < h->W; ++w) h->h_cores[w].E = E[w];
    r = h->push_cores();
    if (r) return r;
  }
  CUDA_TRY(launch_lj_plan(h->d_cores, LjSys{h->d_pos, h->np, h->radius2()}, walker, p->which,
                          (float)p->g[0], (float)p->g[1], (float)p->g[2], p->scale, 0, h->d_tmp,
                          h->stream));
  double o[2];
  CUDA_TRY(cudaMemcpyAsync(o, h->d_tmp, sizeof(o), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  *e_out = o[0];
  *possible = o[1] != 0.0;
  h->pend_walker = *possible ? walker : -1;
  h->pend = *p;
  return SADMC_OK;
}

int32_t sadmc_confirm(sadmc_handle* h, int32_t walker) {
  if (!h || walker < 0 || walker >= h->W) return fail(SADMC_ERR_INVALID, "bad argument");
  if (h->pend_walker != walker) return SADMC_OK;  // ConfirmSystem::confirm with no change
  const sadmc_proposal& p = h->pend;
  CUDA_TRY(launch_lj_plan(h->d_cores, LjSys{h->d_pos, h->np, h->radius2()}, walker, p.which,
                          (float)p.g[0], (float)p.g[1], (float)p.g[2], p.scale, 1, h->d_tmp,
                          h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->pend_walker = -1;
  return SADMC_OK;
}

int32_t sadmc_nbins(sadmc_handle* h, int32_t walker, int64_t* nbins, double* bins_min, double* width) {
  if (!h || walker < 0 || walker >= h->W) return fail(SADMC_ERR_INVALID, "bad argument");
  if (!h->initialized) return fail(SADMC_ERR_STATE, "initialize first");
  WalkerCore k;
  CUDA_TRY(cudaMemcpyAsync(&k, h->d_cores + walker, sizeof(k), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (nbins) *nbins = k.b_hi - k.b_lo + 1;
  if (bins_min) *bins_min = k.cur_min;
  if (width) *width = h->width;
  return SADMC_OK;
}

int32_t sadmc_read_bins(sadmc_handle* h, int32_t walker, double* lnw, uint64_t* hist,
                        uint64_t* t_found, double* sumE, double* sumE2, uint64_t* rt,
                        uint8_t* visited) {
  if (!h || walker < 0 || walker >= h->W) return fail(SADMC_ERR_INVALID, "bad argument");
  if (!h->initialized) return fail(SADMC_ERR_STATE, "initialize first");
  WalkerCore k;
  CUDA_TRY(cudaMemcpyAsync(&k, h->d_cores + walker, sizeof(k), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  const size_t n = (size_t)(k.b_hi - k.b_lo + 1);
  const size_t off = (size_t)walker * h->nb + k.b_lo;
  auto get = [&](void* dst, const void* src) -> cudaError_t {
    if (!dst) return cudaSuccess;
    return cudaMemcpyAsync(dst, (const char*)src + off * 8, n * 8, cudaMemcpyDeviceToHost, h->stream);
  };
  CUDA_TRY(get(lnw, h->planes.lnw));
  CUDA_TRY(get(hist, h->planes.hist));
  CUDA_TRY(get(t_found, h->planes.t_found));
  CUDA_TRY(get(sumE, h->planes.sumE));
  CUDA_TRY(get(sumE2, h->planes.sumE2));
  CUDA_TRY(get(rt, h->planes.round_trips));
  std::vector<uint64_t> st(visited ? n : 0);
  if (visited) CUDA_TRY(get(st.data(), h->planes.visit_stamp));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (visited)
    for (size_t i = 0; i < n; ++i) visited[i] = st[i] == k.fill_gen ? 1 : (uint8_t)(k.fill_val != 0);
  // the cached current bin lives in the planes after each launch (flushed on store)
  return SADMC_OK;
}

int32_t sadmc_read_extra(sadmc_handle* h, int32_t walker, uint64_t* count, double* total) {
  if (!h || walker < 0 || walker >= h->W) return fail(SADMC_ERR_INVALID, "bad argument");
  if (!h->initialized) return fail(SADMC_ERR_STATE, "initialize first");
  if (!h->planes.ex_count) return fail(SADMC_ERR_INVALID, "this system collects no data");
  WalkerCore k;
  CUDA_TRY(cudaMemcpyAsync(&k, h->d_cores + walker, sizeof(k), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  const size_t n = (size_t)(k.b_hi - k.b_lo + 1);
  const size_t off = (size_t)walker * h->nb + k.b_lo;
  if (count)
    CUDA_TRY(cudaMemcpyAsync(count, h->planes.ex_count + off, n * 8, cudaMemcpyDeviceToHost, h->stream));
  if (total)
    CUDA_TRY(cudaMemcpyAsync(total, h->planes.ex_total + off, n * 8, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return SADMC_OK;
}

int32_t sadmc_plane_bins(sadmc_handle* h, int64_t* plane_bins) {
  if (!h || !plane_bins) return fail(SADMC_ERR_INVALID, "null argument");
  *plane_bins = h->nb;
  return SADMC_OK;
}

int32_t sadmc_read_planes(sadmc_handle* h, double* lnw, uint64_t* hist, int32_t* range,
                          double* bins_min) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  if (!h->initialized) return fail(SADMC_ERR_STATE, "initialize first");
  const size_t n = (size_t)h->W * (size_t)h->nb;
  if (lnw) CUDA_TRY(cudaMemcpyAsync(lnw, h->planes.lnw, n * 8, cudaMemcpyDeviceToHost, h->stream));
  if (hist) CUDA_TRY(cudaMemcpyAsync(hist, h->planes.hist, n * 8, cudaMemcpyDeviceToHost, h->stream));
  int32_t r = h->pull_cores();
  if (r) return r;
  for (int w = 0; w < h->W; ++w) {
    if (range) { range[2 * w] = h->h_cores[w].b_lo; range[2 * w + 1] = h->h_cores[w].b_hi; }
    if (bins_min) bins_min[w] = h->h_cores[w].cur_min;
  }
  return SADMC_OK;
}

int32_t sadmc_read_wl_hist(sadmc_handle* h, int32_t walker, uint64_t* hist, int64_t* n, double* min_energy) {
  if (!h || walker < 0 || walker >= h->W || !n) return fail(SADMC_ERR_INVALID, "bad argument");
  WalkerCore k;
  CUDA_TRY(cudaMemcpyAsync(&k, h->d_cores + walker, sizeof(k), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  const int64_t len = k.wl_hi >= k.wl_lo ? (int64_t)(k.wl_hi - k.wl_lo + 1) : 0;
  *n = len;
  if (min_energy) *min_energy = k.min_energy;
  if (hist && len > 0) {
    CUDA_TRY(cudaMemcpyAsync(hist, h->planes.wl_hist + (size_t)walker * h->nb + k.wl_lo, len * 8,
                             cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
  }
  return SADMC_OK;
}

int32_t sadmc_read_scalars(sadmc_handle* h, int32_t walker, double* o) {
  if (!h || !o || walker < 0 || walker >= h->W) return fail(SADMC_ERR_INVALID, "bad argument");
  WalkerCore k;
  CUDA_TRY(cudaMemcpyAsync(&k, h->d_cores + walker, sizeof(k), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  const double kind = k.kind == M_INV_T_WL ? (double)M_WL : (double)k.kind;
  const double v[SADMC_N_SCALARS] = {
      (double)k.moves, (double)k.accepted, k.acc_rate, k.tscale, kind, k.too_lo, k.too_hi,
      (double)k.tL, (double)k.tF, (double)k.num_states, (double)k.highest_hist,
      k.latest_param, k.gamma, (double)k.lowest_hist, (double)k.wl_highest_hist,
      (double)k.total_hist, k.wl_num_states, k.min_energy, k.t0, k.max_S,
      (double)k.max_S_local, k.drift, (double)k.status, k.E};
  std::memcpy(o, v, sizeof(v));
  return SADMC_OK;
}

int32_t sadmc_counters(sadmc_handle* h, uint64_t* moves, uint64_t* accepted) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  int32_t r = h->pull_cores();
  if (r) return r;
  uint64_t m = 0, a = 0;
  for (const auto& k : h->h_cores) { m += k.moves; a += k.accepted; }
  if (moves) *moves = m;
  if (accepted) *accepted = a;
  return SADMC_OK;
}

int32_t sadmc_status(sadmc_handle* h, uint32_t* flags) {
  if (!h || !flags) return fail(SADMC_ERR_INVALID, "null argument");
  int32_t r = h->pull_cores();
  if (r) return r;
  for (int w = 0; w < h->W; ++w) flags[w] = h->h_cores[w].status;
  return SADMC_OK;
}

int32_t sadmc_set_trace(sadmc_handle* h, uint64_t capacity) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  h->drop_graphs();
  cudaFree(h->d_trace);
  cudaFree(h->d_trace_ds);
  h->d_trace = nullptr;
  h->d_trace_ds = nullptr;
  h->trace_cap = 0;
  if (capacity == 0) return SADMC_OK;
  if (dalloc(&h->d_trace, (size_t)h->W * capacity) != cudaSuccess ||
      dalloc(&h->d_trace_ds, (size_t)h->W * capacity) != cudaSuccess)
    return fail(SADMC_ERR_NOMEM, "trace allocation failed");
  CUDA_TRY(cudaMemsetAsync(h->d_trace, 0xff, sizeof(TraceRec) * (size_t)h->W * capacity, h->stream));
  CUDA_TRY(cudaMemsetAsync(h->d_trace_ds, 0, sizeof(float) * (size_t)h->W * capacity, h->stream));
  h->trace_cap = capacity;
  h->trace_t0 = h->moves_done;
  return SADMC_OK;
}

int32_t sadmc_read_trace(sadmc_handle* h, int32_t walker, double* e1, double* e2, uint64_t* count) {
  if (!h || walker < 0 || walker >= h->W) return fail(SADMC_ERR_INVALID, "bad argument");
  if (!h->d_trace) return fail(SADMC_ERR_STATE, "tracing disabled");
  const uint64_t done = h->moves_done > h->trace_t0 ? h->moves_done - h->trace_t0 : 0;
  const uint64_t n = std::min(done, h->trace_cap);
  std::vector<TraceRec> r(n);
  if (n) {
    CUDA_TRY(cudaMemcpyAsync(r.data(), h->d_trace + (size_t)walker * h->trace_cap, n * sizeof(TraceRec),
                             cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
  }
  for (uint64_t k = 0; k < n; ++k) {
    if (e1) e1[k] = r[k].e1;
    if (e2) e2[k] = r[k].e2;
  }
  if (count) *count = n;
  return SADMC_OK;
}

int32_t sadmc_read_trace_ds(sadmc_handle* h, int32_t walker, float* ds, uint64_t* count) {
  if (!h || walker < 0 || walker >= h->W) return fail(SADMC_ERR_INVALID, "bad argument");
  if (!h->d_trace_ds) return fail(SADMC_ERR_STATE, "tracing disabled");
  const uint64_t done = h->moves_done > h->trace_t0 ? h->moves_done - h->trace_t0 : 0;
  const uint64_t n = std::min(done, h->trace_cap);
  if (n && ds) {
    CUDA_TRY(cudaMemcpyAsync(ds, h->d_trace_ds + (size_t)walker * h->trace_cap, n * sizeof(float),
                             cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
  }
  if (count) *count = n;
  return SADMC_OK;
}

int32_t sadmc_lanes_per_walker(sadmc_handle* h) { return h ? h->lpw : 0; }

// Autotuner: each (lanes per walker, warps per block) candidate runs `moves` moves on a
// snapshot of the batch, timed with CUDA events; the snapshot is restored after every
// candidate, the fastest is kept and recorded in the tuning cache
// ($SADMC_TUNE_CACHE or ~/.cache/sadmc_gb300_tune.txt, one "key lpw wpb ms" per line).
int32_t sadmc_autotune(sadmc_handle* h, uint64_t moves, int32_t* best_lpw, double* best_ms) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  if (!h->initialized) return fail(SADMC_ERR_STATE, "initialize first");
  if (moves == 0) moves = 1024;
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  const auto bufs = state_buffers(h);
  std::vector<void*> snap(bufs.size(), nullptr);
  for (size_t i = 0; i < bufs.size(); ++i) {
    if (cudaMalloc(&snap[i], bufs[i].bytes) != cudaSuccess) {
      for (void* p : snap) cudaFree(p);
      return fail(SADMC_ERR_NOMEM, "autotune snapshot allocation failed");
    }
    CUDA_TRY(cudaMemcpyAsync(snap[i], bufs[i].ptr, bufs[i].bytes, cudaMemcpyDeviceToDevice, h->stream));
  }
  auto restore = [&]() -> cudaError_t {
    for (size_t i = 0; i < bufs.size(); ++i) {
      cudaError_t e = cudaMemcpyAsync(bufs[i].ptr, snap[i], bufs[i].bytes, cudaMemcpyDeviceToDevice, h->stream);
      if (e != cudaSuccess) return e;
    }
    return cudaStreamSynchronize(h->stream);
  };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int keep_lpw = h->lpw, keep_wpb = h->wpb;
  int bl = keep_lpw, bw = keep_wpb;
  float bms = 1e30f;
  cudaError_t err = cudaSuccess;
  for (int lpw : lpw_candidates(h)) {
    for (int wpb : {1, 2, 4}) {
      h->lpw = lpw;
      h->wpb = wpb;
      err = launch_chunks(h, std::min<uint64_t>(moves, 256), h->stream);  // warm-up
      if (err == cudaSuccess) err = restore();
      if (err == cudaSuccess) err = cudaEventRecord(e0, h->stream);
      if (err == cudaSuccess) err = launch_chunks(h, moves, h->stream);
      if (err == cudaSuccess) err = cudaEventRecord(e1, h->stream);
      if (err == cudaSuccess) err = cudaEventSynchronize(e1);
      float ms = 0;
      if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
      if (err == cudaSuccess) err = restore();
      if (err != cudaSuccess) break;
      if (ms < bms) { bms = ms; bl = lpw; bw = wpb; }
    }
    if (err != cudaSuccess) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (void* p : snap) cudaFree(p);
  if (err != cudaSuccess) {
    h->lpw = keep_lpw;
    h->wpb = keep_wpb;
    return fail(SADMC_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(err));
  }
  h->lpw = bl;
  h->wpb = bw;
  h->drop_graphs();
  // record (best effort; an unwritable cache directory just skips it)
  const std::string path = tune_cache_path(), key = tune_key(h);
  std::vector<std::string> lines;
  {
    std::ifstream in(path);
    for (std::string line; std::getline(in, line);)
      if (line.rfind(key + " ", 0) != 0) lines.push_back(line);
  }
  std::ostringstream rec;
  rec << key << " " << bl << " " << bw << " " << bms;
  lines.push_back(rec.str());
  std::ofstream out(path);
  for (const auto& l : lines) out << l << "\n";
  if (best_lpw) *best_lpw = bl;
  if (best_ms) *best_ms = bms;
  return SADMC_OK;
}


int32_t sadmc_checkpoint(sadmc_handle* h, const char* path) {
  if (!h || !path) return fail(SADMC_ERR_INVALID, "null argument");
  if (!h->initialized) return fail(SADMC_ERR_STATE, "initialize first");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return fail(SADMC_ERR_INVALID, "cannot open " + tmp);
  bool ok = std::fwrite(kMagic, 1, 8, f) == 8;
  const int32_t W = h->W;
  ok = ok && std::fwrite(&h->cfg, sizeof(h->cfg), 1, f) == 1;
  ok = ok && std::fwrite(&W, sizeof(W), 1, f) == 1;
  ok = ok && std::fwrite(h->geom.data(), sizeof(sadmc_geometry), W, f) == (size_t)W;
  ok = ok && std::fwrite(&h->moves_done, sizeof(h->moves_done), 1, f) == 1;
  ok = ok && std::fwrite(&h->lpw, sizeof(h->lpw), 1, f) == 1;
  std::vector<char> host;
  for (const DevBuf& b : state_buffers(h)) {
    host.resize(b.bytes);
    if (ok && cudaMemcpy(host.data(), b.ptr, b.bytes, cudaMemcpyDeviceToHost) != cudaSuccess) ok = false;
    const uint64_t n = b.bytes;
    ok = ok && std::fwrite(&n, sizeof(n), 1, f) == 1 && std::fwrite(host.data(), 1, b.bytes, f) == b.bytes;
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok || std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return fail(SADMC_ERR_INVALID, std::string("checkpoint write failed: ") + path);
  }
  return SADMC_OK;
}

int32_t sadmc_resume(const char* path, sadmc_handle** out) {
  if (!path || !out) return fail(SADMC_ERR_INVALID, "null argument");
  *out = nullptr;
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(SADMC_ERR_INVALID, std::string("cannot open ") + path);
  char magic[8];
  sadmc_config cfg;
  int32_t W = 0;
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kMagic, 8) == 0 &&
            std::fread(&cfg, sizeof(cfg), 1, f) == 1 && std::fread(&W, sizeof(W), 1, f) == 1 &&
            W == cfg.n_walkers && W > 0;
  std::vector<sadmc_geometry> geom(ok ? W : 0);
  uint64_t moves_done = 0;
  int32_t lpw = 0;
  ok = ok && std::fread(geom.data(), sizeof(sadmc_geometry), W, f) == (size_t)W &&
       std::fread(&moves_done, sizeof(moves_done), 1, f) == 1 && std::fread(&lpw, sizeof(lpw), 1, f) == 1;
  if (!ok) { std::fclose(f); return fail(SADMC_ERR_INVALID, "not a sadmc checkpoint"); }
  cfg.lanes_per_walker = lpw;
  sadmc_handle* h = nullptr;
  int32_t r = sadmc_create(&cfg, geom.data(), &h);
  if (r) { std::fclose(f); return r; }
  std::vector<char> host;
  for (const DevBuf& b : state_buffers(h)) {
    uint64_t n = 0;
    if (std::fread(&n, sizeof(n), 1, f) != 1 || n != b.bytes) { ok = false; break; }
    host.resize(b.bytes);
    if (std::fread(host.data(), 1, b.bytes, f) != b.bytes ||
        cudaMemcpy(b.ptr, host.data(), b.bytes, cudaMemcpyHostToDevice) != cudaSuccess) { ok = false; break; }
  }
  std::fclose(f);
  if (!ok) { sadmc_destroy(h); return fail(SADMC_ERR_INVALID, "truncated or mismatched checkpoint"); }
  h->uploaded = h->initialized = true;
  h->moves_done = moves_done;
  h->h_cores.clear();
  *out = h;
  return SADMC_OK;
}

int32_t sadmc_get_config(sadmc_handle* h, sadmc_config* cfg, sadmc_geometry* geom) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  if (cfg) *cfg = h->cfg;
  if (geom) std::memcpy(geom, h->geom.data(), sizeof(sadmc_geometry) * h->W);
  return SADMC_OK;
}


int32_t sadmc_surrogate_init(sadmc_handle* h, uint64_t seed, int32_t ring_capacity) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  if (h->cfg.system != SADMC_LJ) return fail(SADMC_ERR_INVALID, "the surrogate is for LJ clusters");
  for (int w = 1; w < h->W; ++w)
    if (h->geom[w].n != h->geom[0].n) return fail(SADMC_ERR_INVALID, "surrogate needs walkers of equal N");
  if (h->geom[0].n > SG_MAX_ATOMS)
    return fail(SADMC_ERR_INVALID, "the surrogate supports clusters of up to " + std::to_string(SG_MAX_ATOMS) + " atoms");
  if (ring_capacity <= 0) return fail(SADMC_ERR_INVALID, "ring_capacity must be positive");
  h->free_surrogate();
  const int n = h->geom[0].n;
  cudaError_t e = cudaMalloc(&h->sg_master, sizeof(float) * SG_NPARAM);
  if (e == cudaSuccess) e = cudaMalloc(&h->sg_grad, sizeof(float) * SG_NPARAM);
  if (e == cudaSuccess) e = cudaMalloc(&h->sg_m, sizeof(float) * SG_NPARAM);
  if (e == cudaSuccess) e = cudaMalloc(&h->sg_v, sizeof(float) * SG_NPARAM);
  if (e == cudaSuccess) e = cudaMalloc(&h->sg_w1t, sizeof(__nv_bfloat16) * SG_RBF * SG_H1);
  if (e == cudaSuccess) e = cudaMalloc(&h->sg_w2t, sizeof(__nv_bfloat16) * SG_H1 * SG_H2);
  if (e == cudaSuccess) e = cudaMalloc(&h->sg_wc, sizeof(__nv_bfloat16) * SG_WC_ELEMS);
  if (e == cudaSuccess) e = cudaMalloc(&h->sg_ring_pos, sizeof(float) * 3 * (size_t)n * ring_capacity);
  if (e == cudaSuccess) e = cudaMalloc(&h->sg_ring_e, sizeof(float) * ring_capacity);
  if (e == cudaSuccess) e = cudaMalloc(&h->sg_loss, sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->sg_flag, sizeof(unsigned int));
  if (e != cudaSuccess) { h->free_surrogate(); return fail(SADMC_ERR_NOMEM, "surrogate allocation failed"); }
  // N(0, 1/fan_in) weights, zero biases (a splitmix/Box-Muller host generator)
  std::vector<float> p(SG_NPARAM, 0.0f);
  uint64_t s = seed * 0x9E3779B97F4A7C15ull + 1;
  auto next = [&]() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  };
  auto normal = [&]() { return std::sqrt(-2.0 * std::log(next())) * std::cos(6.283185307179586 * next()); };
  for (int k = 0; k < SG_RBF * SG_H1; ++k) p[SG_OFF_W1 + k] = (float)(normal() / std::sqrt((double)SG_RBF));
  for (int k = 0; k < SG_H1 * SG_H2; ++k) p[SG_OFF_W2 + k] = (float)(normal() / std::sqrt((double)SG_H1));
  for (int k = 0; k < SG_H2; ++k) p[SG_OFF_W3 + k] = (float)(normal() / std::sqrt((double)SG_H2));
  h->sg_cap = ring_capacity;
  h->sg_head = h->sg_count = h->sg_step = 0;
  return sadmc_surrogate_set_params(h, p.data());
}

int32_t sadmc_surrogate_set_params(sadmc_handle* h, const float* params) {
  if (!h || !params) return fail(SADMC_ERR_INVALID, "null argument");
  if (!h->sg_master) return fail(SADMC_ERR_STATE, "call sadmc_surrogate_init first");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  CUDA_TRY(cudaMemcpy(h->sg_master, params, sizeof(float) * SG_NPARAM, cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemset(h->sg_m, 0, sizeof(float) * SG_NPARAM));
  CUDA_TRY(cudaMemset(h->sg_v, 0, sizeof(float) * SG_NPARAM));
  h->sg_step = 0;
  CUDA_TRY(sg_refresh(h->sg_master, h->sg_weights(), h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return SADMC_OK;
}

int32_t sadmc_surrogate_get_params(sadmc_handle* h, float* params) {
  if (!h || !params) return fail(SADMC_ERR_INVALID, "null argument");
  if (!h->sg_master) return fail(SADMC_ERR_STATE, "call sadmc_surrogate_init first");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  CUDA_TRY(cudaMemcpy(params, h->sg_master, sizeof(float) * SG_NPARAM, cudaMemcpyDeviceToHost));
  return SADMC_OK;
}

namespace {

// Append every walker's configuration and energy to the training ring (stream-ordered,
// no host synchronisation: the energies are read from the walker state on the device).
cudaError_t sg_collect_async(sadmc_handle* h) {
  const int take = std::min(h->W, h->sg_cap);
  cudaError_t e = sg_collect(h->d_pos, h->np, h->geom[0].n, h->d_cores, take, h->sg_ring_pos, h->sg_ring_e,
                             h->sg_cap, h->sg_head, h->stream);
  if (e == cudaSuccess) {
    h->sg_head = (h->sg_head + take) % h->sg_cap;
    h->sg_count = std::min(h->sg_cap, h->sg_count + take);
  }
  return e;
}

// `steps` Adam steps on minibatches of `batch` ring configurations (stream-ordered).
cudaError_t sg_train_async(sadmc_handle* h, int steps, int batch, float lr, uint64_t seed) {
  const int n = h->geom[0].n;
  cudaError_t e = h->sg_reserve((size_t)batch * n, batch);
  if (e != cudaSuccess) return e;
  const SgScratch sc = SgScratch::carve(h->sg_scratch, (size_t)batch * n);
  unsigned int* flag = nullptr;
  e = sg_timeout_flag(&flag);
  for (int it = 0; it < steps && e == cudaSuccess; ++it) {
    e = sg_gather(h->sg_ring_pos, h->sg_ring_e, n, h->sg_count, seed, (uint64_t)it, batch, h->sg_batch_pos,
                  h->sg_batch_e, h->stream);
    h->sg_step += 1;
    if (e == cudaSuccess)
      e = sg_train_step(h->sg_batch_pos, h->sg_batch_e, batch, n, h->sg_weights(), h->sg_grad,
                        h->sg_adam(h->sg_step, lr), sc, h->sg_loss, flag, h->stream);
  }
  return e;
}

// Synchronise the handle's stream and report (then clear) a tensor-core wait that ran out.
int32_t sg_check_timeouts(sadmc_handle* h) {
  unsigned int* flag = nullptr;
  CUDA_TRY(sg_timeout_flag(&flag));
  CUDA_TRY(sg_take_flag(flag, h->sg_flag, h->stream));
  unsigned int to = 0;
  CUDA_TRY(cudaMemcpyAsync(&to, h->sg_flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (to) return fail(SADMC_ERR_CUDA, "a tensor-core wait of the surrogate ran out");
  return SADMC_OK;
}

}  // namespace

int32_t sadmc_surrogate_collect(sadmc_handle* h, int32_t* ring_count) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  if (!h->sg_master) return fail(SADMC_ERR_STATE, "call sadmc_surrogate_init first");
  if (!h->initialized) return fail(SADMC_ERR_STATE, "initialize first");
  CUDA_TRY(sg_collect_async(h));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (ring_count) *ring_count = h->sg_count;
  return SADMC_OK;
}

int32_t sadmc_surrogate_train(sadmc_handle* h, int32_t steps, int32_t batch, float lr,
                              uint64_t seed, double* loss) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  if (!h->sg_master) return fail(SADMC_ERR_STATE, "call sadmc_surrogate_init first");
  if (h->sg_count == 0) return fail(SADMC_ERR_STATE, "the training ring is empty");
  if (steps <= 0 || batch <= 0) return fail(SADMC_ERR_INVALID, "steps and batch must be positive");
  CUDA_TRY(sg_train_async(h, steps, batch, lr, seed));
  double l = 0;
  CUDA_TRY(cudaMemcpyAsync(&l, h->sg_loss, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  int32_t r = sg_check_timeouts(h);
  if (r) return r;
  if (loss) *loss = l;
  return SADMC_OK;
}

int32_t sadmc_surrogate_loss_grads(sadmc_handle* h, const float* pos, const float* target,
                                   int32_t configs, double* loss, float* grads) {
  if (!h || !pos || !target || configs <= 0) return fail(SADMC_ERR_INVALID, "bad argument");
  if (!h->sg_master) return fail(SADMC_ERR_STATE, "call sadmc_surrogate_init first");
  const int n = h->geom[0].n;
  CUDA_TRY(h->sg_reserve((size_t)configs * n, configs));
  const SgScratch sc = SgScratch::carve(h->sg_scratch, (size_t)configs * n);
  unsigned int* flag = nullptr;
  CUDA_TRY(sg_timeout_flag(&flag));
  CUDA_TRY(cudaMemcpyAsync(h->sg_batch_pos, pos, sizeof(float) * 3 * (size_t)configs * n, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(cudaMemcpyAsync(h->sg_batch_e, target, sizeof(float) * configs, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(sg_train_step(h->sg_batch_pos, h->sg_batch_e, configs, n, h->sg_weights(), h->sg_grad,
                         h->sg_adam(0, 0.0f), sc, h->sg_loss, flag, h->stream));
  double l = 0;
  CUDA_TRY(cudaMemcpyAsync(&l, h->sg_loss, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (grads) CUDA_TRY(cudaMemcpyAsync(grads, h->sg_grad, sizeof(float) * SG_NPARAM, cudaMemcpyDeviceToHost, h->stream));
  int32_t r = sg_check_timeouts(h);
  if (r) return r;
  if (loss) *loss = l;
  return SADMC_OK;
}

int32_t sadmc_surrogate_loss_grads_noalloc(sadmc_handle* h, const float* pos, const float* target,
                                           int32_t configs, double* loss, float* grads,
                                           void* stream) {
  if (!h || !pos || !target || !loss || !grads || configs <= 0)
    return fail(SADMC_ERR_INVALID, "bad argument");
  if (!h->sg_master) return fail(SADMC_ERR_STATE, "call sadmc_surrogate_init first");
  const size_t rows = (size_t)configs * (size_t)h->geom[0].n;
  if (rows > SG_STATIC_ROWS)
    return fail(SADMC_ERR_INVALID, "configs x atoms exceeds the static scratch of " +
                                       std::to_string(SG_STATIC_ROWS) + " rows");
  void* base = nullptr;
  CUDA_TRY(sg_static_scratch(&base));
  const SgScratch sc = SgScratch::carve(base, rows);
  const cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
  // gradients only, no optimizer state touched; no timeout flag: a tensor-core wait that
  // ran out leaves NaN in the loss and the gradients, the only signal of this path
  CUDA_TRY(sg_train_step(pos, target, configs, h->geom[0].n, h->sg_weights(), grads, h->sg_adam(0, 0.0f),
                         sc, loss, nullptr, st));
  return SADMC_OK;
}

namespace {

// `moves` delayed-acceptance moves of every walker, in launches of at most 8192.
cudaError_t launch_da_chunks(sadmc_handle* h, uint64_t moves, int32_t refresh_interval) {
  MoveLaunch m = h->base_launch();  // traced like sadmc_run, with dS in the second record
  int max_atoms = 0;
  for (const auto& g : h->geom) max_atoms = std::max(max_atoms, (int)g.n);
  cudaError_t e = cudaSuccess;
  for (uint64_t left = moves; left > 0 && e == cudaSuccess;) {
    m.n_moves = std::min<uint64_t>(left, 8192);
    e = launch_lj_da(m, LjSys{h->d_pos, h->np, h->radius2()}, h->sg_weights(), max_atoms, refresh_interval,
                     h->sg_stats, h->stream);
    left -= m.n_moves;
  }
  return e;
}

int32_t da_checks(sadmc_handle* h) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  if (!h->sg_master) return fail(SADMC_ERR_STATE, "call sadmc_surrogate_init first");
  if (!h->initialized) return fail(SADMC_ERR_STATE, "initialize first");
  if (h->cfg.method == SADMC_CANONICAL) return fail(SADMC_ERR_INVALID, "delayed acceptance needs a flat-histogram method");
  if (h->np > 64) return fail(SADMC_ERR_INVALID, "delayed acceptance supports up to 64 atoms");
  if (!h->sg_stats) {
    CUDA_TRY(cudaMalloc(&h->sg_stats, sizeof(uint64_t) * 2 * h->W));
    CUDA_TRY(cudaMemset(h->sg_stats, 0, sizeof(uint64_t) * 2 * h->W));
  }
  return SADMC_OK;
}

}  // namespace

int32_t sadmc_run_da(sadmc_handle* h, uint64_t moves, int32_t refresh_interval, uint64_t* stats) {
  int32_t r = da_checks(h);
  if (r) return r;
  CUDA_TRY(launch_da_chunks(h, moves, refresh_interval));
  h->moves_done += moves;
  if (stats) CUDA_TRY(cudaMemcpyAsync(stats, h->sg_stats, sizeof(uint64_t) * 2 * h->W, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return SADMC_OK;
}

int32_t sadmc_run_online(sadmc_handle* h, uint64_t moves, int32_t delayed, int32_t refresh_interval,
                         const sadmc_online* o, uint64_t* stats) {
  if (!h || !o) return fail(SADMC_ERR_INVALID, "null argument");
  if (!h->sg_master) return fail(SADMC_ERR_STATE, "call sadmc_surrogate_init first");
  if (!h->initialized) return fail(SADMC_ERR_STATE, "initialize first");
  if (o->retrain_interval && (o->train_steps <= 0 || o->batch <= 0))
    return fail(SADMC_ERR_INVALID, "train_steps and batch must be positive");
  if (delayed) {
    int32_t r = da_checks(h);
    if (r) return r;
  }
  // the schedule counts this handle's moves since initialize, so consecutive calls
  // continue it
  const uint64_t t0 = h->moves_done;
  auto next_event = [](uint64_t t, uint64_t every) -> uint64_t {
    return every ? (t / every + 1) * every : ~0ull;
  };
  for (uint64_t t = t0; t < t0 + moves;) {
    const uint64_t stop = std::min({t0 + moves, next_event(t, o->collect_interval), next_event(t, o->retrain_interval)});
    const uint64_t seg = stop - t;
    if (delayed) CUDA_TRY(launch_da_chunks(h, seg, refresh_interval));
    else CUDA_TRY(launch_chunks(h, seg, h->stream));
    t = stop;
    h->moves_done = t;
    if (o->collect_interval && t % o->collect_interval == 0) CUDA_TRY(sg_collect_async(h));
    if (o->retrain_interval && t % o->retrain_interval == 0 && h->sg_count > 0)
      CUDA_TRY(sg_train_async(h, o->train_steps, o->batch, o->lr, o->seed ^ (t * 0x9E3779B97F4A7C15ull)));
  }
  if (stats && delayed)
    CUDA_TRY(cudaMemcpyAsync(stats, h->sg_stats, sizeof(uint64_t) * 2 * h->W, cudaMemcpyDeviceToHost, h->stream));
  return sg_check_timeouts(h);
}

int32_t sadmc_surrogate_predict(sadmc_handle* h, const float* pos, int32_t configs, float* energies) {
  if (!h || !pos || !energies || configs <= 0) return fail(SADMC_ERR_INVALID, "bad argument");
  if (!h->sg_master) return fail(SADMC_ERR_STATE, "call sadmc_surrogate_init first");
  const int n = h->geom[0].n;
  const size_t rows = (size_t)configs * n;
  CUDA_TRY(h->sg_reserve(rows, configs));
  const SgScratch sc = SgScratch::carve(h->sg_scratch, rows);
  unsigned int* flag = nullptr;
  CUDA_TRY(sg_timeout_flag(&flag));
  CUDA_TRY(cudaMemcpyAsync(h->sg_batch_pos, pos, sizeof(float) * 3 * rows, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(sg_descriptors(h->sg_batch_pos, n, (int)rows, sc.gq, nullptr, h->stream));
  CUDA_TRY(sg_forward(sc.gq, (int)rows, h->sg_weights(), sc.e, flag, h->stream));
  std::vector<float> e(rows);
  CUDA_TRY(cudaMemcpyAsync(e.data(), sc.e, sizeof(float) * rows, cudaMemcpyDeviceToHost, h->stream));
  int32_t r = sg_check_timeouts(h);
  if (r) return r;
  for (int c = 0; c < configs; ++c) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += e[(size_t)c * n + i];
    energies[c] = (float)s;
  }
  return SADMC_OK;
}

int32_t sadmc_draws(int32_t system, uint32_t n, uint64_t seed, uint32_t walker, uint64_t t0,
                    int32_t count, uint32_t stream_pair, uint32_t* idx2, float* g3, double* u) {
  if (!idx2 || !g3 || !u || count <= 0 || n == 0) return fail(SADMC_ERR_INVALID, "bad argument");
  uint32_t* di = nullptr;
  float* dg = nullptr;
  double* du = nullptr;
  cudaError_t e = cudaMalloc(&di, sizeof(uint32_t) * 2 * count);
  if (e == cudaSuccess) e = cudaMalloc(&dg, sizeof(float) * 3 * count);
  if (e == cudaSuccess) e = cudaMalloc(&du, sizeof(double) * count);
  if (e == cudaSuccess) e = launch_draws(system, n, seed, walker, t0, count, stream_pair, di, dg, du, 0);
  if (e == cudaSuccess) e = cudaMemcpy(idx2, di, sizeof(uint32_t) * 2 * count, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(g3, dg, sizeof(float) * 3 * count, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(u, du, sizeof(double) * count, cudaMemcpyDeviceToHost);
  cudaFree(di); cudaFree(dg); cudaFree(du);
  if (e != cudaSuccess) return fail(SADMC_ERR_CUDA, cudaGetErrorString(e));
  return SADMC_OK;
}

int32_t sadmc_check_numerics(uint64_t n, uint64_t seed, uint64_t* mismatches, double* first) {
  if (!mismatches) return fail(SADMC_ERR_INVALID, "null argument");
  unsigned long long* d = nullptr;
  double* df = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(unsigned long long) * 5);
  if (e == cudaSuccess) e = cudaMalloc(&df, sizeof(double) * 2);
  if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(unsigned long long) * 5);
  if (e == cudaSuccess) e = cudaMemset(df, 0, sizeof(double) * 2);
  if (e == cudaSuccess) e = launch_numerics_check(n, seed, d, df, 0);
  if (e == cudaSuccess) e = cudaMemcpy(mismatches, d, sizeof(unsigned long long) * 5, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && first) e = cudaMemcpy(first, df, sizeof(double) * 2, cudaMemcpyDeviceToHost);
  cudaFree(d);
  cudaFree(df);
  if (e != cudaSuccess) return fail(SADMC_ERR_CUDA, cudaGetErrorString(e));
  return SADMC_OK;
}

int32_t sadmc_walker_heat_capacity(sadmc_handle* h, const double* T, int32_t nT, double* C) {
  if (!h || !T || !C || nT <= 0) return fail(SADMC_ERR_INVALID, "bad argument");
  if (!h->initialized) return fail(SADMC_ERR_STATE, "initialize first");
  double *dT = nullptr, *dC = nullptr;
  cudaError_t e = cudaMalloc(&dT, sizeof(double) * nT);
  if (e == cudaSuccess) e = cudaMalloc(&dC, sizeof(double) * (size_t)nT * h->W);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dT, T, sizeof(double) * nT, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = launch_walker_cv(h->d_cores, h->planes, h->nb, h->width, h->W, dT, nT, dC, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(C, dC, sizeof(double) * (size_t)nT * h->W, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(dT);
  cudaFree(dC);
  if (e != cudaSuccess) return fail(SADMC_ERR_CUDA, cudaGetErrorString(e));
  return SADMC_OK;
}

int32_t sadmc_heat_capacity(const double* T, int32_t nT, const double* E, const double* S,
                            int32_t n, double* C) {
  if (!T || !E || !S || !C || nT < 0 || n <= 0) return fail(SADMC_ERR_INVALID, "bad argument");
  double *dT = nullptr, *dE = nullptr, *dS = nullptr, *dC = nullptr;
  cudaError_t e = cudaMalloc(&dT, sizeof(double) * (nT + 1));
  if (e == cudaSuccess) e = cudaMalloc(&dE, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&dS, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&dC, sizeof(double) * (nT + 1));
  if (e == cudaSuccess) e = cudaMemcpy(dT, T, sizeof(double) * nT, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dE, E, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dS, S, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = launch_heat_capacity(dT, nT, dE, dS, n, dC, 0);
  if (e == cudaSuccess) e = cudaMemcpy(C, dC, sizeof(double) * nT, cudaMemcpyDeviceToHost);
  cudaFree(dT); cudaFree(dE); cudaFree(dS); cudaFree(dC);
  if (e != cudaSuccess) return fail(SADMC_ERR_CUDA, cudaGetErrorString(e));
  return SADMC_OK;
}


// ---- energy-number MC (grand-canonical LJ cluster) ------------------------------------

int32_t sadmc_grand_create(const sadmc_grand_config* c, sadmc_grand** out) {
  if (!c || !out) return fail(SADMC_ERR_INVALID, "null argument");
  if (c->n_walkers <= 0) return fail(SADMC_ERR_INVALID, "n_walkers must be positive");
  if (c->method != SADMC_SAMC && c->method != SADMC_WL)
    return fail(SADMC_ERR_INVALID, "the energy-number method supports SAMC and WL (energy_number.rs:18-27)");
  const bool wca = c->system == SADMC_WCA;
  if (!wca && c->system != SADMC_LJ) return fail(SADMC_ERR_INVALID, "grand-canonical systems: SADMC_LJ or SADMC_WCA");
  if (c->max_N < 1 || c->max_N > (wca ? 1024 : 63))
    return fail(SADMC_ERR_INVALID, "max_N (the cap on atoms) must be 1..63 (LJ) or 1..1024 (WCA)");
  if (!wca && !(c->radius > 0)) return fail(SADMC_ERR_INVALID, "radius must be positive");
  int ncell[3] = {0, 0, 0};
  if (wca)
    for (int a = 0; a < 3; ++a) {
      ncell[a] = (int)std::floor(c->box[a] / std::pow(2.0, 1.0 / 6.0));  // optcell.rs:64-66
      if (ncell[a] < 3) return fail(SADMC_ERR_INVALID, "box: fewer than 3 subcells per axis");
    }
  const double w = c->energy_bin > 0 ? c->energy_bin : 1.0;
  if (!(c->e_hi > 0.0 && c->e_lo < 0.0)) return fail(SADMC_ERR_INVALID, "need e_lo < 0 < e_hi (walkers start empty, E = 0)");
  if (!wca && c->lanes_per_walker != 0) {
    const int l = c->lanes_per_walker, np = c->max_N < 32 ? 32 : 64;
    if (!(l == 4 || l == 8 || l == 16 || l == 32) || np / l > 8)
      return fail(SADMC_ERR_INVALID, "lanes_per_walker: 32, 16, 8 or 4 (at least 8 when max_N >= 32)");
  }
  if (wca && c->lanes_per_walker != 0) {
    const int l = c->lanes_per_walker;
    if (!(l == 8 || l == 16 || l == 32))
      return fail(SADMC_ERR_INVALID, "lanes_per_walker of the WCA fluid: 32, 16 or 8");
  }
  auto* h = new sadmc_grand();
  h->cfg = *c;
  h->W = c->n_walkers;
  h->np = wca ? (c->max_N + 31) / 32 * 32 : (c->max_N < 32 ? 32 : 64);
  h->lanes = c->lanes_per_walker ? c->lanes_per_walker : (wca ? 32 : 8);
  h->ncol = c->max_N + 1;
  for (int a = 0; a < 3; ++a) h->nc[a] = ncell[a];
  h->cell_cap = ncell[0] * ncell[1] * ncell[2];
  const int below = (int)std::ceil(-c->e_lo / w) + 2, above = (int)std::ceil(c->e_hi / w) + 2;
  h->rows = below + above;
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  const size_t W = h->W, cells = (size_t)h->rows * h->ncol;
  if (e == cudaSuccess) e = cudaMalloc(&h->d_cores, sizeof(GrandCore) * W);
  if (e == cudaSuccess) e = cudaMalloc(&h->plane_mem, W * cells * 8 * 5 + W * h->ncol * 8 * 2);
  if (e == cudaSuccess) e = cudaMalloc(&h->d_pos, sizeof(float) * W * 6 * h->np);
  if (e == cudaSuccess && wca) {
    e = cudaMalloc(&h->d_pos64, sizeof(double) * W * 3 * h->np);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_pos32, sizeof(float) * W * 8 * h->np);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_cell_of, sizeof(int) * W * h->np);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_cnt, sizeof(int) * W * h->cell_cap);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_atoms, sizeof(int) * W * h->cell_cap * h->bucket);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->d_cnt, 0, sizeof(int) * W * h->cell_cap, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->d_pos64, 0, sizeof(double) * W * 3 * h->np, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->d_pos32, 0, sizeof(float) * W * 8 * h->np, h->stream);
  }
  if (e != cudaSuccess) { sadmc_grand_destroy(h); return fail(SADMC_ERR_NOMEM, cudaGetErrorString(e)); }
  char* b = (char*)h->plane_mem;
  h->planes.lnw = (double*)b;
  h->planes.hist = (uint64_t*)(b + 1 * W * cells * 8);
  h->planes.wl_hist = (uint64_t*)(b + 2 * W * cells * 8);
  h->planes.visit = (uint64_t*)(b + 3 * W * cells * 8);
  h->planes.round_trips = (uint64_t*)(b + 4 * W * cells * 8);
  h->planes.tr_att = (uint64_t*)(b + 5 * W * cells * 8);
  h->planes.tr_acc = h->planes.tr_att + W * h->ncol;
  e = cudaMemsetAsync(h->plane_mem, 0, W * cells * 8 * 5 + W * h->ncol * 8 * 2, h->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->d_pos, 0, sizeof(float) * W * 6 * h->np, h->stream);
  // from_params (energy_number.rs:474-533) on the empty GrandLjParams system
  std::vector<GrandCore> cores(W);
  for (size_t k = 0; k < W; ++k) {
    GrandCore& g = cores[k];
    g = GrandCore{};
    g.E = 0.0;
    g.addremove_prob = c->acceptance_rate_mode ? 0.5 : c->addremove_probability;
    g.min = 0.0 - w * 0.5;
    g.gamma = 1.0;
    g.num_states = 1;
    g.t_last = 1;
    g.lowest = 1;
    g.highest = 1;
    g.N = 0;
    g.max_N_ref = 0;
    g.num_E = 1;
    g.e_base = below;
    g.kind = c->method == SADMC_WL ? 2 : 1;
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h->d_cores, cores.data(), sizeof(GrandCore) * W, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = launch_grand_init(h->launch(), h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) { sadmc_grand_destroy(h); return fail(SADMC_ERR_CUDA, cudaGetErrorString(e)); }
  *out = h;
  return SADMC_OK;
}

int32_t sadmc_grand_destroy(sadmc_grand* h) {
  if (!h) return SADMC_OK;
  cudaFree(h->d_cores);
  cudaFree(h->plane_mem);
  cudaFree(h->d_pos);
  cudaFree(h->d_pos64);
  cudaFree(h->d_pos32);
  cudaFree(h->d_cell_of);
  cudaFree(h->d_cnt);
  cudaFree(h->d_atoms);
  cudaFree(h->d_trace);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return SADMC_OK;
}

int32_t sadmc_grand_set_trace(sadmc_grand* h, uint64_t capacity) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  cudaFree(h->d_trace);
  h->d_trace = nullptr;
  h->trace_cap = capacity;
  h->trace_t0 = h->moves_done;
  if (capacity) CUDA_TRY(cudaMalloc(&h->d_trace, sizeof(TraceRec) * capacity * h->W));
  return SADMC_OK;
}

int32_t sadmc_grand_run(sadmc_grand* h, uint64_t moves) {
  if (!h) return fail(SADMC_ERR_INVALID, "null handle");
  GrandLaunch m = h->launch();
  for (uint64_t left = moves; left > 0;) {
    m.n_moves = std::min<uint64_t>(left, 8192);
    CUDA_TRY(h->wca() ? launch_wca_grand_move(m, h->stream) : launch_grand_move(m, h->stream));
    left -= m.n_moves;
  }
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->moves_done += moves;
  return SADMC_OK;
}

int32_t sadmc_grand_read_trace(sadmc_grand* h, int32_t walker, double* e1, double* e2, uint64_t* n) {
  if (!h || walker < 0 || walker >= h->W || !n) return fail(SADMC_ERR_INVALID, "bad argument");
  if (!h->d_trace) return fail(SADMC_ERR_STATE, "tracing disabled");
  const uint64_t cnt = std::min<uint64_t>(h->trace_cap, h->moves_done - h->trace_t0);
  *n = cnt;
  if (!e1 && !e2) return SADMC_OK;
  std::vector<TraceRec> r(cnt);
  CUDA_TRY(cudaMemcpy(r.data(), h->d_trace + (size_t)walker * h->trace_cap, sizeof(TraceRec) * cnt, cudaMemcpyDeviceToHost));
  for (uint64_t k = 0; k < cnt; ++k) {
    if (e1) e1[k] = r[k].e1;
    if (e2) e2[k] = r[k].e2;
  }
  return SADMC_OK;
}

int32_t sadmc_grand_read_state(sadmc_grand* h, int32_t walker, double* pos, int32_t* n) {
  if (!h || walker < 0 || walker >= h->W || !n) return fail(SADMC_ERR_INVALID, "bad argument");
  GrandCore g;
  CUDA_TRY(cudaMemcpy(&g, h->d_cores + walker, sizeof(g), cudaMemcpyDeviceToHost));
  *n = g.N;
  if (pos && h->wca()) {
    std::vector<double> p(3 * (size_t)h->np);
    CUDA_TRY(cudaMemcpy(p.data(), h->d_pos64 + (size_t)walker * 3 * h->np, sizeof(double) * p.size(), cudaMemcpyDeviceToHost));
    for (int j = 0; j < g.N; ++j)
      for (int a = 0; a < 3; ++a) pos[3 * j + a] = p[(size_t)a * h->np + j];
  } else if (pos) {
    std::vector<float> p(6 * (size_t)h->np);
    CUDA_TRY(cudaMemcpy(p.data(), h->d_pos + (size_t)walker * 6 * h->np, sizeof(float) * p.size(), cudaMemcpyDeviceToHost));
    for (int j = 0; j < g.N; ++j)
      for (int a = 0; a < 3; ++a)
        pos[3 * j + a] = (double)p[(size_t)a * h->np + j] + (double)p[(size_t)(3 + a) * h->np + j];
  }
  return SADMC_OK;
}

int32_t sadmc_grand_read_scalars(sadmc_grand* h, int32_t walker, double* o) {
  if (!h || !o || walker < 0 || walker >= h->W) return fail(SADMC_ERR_INVALID, "bad argument");
  GrandCore g;
  CUDA_TRY(cudaMemcpy(&g, h->d_cores + walker, sizeof(g), cudaMemcpyDeviceToHost));
  const double w = h->cfg.energy_bin > 0 ? h->cfg.energy_bin : 1.0;
  const double v[SADMC_GRAND_N_SCALARS] = {
      (double)g.moves, (double)g.accepted, g.addremove_prob, (double)g.N, g.E,
      (double)g.num_states, (double)g.t_last, g.gamma, (double)g.lowest, (double)g.highest,
      (double)g.total, g.max_S, (double)g.max_S_index, g.min, w, (double)g.max_N_ref,
      (double)g.num_E, (double)g.ar_attempts, (double)g.ar_accepted, g.drift, (double)g.status};
  for (int k = 0; k < SADMC_GRAND_N_SCALARS; ++k) o[k] = v[k];
  return SADMC_OK;
}

int32_t sadmc_grand_read_bins(sadmc_grand* h, int32_t walker, double* lnw, uint64_t* hist,
                              uint64_t* wl_hist, uint8_t* visited, uint64_t* round_trips,
                              int64_t* n_e, int64_t* n_n) {
  if (!h || walker < 0 || walker >= h->W || !n_e || !n_n) return fail(SADMC_ERR_INVALID, "bad argument");
  GrandCore g;
  CUDA_TRY(cudaMemcpy(&g, h->d_cores + walker, sizeof(g), cudaMemcpyDeviceToHost));
  *n_e = g.num_E;
  *n_n = g.max_N_ref + 1;
  if (!lnw && !hist && !wl_hist && !visited && !round_trips) return SADMC_OK;
  const size_t cells = (size_t)h->rows * h->ncol, off = (size_t)walker * cells;
  std::vector<double> L(cells);
  std::vector<uint64_t> H(cells), WH(cells), V(cells), R(cells);
  CUDA_TRY(cudaMemcpy(L.data(), h->planes.lnw + off, cells * 8, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(H.data(), h->planes.hist + off, cells * 8, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(WH.data(), h->planes.wl_hist + off, cells * 8, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(V.data(), h->planes.visit + off, cells * 8, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(R.data(), h->planes.round_trips + off, cells * 8, cudaMemcpyDeviceToHost));
  const int nn = g.max_N_ref + 1;
  for (int k = 0; k < g.num_E; ++k)
    for (int q = 0; q < nn; ++q) {
      const size_t src = (size_t)(g.e_base + k) * h->ncol + q, dst = (size_t)k * nn + q;
      if (lnw) lnw[dst] = L[src];
      if (hist) hist[dst] = H[src];
      if (wl_hist) wl_hist[dst] = WH[src];
      if (visited) visited[dst] = (V[src] >> 1) == g.fill_gen ? (uint8_t)(V[src] & 1) : (uint8_t)(g.fill_val != 0);
      if (round_trips) round_trips[dst] = R[src];
    }
  return SADMC_OK;
}

int32_t sadmc_grand_translation_counts(sadmc_grand* h, int32_t walker, uint64_t* attempts,
                                       uint64_t* accepted) {
  if (!h || walker < 0 || walker >= h->W || !attempts || !accepted) return fail(SADMC_ERR_INVALID, "bad argument");
  GrandCore g;
  CUDA_TRY(cudaMemcpy(&g, h->d_cores + walker, sizeof(g), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(attempts, h->planes.tr_att + (size_t)walker * h->ncol, sizeof(uint64_t) * (g.max_N_ref + 1), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(accepted, h->planes.tr_acc + (size_t)walker * h->ncol, sizeof(uint64_t) * (g.max_N_ref + 1), cudaMemcpyDeviceToHost));
  return SADMC_OK;
}

}  // extern "C"

