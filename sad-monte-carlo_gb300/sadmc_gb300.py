"""Python binding of libsadmc_gb300.so (the C ABI in include/sadmc_gpu.h).

`Batch` is a batch of independent flat-histogram walkers on the GPU.  It mirrors the
reference's per-walker Rust surface (src/mc/mod.rs:37-144 MonteCarlo, src/mc/energy.rs
EnergyMC, src/system/mod.rs:54-120 System/MovableSystem) for many walkers at once:

    reference (one walker)                  this binding (a batch)
    EnergyMC::from_params(params, system)   Batch(cfg, geometry); upload(states); initialize()
    loop { mc.move_once() }                 run(moves)
    system().energy() / compute_energy()    energies() / compute_energies()
    system.plan_move(rng, d) / confirm()    plan_move(w, which, g, scale) / confirm(w)
    mc.bins (lnw, histogram, ...)           bins(w)
    num_moves / num_accepted_moves          counters()

There is no CPU fallback: every call runs the CUDA library, which must be built for this
machine (build.build()); a missing library raises RuntimeError.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libsadmc_gb300.so")

ISING, LJ, WCA, SW = 0, 1, 2, 3
SAD, SAMC, WL, INV_T_WL, CANONICAL = 0, 1, 2, 3, 4

ST_BIN_RANGE, ST_NAN_GAMMA, ST_DRIFT, ST_CELL_OVERFLOW = 1, 2, 4, 8
ST_TIMEOUT, ST_DESCENT_FAILED, ST_BAD_INPUT = 16, 32, 64

SCALARS = ["moves", "accepted", "acceptance_rate", "translation_scale", "method_kind",
           "too_lo", "too_hi", "tL", "tF", "num_states", "highest_hist",
           "latest_parameter", "gamma", "lowest_hist", "wl_highest_hist", "total_hist",
           "wl_num_states", "min_energy", "t0", "max_S", "max_S_index", "drift", "status",
           "energy"]


class Config(ctypes.Structure):
    _fields_ = [
        ("system", ctypes.c_int32), ("method", ctypes.c_int32), ("n_walkers", ctypes.c_int32),
        ("max_atoms", ctypes.c_int32), ("min_T", ctypes.c_double), ("t0", ctypes.c_double),
        ("has_min_gamma", ctypes.c_int32), ("pad0", ctypes.c_int32),
        ("min_gamma", ctypes.c_double), ("T", ctypes.c_double),
        ("has_energy_bin", ctypes.c_int32), ("pad1", ctypes.c_int32),
        ("energy_bin", ctypes.c_double),
        ("has_min_allowed", ctypes.c_int32), ("has_max_allowed", ctypes.c_int32),
        ("min_allowed", ctypes.c_double), ("max_allowed", ctypes.c_double),
        ("e_lo", ctypes.c_double), ("e_hi", ctypes.c_double),
        ("acceptance_rate_mode", ctypes.c_int32), ("pad2", ctypes.c_int32),
        ("target_rate", ctypes.c_double), ("translation_scale", ctypes.c_double),
        ("well_width", ctypes.c_double), ("seed", ctypes.c_uint64),
        ("descent_limit", ctypes.c_uint64), ("lanes_per_walker", ctypes.c_int32),
        ("resum_interval", ctypes.c_int32), ("drift_tol", ctypes.c_double),
    ]


class Geometry(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("pad", ctypes.c_int32), ("radius", ctypes.c_double),
                ("box", ctypes.c_double * 3)]


class Online(ctypes.Structure):
    """sadmc_online: the online training schedule of run_online."""
    _fields_ = [("collect_interval", ctypes.c_uint64), ("retrain_interval", ctypes.c_uint64),
                ("train_steps", ctypes.c_int32), ("batch", ctypes.c_int32),
                ("lr", ctypes.c_float), ("pad", ctypes.c_int32), ("seed", ctypes.c_uint64)]


class Proposal(ctypes.Structure):
    _fields_ = [("which", ctypes.c_int32), ("j", ctypes.c_int32), ("g", ctypes.c_double * 3),
                ("scale", ctypes.c_double)]


_lib = None


def lib():
    """Load the CUDA library (raises if it was not built for this machine)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run build.build() (needs nvcc) first")
    L = ctypes.CDLL(LIB_PATH)
    P, I32, U64, D = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint64, ctypes.c_double
    sig = {
        "sadmc_version": (I32, []), "sadmc_last_error": (ctypes.c_char_p, []),
        "sadmc_create": (I32, [P, P, P]), "sadmc_destroy": (I32, [P]),
        "sadmc_upload_state": (I32, [P, I32, I32, P]),
        "sadmc_read_state": (I32, [P, I32, I32, P]),
        "sadmc_initialize": (I32, [P]),
        "sadmc_run": (I32, [P, U64]), "sadmc_run_async": (I32, [P, U64, P]),
        "sadmc_synchronize": (I32, [P]),
        "sadmc_energy": (I32, [P, P]), "sadmc_compute_energy": (I32, [P, P]),
        "sadmc_plan_move_injected": (I32, [P, I32, P, P, P]),
        "sadmc_confirm": (I32, [P, I32]),
        "sadmc_nbins": (I32, [P, I32, P, P, P]),
        "sadmc_read_bins": (I32, [P, I32, P, P, P, P, P, P, P]),
        "sadmc_read_wl_hist": (I32, [P, I32, P, P, P]),
        "sadmc_read_extra": (I32, [P, I32, P, P]),
        "sadmc_plane_bins": (I32, [P, P]), "sadmc_read_planes": (I32, [P, P, P, P, P]),
        "sadmc_read_scalars": (I32, [P, I32, P]),
        "sadmc_counters": (I32, [P, P, P]), "sadmc_status": (I32, [P, P]),
        "sadmc_set_trace": (I32, [P, U64]), "sadmc_read_trace": (I32, [P, I32, P, P, P]),
        "sadmc_read_trace_ds": (I32, [P, I32, P, P]),
        "sadmc_lanes_per_walker": (I32, [P]), "sadmc_autotune": (I32, [P, U64, P, P]),
        "sadmc_heat_capacity": (I32, [P, I32, P, P, I32, P]),
        "sadmc_checkpoint": (I32, [P, ctypes.c_char_p]),
        "sadmc_resume": (I32, [ctypes.c_char_p, P]),
        "sadmc_get_config": (I32, [P, P, P]),
        "sadmc_surrogate_init": (I32, [P, U64, I32]),
        "sadmc_surrogate_get_params": (I32, [P, P]),
        "sadmc_surrogate_set_params": (I32, [P, P]),
        "sadmc_surrogate_collect": (I32, [P, P]),
        "sadmc_surrogate_train": (I32, [P, I32, I32, ctypes.c_float, U64, P]),
        "sadmc_surrogate_loss_grads": (I32, [P, P, P, I32, P, P]),
        "sadmc_surrogate_loss_grads_noalloc": (I32, [P, P, P, I32, P, P, P]),
        "sadmc_check_numerics": (I32, [U64, U64, P, P]),
        "sadmc_grand_create": (I32, [P, P]), "sadmc_grand_destroy": (I32, [P]),
        "sadmc_grand_run": (I32, [P, U64]), "sadmc_grand_set_trace": (I32, [P, U64]),
        "sadmc_grand_read_trace": (I32, [P, I32, P, P, P]),
        "sadmc_grand_read_state": (I32, [P, I32, P, P]),
        "sadmc_grand_read_scalars": (I32, [P, I32, P]),
        "sadmc_grand_read_bins": (I32, [P, I32, P, P, P, P, P, P, P]),
        "sadmc_grand_translation_counts": (I32, [P, I32, P, P]),
        "sadmc_surrogate_predict": (I32, [P, P, I32, P]),
        "sadmc_run_da": (I32, [P, U64, I32, P]),
        "sadmc_run_online": (I32, [P, U64, I32, I32, P, P]),
        "sadmc_walker_heat_capacity": (I32, [P, P, I32, P]),
        "sadmc_draws": (I32, [I32, ctypes.c_uint32, U64, ctypes.c_uint32, U64, I32, ctypes.c_uint32,
                              P, P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    _lib = L
    return L


class SadmcError(RuntimeError):
    pass


def _check(rc):
    if rc != 0:
        raise SadmcError(f"sadmc error {rc}: {lib().sadmc_last_error().decode()}")


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def make_config(system, n_walkers, max_atoms, *, method=SAD, min_T=0.2, t0=1e4, min_gamma=None,
                T=1.0, energy_bin=None, min_allowed=None, max_allowed=None, e_lo, e_hi,
                target_rate=None, translation_scale=0.05, well_width=1.3, seed=0,
                descent_limit=0, lanes_per_walker=0, resum_interval=0, drift_tol=0.0):
    c = Config()
    c.system, c.method, c.n_walkers, c.max_atoms = system, method, n_walkers, max_atoms
    c.min_T, c.t0 = min_T, t0
    c.has_min_gamma, c.min_gamma = int(min_gamma is not None), min_gamma or 0.0
    c.T = T
    c.has_energy_bin, c.energy_bin = int(energy_bin is not None), energy_bin or 0.0
    c.has_min_allowed = int(min_allowed is not None)
    c.min_allowed = 0.0 if min_allowed is None else min_allowed
    c.has_max_allowed = int(max_allowed is not None)
    c.max_allowed = 0.0 if max_allowed is None else max_allowed
    c.e_lo, c.e_hi = e_lo, e_hi
    c.acceptance_rate_mode = int(target_rate is not None)
    c.target_rate = target_rate or 0.5
    c.translation_scale, c.well_width, c.seed = translation_scale, well_width, seed
    c.descent_limit, c.lanes_per_walker = descent_limit, lanes_per_walker
    c.resum_interval, c.drift_tol = resum_interval, drift_tol
    return c


class Batch:
    """A batch of GPU walkers (one sadmc_handle)."""

    def __init__(self, cfg, geometry):
        """geometry: list of (n, radius, (Lx, Ly, Lz)) per walker."""
        self.cfg = cfg
        W = cfg.n_walkers
        if len(geometry) != W:
            raise ValueError("one geometry entry per walker")
        self._geom = (Geometry * W)()
        for w, (n, radius, box) in enumerate(geometry):
            self._geom[w].n, self._geom[w].radius = n, radius
            for a in range(3):
                self._geom[w].box[a] = box[a]
        self.n = np.array([g[0] for g in geometry])
        self.h = ctypes.c_void_p()
        _check(lib().sadmc_create(ctypes.byref(cfg), self._geom, ctypes.byref(self.h)))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().sadmc_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def W(self):
        return self.cfg.n_walkers

    def upload(self, states, begin=0, count=None):
        """states: a list of per-walker arrays, or one packed float64 array for `count`
        walkers (positions x,y,z walker after walker; Ising spins L*L per walker)."""
        if isinstance(states, np.ndarray) and states.ndim == 1:
            flat = np.ascontiguousarray(states, np.float64)
            count = self.W - begin if count is None else count
        else:
            flat = np.ascontiguousarray(np.concatenate([np.ravel(s) for s in states]), np.float64)
            count = len(states)
        _check(lib().sadmc_upload_state(self.h, begin, count, _p(flat)))

    def state(self, w):
        n = int(self.n[w])
        size = n * n if self.cfg.system == ISING else 3 * n
        out = np.zeros(size)
        _check(lib().sadmc_read_state(self.h, w, 1, _p(out)))
        return out if self.cfg.system == ISING else out.reshape(-1, 3)

    def initialize(self):
        _check(lib().sadmc_initialize(self.h))

    def run(self, moves):
        _check(lib().sadmc_run(self.h, int(moves)))

    def run_async(self, moves, stream=None):
        _check(lib().sadmc_run_async(self.h, int(moves), stream))

    def synchronize(self):
        _check(lib().sadmc_synchronize(self.h))

    def energies(self):
        out = np.zeros(self.W)
        _check(lib().sadmc_energy(self.h, _p(out)))
        return out

    def compute_energies(self):
        out = np.zeros(self.W)
        _check(lib().sadmc_compute_energy(self.h, _p(out)))
        return out

    def plan_move(self, w, which, g=(0.0, 0.0, 0.0), scale=0.05, j=0):
        p = Proposal()
        p.which, p.j, p.scale = which, j, scale
        for a in range(3):
            p.g[a] = g[a]
        e = ctypes.c_double(0.0)
        ok = ctypes.c_int32(0)
        _check(lib().sadmc_plan_move_injected(self.h, w, ctypes.byref(p), ctypes.byref(e),
                                              ctypes.byref(ok)))
        return e.value if ok.value else None

    def confirm(self, w):
        _check(lib().sadmc_confirm(self.h, w))

    def bins(self, w):
        n, mn, wd = ctypes.c_int64(0), ctypes.c_double(0), ctypes.c_double(0)
        _check(lib().sadmc_nbins(self.h, w, ctypes.byref(n), ctypes.byref(mn), ctypes.byref(wd)))
        n = n.value
        lnw, sE, sE2 = np.zeros(n), np.zeros(n), np.zeros(n)
        hist, tf, rt = (np.zeros(n, np.uint64) for _ in range(3))
        vis = np.zeros(n, np.uint8)
        _check(lib().sadmc_read_bins(self.h, w, _p(lnw), _p(hist), _p(tf), _p(sE), _p(sE2),
                                     _p(rt), _p(vis)))
        return dict(lnw=lnw, hist=hist, t_found=tf, sumE=sE, sumE2=sE2, round_trips=rt,
                    visited=vis, min=mn.value, width=wd.value)

    def plane_bins(self):
        n = ctypes.c_int64(0)
        _check(lib().sadmc_plane_bins(self.h, ctypes.byref(n)))
        return n.value

    def read_planes(self, lnw=None, hist=None):
        """Copy the whole ln w / histogram planes into (optionally pinned) host arrays."""
        nb = self.plane_bins()
        if lnw is None:
            lnw = np.zeros(self.W * nb)
        if hist is None:
            hist = np.zeros(self.W * nb, np.uint64)
        rng = np.zeros(2 * self.W, np.int32)
        mins = np.zeros(self.W)
        _check(lib().sadmc_read_planes(self.h, _p(lnw), _p(hist), _p(rng), _p(mins)))
        return lnw, hist, rng.reshape(-1, 2), mins

    def wl_hist(self, w):
        n, me = ctypes.c_int64(0), ctypes.c_double(0)
        _check(lib().sadmc_read_wl_hist(self.h, w, None, ctypes.byref(n), ctypes.byref(me)))
        out = np.zeros(max(n.value, 1), np.uint64)
        _check(lib().sadmc_read_wl_hist(self.h, w, _p(out), ctypes.byref(n), ctypes.byref(me)))
        return out[:n.value], me.value

    def extra(self, w):
        """The WCA "pressure" BinCounts of walker w: (count, total) over its bins."""
        n = len(self.bins(w)["lnw"])
        c, t = np.zeros(n, np.uint64), np.zeros(n)
        _check(lib().sadmc_read_extra(self.h, w, _p(c), _p(t)))
        return c, t

    def scalars(self, w):
        o = np.zeros(len(SCALARS))
        _check(lib().sadmc_read_scalars(self.h, w, _p(o)))
        return dict(zip(SCALARS, o))

    def counters(self):
        m, a = ctypes.c_uint64(0), ctypes.c_uint64(0)
        _check(lib().sadmc_counters(self.h, ctypes.byref(m), ctypes.byref(a)))
        return m.value, a.value

    def status(self):
        out = np.zeros(self.W, np.uint32)
        _check(lib().sadmc_status(self.h, _p(out)))
        return out

    def set_trace(self, capacity):
        _check(lib().sadmc_set_trace(self.h, int(capacity)))

    def trace(self, w, capacity):
        e1, e2 = np.zeros(capacity), np.zeros(capacity)
        cnt = ctypes.c_uint64(0)
        _check(lib().sadmc_read_trace(self.h, w, _p(e1), _p(e2), ctypes.byref(cnt)))
        return e1[:cnt.value], e2[:cnt.value]

    def trace_ds(self, w, capacity):
        """dS of each traced delayed-acceptance move of walker w (0 for plain moves)."""
        ds = np.zeros(capacity, np.float32)
        cnt = ctypes.c_uint64(0)
        _check(lib().sadmc_read_trace_ds(self.h, w, _p(ds), ctypes.byref(cnt)))
        return ds[:cnt.value]

    def checkpoint(self, path):
        """Atomic binary checkpoint of the whole batch (write to path.tmp, rename)."""
        _check(lib().sadmc_checkpoint(self.h, os.fsencode(path)))

    @classmethod
    def resume(cls, path):
        """A batch restored from a checkpoint; its runs continue bit for bit."""
        b = cls.__new__(cls)
        b.h = ctypes.c_void_p()
        _check(lib().sadmc_resume(os.fsencode(path), ctypes.byref(b.h)))
        b.cfg = Config()
        _check(lib().sadmc_get_config(b.h, ctypes.byref(b.cfg), None))
        b._geom = (Geometry * b.cfg.n_walkers)()
        _check(lib().sadmc_get_config(b.h, None, b._geom))
        b.n = np.array([g.n for g in b._geom])
        return b

    # ---- learned surrogate (LJ) -------------------------------------------------------
    SG_NPARAM = 6337

    def surrogate_init(self, seed=0, ring_capacity=100000):
        _check(lib().sadmc_surrogate_init(self.h, seed, ring_capacity))

    def surrogate_params(self):
        out = np.zeros(self.SG_NPARAM, np.float32)
        _check(lib().sadmc_surrogate_get_params(self.h, _p(out)))
        return out

    def surrogate_set_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        _check(lib().sadmc_surrogate_set_params(self.h, _p(p)))

    def surrogate_collect(self):
        n = ctypes.c_int32(0)
        _check(lib().sadmc_surrogate_collect(self.h, ctypes.byref(n)))
        return n.value

    def surrogate_train(self, steps, batch=256, lr=1e-3, seed=0):
        loss = ctypes.c_double(0)
        _check(lib().sadmc_surrogate_train(self.h, steps, batch, lr, seed, ctypes.byref(loss)))
        return loss.value

    def surrogate_loss_grads(self, pos, target):
        pos = np.ascontiguousarray(pos, np.float32)
        target = np.ascontiguousarray(target, np.float32)
        g = np.zeros(self.SG_NPARAM, np.float32)
        loss = ctypes.c_double(0)
        _check(lib().sadmc_surrogate_loss_grads(self.h, _p(pos), _p(target), len(target),
                                                ctypes.byref(loss), _p(g)))
        return loss.value, g

    def surrogate_loss_grads_noalloc(self, pos_ptr, target_ptr, configs, loss_ptr, grads_ptr,
                                     stream_ptr=None):
        """sadmc_surrogate_loss_grads_noalloc on device pointers (ints): stream-ordered,
        allocates nothing, returns without synchronising."""
        _check(lib().sadmc_surrogate_loss_grads_noalloc(
            self.h, ctypes.c_void_p(pos_ptr), ctypes.c_void_p(target_ptr), int(configs),
            ctypes.c_void_p(loss_ptr), ctypes.c_void_p(grads_ptr),
            ctypes.c_void_p(stream_ptr) if stream_ptr else None))

    def run_da(self, moves, refresh_interval=2048):
        """Delayed-acceptance moves; returns per-walker (stage-1 rejections, exact evaluations)."""
        st = np.zeros(2 * self.W, np.uint64)
        _check(lib().sadmc_run_da(self.h, int(moves), refresh_interval, _p(st)))
        return st.reshape(-1, 2)

    def run_online(self, moves, delayed, collect_interval=0, retrain_interval=0, train_steps=0,
                   batch=256, lr=1e-3, seed=0, refresh_interval=2048):
        """Plain (delayed=False) or delayed-acceptance moves while the surrogate trains
        online on the device (sadmc_run_online); returns the delayed-acceptance counters
        (stage-1 rejections, exact evaluations) per walker, or None for plain moves."""
        o = Online(int(collect_interval), int(retrain_interval), int(train_steps), int(batch),
                   float(lr), 0, int(seed))
        st = np.zeros(2 * self.W, np.uint64)
        _check(lib().sadmc_run_online(self.h, int(moves), int(bool(delayed)), int(refresh_interval),
                                      ctypes.byref(o), _p(st)))
        return st.reshape(-1, 2) if delayed else None

    def surrogate_predict(self, pos):
        pos = np.ascontiguousarray(pos, np.float32)
        out = np.zeros(pos.shape[0], np.float32)
        _check(lib().sadmc_surrogate_predict(self.h, _p(pos), pos.shape[0], _p(out)))
        return out

    def heat_capacities(self, T):
        """Per-walker heat capacity C[w, t] from each walker's own bins, FP64 on the device
        (sadmc_walker_heat_capacity)."""
        T = np.ascontiguousarray(T, np.float64)
        out = np.zeros((self.W, len(T)))
        _check(lib().sadmc_walker_heat_capacity(self.h, _p(T), len(T), _p(out)))
        return out

    def lanes_per_walker(self):
        return lib().sadmc_lanes_per_walker(self.h)

    def autotune(self, moves=2048):
        lpw, ms = ctypes.c_int32(0), ctypes.c_double(0)
        _check(lib().sadmc_autotune(self.h, int(moves), ctypes.byref(lpw), ctypes.byref(ms)))
        return lpw.value, ms.value


def unpack_params(flat):
    """Flat surrogate parameters -> dict (W1 [32,64], b1, W2 [64,64], b2, w3, b3)."""
    f = np.asarray(flat, np.float64)
    o = 0
    out = {}
    for name, shape in [("W1", (32, 64)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)),
                        ("w3", (64,)), ("b3", (1,))]:
        size = int(np.prod(shape))
        out[name] = f[o:o + size].reshape(shape)
        o += size
    return out


def pack_params(d):
    return np.concatenate([np.ravel(d[k]) for k in ("W1", "b1", "W2", "b2", "w3", "b3")]).astype(np.float32)


def draws(system, n, seed, walker, t0, count, stream_pair=0):
    """The device-side per-move draws (diagnostic): (idx [count,2], g [count,3], u [count])."""
    idx = np.zeros(2 * count, np.uint32)
    g = np.zeros(3 * count, np.float32)
    u = np.zeros(count)
    _check(lib().sadmc_draws(system, n, seed, walker, t0, count, stream_pair, _p(idx), _p(g), _p(u)))
    return idx.reshape(-1, 2), g.reshape(-1, 3), u


def heat_capacity(T, E, S):
    """C(T) on the GPU in FP64 (plotting/final_heat_capacity.py:79-88)."""
    T = np.ascontiguousarray(T, np.float64)
    E = np.ascontiguousarray(E, np.float64)
    S = np.ascontiguousarray(S, np.float64)
    C = np.zeros(len(T))
    _check(lib().sadmc_heat_capacity(_p(T), len(T), _p(E), _p(S), len(E), _p(C)))
    return C


class GrandConfig(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int32), ("n_walkers", ctypes.c_int32),
                ("max_N", ctypes.c_int32), ("acceptance_rate_mode", ctypes.c_int32),
                ("t0", ctypes.c_double), ("energy_bin", ctypes.c_double),
                ("radius", ctypes.c_double),
                ("has_min_allowed", ctypes.c_int32), ("has_max_allowed", ctypes.c_int32),
                ("min_allowed", ctypes.c_double), ("max_allowed", ctypes.c_double),
                ("target_rate", ctypes.c_double), ("translation_scale", ctypes.c_double),
                ("addremove_probability", ctypes.c_double),
                ("e_lo", ctypes.c_double), ("e_hi", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("resum_interval", ctypes.c_int32),
                ("system", ctypes.c_int32), ("drift_tol", ctypes.c_double),
                ("box", ctypes.c_double * 3), ("lanes_per_walker", ctypes.c_int32)]


GRAND_SCALARS = ["moves", "accepted", "addremove_probability", "N", "energy", "num_states",
                 "t_last", "gamma", "lowest_hist", "highest_hist", "total_hist", "max_S",
                 "max_S_index", "min", "width", "max_N", "num_E", "addremove_attempts",
                 "addremove_accepted", "drift", "status"]


def make_grand_config(n_walkers, max_N, radius=0.0, *, box=None, method=SAMC, t0=1e4,
                      energy_bin=1.0, min_allowed=None, max_allowed=None, target_rate=None,
                      translation_scale=0.05, addremove_probability=0.05, e_lo=-200.0,
                      e_hi=50.0, seed=0, resum_interval=0, drift_tol=0.0, lanes_per_walker=0):
    """Energy-number walkers: the LJ cluster of `radius`, or (box given) the WCA fluid.
    lanes_per_walker: lanes per walker (LJ: 32, 16, 8, 4, 0 = 8; WCA: 32, 16, 8, 0 = 32)."""
    c = GrandConfig()
    c.system = WCA if box is not None else LJ
    if box is not None:
        c.box[0], c.box[1], c.box[2] = box
    c.method, c.n_walkers, c.max_N = method, n_walkers, max_N
    c.acceptance_rate_mode, c.target_rate = int(target_rate is not None), target_rate or 0.5
    c.t0, c.energy_bin, c.radius = t0, energy_bin, radius
    c.has_min_allowed, c.min_allowed = int(min_allowed is not None), min_allowed or 0.0
    c.has_max_allowed = int(max_allowed is not None)
    c.max_allowed = max_allowed if max_allowed is not None else 0.0
    c.translation_scale, c.addremove_probability = translation_scale, addremove_probability
    c.e_lo, c.e_hi, c.seed = e_lo, e_hi, seed
    c.resum_interval, c.drift_tol = resum_interval, drift_tol
    c.lanes_per_walker = lanes_per_walker
    return c


class GrandBatch:
    """Energy-number walkers of a grand-canonical LJ cluster (one sadmc_grand handle)."""

    def __init__(self, cfg):
        self.cfg = cfg
        self.h = ctypes.c_void_p()
        _check(lib().sadmc_grand_create(ctypes.byref(cfg), ctypes.byref(self.h)))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().sadmc_grand_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, moves):
        _check(lib().sadmc_grand_run(self.h, int(moves)))

    def set_trace(self, capacity):
        _check(lib().sadmc_grand_set_trace(self.h, int(capacity)))

    def trace(self, w, n):
        e1, e2 = np.zeros(n), np.zeros(n)
        cnt = ctypes.c_uint64(0)
        _check(lib().sadmc_grand_read_trace(self.h, w, _p(e1), _p(e2), ctypes.byref(cnt)))
        return e1[:cnt.value], e2[:cnt.value]

    def state(self, w):
        n = ctypes.c_int32(0)
        out = np.zeros((max(64, int(self.cfg.max_N)), 3))
        _check(lib().sadmc_grand_read_state(self.h, w, _p(out), ctypes.byref(n)))
        return out[:n.value]

    def scalars(self, w):
        o = np.zeros(len(GRAND_SCALARS))
        _check(lib().sadmc_grand_read_scalars(self.h, w, _p(o)))
        return dict(zip(GRAND_SCALARS, o))

    def bins(self, w):
        ne, nn = ctypes.c_int64(0), ctypes.c_int64(0)
        _check(lib().sadmc_grand_read_bins(self.h, w, None, None, None, None, None,
                                          ctypes.byref(ne), ctypes.byref(nn)))
        n = ne.value * nn.value
        lnw = np.zeros(n)
        hist, wlh, rt = (np.zeros(n, np.uint64) for _ in range(3))
        vis = np.zeros(n, np.uint8)
        _check(lib().sadmc_grand_read_bins(self.h, w, _p(lnw), _p(hist), _p(wlh), _p(vis), _p(rt),
                                          ctypes.byref(ne), ctypes.byref(nn)))
        shape = (ne.value, nn.value)
        return dict(lnw=lnw.reshape(shape), hist=hist.reshape(shape), wl_hist=wlh.reshape(shape),
                    visited=vis.reshape(shape), round_trips=rt.reshape(shape))

    def translation_counts(self, w):
        nn = int(self.scalars(w)["max_N"]) + 1
        a, b = np.zeros(nn, np.uint64), np.zeros(nn, np.uint64)
        _check(lib().sadmc_grand_translation_counts(self.h, w, _p(a), _p(b)))
        return a, b


def check_numerics(n, seed=1):
    """Mismatch counts of the exact FP64 rewrites against CUDA's own operations (see
    sadmc_check_numerics) and the first mismatching division (a, b)."""
    out = np.zeros(5, np.uint64)
    first = np.zeros(2)
    _check(lib().sadmc_check_numerics(int(n), int(seed), _p(out), _p(first)))
    return out, first


def cv_from_bins(bins, T):
    """Heat capacity from a walker's visited bins (centres as E, lnw as S)."""
    m = bins["hist"] > 0
    E = bins["min"] + (np.nonzero(m)[0] + 0.5) * bins["width"]
    return heat_capacity(T, E, bins["lnw"][m])
