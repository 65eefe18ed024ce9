"""ctypes binding of the FP64 oracle (test infrastructure only).

The oracle is a C++ restatement of the reference's flat-histogram driver
(src/mc/energy.rs) and systems (src/system/{ising,lj,wca,optcell,optsquare}.rs).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module; the CUDA product never calls it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle_sadmc.so")

ISING, LJ, WCA, SW = 0, 1, 2, 3
M_SAD, M_SAMC, M_WL, M_INV_T_WL, M_CANONICAL = 0, 1, 2, 3, 4

SCALARS = ["moves", "accepted", "acceptance_rate", "translation_scale", "method_kind",
           "too_lo", "too_hi", "tL", "tF", "num_states", "highest_hist",
           "latest_parameter", "gamma", "lowest_hist", "wl_highest_hist", "total_hist",
           "wl_num_states", "min_energy", "t0", "max_S", "max_S_index",
           "verify_failures", "nan_gamma", "energy"]


class Config(ctypes.Structure):
    _fields_ = [
        ("system", ctypes.c_int32), ("n", ctypes.c_int32), ("radius", ctypes.c_double),
        ("box", ctypes.c_double * 3), ("well_width", ctypes.c_double),
        ("method", ctypes.c_int32), ("min_T", ctypes.c_double), ("t0", ctypes.c_double),
        ("has_min_gamma", ctypes.c_int32), ("min_gamma", ctypes.c_double),
        ("T", ctypes.c_double), ("seed", ctypes.c_uint64), ("walker", ctypes.c_uint32),
        ("has_energy_bin", ctypes.c_int32), ("energy_bin", ctypes.c_double),
        ("has_min_allowed", ctypes.c_int32), ("has_max_allowed", ctypes.c_int32),
        ("min_allowed", ctypes.c_double), ("max_allowed", ctypes.c_double),
        ("acceptance_rate_mode", ctypes.c_int32), ("target_rate", ctypes.c_double),
        ("translation_scale", ctypes.c_double), ("descent_limit", ctypes.c_uint64),
        ("has_e0", ctypes.c_int32), ("e0", ctypes.c_double),
    ]


def build():
    """Compile the oracle with its Makefile (g++, no GPU needed)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


_libs = {}
# the timed CPU baseline: the same sources built for the host's own cores (oracle/Makefile)
NATIVE_FLAGS = "g++ -O3 -ffp-contract=off -mcpu=native (Arm) / -march=native (x86)"


def lib(native=False):
    """The oracle library; native=True loads the host-tuned build of the same sources,
    which the CPU baseline times (its results are the checker's)."""
    key = bool(native)
    if key not in _libs:
        path = _LIB_PATH.replace(".so", "_native.so") if native else _LIB_PATH
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        P, D, U64, I32, U32, I64 = (ctypes.c_void_p, ctypes.c_double, ctypes.c_uint64,
                                    ctypes.c_int32, ctypes.c_uint32, ctypes.c_int64)
        sig = {
            "orc_create": (P, [ctypes.POINTER(Config), P]),
            "orc_destroy": (None, [P]),
            "orc_run": (None, [P, U64]),
            "orc_run_override": (D, [P, U64, P, P, P]),
            "orc_run_override_da": (D, [P, U64, P, P, P, P]),
            "orc_energy": (D, [P]), "orc_compute_energy": (D, [P]),
            "orc_override_worst": (None, [P, P]),
            "orc_extra": (I64, [P, P, P]),
            "orc_grand_create": (P, [P]), "orc_grand_destroy": (None, [P]),
            "orc_grand_run": (None, [P, U64]),
            "orc_grand_run_override": (D, [P, U64, P, P, P]),
            "orc_grand_worst": (None, [P, P]), "orc_grand_state": (I64, [P, P]),
            "orc_grand_compute_energy": (D, [P]), "orc_grand_scalars": (None, [P, P]),
            "orc_grand_bins": (I64, [P, P, P, P, P, P]),
            "orc_grand_translation": (None, [P, P, P]),
            "orc_grand_check_cells": (I64, [P]),
            "orc_grand_draws": (None, [U64, ctypes.c_uint32, U64, P, P, P, P]),
            "orc_verify_energy": (ctypes.c_int, [P]),
            "orc_get_state": (None, [P, P]),
            "orc_plan_move": (ctypes.c_int, [P, U32, U32, D, D, D, D, P]),
            "orc_confirm": (None, [P]),
            "orc_nbins": (I64, [P]),
            "orc_get_bins": (None, [P, P, P, P, P, P, P, P, P]),
            "orc_wl_hist": (I64, [P, P, P]),
            "orc_get_scalars": (None, [P, P]),
            "orc_temperature": (D, [P, D]),
            "orc_pressure": (D, [P]),
            "orc_philox": (None, [P, P, P]),
            "orc_draws": (None, [I32, U32, U64, U32, U64, U32, P, P, P]),
            "orc_normal_pairs": (None, [P, P, ctypes.c_size_t, P, P]),
            "orc_heat_capacity": (None, [P, ctypes.c_size_t, P, P, ctypes.c_size_t, P]),
            "orc_max_balls_within": (U64, [D]),
            "orc_lj_potential": (D, [D]), "orc_wca_potential": (D, [D]),
            "orc_selftest_ising": (I64, [I32, U64, U64]),
            "orc_init_lj": (ctypes.c_int, [I32, D, U64, P]),
            "orc_init_sw_fcc": (ctypes.c_int, [I32, D, D, U64, P, P]),
            "orc_selftest_moves": (I64, [P, U64, D, D, U64]),
            "orc_selftest_cell": (I64, [P]),
            "orc_bench": (D, [P, P, I32, U64, I32, P, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _libs[key] = L
    return _libs[key]


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def make_config(system, n, *, radius=0.0, box=(0.0, 0.0, 0.0), well_width=1.3,
                method=M_SAD, min_T=0.2, t0=1e4, min_gamma=None, T=1.0, seed=0, walker=0,
                energy_bin=None, min_allowed=None, max_allowed=None,
                target_rate=None, translation_scale=0.05, descent_limit=0, e0=None):
    c = Config()
    c.system, c.n, c.radius = system, n, radius
    c.box[0], c.box[1], c.box[2] = box
    c.well_width = well_width
    c.method, c.min_T, c.t0 = method, min_T, t0
    c.has_min_gamma = int(min_gamma is not None)
    c.min_gamma = min_gamma or 0.0
    c.T, c.seed, c.walker = T, seed, walker
    c.has_energy_bin = int(energy_bin is not None)
    c.energy_bin = energy_bin or 0.0
    c.has_min_allowed = int(min_allowed is not None)
    c.min_allowed = min_allowed if min_allowed is not None else 0.0
    c.has_max_allowed = int(max_allowed is not None)
    c.max_allowed = max_allowed if max_allowed is not None else 0.0
    c.acceptance_rate_mode = int(target_rate is not None)
    c.target_rate = target_rate or 0.5
    c.translation_scale = translation_scale
    c.descent_limit = descent_limit
    c.has_e0 = int(e0 is not None)
    c.e0 = e0 if e0 is not None else 0.0
    return c


class Walker:
    """One oracle EnergyMC walker."""

    def __init__(self, cfg, state):
        self.cfg = cfg
        self._state = np.ascontiguousarray(state, dtype=np.float64)
        self.h = lib().orc_create(ctypes.byref(cfg), _p(self._state))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def run(self, n):
        lib().orc_run(self.h, int(n))

    def run_override(self, e1, e2):
        """Replay a GPU trace; returns (max |e2 - own e2|, possibility mismatches)."""
        e1 = np.ascontiguousarray(e1, dtype=np.float64)
        e2 = np.ascontiguousarray(e2, dtype=np.float64)
        mm = ctypes.c_uint64(0)
        d = lib().orc_run_override(self.h, len(e2), _p(e1), _p(e2), ctypes.byref(mm))
        return d, mm.value

    def run_override_da(self, e1, e2, ds):
        """Replay a traced delayed-acceptance run (e2 NaN where the first stage screened the
        move out, ds the GPU surrogate's change); returns (max |e2 - own e2|, mismatches)."""
        e1 = np.ascontiguousarray(e1, dtype=np.float64)
        e2 = np.ascontiguousarray(e2, dtype=np.float64)
        ds = np.ascontiguousarray(ds, dtype=np.float32)
        mm = ctypes.c_uint64(0)
        d = lib().orc_run_override_da(self.h, len(e2), _p(e1), _p(e2), _p(ds), ctypes.byref(mm))
        return d, mm.value

    def extra(self):
        """The WCA pressure BinCounts: (count, total) per bin (empty arrays if none)."""
        n = lib().orc_extra(self.h, None, None)
        c = np.zeros(max(n, 1), np.uint64)
        t = np.zeros(max(n, 1))
        lib().orc_extra(self.h, _p(c), _p(t))
        return c[:n], t[:n]

    def override_worst(self):
        """(move, e2 given, e2 own, gross pair-term magnitude) of the largest replay gap."""
        o = np.zeros(4)
        lib().orc_override_worst(self.h, _p(o))
        return o

    def energy(self):
        return lib().orc_energy(self.h)

    def compute_energy(self):
        return lib().orc_compute_energy(self.h)

    def verify_energy(self):
        return bool(lib().orc_verify_energy(self.h))

    def state(self):
        n = self.cfg.n * self.cfg.n if self.cfg.system == ISING else 3 * self.cfg.n
        out = np.zeros(n)
        lib().orc_get_state(self.h, _p(out))
        return out if self.cfg.system == ISING else out.reshape(-1, 3)

    def plan_move(self, which, g=(0.0, 0.0, 0.0), j=0, scale=0.05):
        e = ctypes.c_double(0.0)
        ok = lib().orc_plan_move(self.h, which, j, g[0], g[1], g[2], scale, ctypes.byref(e))
        return e.value if ok else None

    def confirm(self):
        lib().orc_confirm(self.h)

    def bins(self):
        n = lib().orc_nbins(self.h)
        lnw, sumE, sumE2 = np.zeros(n), np.zeros(n), np.zeros(n)
        hist, tf, rt = (np.zeros(n, np.uint64) for _ in range(3))
        vis = np.zeros(n, np.uint8)
        mw = np.zeros(2)
        lib().orc_get_bins(self.h, _p(lnw), _p(hist), _p(tf), _p(sumE), _p(sumE2), _p(rt),
                           _p(vis), _p(mw))
        return dict(lnw=lnw, hist=hist, t_found=tf, sumE=sumE, sumE2=sumE2,
                    round_trips=rt, visited=vis, min=mw[0], width=mw[1])

    def wl_hist(self):
        n = lib().orc_wl_hist(self.h, None, None)
        out = np.zeros(max(n, 1), np.uint64)
        me = ctypes.c_double(0.0)
        lib().orc_wl_hist(self.h, _p(out), ctypes.byref(me))
        return out[:n], me.value

    def scalars(self):
        o = np.zeros(len(SCALARS))
        lib().orc_get_scalars(self.h, _p(o))
        return dict(zip(SCALARS, o))

    def temperature(self, e):
        return lib().orc_temperature(self.h, e)

    def pressure(self):
        return lib().orc_pressure(self.h)


class GrandConfig(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("has_energy_bin", ctypes.c_int32),
                ("t0", ctypes.c_double), ("energy_bin", ctypes.c_double),
                ("has_max_N", ctypes.c_int32), ("max_N", ctypes.c_int32),
                ("has_min_allowed", ctypes.c_int32), ("has_max_allowed", ctypes.c_int32),
                ("min_allowed", ctypes.c_double), ("max_allowed", ctypes.c_double),
                ("acc_mode", ctypes.c_int32), ("system", ctypes.c_int32),
                ("target_rate", ctypes.c_double), ("translation_scale", ctypes.c_double),
                ("addremove_probability", ctypes.c_double), ("radius", ctypes.c_double),
                ("box", ctypes.c_double * 3),
                ("seed", ctypes.c_uint64), ("walker", ctypes.c_uint32), ("pad2", ctypes.c_uint32)]


GRAND_SCALARS = ["moves", "accepted", "addremove_probability", "N", "energy", "num_states",
                 "t_last", "gamma", "lowest_hist", "highest_hist", "total_hist", "max_S",
                 "max_S_index", "min", "width", "max_N", "num_E", "addremove_attempts",
                 "addremove_accepted"]


def make_grand_config(radius=0.0, *, box=None, method=M_SAMC, t0=1e4, energy_bin=None,
                      max_N=None, min_allowed=None, max_allowed=None, target_rate=None,
                      translation_scale=0.05, addremove_probability=0.05, seed=0, walker=0):
    """Energy-number walker: the LJ cluster of `radius`, or (box given) the WCA fluid."""
    c = GrandConfig()
    c.system = 2 if box is not None else 1
    if box is not None:
        c.box[0], c.box[1], c.box[2] = box
    c.kind = method
    c.t0 = t0
    c.has_energy_bin, c.energy_bin = int(energy_bin is not None), energy_bin or 0.0
    c.has_max_N, c.max_N = int(max_N is not None), max_N or 0
    c.has_min_allowed, c.min_allowed = int(min_allowed is not None), min_allowed or 0.0
    c.has_max_allowed = int(max_allowed is not None)
    c.max_allowed = max_allowed if max_allowed is not None else 0.0
    c.acc_mode, c.target_rate = int(target_rate is not None), target_rate or 0.5
    c.translation_scale, c.addremove_probability = translation_scale, addremove_probability
    c.radius, c.seed, c.walker = radius, seed, walker
    return c


class GrandWalker:
    """One oracle energy-number walker (grand-canonical LJ cluster, starting empty)."""

    def __init__(self, cfg):
        self.cfg = cfg
        self.h = lib().orc_grand_create(ctypes.byref(cfg))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_grand_destroy(self.h)
            self.h = None

    def run(self, n):
        lib().orc_grand_run(self.h, int(n))

    def run_override(self, e1, e2):
        e1 = np.ascontiguousarray(e1, dtype=np.float64)
        e2 = np.ascontiguousarray(e2, dtype=np.float64)
        mm = ctypes.c_uint64(0)
        d = lib().orc_grand_run_override(self.h, len(e2), _p(e1), _p(e2), ctypes.byref(mm))
        return d, mm.value

    def worst(self):
        o = np.zeros(4)
        lib().orc_grand_worst(self.h, _p(o))
        return o

    def state(self):
        n = lib().orc_grand_state(self.h, None)
        out = np.zeros((max(n, 1), 3))
        lib().orc_grand_state(self.h, _p(out))
        return out[:n]

    def compute_energy(self):
        return lib().orc_grand_compute_energy(self.h)

    def scalars(self):
        o = np.zeros(len(GRAND_SCALARS))
        lib().orc_grand_scalars(self.h, _p(o))
        return dict(zip(GRAND_SCALARS, o))

    def bins(self):
        n = lib().orc_grand_bins(self.h, None, None, None, None, None)
        lnw = np.zeros(n)
        hist, wlh, rt = (np.zeros(n, np.uint64) for _ in range(3))
        vis = np.zeros(n, np.uint8)
        lib().orc_grand_bins(self.h, _p(lnw), _p(hist), _p(wlh), _p(vis), _p(rt))
        s = self.scalars()
        nN = int(s["max_N"]) + 1
        return dict(lnw=lnw.reshape(-1, nN), hist=hist.reshape(-1, nN), wl_hist=wlh.reshape(-1, nN),
                    visited=vis.reshape(-1, nN), round_trips=rt.reshape(-1, nN), min=s["min"],
                    width=s["width"])

    def check_cells(self):
        """Subcells whose lists differ from a rebuild (WCA; 0 for the LJ cluster)."""
        return lib().orc_grand_check_cells(self.h)

    def translation_counts(self):
        nN = int(self.scalars()["max_N"]) + 1
        a, b = np.zeros(nN, np.uint64), np.zeros(nN, np.uint64)
        lib().orc_grand_translation(self.h, _p(a), _p(b))
        return a, b


def grand_draws(seed, walker, t):
    d = np.zeros(2)
    u = np.zeros(2, np.uint32)
    g = np.zeros(3, np.float32)
    c = np.zeros(3)
    lib().orc_grand_draws(seed, walker, t, _p(d), _p(u), _p(g), _p(c))
    return dict(u_choice=d[0], u=d[1], add_bit=int(u[0]), pick=int(u[1]), g=g, cand0=c)


def philox(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().orc_philox(_p(c), _p(k), _p(o))
    return o


def draws(system, n, seed, walker, t, stream_pair=0):
    idx = np.zeros(2, np.uint32)
    g = np.zeros(3, np.float32)
    u = ctypes.c_double(0.0)
    lib().orc_draws(system, n, seed, walker, t, stream_pair, _p(idx), _p(g), ctypes.byref(u))
    return idx, g, u.value


def normal_pairs(a, b):
    a = np.ascontiguousarray(a, np.uint32)
    b = np.ascontiguousarray(b, np.uint32)
    z0 = np.zeros(len(a), np.float32)
    z1 = np.zeros(len(a), np.float32)
    lib().orc_normal_pairs(_p(a), _p(b), len(a), _p(z0), _p(z1))
    return z0, z1


def heat_capacity(T, E, S):
    T = np.ascontiguousarray(T, np.float64)
    E = np.ascontiguousarray(E, np.float64)
    S = np.ascontiguousarray(S, np.float64)
    C = np.zeros(len(T))
    lib().orc_heat_capacity(_p(T), len(T), _p(E), _p(S), len(E), _p(C))
    return C


def max_balls_within(d):
    return lib().orc_max_balls_within(d)


def init_lj(n, radius, seed):
    out = np.zeros(3 * n)
    ok = lib().orc_init_lj(n, radius, seed, _p(out))
    return out.reshape(-1, 3), bool(ok)


def init_sw_fcc(n, filling_fraction, well_width=1.3, seed=0):
    box = np.zeros(3)
    out = np.zeros(3 * n)
    ok = lib().orc_init_sw_fcc(n, filling_fraction, well_width, seed, _p(box), _p(out))
    if not ok:
        raise ValueError("FCC initialisation failed")
    return out.reshape(-1, 3), tuple(box)


def selftest_ising(L, flips, seed=1):
    return lib().orc_selftest_ising(L, flips, seed)


def selftest_moves(walker, nmoves, scale, maxe_per_atom=16.0, seed=1):
    return lib().orc_selftest_moves(walker.h, nmoves, scale, maxe_per_atom, seed)


def selftest_cell(walker):
    return lib().orc_selftest_cell(walker.h)


def bench(cfgs, states, moves, threads, native=False):
    """Time `moves` moves of each walker on `threads` host threads; returns
    (seconds, total_moves, total_accepted).  native: the host-tuned build."""
    n = len(cfgs)
    arr = (Config * n)(*cfgs)
    keep = [np.ascontiguousarray(s, np.float64) for s in states]
    ptrs = (ctypes.c_void_p * n)(*[k.ctypes.data for k in keep])
    tm, ta = ctypes.c_uint64(0), ctypes.c_uint64(0)
    sec = lib(native).orc_bench(arr, ptrs, n, int(moves), threads, ctypes.byref(tm), ctypes.byref(ta))
    return sec, tm.value, ta.value
