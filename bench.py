"""Benchmark of the flat-histogram hot path on one GB300.

Workload (C2): LJ cluster N=31 in a sphere of radius 2.5 sigma, plain SAD (min_T 0.2 ...
see WORKLOAD) over [-134, 0] with 1000 FP64 bins, 4096 independent walkers, Gaussian
single-atom moves of initial rms 0.1 adapted toward 50% acceptance.  One step = 24,414
moves of every walker = 1.0e8 moves (the C2 budget).

  value   moves/s with the batch resident in HBM (CUDA events on the launching stream)
  e2e     moves/s through the C ABI from pinned host buffers: upload configurations,
          initialize (FP64 energies, descent below E=0, bins), run, read back all ln w
          and histogram planes -- every step
  roofline  FP32 pair work of the move kernel (30 (N-1) FLOP per move) against the FP32
          issue peak; HBM traffic per launch from the committed ncu summary

`--impl reference` times the FP64 CPU oracle (the C++ restatement of the reference's
Rust path, which cannot be built here) on all host cores on a bounded sample.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "sad-monte-carlo_gb300"))

N_ATOMS, RADIUS, WALKERS = 31, 2.5, 4096
MOVES_PER_STEP = 24414                       # per walker: 4096 * 24414 = 1.0e8 moves
E_LO, E_HI, NBINS = -134.0, 0.0, 1000
WIDTH = (E_HI - E_LO) / NBINS                # 0.134
FLOP_PER_MOVE = 30 * (N_ATOMS - 1)           # 2 (N-1) pair terms x 15 FLOP
WORKLOAD = (f"C2 LJ{N_ATOMS} cluster (R={RADIUS}), SAD min_T=0.2, {NBINS} bins of "
            f"{WIDTH:g} over [{E_LO:g},{E_HI:g}], max_allowed_energy 0, {WALKERS} walkers, "
            f"{MOVES_PER_STEP} moves/walker per step, step 0.1 adapted to 50% acceptance")


def lj_configs(n_walkers, seed):
    """Uniform in the sphere with random sequential rejection of pairs closer than 0.8."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n_walkers, N_ATOMS, 3))
    for w in range(n_walkers):
        pts = []
        while len(pts) < N_ATOMS:
            p = rng.uniform(-RADIUS, RADIUS, 3)
            if p @ p >= RADIUS * RADIUS:
                continue
            if pts and np.min(np.sum((np.array(pts) - p) ** 2, axis=1)) < 0.64:
                continue
            pts.append(p)
        out[w] = pts
    return out


def _time_run(b, moves, warm):
    """Seconds for `moves` moves per walker after `warm` warm-up moves: CUDA events on the
    stream the kernels are launched on (a batch's run_async takes the stream; a grand batch
    runs on its own stream and returns when done, so its events bracket the whole call)."""
    import ctypes
    import torch
    b.run(warm)
    torch.cuda.synchronize()
    st = torch.cuda.Stream()  # a stream of its own: a null handle means the library's stream
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed")
    e0.record(st)
    if hasattr(b, "run_async"):
        b.run_async(moves, ctypes.c_void_p(st.cuda_stream))
    else:
        b.run(moves)
    e1.record(st)
    torch.cuda.nvtx.range_pop()
    e1.synchronize()
    return e0.elapsed_time(e1) * 1e-3


def _lanes(b, lpw, tune_moves):
    """The shape: fixed by --lpw, else autotuned on a snapshot of the batch."""
    if not lpw:
        b.autotune(tune_moves)
    return b.lanes_per_walker()


def c1_inputs(seed=11):
    """C1: one 32x32 Ising lattice, uniform random spins from the seed."""
    rng = np.random.default_rng(seed)
    return 32, np.where(rng.random(32 * 32) < 0.5, -1.0, 1.0)


def c3_inputs(seed=11, walkers=2048):
    """C3: WCA, N in {64,128,256,512}, density U[0.6, 0.9], a random subset of a
    jittered simple-cubic lattice filling each box: [(n, box edge, positions)]."""
    rng = np.random.default_rng(seed)
    rng.random(32 * 32)  # the C1 spins come first from this seed
    ns = rng.choice([64, 128, 256, 512], walkers)
    rhos = rng.uniform(0.6, 0.9, walkers)
    out = []
    for n, rho in zip(ns, rhos):
        Lb = (n / rho) ** (1 / 3)
        m = int(np.ceil(n ** (1 / 3)))
        g = np.array([(i, j, k) for i in range(m) for j in range(m) for k in range(m)], float)
        g = g[rng.permutation(len(g))[:n]]
        out.append((int(n), Lb, np.mod((g + 0.5 + rng.uniform(-0.05, 0.05, g.shape)) * (Lb / m), Lb)))
    return out


def c5_inputs(seed=11, walkers=1024):
    """C5: N = 1024 hard-core square-well atoms on a jittered FCC lattice, packing
    fraction U[0.30, 0.50]: [(box edge, positions)]."""
    rng = np.random.default_rng(seed + 1)
    n5 = 1024
    m = int(np.ceil((n5 / 4) ** (1 / 3)))
    base = np.array([(0, 0, 0), (0.5, 0.5, 0), (0.5, 0, 0.5), (0, 0.5, 0.5)])
    sites = (np.array([(i, j, k) for i in range(m) for j in range(m) for k in range(m)], float)[:, None, :]
             + base[None]).reshape(-1, 3)
    out = []
    for eta in rng.uniform(0.30, 0.50, walkers):
        Lb = (n5 * np.pi / (6 * eta)) ** (1 / 3)
        pick = sites[rng.permutation(len(sites))[:n5]]
        out.append((Lb, np.mod((pick + rng.uniform(-0.004, 0.004, pick.shape)) * (Lb / m), Lb)))
    return out


# Peaks for the roofline of the other workloads: FP32 FFMA issue (152 SMs x 128 lanes x
# 2 FLOP x max SM clock), FP64 from the DFMA throughput probe (0.052 warp instructions per
# clock per SM: 152 x 0.052 x 32 lanes x 2 FLOP x clock), one SM's shared-memory port
# (128 B per clock).
SM_HZ = 2.07e9
FP32_PEAK = 152 * 128 * 2 * SM_HZ
FP64_PEAK = 152 * 0.052 * 32 * 2 * SM_HZ
SMEM_SM_PEAK = 128 * SM_HZ


def _roof(achieved, peak, unit, note):
    return {"achieved": achieved, "peak": peak, "unit": unit, "frac": achieved / peak, "note": note}


def status_summary(b, ignore=0):
    """Walkers whose device status word is set after a run, and the bits seen."""
    st = b.status() & ~np.uint32(ignore)
    bits = int(np.bitwise_or.reduce(st)) if len(st) else 0
    return {"walkers_with_status": int((st != 0).sum()), "status_bits": bits}


def candidates(n, L, r_cut):
    """C = 27 N / n_c^3 - 1 candidate partners of a query, n_c = floor(L / r_cut)."""
    nc = np.floor(np.asarray(L) / r_cut)
    return 27.0 * np.asarray(n) / nc ** 3 - 1.0


C3_METHOD = dict(t0=1e4, energy_bin=1.0, max_allowed=500.0, translation_scale=0.1)
C5_METHOD = dict(well_width=1.3, translation_scale=0.05)


O_FLAGS = "g++ -O3 -ffp-contract=off -mcpu=native (Arm host; -march=native on x86)"


def case_c1(G, seed=11, moves=10_000_000, lpw=0, **_):
    """C1: plain SAD, Ising 32x32, one walker, bins of 4 over [-2N, 2N]."""
    L, spins = c1_inputs(seed)
    b = G.Batch(G.make_config(G.ISING, 1, L, method=G.SAD, min_T=0.2, e_lo=-2.0 * L * L - 8,
                              e_hi=2.0 * L * L + 8, seed=seed, lanes_per_walker=lpw),
                [(L, 0.0, (0, 0, 0))])
    b.upload([spins])
    b.initialize()
    lanes = _lanes(b, lpw, 20000)
    sec = _time_run(b, moves, 100_000)
    flagged = int((b.status() != 0).sum())
    b.close()
    rate = moves / sec
    return {"workload": "Ising 32x32, plain SAD (min_T 0.2), 1 walker", "moves": moves,
            "moves_per_s": rate, "ns_per_move": 1e9 * sec / moves, "lanes_per_walker": lanes,
            "walkers_with_status": flagged,
            "roofline": _roof(48 * rate / 1e9, SMEM_SM_PEAK / 1e9, "GB/s",
                              "48 B of shared-memory traffic per move against one SM's "
                              "port; not meaningful for one serial walker")}


def case_c1_batch(G, seed=11, walkers=4096, moves=20000, lpw=0):
    """The C1 lattice and method for many independent walkers (spins from seed + walker):
    the shape in which a GPU runs Ising work; C1 itself is one serial chain."""
    L = 32
    b = G.Batch(G.make_config(G.ISING, walkers, L, method=G.SAD, min_T=0.2,
                              e_lo=-2.0 * L * L - 8, e_hi=2.0 * L * L + 8, seed=seed,
                              lanes_per_walker=lpw),
                [(L, 0.0, (0, 0, 0))] * walkers)
    b.upload([c1_inputs(seed + w)[1] for w in range(walkers)])
    b.initialize()
    lanes = _lanes(b, lpw, 2000)
    sec = _time_run(b, moves, 4000)
    flagged = int((b.status() != 0).sum())
    b.close()
    return {"workload": f"Ising 32x32, plain SAD (min_T 0.2), {walkers} independent walkers",
            "moves": walkers * moves, "moves_per_s": walkers * moves / sec,
            "lanes_per_walker": lanes, "walkers_with_status": flagged}


def case_c3(G, seed=11, walkers=2048, moves=2048, lpw=0):
    """C3: WCA, SAMC t0 = 1e4, 500 bins over [0, 500) (a range fixed here; the workload
    states none); the descent of initialize() brings each walker below 500."""
    inp = c3_inputs(seed, walkers)
    nmax = max(n for n, _, _ in inp)
    b = G.Batch(G.make_config(G.WCA, walkers, nmax, method=G.SAMC, e_lo=-1.0, e_hi=501.0,
                              seed=seed, resum_interval=4096, lanes_per_walker=lpw, **C3_METHOD),
                [(n, 0.0, (Lb, Lb, Lb)) for n, Lb, _ in inp])
    b.upload([p for _, _, p in inp])
    b.initialize()
    lanes = _lanes(b, lpw, 256)
    sec = _time_run(b, moves, 512)
    flagged = status_summary(b)
    b.close()
    rate = walkers * moves / sec
    flop = float(np.mean(2 * 15 * candidates([n for n, _, _ in inp], [Lb for _, Lb, _ in inp],
                                              2 ** (1 / 6))))
    return {"workload": f"WCA, N in {{64,128,256,512}}, density U[0.6,0.9], {walkers} walkers, "
                        "SAMC t0=1e4, 500 bins over [0,500)",
            "moves": walkers * moves, "moves_per_s": rate, "lanes_per_walker": lanes,
            **flagged,
            "roofline": _roof(rate * flop / 1e12, FP32_PEAK / 1e12, "TFLOP/s",
                              f"2 C x 15 FP32 FLOP per move, C = 27 N / n_c^3 - 1 per walker "
                              f"(mean {flop:.0f} FLOP)")}


def case_c5(G, seed=11, walkers=1024, moves=2048, lpw=0):
    """C5: hard-core square well (lambda 1.3), Wang-Landau over contact-count bins of
    width 1."""
    inp = c5_inputs(seed, walkers)
    b = G.Batch(G.make_config(G.SW, walkers, 1024, method=G.WL, e_lo=-6.0 * 1024 - 2, e_hi=2.0,
                              seed=seed, lanes_per_walker=lpw, **C5_METHOD),
                [(1024, 0.0, (Lb, Lb, Lb)) for Lb, _ in inp])
    b.upload([p for _, p in inp])
    b.initialize()
    lanes = _lanes(b, lpw, 256)
    sec = _time_run(b, moves, 512)
    flagged = status_summary(b)
    b.close()
    rate = walkers * moves / sec
    flop = float(np.mean(2 * 8 * candidates(1024, [Lb for Lb, _ in inp], 1.3)))
    return {"workload": f"hard-core square well lambda=1.3, N=1024, packing U[0.30,0.50], "
                        f"jittered FCC, WL on contact bins, {walkers} walkers",
            "moves": walkers * moves, "moves_per_s": rate, "lanes_per_walker": lanes,
            **flagged,
            "roofline": _roof(rate * flop / 1e12, FP64_PEAK / 1e12, "TFLOP/s",
                              f"2 C x 8 FP64 FLOP per move (C = 27 N / n_c^3 - 1, mean {flop:.0f} "
                              "FLOP) against the FP64 peak; the kernel decides most pairs with "
                              "binary32 screens, so this counts the reference's work")}


def case_grand(G, seed=11, walkers=4096, moves=4096, lpw=0):
    """Grand-canonical LJ cluster, energy-number SAMC (src/mc/energy_number.rs): walkers
    start empty and grow to at most 31 atoms in a sphere of radius 2.5."""
    gb = G.GrandBatch(G.make_grand_config(walkers, 31, 2.5, method=G.SAMC, t0=1e4,
                                          energy_bin=0.5, max_allowed=10.0,
                                          translation_scale=0.1, addremove_probability=0.1,
                                          e_lo=-150.0, e_hi=12.0, seed=seed,
                                          lanes_per_walker=lpw))
    sec = _time_run(gb, moves, 4096)
    out = {"workload": f"grand-canonical LJ cluster (R=2.5, N <= 31), energy-number SAMC "
                       f"t0=1e4, {walkers} walkers",
           "moves": walkers * moves, "moves_per_s": walkers * moves / sec,
           "mean_N": float(np.mean([gb.scalars(w)["N"] for w in range(0, walkers, 256)])),
           "lanes_per_walker": lpw or 8}
    gb.close()
    return out


def case_da(G, seed=11, walkers=8192, moves=100_000, **_):
    """C4 shape: the plain and delayed-acceptance arms of da_compare, alone."""
    return da_compare(G, 0, walkers, moves)


def case_north_star(G, seed=31, walkers=1024, moves=1_000_000, **_):
    """Plain against delayed acceptance at equal heat-capacity error (the benchmark spec), alone."""
    return north_star(G, walkers=walkers, warm=moves, seed=seed)


def case_grand_wca(G, seed=11, walkers=512, moves=2048, lpw=0):
    """Grand-canonical WCA fluid, energy-number SAMC (wca.rs:307-323): walkers start empty
    in a periodic box of edge 6 and grow to at most 200 atoms (density up to 0.93)."""
    gb = G.GrandBatch(G.make_grand_config(walkers, 200, box=(6.0, 6.0, 6.0), method=G.SAMC,
                                          t0=1e4, energy_bin=1.0, max_allowed=400.0,
                                          translation_scale=0.1, addremove_probability=0.2,
                                          e_lo=-1.0, e_hi=402.0, seed=seed, lanes_per_walker=lpw))
    sec = _time_run(gb, moves, 4096)
    out = {"workload": f"grand-canonical WCA fluid (box 6^3, N <= 200), energy-number SAMC "
                       f"t0=1e4, {walkers} walkers",
           "moves": walkers * moves, "moves_per_s": walkers * moves / sec,
           "mean_N": float(np.mean([gb.scalars(w)["N"] for w in range(0, walkers, 64)])),
           "lanes_per_walker": lpw or 32}
    gb.close()
    return out


CASES = {"C1": case_c1, "C1_batch": case_c1_batch, "C3": case_c3, "C5": case_c5,
         "grand": case_grand, "grand_wca": case_grand_wca}
ONLY = dict(CASES, DA=case_da, NORTH_STAR=case_north_star)


def cpu_cases(seed=11):
    """The FP64 oracle on the same inputs as C1, C3 and C5, each on a bounded sample (its
    first walkers, fewer moves), on the host threads: the reference's CPU algorithm
    beside the GPU numbers."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    out = {}
    L, spins = c1_inputs(seed)
    moves = 2_000_000
    cfg = O.make_config(O.ISING, L, method=O.M_SAD, min_T=0.2, seed=seed, walker=0)
    sec, tm, _ = O.bench([cfg], [spins], moves, 1, native=True)
    out["C1"] = {"moves_per_s": tm / sec, "threads": 1, "sample": f"1 walker x {moves} moves"}
    w3, m3 = 256, 8000
    inp = c3_inputs(seed, w3)
    cfgs = [O.make_config(O.WCA, n, box=(Lb, Lb, Lb), method=O.M_SAMC, seed=seed, walker=w,
                          **C3_METHOD) for w, (n, Lb, _) in enumerate(inp)]
    sec, tm, _ = O.bench(cfgs, [p for _, _, p in inp], m3, threads, native=True)
    out["C3"] = {"moves_per_s": tm / sec, "threads": threads,
                 "sample": f"first {w3} walkers x {m3} moves"}
    w5, m5 = 128, 8000
    inp = c5_inputs(seed, w5)
    cfgs = [O.make_config(O.SW, 1024, box=(Lb, Lb, Lb), method=O.M_WL, seed=seed, walker=w,
                          **C5_METHOD) for w, (Lb, _) in enumerate(inp)]
    sec, tm, _ = O.bench(cfgs, [p for _, p in inp], m5, threads, native=True)
    out["C5"] = {"moves_per_s": tm / sec, "threads": threads,
                 "sample": f"first {w5} walkers x {m5} moves"}
    return out


def other_configs(G, seed=11, cpu=True):
    """Device-resident moves/s of the other workloads (synthetic seeded inputs with their
    shapes): C1 one Ising 32x32 walker, C3 an uneven WCA batch, C5 a hard-core square-well
    batch, and the grand-canonical LJ cluster.  Each is a short run after a warm-up, timed
    with CUDA events.  With cpu, the oracle's moves/s on a sample of the same inputs sits
    beside C1, C3 and C5 (`cpu`)."""
    out = {k: f(G, seed) for k, f in CASES.items()}
    if cpu:
        for k, v in cpu_cases(seed).items():
            out[k]["cpu"] = v
    return out


def sphere_configs(n, R, count, seed):
    """Uniform in the sphere with sequential rejection of pairs closer than 0.8."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        pts = np.empty((n, 3))
        k = 0
        while k < n:
            p = rng.uniform(-R, R, 3)
            if p @ p >= R * R or (k and np.min(((pts[:k] - p) ** 2).sum(axis=1)) < 0.64):
                continue
            pts[k] = p
            k += 1
        out.append(pts)
    return out


def _timed(f):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = f()
    torch.cuda.synchronize()
    return r, time.perf_counter() - t0


def da_compare(G, rank=0, walkers=8192, moves=100_000):
    """C4 shape: LJ38 (R = 3.5), SAD min_T 0.05, bins of 0.2, 8192 walkers.  The surrogate
    is trained online on configurations the walkers' own SAD run visits (a ring of 1e6,
    every walker collected every 4000 moves, retrained every 2e4 moves of the warm-up),
    then the plain arm (at its autotuned shape) and the delayed-acceptance arm (retrained
    every 5e4 moves, inside its timed region) each run `moves` moves per walker."""
    n, R = 38, 3.5
    cfg = G.make_config(G.LJ, walkers, n, method=G.SAD, min_T=0.05, energy_bin=0.2,
                        max_allowed=0.0, e_lo=-180.0, e_hi=1.0, target_rate=0.5,
                        translation_scale=0.1, seed=21 + rank)
    b = G.Batch(cfg, [(n, R, (0, 0, 0))] * walkers)
    b.upload(sphere_configs(n, R, walkers, 77 + rank))
    b.initialize()
    b.surrogate_init(seed=3, ring_capacity=1_000_000)
    _, warm_s = _timed(lambda: b.run_online(40_000, False, collect_interval=4000, retrain_interval=20_000,
                                            train_steps=400, batch=512, lr=2e-3, seed=5))
    _, train_s = _timed(lambda: b.surrogate_train(200, batch=512, lr=1e-3, seed=6))
    loss = b.surrogate_train(1, batch=4096, lr=0.0, seed=7)
    b.autotune(2048)
    m0, a0 = b.counters()
    _, plain_s = _timed(lambda: b.run(moves))
    m1, a1 = b.counters()
    st0 = b.run_da(0)
    st, da_s = _timed(lambda: b.run_online(moves, True, collect_interval=10_000, retrain_interval=50_000,
                                           train_steps=100, batch=512, lr=1e-3, seed=8))
    m2, a2 = b.counters()
    flagged = status_summary(b)
    lanes = b.lanes_per_walker()
    b.close()
    st = st.astype(np.float64) - st0.astype(np.float64)
    screened = float(st[:, 0].sum()) / float(st.sum())
    exact = float(st[:, 1].sum()) / float(m2 - m1)
    return {"workload": f"C4 shape: LJ{n} (R={R}), SAD min_T 0.05, bins of 0.2, {walkers} walkers, "
                        f"{moves} moves/walker per arm",
            "plain_moves_per_s": (m1 - m0) / plain_s, "plain_accepted_per_s": (a1 - a0) / plain_s,
            "plain_lanes_per_walker": lanes,
            "da_moves_per_s": (m2 - m1) / da_s, "da_accepted_per_s": (a2 - a1) / da_s,
            "da_vs_plain": ((m2 - m1) / da_s) / ((m1 - m0) / plain_s),
            "da_accepted_vs_plain": ((a2 - a1) / da_s) / ((a1 - a0) / plain_s),
            "screened_fraction": screened, "exact_evaluations_per_move": exact,
            "surrogate_rmse": float(np.sqrt(loss)),
            "train_us_per_step": 1e6 * train_s / 200, "train_batch_rows": 512 * n,
            "warmup_s": warm_s, **flagged,
            "online": "ring 1e6 configurations; warm-up collects every 4000 moves and retrains every "
                      "20000 (400 Adam steps of 512); the DA arm collects every 10000 and retrains "
                      "every 50000 moves (100 steps) inside its timed region",
            "roofline": _roof((m2 - m1) / da_s * 2 * n * 6208 / 1e12,
                              float(peaks().get("bf16_tflops", 1900.0)), "TFLOP/s",
                              f"stage 1: the MLP on all {n} descriptor rows, 2 x 6208 BF16 FLOP "
                              "per row, against the measured bf16 peak (mma.sync m16n8k16, one "
                              "walker per warp)")}


CV_T = np.array([0.25, 0.28, 0.30, 0.33, 0.36])


def lj31_reference_cv(T=CV_T):
    """Mean of the reference's Rc = 2.5 LJ31 curves (RESTMC and t-REM) at T, from the
    committed fixture of the reference's CSV files."""
    import cv as CVM
    g = json.load(open(os.path.join(REPO, "tests", "golden", "lj31_cv_reference.json")))
    return CVM.interp_reference(T, [(g["curves"][k]["T"], g["curves"][k]["Cv"]) for k in ("RESTMC", "t-REM")])


def north_star(G, walkers=1024, warm=1_000_000, seconds=20.0, seed=31):
    """Plain against delayed-acceptance moves at equal heat-capacity error, on the LJ31
    workload's configuration (R = 2.5, SAD min_T 0.2, bins of 0.134), whose heat capacity
    the reference holds (its Rc = 2.5 curves, RESTMC and t-REM, T = 0.25-0.36).  Both arms
    continue from one checkpoint after a shared warm-up in which the surrogate trains
    online on the walkers' own configurations; each arm runs for `seconds` of wall time in
    segments, and after each segment every walker's Cv is rebuilt on the device from its
    own bins.  The error is that of the walker-median Cv curve against the reference
    (max over T of the relative error).  The comparison is the time each arm needs to
    reach the error both reach (the larger of the two arms' smallest errors), and at a
    few coarser levels.  1024 walkers: the delayed-acceptance kernel (a warp per walker,
    8 per SM) still runs them in one wave, and the median over walkers is steadier than
    at fewer."""
    import tempfile
    import cv as CVM
    ref = lj31_reference_cv()
    width = 0.134
    cfg = G.make_config(G.LJ, walkers, 31, method=G.SAD, min_T=0.2, energy_bin=width, max_allowed=0.0,
                        e_lo=-134.0 - 2 * width, e_hi=2 * width, target_rate=0.5,
                        translation_scale=0.1, seed=seed)
    b = G.Batch(cfg, [(31, 2.5, (0, 0, 0))] * walkers)
    b.upload(sphere_configs(31, 2.5, walkers, 900 + seed))
    b.initialize()
    b.surrogate_init(seed=4, ring_capacity=1 << 18)
    b.run_online(warm, False, collect_interval=warm // 10, retrain_interval=warm // 5, train_steps=300,
                 batch=512, lr=2e-3, seed=9)
    path = os.path.join(tempfile.gettempdir(), f"sadmc_north_star_{os.getpid()}.ck")
    b.checkpoint(path)
    plain = G.Batch.resume(path)
    os.remove(path)

    def arm(step, seg):
        rows, t, m_start, a_start = [], 0.0, *b_counters(step)
        while t < seconds:
            _, dt = _timed(lambda: step["run"](seg))
            t += dt
            m, a = b_counters(step)
            e = CVM.cv_error(step["batch"].heat_capacities(CV_T), ref)
            rows.append({"t": t, "moves_per_walker": (m - m_start) / walkers, "accepted": a - a_start,
                         "err": e["max_rel_of_median"], "median_walker_err": e["median_max_rel"]})
        return rows

    def b_counters(step):
        return step["batch"].counters()

    p_rows = arm({"batch": plain, "run": lambda k: plain.run(k)}, 1_000_000)
    d_rows = arm({"batch": b, "run": lambda k: b.run_online(k, True, collect_interval=100_000,
                                                             retrain_interval=100_000, train_steps=100,
                                                             batch=512, lr=1e-3, seed=10)}, 200_000)
    # the levels both arms reach: the larger final error (the common level), and coarser
    # levels up to the larger first error, each crossed by the running minimum
    eps = max(min(r["err"] for r in p_rows), min(r["err"] for r in d_rows))
    top = min(max(r["err"] for r in p_rows), max(r["err"] for r in d_rows))
    levels = [float(x) for x in np.geomspace(eps, max(top, eps), 4)]
    tt = lambda rows, e: CVM.time_to_error([r["t"] for r in rows], [r["err"] for r in rows], e)
    tp, td = tt(p_rows, eps), tt(d_rows, eps)
    by_level = [{"cv_error": e, "plain_s": tt(p_rows, e), "da_s": tt(d_rows, e)} for e in levels]
    for x in by_level:
        x["da_speedup"] = (x["plain_s"] / x["da_s"]) if (x["plain_s"] and x["da_s"]) else None
    flagged = {"plain": status_summary(plain), "da": status_summary(b)}
    plain.close()
    b.close()

    def summary(rows):
        t = rows[-1]["t"]
        return {"seconds": t, "moves_per_s": rows[-1]["moves_per_walker"] * walkers / t,
                "accepted_moves_per_s": rows[-1]["accepted"] / t, "cv_error": rows[-1]["err"],
                "median_walker_cv_error": rows[-1]["median_walker_err"],
                "curve": [(round(r["t"], 2), round(r["moves_per_walker"]), round(r["err"], 4)) for r in rows]}
    out = {"workload": f"LJ31 (R=2.5), SAD min_T 0.2, bins of 0.134, {walkers} walkers, {warm} shared "
                       f"warm-up moves/walker with online training, then {seconds:g} s per arm",
           "cv_reference": "mean of the reference's Rc = 2.5 curves (RESTMC, t-REM) at T = "
                           + ", ".join(f"{t:g}" for t in CV_T),
           "cv_error_metric": "max over T of |median-walker Cv - reference| / reference",
           "plain": summary(p_rows), "da": summary(d_rows), "equal_cv_error": eps,
           "plain_seconds_to_equal_error": tp, "da_seconds_to_equal_error": td,
           "da_speedup_at_equal_cv_error": (tp / td) if (tp and td) else None,
           "by_error_level": by_level,
           "status": flagged}
    out["da_wins"] = bool(out["da_speedup_at_equal_cv_error"] and out["da_speedup_at_equal_cv_error"] > 1.0)
    for k in ("plain", "da"):
        out[k]["accepted_moves_per_s_at_equal_cv_error"] = out[k]["accepted_moves_per_s"]
    return out


def make_batch(G, n_walkers, seed=1, lpw=0):
    cfg = G.make_config(G.LJ, n_walkers, N_ATOMS, method=G.SAD, min_T=0.2, energy_bin=WIDTH,
                        max_allowed=0.0, e_lo=E_LO - 2 * WIDTH, e_hi=E_HI + 2 * WIDTH,
                        target_rate=0.5, translation_scale=0.1, seed=seed,
                        lanes_per_walker=lpw)
    return G.Batch(cfg, [(N_ATOMS, RADIUS, (0, 0, 0))] * n_walkers)


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"sadmc_bench_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", "0", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def profile_value(key, kernel="lj_move_kernel_lj31_4096w"):
    """A figure of the last ncu capture of a kernel (profiles/ncu_figures.json, written
    from the capture that the summary of the same name describes), if present."""
    try:
        return json.load(open(os.path.join(REPO, "profiles", "ncu_figures.json")))[kernel].get(key)
    except (OSError, ValueError, KeyError):
        return None


def profile_traffic():
    """DRAM bytes per move-kernel launch from the last ncu capture, if present."""
    return profile_value("traffic_bytes_per_launch")


def peaks():
    try:
        return json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def cpu_sample(threads, walkers=128, moves=100000, seed=7):
    """The FP64 oracle on host threads, on `walkers` C2 walkers x `moves` moves."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    O.build()
    confs = lj_configs(walkers, seed)
    cfgs = [O.make_config(O.LJ, N_ATOMS, radius=RADIUS, method=O.M_SAD, min_T=0.2,
                          energy_bin=WIDTH, max_allowed=0.0, target_rate=0.5,
                          translation_scale=0.1, seed=seed, walker=w) for w in range(walkers)]
    sec, tm, ta = O.bench(cfgs, [c.reshape(-1) for c in confs], moves, threads, native=True)
    return tm / sec, ta / sec, sec, tm


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    walkers, moves = 256, 100000
    vals = []
    for k in range(args.warmup + args.steps):
        v, _, sec, tm = cpu_sample(threads, walkers=walkers, moves=moves, seed=11 + k)
        if k >= args.warmup:
            vals.append((v, sec))
    value = statistics.mean(v for v, _ in vals)
    line = {
        "impl": "reference", "metric": "moves/s", "value": value, "unit": "moves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.mean(s for _, s in vals),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded uniform-in-sphere LJ31 configurations)",
        "config": {"workload": WORKLOAD, "sample": f"{walkers} walkers x {moves} moves per step"},
        "cpu_baseline": {"value": value, "unit": "moves/s", "cores": threads, "kind": "port",
                         "per_core": value / threads,
                         "sample": f"{walkers} C2 walkers x {moves} moves per step, FP64 C++ "
                                   "restatement of the reference (Rust toolchain absent), built "
                                   f"{O_FLAGS}"},
        "e2e": {"value": value, "unit": "moves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_gpu(args):
    import ctypes

    import torch
    import sadmc_gb300 as G
    import build as B
    import replicas as Rp

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    B.build()
    G.lib()

    # ---- device-resident throughput -------------------------------------------------
    confs = lj_configs(WALKERS, 1000 + rank)
    b = make_batch(G, WALKERS, seed=Rp.rank_seed(1, rank), lpw=args.lpw)
    b.upload(list(confs))
    b.initialize()
    if not args.lpw:
        # the library's autotuner picks lanes per walker x warps per block on a snapshot of
        # this batch (state restored), outside the timed region; cached per shape
        b.autotune(2048)
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    chunk = 8192
    launches_per_step = math.ceil(MOVES_PER_STEP / chunk)
    for _ in range(args.warmup):
        b.run_async(MOVES_PER_STEP, sp)
    stream.synchronize()
    clocks = Clocks()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    m0, a0 = b.counters()
    ev0.record(stream)
    for _ in range(args.steps):
        b.run_async(MOVES_PER_STEP, sp)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    m1, a1 = b.counters()
    moves = m1 - m0
    if moves != WALKERS * MOVES_PER_STEP * args.steps:
        raise RuntimeError(f"move count {moves} != expected")
    ms = Rp.max_over_ranks(ms, device="cuda")
    value = moves * world / (ms * 1e-3)
    acc_rate = (a1 - a0) / moves
    status = b.status()
    launch_ms = ms / (args.steps * launches_per_step)
    flop_per_launch = FLOP_PER_MOVE * WALKERS * (MOVES_PER_STEP / launches_per_step)
    achieved_tflops = flop_per_launch / (launch_ms * 1e-3) / 1e12
    pk = peaks()
    sm_mhz = clk.get("sm_max_mhz") or pk.get("sm_max_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12  # FFMA issue peak, TFLOP/s
    traffic = profile_traffic()
    lanes_per_walker = b.lanes_per_walker()
    b.close()

    # ---- end to end through the C ABI with host buffers ------------------------------
    e2e = None
    if not args.no_e2e:
        n_e2e = WALKERS
        host_conf = torch.from_numpy(lj_configs(n_e2e, 5000 + rank).reshape(-1)).pin_memory()
        be = make_batch(G, n_e2e, seed=7 + rank, lpw=args.lpw)
        nb = be.plane_bins()
        lnw_h = torch.empty(n_e2e * nb, dtype=torch.float64).pin_memory()
        hist_h = torch.empty(n_e2e * nb, dtype=torch.int64).pin_memory()
        lnw_np, hist_np = lnw_h.numpy(), hist_h.numpy().view(np.uint64)
        conf_np = host_conf.numpy()

        def e2e_step():
            be.upload(conf_np)  # all walkers, packed, from pinned memory
            be.initialize()
            be.run(MOVES_PER_STEP)
            be.read_planes(lnw_np, hist_np)
        for _ in range(max(1, args.warmup // 2)):
            e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e_steps = max(1, args.steps // 2)
        for _ in range(e_steps):
            e2e_step()
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        e2e = {"value": n_e2e * MOVES_PER_STEP * e_steps * world / sec, "unit": "moves/s",
               "h2d_bytes_per_step": int(conf_np.nbytes),
               "d2h_bytes_per_step": int(lnw_np.nbytes + hist_np.nbytes),
               "ms_per_step": 1e3 * sec / e_steps,
               "includes": "upload, initialize (FP64 energies, descent, bins), run, read planes"}
        be.close()

    da = None
    if not args.no_da and world == 1:
        da = {"c4_shape": da_compare(G, rank), "equal_cv_error": north_star(G)}
    others = None
    if not args.no_other and rank == 0:
        others = other_configs(G, cpu=not args.no_cpu)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, va, sec, tm = cpu_sample(threads, walkers=256, moves=200000)
        cpu = {"value": v, "unit": "moves/s", "cores": threads, "kind": "port",
               "per_core": v / threads, "accepted_moves_per_s": va,
               "sample": f"256 C2 walkers x 200000 moves ({tm} moves, {sec:.2f} s wall), FP64 "
                         f"C++ restatement of the reference (Rust toolchain absent), built {O_FLAGS}"}

    if rank == 0:
        line = {
            "metric": "moves/s", "value": value, "unit": "moves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 pair energies, f64 ln g / gamma / energy",
            "data": "synthetic (seeded uniform-in-sphere LJ31 configurations)",
            "config": {"workload": WORKLOAD, "walkers": WALKERS, "moves_per_step": WALKERS * MOVES_PER_STEP,
                       "lanes_per_walker": lanes_per_walker,
                       "launch_shape": "fixed by --lpw" if args.lpw else "autotuned",
                       "l2": "bin planes 4096 x 1004 x 64 B = 263 MB > 129 MB L2 (inputs larger than L2)"},
            "accepted_moves_per_s": value * acc_rate,
            "acceptance": acc_rate,
            "walkers_with_status": int((status != 0).sum()),
            "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": fp32_peak,
                         "unit": "TFLOP/s", "frac": achieved_tflops / fp32_peak,
                         "traffic": traffic,
                         "limiter": {"fp64_pipe_active": profile_value("fp64_pipe_active_frac"),
                                     "issue_active": profile_value("issue_active_frac"),
                                     "source": "ncu capture summarised in profiles/lj_move_kernel_lj31_4096w.md"},
                         "note": "30(N-1) FLOP/move algorithmic; peak = 152 SM x 128 FFMA x 2 x "
                                 "max SM clock (FP32 issue, not in MEASURED_PEAKS.json); the "
                                 "kernel is bound by the FP64 pipe and the latency of the per-move "
                                 "bookkeeping (limiter: fractions of peak from ncu)"},
            "launch_ms": launch_ms,
            "clocks": clk,
            "gpu_launches": args.steps * launches_per_step,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "delayed_acceptance": da,
            "other_configs": others,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_case(args):
    import torch
    import build as B
    import sadmc_gb300 as G
    torch.cuda.set_device(0)
    B.build()
    G.lib()
    kw = {"lpw": args.lpw}
    if args.walkers:
        kw["walkers"] = args.walkers
    if args.moves:
        kw["moves"] = args.moves
    out = ONLY[args.only](G, **kw)
    print(json.dumps({"case": args.only, **out}))


def main():
    global WALKERS, MOVES_PER_STEP
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--lpw", type=int, default=0, help="lanes per walker (0: library default)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--walkers", type=int, default=None,
                    help="walkers (profiling a smaller case; the bench line uses 4096)")
    ap.add_argument("--moves", type=int, default=None, help="moves per walker per step")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-da", action="store_true", help="skip the delayed-acceptance comparison")
    ap.add_argument("--no-other", action="store_true", help="skip the C1/C3/C5 measurements")
    ap.add_argument("--only", choices=sorted(ONLY),
                    help="time one other workload alone (with --walkers, --moves, --lpw) and "
                         "print its line; for profiling a small case")
    args = ap.parse_args()
    if args.only:
        run_case(args)
        return
    WALKERS = args.walkers or WALKERS
    MOVES_PER_STEP = args.moves or MOVES_PER_STEP
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
