"""Heat-capacity error of a batch of flat-histogram walkers against a reference curve.

The reference's convergence measure is |C_ref(T_peak) - C(T_peak)| for one run's
entropy estimate (lj/convergence-for-proposal.py:119-120, with C from
lj/heat_capacity.py:11-34).  A batch here holds thousands of independent runs, so the
error is taken per walker (each walker's own Cv from sadmc_walker_heat_capacity) and
summarised over the batch:

  median_max_rel   median over walkers of max_T |C_w(T) - C_ref(T)| / C_ref(T)
  median_rel[T]    median over walkers of |C_w(T) - C_ref(T)| / C_ref(T), per T
  median_curve     the per-T median of C_w, and its relative error max_rel_of_median
"""
import numpy as np


def interp_reference(T, curves):
    """Mean of the reference curves (each a (T, Cv) pair of arrays) at T."""
    return np.mean([np.interp(T, np.asarray(t), np.asarray(c)) for t, c in curves], axis=0)


def cv_error(C, C_ref):
    """C: [walkers, len(T)] per-walker heat capacities; C_ref: [len(T)]."""
    C = np.asarray(C, float)
    C_ref = np.asarray(C_ref, float)
    rel = np.abs(C - C_ref[None, :]) / C_ref[None, :]
    rel = np.where(np.isfinite(rel), rel, np.inf)
    med = np.median(C, axis=0)
    return {"median_max_rel": float(np.median(rel.max(axis=1))),
            "median_rel": [float(x) for x in np.median(rel, axis=0)],
            "median_curve": [float(x) for x in med],
            "max_rel_of_median": float(np.max(np.abs(med - C_ref) / C_ref))}


def time_to_error(times, errors, target):
    """First time at which the running minimum of errors reaches target (linear in
    log error between checkpoints), or None if it never does."""
    best = np.minimum.accumulate(np.asarray(errors, float))
    for k, e in enumerate(best):
        if e <= target:
            if k == 0:
                return float(times[0])
            e0, e1 = np.log(best[k - 1]), np.log(max(e, 1e-300))
            f = 0.0 if e0 == e1 else (e0 - np.log(target)) / (e0 - e1)
            return float(times[k - 1] + f * (times[k] - times[k - 1]))
    return None
