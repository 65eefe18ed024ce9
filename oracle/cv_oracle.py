"""ORACLE / TEST INFRASTRUCTURE ONLY: FP64 numpy statement of the heat-capacity
reconstruction from one walker's bins, against which the GPU's per-walker kernel
(sadmc_walker_heat_capacity) and the Cv-error harness are checked.

  entropy   plotting/parse-binning.py:136-160: ln w inside SAD's [too_lo, too_hi]; below
            it ln w(too_lo) + (E - too_lo)/min_T + ln(hist / mean hist over the window),
            above it ln w(too_hi) + ln(hist / mean hist); a Wang-Landau production run
            (gamma == 0) adds ln of its production histogram; unvisited bins dropped
  Cv(T)     plotting/final_heat_capacity.py:79-88: P ~ exp(S - E/T - max),
            C = sum (E - <E>)^2 P / T^2
"""
import numpy as np


def walker_entropy(bins, scalars, min_T=None, wl_hist=None):
    """(E, S) over the visited bins of one walker: bins as returned by the walkers'
    bins() (lnw, hist, min, width), scalars as by scalars()."""
    lnw = np.asarray(bins["lnw"], float)
    h = np.asarray(bins["hist"], float)
    E = bins["min"] + (np.arange(len(lnw)) + 0.5) * bins["width"]
    S = lnw.copy()
    kind = int(scalars["method_kind"])
    if kind == 0:
        lo, hi = scalars["too_lo"], scalars["too_hi"]
        i_lo = int(np.floor((lo - bins["min"]) / bins["width"]))
        i_hi = int(np.floor((hi - bins["min"]) / bins["width"]))
        i_lo = min(max(i_lo, 0), len(E) - 1)
        i_hi = min(max(i_hi, 0), len(E) - 1)
        mean = h[i_lo:i_hi + 1].mean()
        below, above = E < lo, E > hi
        with np.errstate(divide="ignore"):
            S[below] = lnw[i_lo] + (E[below] - lo) / min_T + np.log(h[below] / mean)
            S[above] = lnw[i_hi] + np.log(h[above] / mean)
    elif kind in (2, 3) and scalars["gamma"] == 0.0 and wl_hist is not None:
        p = np.asarray(wl_hist, float)
        S[p > 0] += np.log(p[p > 0])
    keep = h > 0
    return E[keep], S[keep]


def heat_capacity(T, E, S):
    out = []
    for t in np.atleast_1d(T):
        b = S - E / t
        P = np.exp(b - b.max())
        P /= P.sum()
        U = (E * P).sum()
        out.append(((E - U) ** 2 * P).sum() / t ** 2)
    return np.array(out)
