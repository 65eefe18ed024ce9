"""Walker state in the reference's save and analysis formats.

The reference saves a run as its `EnergyMC<Any>` serialised to YAML or CBOR: the serde
field names of src/mc/energy.rs:145-163 (Bins), 136-142 (BinCounts), 167-210
(EnergyMC) and 213-243 (Method), with the system as the externally tagged enum of
src/system/any.rs:61-78.  Its analysis turns such a file into plain text through
plotting/parse-binning.py:176-190, and lj/compute.py:4-26 and the convergence scripts
load those text files.  This module writes both, from a walker of a `Batch`:

- `document(view)`: the EnergyMC<Any> field tree.  Every field the analysis reads is
  present, together with the method and bin state.  The RNG, the move plan, the save
  path and the plugin fields are left out: they describe one CPU process, not a walker
  of the batch.
- `write_yaml(doc, path)`: one `key: value` line per field, each value in YAML flow
  style with quoted keys (JSON apart from .nan / .inf), which PyYAML's safe_load and
  full_load read, as does any YAML 1.2 parser.
- `write_dat(doc, base)`: the text files parse-binning.py writes from such a
  document: -histogram, -energy-boundaries, -mean-energy, -mean-energy-squared, one
  per collected datum (-pressure for the WCA fluid), -lnw, and -system.
- `movie_times` / `run_with_movie`: the geometric movie frames of
  src/mc/plugin.rs:447-477, each frame a document in the movie directory.
"""
import math
import os

import numpy as np

from sadmc_gb300 import ISING, LJ, WCA, SW, SAD, SAMC, WL, INV_T_WL, CANONICAL

_SYSTEM_TAG = {ISING: "Ising", LJ: "Lj", WCA: "Wca", SW: "Sw"}


class BatchWalker:
    """Walker w of a Batch, seen through the accessors the export reads."""

    def __init__(self, batch, w):
        self.batch, self.w = batch, w
        self.cfg = batch.cfg
        g = batch._geom[w]
        self.system = batch.cfg.system
        self.n = int(g.n)
        self.radius = float(g.radius)
        self.box = (float(g.box[0]), float(g.box[1]), float(g.box[2]))

    def bins(self):
        return self.batch.bins(self.w)

    def scalars(self):
        return self.batch.scalars(self.w)

    def state(self):
        return self.batch.state(self.w)

    def wl_hist(self):
        return self.batch.wl_hist(self.w)

    def extra(self):
        if self.system != WCA:
            return None
        return self.batch.extra(self.w)


# ---------------------------------------------------------------------------------
# the document

def _vec(p):
    return {"x": float(p[0]), "y": float(p[1]), "z": float(p[2])}


def _system(view, s):
    """The system field (any.rs:61-78): Ising ising.rs:20-29, Lj lj.rs:32-45, Wca
    wca.rs:23-32 and Sw optsquare.rs:24-31, with Cell optcell.rs:27-40."""
    E = float(s["energy"])
    st = view.state()
    if view.system == ISING:
        body = {"E": E, "N": int(view.n), "S": [int(v) for v in np.ravel(st)],
                "possible_change": None}
    elif view.system == LJ:
        body = {"E": E, "error": 0.0, "possible_change": "None",
                "positions": [_vec(p) for p in st],
                "max_radius_squared": view.radius * view.radius, "max_radius": view.radius}
    else:
        r_cut = 2.0 ** (1.0 / 6.0) if view.system == WCA else float(view.cfg.well_width)
        cell = {"box_diagonal": _vec(view.box), "r_cutoff": r_cut,
                "positions": [_vec(p) for p in st]}
        body = {"E": E, "cell": cell, "possible_change": "None"}
        if view.system == WCA:
            body["error"] = 0.0
    return {_SYSTEM_TAG[view.system]: body}


def _method(view, s):
    """The method field (energy.rs:213-243)."""
    c = view.cfg
    if c.method == SAD:
        return {"Sad": {"min_T": float(c.min_T), "too_lo": float(s["too_lo"]),
                        "too_hi": float(s["too_hi"]), "tL": int(s["tL"]), "tF": int(s["tF"]),
                        "num_states": int(s["num_states"]),
                        "highest_hist": int(s["highest_hist"]), "version": "Sad",
                        "latest_parameter": float(s["latest_parameter"])}}
    if c.method == SAMC:
        return {"Samc": {"t0": float(c.t0)}}
    if c.method in (WL, INV_T_WL):
        hist, min_energy = view.wl_hist()
        return {"WL": {"gamma": float(s["gamma"]), "lowest_hist": int(s["lowest_hist"]),
                       "highest_hist": int(s["wl_highest_hist"]),
                       "total_hist": int(s["total_hist"]),
                       "num_states": float(s["wl_num_states"]),
                       "hist": [int(v) for v in hist], "min_energy": float(min_energy),
                       "inv_t": c.method == INV_T_WL,
                       "min_gamma": float(c.min_gamma) if c.has_min_gamma else None}}
    if c.method == CANONICAL:
        return {"Canonical": {"temperature": float(c.T)}}
    raise ValueError(f"unknown method {c.method}")


def document(view):
    """The EnergyMC<Any> field tree of one walker (see the module docstring)."""
    s = view.scalars()
    b = view.bins()
    c = view.cfg
    extra = {}
    ex = view.extra()
    if ex is not None:
        count, total = ex
        if int(np.sum(count)) > 0:  # the reference creates a BinCounts at its first datum
            extra["pressure"] = {"total": [float(v) for v in total],
                                 "count": [int(v) for v in count]}
    bins = {"min": float(b["min"]), "width": float(b["width"]),
            "histogram": [int(v) for v in b["hist"]],
            "t_found": [int(v) for v in b["t_found"]],
            "lnw": [float(v) for v in b["lnw"]],
            "energy_total": [float(v) for v in b["sumE"]],
            "energy_squared_total": [float(v) for v in b["sumE2"]],
            "extra": extra}
    return {
        "system": _system(view, s),
        "method": _method(view, s),
        "moves": int(s["moves"]),
        "accepted_moves": int(s["accepted"]),
        "min_allowed_energy": float(c.min_allowed) if c.has_min_allowed else None,
        "max_allowed_energy": float(c.max_allowed) if c.has_max_allowed else None,
        "translation_scale": float(s["translation_scale"]),
        "acceptance_rate": float(s["acceptance_rate"]),
        "bins": bins,
        "have_visited_since_maxentropy": [bool(v) for v in b["visited"]],
        "round_trips": [int(v) for v in b["round_trips"]],
        "max_S": float(s["max_S"]),
        "max_S_index": int(s["max_S_index"]),
    }


# ---------------------------------------------------------------------------------
# YAML in flow style

def _yaml_float(x):
    if math.isnan(x):
        return ".nan"
    if math.isinf(x):
        return ".inf" if x > 0 else "-.inf"
    r = repr(float(x))
    if "e" in r and "." not in r.split("e")[0]:
        m, e = r.split("e")
        r = m + ".0e" + e  # YAML 1.1 resolvers want a point in the mantissa
    return r


def _yaml(v):
    if v is None:
        return "null"
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, int):
        return str(v)
    if isinstance(v, float):
        return _yaml_float(v)
    if isinstance(v, str):
        return '"' + v.replace("\\", "\\\\").replace('"', '\\"') + '"'
    if isinstance(v, dict):
        return "{" + ", ".join(f"{_yaml(str(k))}: {_yaml(x)}" for k, x in v.items()) + "}"
    if isinstance(v, (list, tuple)):
        return "[" + ", ".join(_yaml(x) for x in v) + "]"
    raise TypeError(f"cannot write {type(v)}")


def write_yaml(doc, path):
    """Write a document as one YAML mapping per top-level key (flow style values)."""
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        for k, v in doc.items():
            f.write(f"{k}: {_yaml(v)}\n")
    os.replace(tmp, path)  # atomic, as the reference's AtomicFile


# ---------------------------------------------------------------------------------
# the analysis text files

def excess_entropy(doc):
    """ln w made into an entropy estimate the way plotting/parse-binning.py:136-160 does:
    SAD extends it below too_lo with slope 1/min_T and above too_hi flat, both corrected
    by ln(hist / mean hist over the window); a Wang-Landau production run (gamma == 0)
    adds ln of its production histogram.  Shifted so the maximum is 0."""
    b = doc["bins"]
    lnw = np.array(b["lnw"], dtype=float)
    width, emin = b["width"], b["min"]
    E = emin + (np.arange(len(lnw)) + 0.5) * width
    m = doc["method"]
    if "Sad" in m:
        sad = m["Sad"]
        hist = np.array(b["histogram"], dtype=float)
        i_lo = int(np.abs(E - sad["too_lo"]).argmin())
        i_hi = int(np.abs(E - sad["too_hi"]).argmin())
        mean_hist = hist[i_lo:i_hi + 1].mean()
        lo, hi = E < sad["too_lo"], E > sad["too_hi"]
        with np.errstate(divide="ignore", invalid="ignore"):
            lnw[lo] = lnw[i_lo] + (E[lo] - sad["too_lo"]) / sad["min_T"] + np.log(hist[lo] / mean_hist)
            lnw[hi] = lnw[i_hi] + np.log(hist[hi] / mean_hist)
        lnw[~np.isfinite(lnw)] = 0.0
    elif "WL" in m and m["WL"]["gamma"] == 0:
        hist = wl_hist_on_bins(doc)
        pos = hist > 0
        lnw[pos] += np.log(hist[pos])
    return lnw - lnw.max()


def wl_hist_on_bins(doc):
    """The Wang-Landau histogram placed on the bins (it starts at its own min_energy)."""
    b, wl = doc["bins"], doc["method"]["WL"]
    out = np.zeros(len(b["lnw"]))
    h = np.array(wl["hist"], dtype=float)
    off = int(round((wl["min_energy"] - b["min"]) / b["width"]))
    for k, v in enumerate(h):
        if 0 <= off + k < len(out):
            out[off + k] = v
    return out


def system_summary(doc):
    """plotting/readsystem.py: kind, and volume, N and density for the WCA fluid."""
    sysd = doc["system"]
    out = {"kind": "unknown"}
    if "Wca" in sysd:
        a = sysd["Wca"]["cell"]["box_diagonal"]
        out["kind"] = "WCA"
        out["volume"] = a["x"] * a["y"] * a["z"]
        out["N"] = len(sysd["Wca"]["cell"]["positions"])
        out["density"] = out["N"] / out["volume"]
    return out


def write_dat(doc, base):
    """The text files of plotting/parse-binning.py:176-190 for one document.  Bins run
    upward from bins.min; the unbounded bins at either end are padded (histogram 0, mean
    energy NaN, ln w -inf); each collected datum is written high energy first, as there."""
    b = doc["bins"]
    n = len(b["lnw"])
    hist = np.array(b["histogram"], dtype=float)
    boundaries = b["min"] + np.arange(n + 1) * b["width"]
    with np.errstate(divide="ignore", invalid="ignore"):
        mean_e = np.array(b["energy_total"]) / hist
        mean_e2 = np.array(b["energy_squared_total"]) / hist
    pad = np.array([np.nan])
    np.savetxt(base + "-histogram.dat", np.concatenate([[0], hist, [0]]))
    np.savetxt(base + "-energy-boundaries.dat", boundaries)
    np.savetxt(base + "-mean-energy.dat", np.concatenate([pad, mean_e, pad]))
    np.savetxt(base + "-mean-energy-squared.dat", np.concatenate([pad, mean_e2, pad]))
    for name, bc in b["extra"].items():
        with np.errstate(divide="ignore", invalid="ignore"):
            mean = np.array(bc["total"]) / np.array(bc["count"], dtype=float)
        np.savetxt(base + f"-{name}.dat", np.concatenate([[-np.inf], mean, [-np.inf]])[::-1])
    s = excess_entropy(doc)
    s = s - s.max()
    s = s - np.log(np.sum(np.exp(s)))
    np.savetxt(base + "-lnw.dat", np.concatenate([[-np.inf], s, [-np.inf]]))
    write_yaml(system_summary(doc), base + "-system.dat")


# ---------------------------------------------------------------------------------
# movies

def movie_times(movie_time, max_moves):
    """Moves at which the movie plugin of plugin.rs:447-477 saves a frame, up to
    max_moves: the first move, then each next frame at the first (movie_time^k + 0.5)
    truncated that lies beyond the current move."""
    if movie_time is None or max_moves < 1:
        return []
    out, t, k = [1], 1, 0
    while True:
        k += 1
        nxt = int(movie_time ** k + 0.5)
        while nxt <= t:
            k += 1
            nxt = int(movie_time ** k + 0.5)
        if nxt > max_moves:
            return out
        out.append(nxt)
        t = nxt


def movie_dir(save_as):
    """save_as without its extension, the movie directory of plugin.rs:447-452."""
    return os.path.splitext(save_as)[0]


def run_with_movie(batch, moves, movie_time, save_as="walker-{walker:05d}.yaml"):
    """Run every walker of an initialised batch `moves` more moves, saving a frame of
    each walker at the movie times (counted on each walker's move counter, which all
    walkers of a batch share): `{movie_dir(save_as)}/{moves:014}.yaml`.  The final state
    is saved as save_as itself, as the reference's save plugin does at the end."""
    start = int(batch.scalars(0)["moves"])
    frames = [t for t in movie_times(movie_time, start + moves) if t > start]
    done = start
    for t in frames + [start + moves]:
        if t > done:
            batch.run(t - done)
            done = t
        if t in frames:
            for w in range(batch.W):
                d = movie_dir(save_as.format(walker=w))
                os.makedirs(d, exist_ok=True)
                write_yaml(document(BatchWalker(batch, w)), os.path.join(d, f"{t:014d}.yaml"))
    for w in range(batch.W):
        write_yaml(document(BatchWalker(batch, w)), save_as.format(walker=w))
    return frames
