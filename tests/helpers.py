"""Shared set-up for the GPU parity tests: the same seeded inputs for the CUDA batch and
the FP64 oracle walkers."""
import numpy as np

BIN_KEYS = ["lnw", "hist", "t_found", "sumE", "sumE2", "round_trips", "visited"]
EXACT_SCALARS = ["moves", "accepted", "acceptance_rate", "translation_scale", "method_kind",
                 "too_lo", "too_hi", "tL", "tF", "num_states", "highest_hist",
                 "latest_parameter", "gamma", "lowest_hist", "wl_highest_hist", "total_hist",
                 "wl_num_states", "min_energy", "t0", "max_S", "max_S_index", "energy"]

METHOD_KW = {
    "sad": dict(method=0, min_T=0.2),
    "samc": dict(method=1, t0=500.0),
    "wl": dict(method=2),
    "inv_t_wl": dict(method=3),
    "canonical": dict(method=4, T=3.0),
}


def ising_spins(L, seed):
    return np.where(np.random.default_rng(seed).random(L * L) < 0.5, -1.0, 1.0)


def assert_bins_equal(gb, ob, keys=BIN_KEYS, label=""):
    assert gb["min"] == ob["min"], label
    assert gb["width"] == ob["width"], label
    for k in keys:
        a, b = np.asarray(gb[k]), np.asarray(ob[k])
        assert a.shape == b.shape, (label, k, a.shape, b.shape)
        if not np.array_equal(a, b):
            bad = np.nonzero(a != b)[0][:5]
            raise AssertionError(f"{label} bins[{k}] differ at {bad}: gpu {a[bad]} oracle {b[bad]}")


COMMON_SCALARS = ["moves", "accepted", "acceptance_rate", "translation_scale", "method_kind",
                  "max_S", "max_S_index", "energy"]
METHOD_SCALARS = {  # Method fields per variant (energy.rs:212-244)
    0: ["too_lo", "too_hi", "tL", "tF", "num_states", "highest_hist", "latest_parameter"],
    1: ["t0"],
    2: ["gamma", "lowest_hist", "wl_highest_hist", "total_hist", "wl_num_states", "min_energy"],
    4: [],
}


def assert_scalars_equal(gs, os_, keys=None, label=""):
    if keys is None:
        keys = COMMON_SCALARS + METHOD_SCALARS[int(os_["method_kind"])]
    for k in keys:
        assert gs[k] == os_[k], f"{label} scalar {k}: gpu {gs[k]!r} oracle {os_[k]!r}"


def sphere_configs(n, radius, count, seed, dmin=0.8):
    """`count` LJ-cluster configurations for large batches: atoms uniform in the sphere,
    each redrawn while closer than dmin to an earlier one (the rule of the LJ workloads),
    from one seeded numpy generator.  Far quicker than the oracle's initialiser, which
    follows the reference's (lj.rs:126-204) at about 0.3 s per configuration."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        pts = np.empty((n, 3))
        k = 0
        while k < n:
            p = rng.uniform(-radius, radius, 3)
            if p @ p >= radius * radius:
                continue
            if k and np.min(((pts[:k] - p) ** 2).sum(axis=1)) < dmin * dmin:
                continue
            pts[k] = p
            k += 1
        out.append(pts)
    return out


def lj_configs(oracle, n, radius, seeds):
    out = []
    for s in seeds:
        pos, ok = oracle.init_lj(n, radius, s)
        assert ok
        out.append(pos)
    return out


class OracleView:
    """An oracle walker seen through the accessors of export.BatchWalker."""

    def __init__(self, walker):
        self.wk = walker
        self.cfg = walker.cfg
        self.system = walker.cfg.system
        self.n = int(walker.cfg.n)
        self.radius = float(walker.cfg.radius)
        self.box = tuple(float(x) for x in walker.cfg.box)

    def bins(self):
        return self.wk.bins()

    def scalars(self):
        return self.wk.scalars()

    def state(self):
        return self.wk.state()

    def wl_hist(self):
        return self.wk.wl_hist()

    def extra(self):
        return self.wk.extra() if self.system == 2 else None


def read_flow_yaml(path):
    """Read a file written by export.write_yaml (its values are JSON apart from the
    YAML spellings of non-finite floats)."""
    import json
    out = {}
    with open(path) as f:
        for line in f:
            k, v = line.rstrip("\n").split(": ", 1)
            v = v.replace("-.inf", "-Infinity").replace(".inf", "Infinity").replace(".nan", "NaN")
            out[k] = json.loads(v)
    return out
