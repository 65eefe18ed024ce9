"""CPU checks of the C ABI: the library builds for sm_103a, loads, and exports every
function that include/sadmc_gpu.h declares (no compute call is made without a GPU)."""
import ctypes
import os
import re

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(REPO, "include", "sadmc_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int32_t|const char\*)\s+(sadmc_\w+)\(", text, re.M)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ["sadmc_create", "sadmc_destroy", "sadmc_upload_state", "sadmc_initialize",
                 "sadmc_run", "sadmc_energy", "sadmc_compute_energy", "sadmc_plan_move_injected",
                 "sadmc_confirm", "sadmc_read_bins", "sadmc_counters", "sadmc_status"]:
        assert must in names


def test_library_exports_every_declared_symbol():
    import build as B
    lib_path = B.build()
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    lib.sadmc_version.restype = ctypes.c_int32
    assert lib.sadmc_version() >= 1


def test_rust_binding_covers_the_header():
    """The Rust binding's extern "C" blocks bind every declared entry point, and nothing
    else."""
    text = open(os.path.join(REPO, "include", "sadmc_gpu.rs")).read()
    bound = sorted(set(re.findall(r"pub fn (sadmc_\w+)\(", text)))
    assert bound == declared_functions(), (set(declared_functions()) ^ set(bound))


def test_no_oracle_in_product():
    """The product sources never include, link or load the oracle."""
    pkg = os.path.join(REPO, "sad-monte-carlo_gb300")
    for root, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".cu", ".cuh", ".cpp", ".h", ".py")):
                text = open(os.path.join(root, f)).read()
                for pat in (r"import\s+oracle", r"from\s+oracle", r"liboracle", r"#include\s+\S*oracle"):
                    assert not re.search(pat, text), (f, pat)


def test_create_refuses_a_target_rate_it_cannot_divide_by():
    """In acceptance-rate mode the translation-scale update divides by target_rate through
    its reciprocal; sadmc_create refuses a target rate that is not a positive number before
    it touches the device (so this runs without a GPU)."""
    import ctypes
    import sadmc_gb300 as G
    for bad in (0.0, -0.5, float("nan")):
        cfg = G.make_config(G.LJ, 4, 13, method=G.SAD, e_lo=-50.0, e_hi=0.0, target_rate=0.5)
        cfg.target_rate = bad
        geom = (G.Geometry * 4)()
        for g in geom:
            g.n, g.radius = 13, 2.5
        h = ctypes.c_void_p()
        rc = G.lib().sadmc_create(ctypes.byref(cfg), geom, ctypes.byref(h))
        assert rc == -1 and not h.value, (bad, rc)
        assert b"target_rate" in G.lib().sadmc_last_error()


def test_create_refuses_malformed_configurations_before_touching_the_device():
    """sadmc_create checks the configuration before it looks for a device (so this runs
    without a GPU): walker count, system, method and energy range."""
    import ctypes
    import sadmc_gb300 as G
    cases = [("n_walkers", 0, b"n_walkers"), ("system", 9, b"system"), ("method", 7, b"method"),
             ("e_hi", -60.0, b"e_hi")]
    for field, value, word in cases:
        cfg = G.make_config(G.LJ, 4, 13, method=G.SAD, e_lo=-50.0, e_hi=0.0)
        setattr(cfg, field, value)
        geom = (G.Geometry * 4)()
        for g in geom:
            g.n, g.radius = 13, 2.5
        h = ctypes.c_void_p()
        rc = G.lib().sadmc_create(ctypes.byref(cfg), geom, ctypes.byref(h))
        assert rc == -1 and not h.value, (field, rc)
        assert word in G.lib().sadmc_last_error(), (field, G.lib().sadmc_last_error())
