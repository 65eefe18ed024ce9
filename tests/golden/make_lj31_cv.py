"""Writes tests/golden/lj31_cv_reference.json from the reference's own LJ31 heat-capacity
curves (the CSV files at the top of droundy/sad-monte-carlo).  Run from the repository
root with the reference checked out at REF (default /root/reference):

    python tests/golden/make_lj31_cv.py [REF]

Each curve is stored as (T, Cv) in the reference's units (k_B = epsilon = 1).  The
transform is the one plotting/final_heat_capacity.py:29-53 applies before plotting: the
per-atom curves that include the kinetic 3/2 (LJ31_Cv_Reference, _3, _4) become the
configurational heat capacity of the cluster, (Cv - 3/2) * 31; the RESTMC (_alt) and
t-REM (tRem_Ref) curves are already in that form.  The comments at
final_heat_capacity.py:141-156 give the confining radius Rc = 2.5 sigma for RESTMC and
EMC (t-REM comes from the RESTMC paper); the curves agree to a few per cent below
T = 0.25 and split by about 12 % at the melting peak (T ~ 0.33), where the container
matters: RESTMC and t-REM near 120, REM and EMC near 134.
"""
import json
import os
import sys

import numpy as np

CURVES = [  # file, per-atom with the kinetic term, method, confining radius
    ("LJ31_Cv_Reference.csv", True, "REM", None),
    ("LJ31_Cv_Reference_alt.csv", False, "RESTMC", 2.5),
    ("LJ31_Cv_Reference_3.csv", True, "MCET", None),
    ("LJ31_Cv_Reference_4.csv", True, "EMC", 2.5),
    ("tRem_Ref.csv", False, "t-REM", 2.5),  # the RESTMC paper
]


def main(ref):
    out = {"source": "droundy/sad-monte-carlo top-level CSV files; transform of "
                     "plotting/final_heat_capacity.py:29-53",
           "ground_state": -133.586422,
           "ground_state_source": "big-lj-31.sh:16 (comment), lj/convergence-for-proposal.py:144",
           "T_peak": 0.025, "T_peak_source": "lj/heat_capacity.py:9",
           "curves": {}}
    for name, per_atom, method, radius in CURVES:
        d = np.loadtxt(os.path.join(ref, name), delimiter=",")
        d = d[np.argsort(d[:, 0])]
        cv = (d[:, 1] - 1.5) * 31 if per_atom else d[:, 1]
        out["curves"][method] = {"file": name, "radius": radius,
                                 "T": [float(x) for x in d[:, 0]], "Cv": [float(x) for x in cv]}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lj31_cv_reference.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
