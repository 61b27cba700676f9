"""Extracts the reference's regression gold values used to pin the oracle.

Reads MrHyDE's regression/thermal/<case>/mrhyde.gold (and input.yaml for the case parameters,
transcribed by hand into CASES below) from a checkout of the reference and writes
regression_goldens.json next to this script.  Run once in a container that has the reference;
the JSON is what the tests read.

    python tests/golden/make_goldens.py /path/to/MrHyDE
"""
import json
import os
import re
import sys

# case -> parameters of its input.yaml, in the oracle's vocabulary
CASES = {
    "3D_verification": dict(dim=3, order=1, n=[10, 10, 10], quad_order=2, source=["sinprod", "12*pi^2", "2*pi"],
                            dirichlet=["const", 0.0], exact=["1", "2*pi"]),
    "2D_verification": dict(dim=2, order=1, n=[40, 40], quad_order=2, source=["sinprod", "8*pi^2", "2*pi"],
                            dirichlet=["const", 0.0], exact=["1", "2*pi"]),
    "2D_verification_highorder": dict(dim=2, order=4, n=[10, 10], quad_order=8,
                                      source=["sinprod", "8*pi^2", "2*pi"], dirichlet=["const", 0.0],
                                      exact=["1", "2*pi"]),
    "2D_verification_nonzeroDBC": dict(dim=2, order=1, n=[40, 40], quad_order=2, source=["sinprod", "2", "1"],
                                       dirichlet=["sinprod_l2", 1.0, 1.0], exact=["1", "1"]),
    "3D-Multiblock": dict(dim=3, order=1, n=[10, 10, 10], quad_order=2, source=["sinprod", "12*pi^2", "2*pi"],
                          dirichlet=["const", 0.0], exact=["1", "2*pi"], workset_size=1),
    # strong Dirichlet on left/right only (faces x-, x+), Neumann data on bottom (y-) / top (y+)
    "2D_mixed_bcs": dict(dim=2, order=1, n=[40, 40], quad_order=2, source=["sinprod", "8*pi^2", "2*pi"],
                         dirichlet=["const", 0.0], dirichlet_faces=3, exact=["1", "2*pi"],
                         neumann=[[2, "-2*pi*sin(2*pi*x)*cos(2*pi*y)"], [3, "2*pi*sin(2*pi*x)*cos(2*pi*y)"]]),
}


def main(ref):
    out = {}
    for case, params in CASES.items():
        gold = open(os.path.join(ref, "regression", "thermal", case, "mrhyde.gold")).read()
        l2 = re.findall(r"L2 norm of the error for T = ([0-9.eE+-]+)", gold)
        grad = re.findall(r"L2 norm of the error for grad\(T\) = ([0-9.eE+-]+)", gold)
        rec = dict(params)
        rec["source_file"] = f"regression/thermal/{case}/mrhyde.gold"
        rec["l2_T"] = float(l2[0])
        if grad:
            rec["l2_gradT"] = float(grad[0])
        out[case] = rec
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "regression_goldens.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print(path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_goldens.py <path of the MrHyDE source tree>")
    main(sys.argv[1])
