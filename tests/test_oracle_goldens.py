"""The oracle reproduces the reference's regression goldens (6 significant digits).

Each case restates one regression/thermal/<case>/input.yaml of MrHyDE; the gold L2 errors are in
tests/golden/regression_goldens.json (extracted by tests/golden/make_goldens.py).  These pin the
oracle's bases, quadrature, geometry, assembly, Dirichlet handling, Newton and PCG.
"""
import json
import math
import os

import numpy as np
import pytest

from tests.cases import oracle_problem

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "regression_goldens.json")))


def _num(s):
    return float(eval(str(s).replace("^", "**"), {"pi": math.pi}))


def side_values(xyz, expr):
    """Evaluates a boundary-data expression of the case's input.yaml at side points [n, 3]."""
    env = {"sin": np.sin, "cos": np.cos, "exp": np.exp, "pi": math.pi,
           "x": xyz[:, 0], "y": xyz[:, 1], "z": xyz[:, 2]}
    return np.asarray(eval(expr.replace("^", "**"), {"__builtins__": {}}, env), dtype=np.float64) * np.ones(len(xyz))


def _sig6(x):
    return float(f"{x:.6g}")


@pytest.mark.parametrize("case", sorted(GOLD))
def test_oracle_matches_regression_gold(case):
    g = GOLD[case]
    d = g["dirichlet"]
    dirichlet = ("const", d[1]) if d[0] == "const" else (d[0], d[1], d[2])
    cfg = dict(dim=g["dim"], order=g["order"], n=tuple(g["n"]), quad_order=g["quad_order"],
               source=(g["source"][0], _num(g["source"][1]), _num(g["source"][2])), dirichlet=dirichlet,
               dirichlet_faces=g.get("dirichlet_faces", 63 if g["dim"] == 3 else 15),
               workset_size=g.get("workset_size", 0))
    P = oracle_problem(cfg)
    for face, expr in g.get("neumann", []):
        P.set_face_bc(face, 1, side_values(P.side_points(face), expr))
    u = P.set_dirichlet(np.zeros(P.ndof))
    u, rc, st = P.newton(u, nltol=1e-12, maxiter=4, lintol=1e-13, linmaxiter=100000, nthreads=2)
    assert rc == 0
    l2, h1 = P.errors(u, _num(g["exact"][0]), _num(g["exact"][1]))
    assert _sig6(l2) == g["l2_T"], (case, l2)
    if "l2_gradT" in g:
        assert _sig6(h1) == g["l2_gradT"], (case, h1)
