"""Host logic of bench.py's roofline: the FP64 instruction count of the factored Q1 Jacobian+residual
assembly, against a brute-force enumeration of the free rows' entries (rows on x = 0 and x = 1 are
Dirichlet).  Box cells: a multiply and an FMA per entry.  Cubic cells: none for the axis-neighbour entries
(coefficient +0), an FMA for each other entry (the entries are exact sums of scaled conductances) and one
multiply per cell (the scaling)."""
import itertools

import pytest

import bench


def _brute(n, hi):
    nn = [c + 1 for c in n]
    h = [hi[k] / n[k] for k in range(3)]
    cubic = h[0] == h[1] == h[2]
    count = 0
    for iz, iy, ix in itertools.product(range(nn[2]), range(nn[1]), range(nn[0])):
        if ix == 0 or ix == nn[0] - 1:
            continue
        for dz, dy, dx in itertools.product((-1, 0, 1), repeat=3):
            jx, jy, jz = ix + dx, iy + dy, iz + dz
            if not (0 <= jx < nn[0] and 0 <= jy < nn[1] and 0 <= jz < nn[2]):
                continue
            if cubic and (dx != 0) + (dy != 0) + (dz != 0) == 1:
                continue
            count += 1 if cubic else 2
    return count + (n[0] * n[1] * n[2] if cubic else 0)


@pytest.mark.parametrize("n,hi", [((4, 4, 4), (1.0, 1.0, 1.0)), ((5, 3, 4), (1.0, 1.0, 1.0)),
                                  ((6, 6, 6), (0.5, 0.5, 0.5)), ((3, 7, 2), (0.3, 0.7, 0.2))])
def test_fp64_instruction_count(n, hi):
    cfg = dict(n=n, lo=(0.0, 0.0, 0.0), hi=hi)
    assert bench.fp64_instructions(cfg) == _brute(n, hi)


def test_targets_summary_survives_failed_extras():
    """The bench line's last key is built from whatever the run produced: extras that failed (an "error"
    entry) or were skipped leave their targets out instead of breaking the line."""
    import json

    out = {"ms_per_step": 0.1373, "mixed": {"ms_per_step": 0.142},
           "roofline": {"frac": 0.67, "fp64_pipe": {"frac": 0.63}}, "e2e": {"value": 8.4e8},
           "solve": {"error": "RuntimeError: x"}, "c3": {"error": "MrgError: y"}, "general": {},
           "c4": {"error": "z"}, "c5": {"error": "w"}}
    t = bench.targets_summary(out)
    json.dumps(t)
    assert t["c2_fp64_jacres_ms"] == 0.1373 and t["c2_mixed_jacres_ms"] == 0.142
    for k in ("c3", "c4", "c5", "general_noaffine"):
        assert k not in t
    assert bench.targets_summary({"ms_per_step": 1.0})["c2_fp64_jacres_ms"] == 1.0
