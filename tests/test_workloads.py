"""Host logic of the bench and test workloads (mrhyde_gb300/workloads.py): the non-affine meshes keep the
box's boundary vertices, move every interior vertex by at most amp * h per axis, order vertices with x
fastest, and are reproducible from their seed; the general-geometry configurations carry the box
configurations' coefficients."""
import numpy as np
import pytest

from mrhyde_gb300 import workloads as W


def _box(n, lo, hi):
    d = len(n)
    axes = [np.linspace(lo[k], hi[k], n[k] + 1) for k in range(d)]
    idx = np.indices([n[k] + 1 for k in reversed(range(d))]).reshape(d, -1)[::-1]  # x fastest
    return np.stack([axes[k][idx[k]] for k in range(d)], axis=1), idx.T


@pytest.mark.parametrize("n,lo,hi", [((4, 3), (0.0, 0.0), (1.0, 2.0)), ((3, 4, 2), (0.0, -1.0, 0.5), (1.0, 1.0, 1.0))])
def test_perturbed_vertices_move_interior_only(n, lo, hi):
    amp = 0.2
    v = W.perturbed_vertices(n, amp, 7, lo=lo, hi=hi)
    box, idx = _box(n, lo, hi)
    assert v.shape == box.shape
    interior = np.all((idx > 0) & (idx < np.array(n)), axis=1)
    np.testing.assert_array_equal(v[~interior], box[~interior])
    h = np.array([(hi[k] - lo[k]) / n[k] for k in range(len(n))])
    d = np.abs(v[interior] - box[interior])
    assert np.all(d <= amp * h + 1e-15) and np.all(d.max(axis=0) > 0)
    np.testing.assert_array_equal(v, W.perturbed_vertices(n, amp, 7, lo=lo, hi=hi))
    assert not np.array_equal(v, W.perturbed_vertices(n, amp, 8, lo=lo, hi=hi))


def test_general_configs_keep_box_coefficients():
    g1, b1 = W.c1_general(seed=1, n=16), W.c1(seed=1, n=16)
    assert g1["vertex_coords"].shape == (17 * 17, 2)
    for k in ("dim", "order", "n", "kind", "source", "dirichlet_faces", "dirichlet"):
        assert g1[k] == b1[k]
    np.testing.assert_array_equal(g1["kappa"], b1["kappa"])
    g2, b2 = W.c2_general(seed=2, n=8), W.c2(seed=2, n=8)
    assert g2["vertex_coords"].shape == (9 ** 3, 3)
    np.testing.assert_array_equal(g2["kappa"], b2["kappa"])
