"""Exodus II writer (host only): structure, coordinates, element orientation and values read back."""
import numpy as np
import pytest

from mrhyde_gb300.exodus import ExodusWriter, linear_connectivity, node_coordinates


def _read(path):
    from scipy.io import netcdf_file

    return netcdf_file(path, "r", mmap=False)


def _chars(a):
    return ["".join(c.decode() for c in row if c) for row in a]


def _hex_volume(x, c):
    """Volume of a trilinear HEX8 (Exodus order) by 2x2x2 Gauss quadrature of det(dx/dxi)."""
    pts = [-1 / np.sqrt(3), 1 / np.sqrt(3)]
    sgn = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]])
    vol = 0.0
    for a in pts:
        for b in pts:
            for g in pts:
                xi = np.array([a, b, g])
                dN = np.zeros((8, 3))
                for i in range(8):
                    f = (1 + sgn[i] * xi) / 2
                    for k in range(3):
                        dN[i, k] = sgn[i, k] / 2 * np.prod([f[m] for m in range(3) if m != k])
                vol += np.linalg.det(x[c - 1].T @ dN)
    return vol


@pytest.mark.parametrize("order", [1, 2])
def test_hex_mesh_round_trip(tmp_path, order):
    from tests.cases import perturbed_vertices

    n = (3, 2, 4)
    vc = perturbed_vertices(3, n, (0, 0, 0), (1.5, 1.0, 2.0), 0.2, 5)
    nn = [order * k + 1 for k in n]
    nnodes = int(np.prod(nn))
    ncell = int(np.prod(n))
    u = np.random.default_rng(1).standard_normal(nnodes)
    kap = np.arange(ncell, dtype=np.float64) + 0.5
    path = str(tmp_path / "sol.exo")
    with ExodusWriter(path, dim=3, order=order, n=n, lo=(0, 0, 0), hi=(1.5, 1.0, 2.0), vertex_coords=vc,
                      nodal_names=("T",), elem_names=("kappa",)) as w:
        w.write_step(0.0, {"T": u}, {"kappa": kap})
        w.write_step(1.0, {"T": 2 * u}, {"kappa": kap})
    f = _read(path)
    assert f.dimensions["num_nodes"] == nnodes
    assert f.dimensions["num_elem"] == ncell * order ** 3
    assert f.floating_point_word_size == 8
    assert _chars(f.variables["name_nod_var"][:]) == ["T"]
    assert _chars(f.variables["coor_names"][:]) == ["x", "y", "z"]
    assert f.variables["connect1"].elem_type == b"HEX8"
    np.testing.assert_array_equal(f.variables["time_whole"][:], [0.0, 1.0])
    np.testing.assert_array_equal(f.variables["vals_nod_var1"][1], 2 * u)
    x = np.stack([f.variables[f"coord{a}"][:] for a in "xyz"], axis=1)
    # vertex nodes carry the given vertex coordinates
    V = vc.reshape(n[2] + 1, n[1] + 1, n[0] + 1, 3)
    Xg = x.reshape(nn[2], nn[1], nn[0], 3)
    np.testing.assert_allclose(Xg[::order, ::order, ::order], V, rtol=0, atol=1e-15)
    conn = f.variables["connect1"][:]
    vols = [_hex_volume(x, c) for c in conn]
    assert min(vols) > 0  # Exodus HEX8 order gives positive orientation
    np.testing.assert_allclose(sum(vols), np.sum([_hex_volume(x, c) for c in conn]))
    # element values: each sub-cell carries its cell's value
    ev = f.variables["vals_elem_var1eb1"][0]
    _, parent = linear_connectivity(3, order, n)
    np.testing.assert_array_equal(ev, kap[parent])
    f.close()


def test_quad_mesh_uniform_coordinates(tmp_path):
    path = str(tmp_path / "q.exo")
    with ExodusWriter(path, dim=2, order=1, n=(4, 3), lo=(0.0, -1.0), hi=(2.0, 0.5)) as w:
        w.write_step(0.5, {"T": np.arange(20.0)})
    f = _read(path)
    assert f.variables["connect1"].elem_type == b"QUAD4"
    x, y = f.variables["coordx"][:], f.variables["coordy"][:]
    np.testing.assert_allclose(x[:5], np.linspace(0, 2, 5))
    np.testing.assert_allclose(y[::5], np.linspace(-1, 0.5, 4))
    c = f.variables["connect1"][:] - 1
    # counter-clockwise: positive signed area of every quad
    area = 0.5 * sum(x[c[:, k]] * y[c[:, (k + 1) % 4]] - x[c[:, (k + 1) % 4]] * y[c[:, k]] for k in range(4))
    assert np.all(area > 0)
    f.close()


def test_node_coordinates_uniform_match_linspace():
    xyz = node_coordinates(3, 2, (2, 2, 2), (0, 0, 0), (1, 2, 3))
    assert xyz.shape == (125, 3)
    np.testing.assert_allclose(xyz[:5, 0], np.linspace(0, 1, 5))
    np.testing.assert_allclose(xyz[::25, 2], np.linspace(0, 3, 5))


def test_wrong_sizes_rejected(tmp_path):
    with ExodusWriter(str(tmp_path / "e.exo"), dim=2, order=1, n=(2, 2), elem_names=("k",)) as w:
        with pytest.raises(ValueError):
            w.write_step(0.0, {"T": np.zeros(8)}, {"k": np.zeros(4)})
        with pytest.raises(ValueError):
            w.write_step(0.0, {"T": np.zeros(9)}, {"k": np.zeros(3)})


@pytest.mark.gpu
def test_device_solution_written(cuda, tmp_path):
    """A solved problem's device solution and per-cell kappa written through the Problem handle."""
    import torch

    from mrhyde_gb300 import Problem, SolverManager
    from mrhyde_gb300.exodus import write_solution

    kap = np.exp(0.5 * np.random.default_rng(3).standard_normal(6 * 5 * 4))
    P = Problem(dim=3, order=1, n=(6, 5, 4), kappa=kap, dirichlet_faces=3)
    u = P.new_vector()
    SolverManager(P, nonlinear_tol=1e-10, linear_tol=1e-12).nonlinearSolver(u)
    path = str(tmp_path / "dev.exo")
    write_solution(path, P, u, time=1.0, elem={"kappa": kap})
    f = _read(path)
    np.testing.assert_array_equal(f.variables["vals_nod_var1"][0], u.cpu().numpy())
    np.testing.assert_array_equal(f.variables["vals_elem_var1eb1"][0], kap)
    f.close()
    assert torch.isfinite(u).all()
