"""Exodus II output of nodal and element fields on the structured mesh.

The reference writes its solution for visualisation through the STK mesh's Exodus writer
(PostprocessManager::writeSolution, src/managers/postprocess/postprocessManager_exodus.hpp:14-671, which
ends in MeshInterface::writeToExodus, src/interfaces/mesh/meshInterface_exodus.hpp:225-240): one
element block, the node coordinates, nodal solution fields ("T" for the thermal module) and element
fields, one record per output time.  This module writes the same content as an Exodus II file
(netCDF-3 64-bit-offset container, written with scipy.io.netcdf_file):

* dimensions len_string, len_line, four, len_name, time_step (unlimited), num_dim, num_nodes, num_elem,
  num_el_blk = 1, num_el_in_blk1, num_nod_per_el1, num_nod_var, num_elem_var;
* variables time_whole, coordx/coordy/coordz, coor_names, eb_status, eb_prop1 (attribute name "ID"),
  eb_names, connect1 (attribute elem_type), name_nod_var, vals_nod_var<k>, name_elem_var, elem_var_tab,
  vals_elem_var<k>eb1;
* global attributes api_version, version, floating_point_word_size = 8, file_size = 1,
  maximum_name_length = 32, int64_status = 0, title.

Elements are linear (QUAD4 / HEX8, Exodus node order: the bottom face counter-clockwise seen from
above, then the top face).  A Q2 mesh is written on its node grid, i.e. every Q2 cell as 2^dim linear
sub-cells that carry the cell's element values, so nodal values are exact and no HEX27 ordering is
needed.  Node numbering follows the library's canonical numbering (x fastest), 1-based in connect1.
"""
from __future__ import annotations

import numpy as np

LEN_NAME = 33


def _np(a):
    try:
        import torch

        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except ImportError:
        pass
    return np.asarray(a)


def _names(names, width=LEN_NAME):
    out = np.zeros((len(names), width), dtype="S1")
    for i, nm in enumerate(names):
        b = nm.encode()[: width - 1]
        out[i, : len(b)] = np.frombuffer(b, dtype="S1")
    return out


def node_coordinates(dim, order, n, lo, hi, vertex_coords=None):
    """Coordinates [n_nodes, dim] of the order-p node grid (x fastest); with vertex coordinates the nodes
    of each cell are the images of the equispaced reference nodes under the cell's (bi/tri)linear map."""
    n = tuple(int(v) for v in n[:dim])
    nn = [order * n[k] + 1 for k in range(dim)]
    if vertex_coords is None:
        axes = [np.linspace(lo[k], hi[k], nn[k]) for k in range(dim)]
        grids = np.meshgrid(*reversed(axes), indexing="ij")  # slowest axis first
        return np.stack([g.reshape(-1) for g in reversed(grids)], axis=1)
    V = np.asarray(vertex_coords, dtype=np.float64).reshape(*[n[k] + 1 for k in reversed(range(dim))], dim)
    idx = np.meshgrid(*[np.arange(m) for m in reversed(nn)], indexing="ij")
    idx = [i.reshape(-1) for i in reversed(idx)]  # ix, iy(, iz) per node
    cell = [np.minimum(idx[k] // order, n[k] - 1) for k in range(dim)]
    t = [(idx[k] - order * cell[k]) / order for k in range(dim)]  # local coordinate in [0, 1]
    out = np.zeros((len(idx[0]), dim))
    for corner in range(2 ** dim):
        bits = [(corner >> k) & 1 for k in range(dim)]
        wgt = np.ones(len(idx[0]))
        for k in range(dim):
            wgt *= t[k] if bits[k] else 1.0 - t[k]
        vi = tuple((cell[k] + bits[k]) for k in reversed(range(dim)))
        out += wgt[:, None] * V[vi]
    return out


def linear_connectivity(dim, order, n):
    """1-based QUAD4 / HEX8 connectivity of the sub-cells of the node grid, and for each sub-cell the
    index of the order-p cell that contains it."""
    n = tuple(int(v) for v in n[:dim])
    m = [order * n[k] for k in range(dim)]        # sub-cells per axis
    nn = [m[k] + 1 for k in range(dim)]
    grid = np.meshgrid(*[np.arange(c) for c in reversed(m)], indexing="ij")
    sc = [g.reshape(-1) for g in reversed(grid)]  # sub-cell coordinates, x fastest
    def node(dx, dy, dz=0):
        i = (sc[0] + dx) + nn[0] * (sc[1] + dy)
        if dim == 3:
            i = i + nn[0] * nn[1] * (sc[2] + dz)
        return i + 1
    if dim == 2:
        conn = np.stack([node(0, 0), node(1, 0), node(1, 1), node(0, 1)], axis=1)
    else:
        conn = np.stack([node(0, 0, 0), node(1, 0, 0), node(1, 1, 0), node(0, 1, 0),
                         node(0, 0, 1), node(1, 0, 1), node(1, 1, 1), node(0, 1, 1)], axis=1)
    parent = sc[0] // order + n[0] * (sc[1] // order)
    if dim == 3:
        parent = parent + n[0] * n[1] * (sc[2] // order)
    return conn.astype(np.int32), parent


class ExodusWriter:
    """Exodus II file of one structured problem; write_step() appends one output time."""

    def __init__(self, path, problem=None, *, dim=None, order=None, n=None, lo=None, hi=None, vertex_coords=None,
                 nodal_names=("T",), elem_names=(), title="mrhyde_gb300 solution"):
        from scipy.io import netcdf_file

        if problem is not None:
            dim, order, n = problem.dim, problem.order, problem.n
            lo, hi, vertex_coords = problem.lo, problem.hi, problem.vertex_coords
        lo = tuple(lo) if lo is not None else (0.0,) * dim
        hi = tuple(hi) if hi is not None else (1.0,) * dim
        self.dim, self.order, self.n = dim, order, tuple(n[:dim])
        xyz = node_coordinates(dim, order, n, lo, hi, vertex_coords)
        conn, self.parent = linear_connectivity(dim, order, n)
        self.n_nodes, self.n_elem = xyz.shape[0], conn.shape[0]
        self.n_cells = int(np.prod(self.n))
        self.nodal_names, self.elem_names = list(nodal_names), list(elem_names)
        f = self.f = netcdf_file(path, "w", version=2)
        f.api_version = np.float32(8.0)
        f.version = np.float32(8.0)
        f.floating_point_word_size = np.int32(8)
        f.file_size = np.int32(1)
        f.maximum_name_length = np.int32(32)
        f.int64_status = np.int32(0)
        f.title = title
        # the record (unlimited) dimension is created first, as the netCDF-3 writer requires
        for name, size in (("time_step", None), ("len_string", 33), ("len_line", 81), ("four", 4),
                           ("len_name", LEN_NAME), ("num_dim", dim), ("num_nodes", self.n_nodes),
                           ("num_elem", self.n_elem), ("num_el_blk", 1), ("num_el_in_blk1", self.n_elem),
                           ("num_nod_per_el1", conn.shape[1])):
            f.createDimension(name, size)
        f.createVariable("time_whole", "d", ("time_step",))
        v = f.createVariable("eb_status", "i", ("num_el_blk",))
        v[:] = 1
        v = f.createVariable("eb_prop1", "i", ("num_el_blk",))
        v[:] = 1
        v.name = "ID"
        f.createVariable("eb_names", "c", ("num_el_blk", "len_name"))[:] = _names(["eblock-0_0"])
        for k, ax in enumerate("xyz"[:dim]):
            f.createVariable("coord" + ax, "d", ("num_nodes",))[:] = xyz[:, k]
        f.createVariable("coor_names", "c", ("num_dim", "len_name"))[:] = _names(list("xyz"[:dim]))
        v = f.createVariable("connect1", "i", ("num_el_in_blk1", "num_nod_per_el1"))
        v[:] = conn
        v.elem_type = "QUAD4" if dim == 2 else "HEX8"
        if self.nodal_names:
            f.createDimension("num_nod_var", len(self.nodal_names))
            f.createVariable("name_nod_var", "c", ("num_nod_var", "len_name"))[:] = _names(self.nodal_names)
            for k in range(len(self.nodal_names)):
                f.createVariable(f"vals_nod_var{k + 1}", "d", ("time_step", "num_nodes"))
        if self.elem_names:
            f.createDimension("num_elem_var", len(self.elem_names))
            f.createVariable("name_elem_var", "c", ("num_elem_var", "len_name"))[:] = _names(self.elem_names)
            f.createVariable("elem_var_tab", "i", ("num_el_blk", "num_elem_var"))[:] = np.ones(
                (1, len(self.elem_names)), np.int32)
            for k in range(len(self.elem_names)):
                f.createVariable(f"vals_elem_var{k + 1}eb1", "d", ("time_step", "num_el_in_blk1"))
        self.steps = 0

    def write_step(self, time, nodal=None, elem=None):
        """nodal: {name: values per node (canonical numbering)}; elem: {name: values per cell of the
        problem}; arrays may be torch tensors on the device."""
        f, k = self.f, self.steps
        f.variables["time_whole"][k] = float(time)
        nodal = nodal or {}
        elem = elem or {}
        for i, nm in enumerate(self.nodal_names):
            a = _np(nodal[nm]).astype(np.float64).reshape(-1)
            if a.size != self.n_nodes:
                raise ValueError(f"nodal field {nm!r}: {a.size} values for {self.n_nodes} nodes")
            f.variables[f"vals_nod_var{i + 1}"][k, :] = a
        for i, nm in enumerate(self.elem_names):
            a = _np(elem[nm]).astype(np.float64).reshape(-1)
            if a.size != self.n_cells:
                raise ValueError(f"element field {nm!r}: {a.size} values for {self.n_cells} cells")
            f.variables[f"vals_elem_var{i + 1}eb1"][k, :] = a[self.parent]
        self.steps += 1
        f.flush()

    def close(self):
        if self.f is not None:
            self.f.close()
            self.f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def write_solution(path, problem, u, time=0.0, name="T", elem=None):
    """One-step file: nodal field `name` = u, optional element fields {name: per-cell values}."""
    elem = elem or {}
    with ExodusWriter(path, problem, nodal_names=(name,), elem_names=tuple(elem)) as w:
        w.write_step(time, {name: u}, elem)
