"""Host-side mirror of MrHyDE's AssemblyManager for the GB300 workset assembly path.

Names and argument meaning follow the reference (src/managers/assembly/assemblyManager.hpp:237-259,
:330-380): ``assembleJacRes`` adds the residual ``-res.val()`` into ``res`` and the Jacobian
``res.dx()`` into ``J`` (sum-into semantics; Dirichlet rows skipped, then ``J(d,d) = 1``);
``assembleRes`` adds only the residual.  All arrays are CUDA tensors owned by the caller; the work
is enqueued on the current torch stream and runs in the hand-written sm_103a kernels of
libmrhyde_gb.so.  There is no CPU path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L


def _stream(stream=None) -> int:
    if stream is None:
        stream = torch.cuda.current_stream()
    return stream.cuda_stream


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _require_cuda(t, name, dtype=None, numel=None):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise ValueError(f"{name} must have dtype {dtype}, got {t.dtype}")
    if numel is not None and t.numel() != numel:
        raise ValueError(f"{name} must have {numel} entries, got {t.numel()}")


@dataclass
class ProblemInfo:
    n_dofs: int
    n_cells: int
    nnz: int
    n_fixed: int
    nodes_per_cell: int
    qp_per_cell: int
    path: int


class Problem:
    """A structured Q1/Q2 problem: mesh, DOF map, CSR graph, coefficients and Dirichlet data.

    Mirrors what the reference's driver builds before the solve: the mesh factory
    (src/interfaces/mesh/meshInterface_construct.hpp:120-175), the DOF managers
    (src/interfaces/discretization/discretizationInterface_dof.hpp:14-243), the worksets
    (src/managers/assembly/assemblyManager_groups.hpp:14-286) and the overlapped graph
    (src/interfaces/linear_algebra/linearAlgebraInterface_construct.hpp:214-265).
    """

    def __init__(self, dim=3, order=1, n=(8, 8, 8), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), kind="thermal",
                 source=("const", 1.0, 0.0), kappa=1.0, dirichlet_faces=L.MRG_FACE_ALL, dirichlet=("const", 0.0),
                 quad_order=0, vertex_coords=None, stream=None):
        lib = L.lib()
        m = L.MeshDesc()
        m.dim, m.order = dim, order
        m.nx, m.ny = int(n[0]), int(n[1])
        m.nz = int(n[2]) if dim == 3 else 1
        for k in range(3):
            m.lo[k] = float(lo[k]) if k < len(lo) else 0.0
            m.hi[k] = float(hi[k]) if k < len(hi) else 1.0
        keep = []
        if vertex_coords is not None:
            vc = np.ascontiguousarray(vertex_coords, dtype=np.float64)
            keep.append(vc)
            m.vertex_coords = vc.ctypes.data_as(C.POINTER(C.c_double))
        ph = L.PhysicsDesc()
        ph.kind = {"thermal": L.MRG_THERMAL, "diffusion_1pu2": L.MRG_DIFFUSION_1PU2}[kind]
        skind, amp, freq = source
        ph.source_kind = {"const": L.MRG_SRC_CONST, "sinprod": L.MRG_SRC_SINPROD}[skind]
        ph.source_amp, ph.source_freq = float(amp), float(freq)
        if np.isscalar(kappa):
            ph.kappa_const = float(kappa)
        else:
            kc = np.ascontiguousarray(kappa, dtype=np.float64)
            keep.append(kc)
            ph.kappa_cell = kc.ctypes.data_as(C.POINTER(C.c_double))
            ph.kappa_const = 1.0
        ph.dirichlet_faces = int(dirichlet_faces)
        if dirichlet[0] == "const":
            ph.dirichlet_kind, ph.dirichlet_const = L.MRG_DBC_CONST, float(dirichlet[1])
        elif dirichlet[0] == "node":
            arr = np.ascontiguousarray(dirichlet[1], dtype=np.float64)
            keep.append(arr)
            ph.dirichlet_kind = L.MRG_DBC_NODE
            ph.dirichlet_node = arr.ctypes.data_as(C.POINTER(C.c_double))
        else:
            raise ValueError(f"unknown Dirichlet form {dirichlet[0]!r}")
        ph.quad_order = int(quad_order)
        h = C.c_void_p()
        if stream is None:
            L.check(lib.mrg_problem_create(C.byref(m), C.byref(ph), C.byref(h)), "mrg_problem_create")
        else:
            L.check(lib.mrg_problem_create_on_stream(C.byref(m), C.byref(ph), stream.cuda_stream, C.byref(h)),
                    "mrg_problem_create_on_stream")
        self._h = h
        self.dim, self.order = dim, order
        self.n = tuple(int(v) for v in n[:dim])
        self.lo = tuple(float(lo[k]) if k < len(lo) else 0.0 for k in range(dim))
        self.hi = tuple(float(hi[k]) if k < len(hi) else 1.0 for k in range(dim))
        self.vertex_coords = keep[0] if vertex_coords is not None else None  # host copy, x fastest
        info = L.ProblemInfo()
        L.check(lib.mrg_problem_get_info(self._h, C.byref(info)), "mrg_problem_get_info")
        self.info = ProblemInfo(info.n_dofs, info.n_cells, info.nnz, info.n_fixed, info.nodes_per_cell,
                                info.qp_per_cell, info.path)

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().mrg_problem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- structure -----------------------------------------------------------------------------
    def graph(self, device="cuda", stream=None):
        rp = torch.empty(self.info.n_dofs + 1, dtype=torch.int64, device=device)
        ci = torch.empty(self.info.nnz, dtype=torch.int32, device=device)
        L.check(L.lib().mrg_get_graph(self._h, _ptr(rp), _ptr(ci), _stream(stream)), "mrg_get_graph")
        return rp, ci

    def dof_map(self, device="cuda", stream=None):
        lids = torch.empty(self.info.n_cells * self.info.nodes_per_cell, dtype=torch.int32, device=device)
        L.check(L.lib().mrg_get_dof_map(self._h, _ptr(lids), _stream(stream)), "mrg_get_dof_map")
        return lids.view(self.info.n_cells, self.info.nodes_per_cell)

    def fixed_dofs(self, device="cuda", stream=None):
        d = torch.empty(self.info.n_fixed, dtype=torch.int32, device=device)
        v = torch.empty(self.info.n_fixed, dtype=torch.float64, device=device)
        if self.info.n_fixed:
            L.check(L.lib().mrg_get_fixed_dofs(self._h, _ptr(d), _ptr(v), _stream(stream)), "mrg_get_fixed_dofs")
        return d, v

    # ---- data ----------------------------------------------------------------------------------
    def set_kappa(self, kappa: torch.Tensor, stream=None):
        _require_cuda(kappa, "kappa", torch.float64, self.info.n_cells)
        L.check(L.lib().mrg_set_kappa(self._h, _ptr(kappa), _stream(stream)), "mrg_set_kappa")

    def set_wait_policy(self, limit_ns: int = 0, withhold_copy: bool = False):
        """Time limit of the device-side waits of this problem's kernels (0 = defaults); withhold_copy is
        a testing switch that makes the first staged copy never be issued, so that its wait runs out."""
        L.check(L.lib().mrg_set_wait_policy(self._h, int(limit_ns), 1 if withhold_copy else 0),
                "mrg_set_wait_policy")

    def side_points(self, face: int) -> np.ndarray:
        """Coordinates [npts, 3] of the side quadrature points of `face` (0..2*dim-1 = x-, x+, y-, y+,
        z-, z+), ordered as mrg_set_face_bc expects its data."""
        n = C.c_int64(0)
        L.check(L.lib().mrg_get_side_points(self._h, int(face), C.byref(n), None), "mrg_get_side_points")
        xyz = np.zeros((n.value, 3))
        L.check(L.lib().mrg_get_side_points(self._h, int(face), C.byref(n), xyz.ctypes.data_as(C.c_void_p)),
                "mrg_get_side_points")
        return xyz

    def set_face_bc(self, face: int, kind: str, g=None):
        """Neumann ("neumann") or weakly imposed Dirichlet ("weak_dirichlet") data on a face, one value per
        side point (None = 0); "none" removes it.  Reference: thermal::boundaryResidual."""
        k = {"none": L.MRG_BC_NONE, "neumann": L.MRG_BC_NEUMANN, "weak_dirichlet": L.MRG_BC_WEAK_DIRICHLET}[kind]
        ga = None if g is None else np.ascontiguousarray(g, dtype=np.float64)
        L.check(L.lib().mrg_set_face_bc(self._h, int(face), k, None if ga is None else ga.ctypes.data_as(C.c_void_p)),
                "mrg_set_face_bc")

    def new_vector(self, dtype=torch.float64):
        return torch.zeros(self.info.n_dofs, dtype=dtype, device="cuda")

    def new_matrix_values(self, fp32=False):
        return torch.zeros(self.info.nnz, dtype=torch.float32 if fp32 else torch.float64, device="cuda")


class AssemblyManager:
    """assembleJacRes / assembleRes over one Problem (src/managers/assembly/assemblyManager.hpp)."""

    def __init__(self, problem: Problem):
        self.problem = problem

    def _check_args(self, u, res, J, want_res, want_jac, fp32):
        info = self.problem.info
        _require_cuda(u, "u", torch.float64, info.n_dofs)
        if want_res:
            _require_cuda(res, "res", torch.float64, info.n_dofs)
        if want_jac:
            _require_cuda(J, "J", torch.float32 if fp32 else torch.float64, info.nnz)

    def assembleJacRes(self, u, res, J, compute_jacobian=True, fp32_jacobian=False, overwrite=False,
                       compute_sens=False, is_adjoint=False, fix_zero_rows=False, force_cell=False, atomic=False,
                       stream=None, tensor_cores=None, native_fp64=False):
        """r += -res.val(), J += res.dx(); Dirichlet rows skipped, then J(d,d) = 1.

        ``overwrite=True`` fuses the caller's ``J.setAllToScalar(0); r.putScalar(0)``.
        ``native_fp64=True`` forms the factored path's kappa sums with FP64 additions instead of exact
        fixed-point sums rounded once to FP64 (the default).
        """
        flags = L.MRG_ASM_RES
        if compute_jacobian:
            flags |= L.MRG_ASM_JAC
        if fp32_jacobian:
            flags |= L.MRG_ASM_J_FP32
        if overwrite:
            flags |= L.MRG_ASM_OVERWRITE
        if fix_zero_rows:
            flags |= L.MRG_ASM_FIX_ZERO_ROWS
        if force_cell:
            flags |= L.MRG_ASM_FORCE_CELL
        if atomic:
            flags |= L.MRG_ASM_ATOMIC
        if tensor_cores is not None:  # Q2 FP32 Jacobians use the tensor cores unless told otherwise
            flags |= L.MRG_ASM_TENSOR_CORES if tensor_cores else L.MRG_ASM_CUDA_CORES
        if native_fp64:
            flags |= L.MRG_ASM_NATIVE_FP64
        if compute_sens:
            flags |= L.MRG_ASM_SENS
        if is_adjoint:
            flags |= L.MRG_ASM_ADJOINT
        if not (compute_sens or is_adjoint):
            self._check_args(u, res, J, True, compute_jacobian, fp32_jacobian)
        L.check(L.lib().mrg_assemble(self.problem.handle, _ptr(u), _ptr(res), _ptr(J) if compute_jacobian else None,
                                     flags, _stream(stream)), "mrg_assemble")

    def assembleJac(self, u, J, fp32_jacobian=False, overwrite=False, force_cell=False, atomic=False, stream=None,
                    tensor_cores=None):
        flags = L.MRG_ASM_JAC | (L.MRG_ASM_J_FP32 if fp32_jacobian else 0) | (L.MRG_ASM_OVERWRITE if overwrite else 0)
        if tensor_cores is not None:
            flags |= L.MRG_ASM_TENSOR_CORES if tensor_cores else L.MRG_ASM_CUDA_CORES
        flags |= (L.MRG_ASM_FORCE_CELL if force_cell else 0) | (L.MRG_ASM_ATOMIC if atomic else 0)
        self._check_args(u, None, J, False, True, fp32_jacobian)
        L.check(L.lib().mrg_assemble(self.problem.handle, _ptr(u), None, _ptr(J), flags, _stream(stream)),
                "mrg_assemble")

    def assembleRes(self, u, res, overwrite=False, force_cell=False, atomic=False, stream=None, native_fp64=False):
        flags = L.MRG_ASM_RES | (L.MRG_ASM_OVERWRITE if overwrite else 0)
        flags |= L.MRG_ASM_NATIVE_FP64 if native_fp64 else 0
        flags |= (L.MRG_ASM_FORCE_CELL if force_cell else 0) | (L.MRG_ASM_ATOMIC if atomic else 0)
        self._check_args(u, res, None, True, False, False)
        L.check(L.lib().mrg_assemble_residual(self.problem.handle, _ptr(u), _ptr(res), flags, _stream(stream)),
                "mrg_assemble_residual")
