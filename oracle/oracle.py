"""ctypes wrapper of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, never by the mrhyde_gb300 package.  The oracle restates MrHyDE's workset assembly path
(src/managers/assembly/assemblyManager_jacres.hpp:121-630) in plain FP64 C++; see the header of
oracle.cpp for the per-function citations.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None


class OrcDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("order", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("lo", C.c_double * 3), ("hi", C.c_double * 3),
        ("vertex_coords", C.POINTER(C.c_double)),
        ("kind", C.c_int32), ("source_kind", C.c_int32),
        ("source_amp", C.c_double), ("source_freq", C.c_double),
        ("kappa_const", C.c_double), ("kappa_cell", C.POINTER(C.c_double)),
        ("dirichlet_faces", C.c_uint32), ("dirichlet_kind", C.c_int32),
        ("dirichlet_const", C.c_double), ("dirichlet_node", C.POINTER(C.c_double)),
        ("dirichlet_amp", C.c_double), ("dirichlet_freq", C.c_double),
        ("quad_order", C.c_int32), ("workset_size", C.c_int32),
    ]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (portable flags, x86_64 or aarch64)."""
    src = os.path.join(_HERE, "oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        P = C.c_void_p
        dp = C.POINTER(C.c_double)
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.POINTER(OrcDesc)]
        L.orc_destroy.argtypes = [P]
        L.orc_sizes.argtypes = [P, C.POINTER(C.c_int64)]
        L.orc_graph.argtypes = [P, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
        L.orc_dof_map.argtypes = [P, C.POINTER(C.c_int32)]
        L.orc_fixed.argtypes = [P, C.POINTER(C.c_int32), dp]
        L.orc_set_kappa.argtypes = [P, dp]
        L.orc_set_dirichlet.argtypes = [P, dp]
        L.orc_assemble.argtypes = [P, dp, dp, dp, C.c_int, C.c_int]
        L.orc_assemble.restype = C.c_int
        L.orc_assemble_sample.argtypes = [P, dp, dp, dp, C.c_int, C.c_int, C.c_int64]
        L.orc_assemble_sample.restype = C.c_int
        L.orc_spmv.argtypes = [P, dp, dp, dp, C.c_int]
        L.orc_pcg.argtypes = [P, dp, dp, dp, C.c_double, C.c_int, C.c_int, dp]
        L.orc_pcg.restype = C.c_int
        L.orc_newton.argtypes = [P, dp, C.c_double, C.c_int, C.c_double, C.c_int, C.c_int, dp]
        L.orc_newton.restype = C.c_int
        L.orc_errors.argtypes = [P, dp, C.c_double, C.c_double, dp, dp]
        L.orc_tables.argtypes = [P, dp, dp, dp]
        L.orc_max_threads.restype = C.c_int
        L.orc_side_points.argtypes = [P, C.c_int, dp]
        L.orc_side_points.restype = C.c_int64
        L.orc_set_face_bc.argtypes = [P, C.c_int, C.c_int, dp]
        L.orc_set_face_bc.restype = C.c_int
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


class OracleProblem:
    """One structured-mesh problem in the oracle.  Arguments mirror mrhyde_gb300.Problem."""

    def __init__(self, dim=3, order=1, n=(4, 4, 4), lo=(0, 0, 0), hi=(1, 1, 1), kind=0,
                 source=("const", 1.0, 0.0), kappa=1.0, dirichlet_faces=63, dirichlet=("const", 0.0),
                 quad_order=0, workset_size=0, vertex_coords=None):
        L = lib()
        d = OrcDesc()
        d.dim, d.order = dim, order
        d.nx, d.ny = n[0], n[1]
        d.nz = n[2] if dim == 3 else 1
        for k in range(3):
            d.lo[k] = float(lo[k]) if k < len(lo) else 0.0
            d.hi[k] = float(hi[k]) if k < len(hi) else 1.0
        self._keep = []
        if vertex_coords is not None:
            vc = np.ascontiguousarray(vertex_coords, dtype=np.float64)
            self._keep.append(vc)
            d.vertex_coords = _dp(vc)
        d.kind = kind
        skind, amp, freq = source
        d.source_kind = {"const": 0, "sinprod": 1}[skind]
        d.source_amp, d.source_freq = amp, freq
        if np.isscalar(kappa):
            d.kappa_const = float(kappa)
        else:
            kc = np.ascontiguousarray(kappa, dtype=np.float64)
            self._keep.append(kc)
            d.kappa_cell = _dp(kc)
            d.kappa_const = 1.0
        d.dirichlet_faces = dirichlet_faces
        dk = dirichlet[0]
        if dk == "const":
            d.dirichlet_kind, d.dirichlet_const = 0, dirichlet[1]
        elif dk == "node":
            arr = np.ascontiguousarray(dirichlet[1], dtype=np.float64)
            self._keep.append(arr)
            d.dirichlet_kind, d.dirichlet_node = 1, _dp(arr)
        elif dk in ("sinprod", "sinprod_l2"):
            d.dirichlet_kind = 2 if dk == "sinprod" else 3
            d.dirichlet_amp, d.dirichlet_freq = dirichlet[1], dirichlet[2]
        d.quad_order, d.workset_size = quad_order, workset_size
        self.desc = d
        self.h = L.orc_create(C.byref(d))
        if not self.h:
            raise ValueError("oracle rejected the problem description")
        s = (C.c_int64 * 6)()
        L.orc_sizes(self.h, s)
        self.ndof, self.ncell, self.nnz, self.nfixed, self.npe, self.nq = [int(v) for v in s]

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def graph(self):
        rp = np.zeros(self.ndof + 1, np.int64)
        ci = np.zeros(self.nnz, np.int32)
        lib().orc_graph(self.h, rp.ctypes.data_as(C.POINTER(C.c_int64)), ci.ctypes.data_as(C.POINTER(C.c_int32)))
        return rp, ci

    def dof_map(self):
        lids = np.zeros(self.ncell * self.npe, np.int32)
        lib().orc_dof_map(self.h, lids.ctypes.data_as(C.POINTER(C.c_int32)))
        return lids.reshape(self.ncell, self.npe)

    def fixed(self):
        dofs = np.zeros(self.nfixed, np.int32)
        vals = np.zeros(self.nfixed, np.float64)
        lib().orc_fixed(self.h, dofs.ctypes.data_as(C.POINTER(C.c_int32)), _dp(vals))
        return dofs, vals

    def set_dirichlet(self, u):
        lib().orc_set_dirichlet(self.h, _dp(u))
        return u

    def assemble(self, u, jac=True, res=True, nthreads=1, fix_zero_rows=False):
        """Zero-then-sum-into assembly; returns (r, J values)."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        r = np.zeros(self.ndof) if res else None
        J = np.zeros(self.nnz) if jac else None
        flags = (1 if res else 0) | (2 if jac else 0) | (16 if fix_zero_rows else 0)
        rc = lib().orc_assemble(self.h, _dp(u), _dp(r), _dp(J), flags, nthreads)
        if rc:
            raise RuntimeError("oracle assemble failed")
        return r, J

    def assemble_sample(self, u, ncell, nthreads=1, jac=True):
        r = np.zeros(self.ndof)
        J = np.zeros(self.nnz) if jac else None
        lib().orc_assemble_sample(self.h, _dp(u), _dp(r), _dp(J), 3 if jac else 1, nthreads, ncell)
        return r, J

    def spmv(self, J, x, nthreads=1):
        y = np.zeros(self.ndof)
        lib().orc_spmv(self.h, _dp(J), _dp(np.ascontiguousarray(x, np.float64)), _dp(y), nthreads)
        return y

    def pcg(self, J, b, x0=None, tol=1e-10, maxiter=10000, nthreads=1):
        x = np.zeros(self.ndof) if x0 is None else np.array(x0, dtype=np.float64)
        rr = np.zeros(1)
        it = lib().orc_pcg(self.h, _dp(J), _dp(np.ascontiguousarray(b, np.float64)), _dp(x), tol, maxiter,
                           nthreads, _dp(rr))
        return x, it, float(rr[0])

    def newton(self, u, nltol=1e-10, maxiter=10, lintol=1e-12, linmaxiter=20000, nthreads=1):
        u = np.array(u, dtype=np.float64)
        st = np.zeros(3)
        rc = lib().orc_newton(self.h, _dp(u), nltol, maxiter, lintol, linmaxiter, nthreads, _dp(st))
        return u, rc, st

    def side_points(self, face):
        """Coordinates [npts, 3] of the side quadrature points of `face` (face-cell order)."""
        n = lib().orc_side_points(self.h, int(face), None)
        if n < 0:
            raise ValueError(f"bad face {face}")
        xyz = np.zeros((n, 3))
        lib().orc_side_points(self.h, int(face), _dp(xyz))
        return xyz

    def set_face_bc(self, face, kind, g=None):
        """kind: 0 none, 1 Neumann, 2 weak Dirichlet; g: one value per side point (None = 0)."""
        ga = None if g is None else np.ascontiguousarray(g, dtype=np.float64)
        if lib().orc_set_face_bc(self.h, int(face), int(kind), None if ga is None else _dp(ga)) != 0:
            raise ValueError("bad face boundary condition")

    def errors(self, u, amp, freq):
        l2 = np.zeros(1)
        h1 = np.zeros(1)
        lib().orc_errors(self.h, _dp(np.ascontiguousarray(u, np.float64)), amp, freq, _dp(l2), _dp(h1))
        return float(l2[0]), float(h1[0])

    def tables(self):
        qw = np.zeros(self.nq)
        phi = np.zeros(self.npe * self.nq)
        dphi = np.zeros(self.npe * self.nq * self.desc.dim)
        lib().orc_tables(self.h, _dp(qw), _dp(phi), _dp(dphi))
        return qw, phi.reshape(self.npe, self.nq), dphi.reshape(self.npe, self.nq, self.desc.dim)


def max_threads() -> int:
    return int(lib().orc_max_threads())
