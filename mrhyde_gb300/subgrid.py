"""Batched multiscale-subgrid local solves (the per-macro-element loop of the reference's multiscale
manager, src/managers/multiscale/multiscaleManager.cpp:866 -> src/subgrid/subgridDtN_solver.cpp:136,
done as one persistent GPU launch).

``SubgridBatch(sizes, kappa_list, dirichlet_list, source)`` holds the problems on the device;
``solve()`` assembles every local FP32 Jacobian and solves every problem (FP32 Jacobi-PCG with FP64
refinement to ``tol`` in the reference's relative inf-norm); ``autotune()`` picks the launch shape.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .assembly import _stream


class SubgridBatch:
    def __init__(self, sizes, kappa_list, dirichlet_list, source=1.0):
        sizes = np.ascontiguousarray(np.asarray(sizes, dtype=np.int32).reshape(-1, 3))
        kap = np.ascontiguousarray(np.concatenate([np.asarray(k, np.float64).ravel() for k in kappa_list]))
        dbc = np.ascontiguousarray(np.concatenate([np.asarray(d, np.float64).ravel() for d in dirichlet_list]))
        d = L.BatchDesc()
        d.n_problems = len(sizes)
        d.sizes = sizes.ctypes.data_as(C.POINTER(C.c_int32))
        d.kappa = kap.ctypes.data_as(C.POINTER(C.c_double))
        d.dirichlet = dbc.ctypes.data_as(C.POINTER(C.c_double))
        d.source = float(source)
        h = C.c_void_p()
        L.check(L.lib().mrg_batch_create(C.byref(d), C.byref(h)), "mrg_batch_create")
        self._h = h
        self.sizes = sizes
        self.n = len(sizes)
        info = L.BatchInfo()
        self.node_off = np.zeros(self.n, np.int64)
        self.nnz_off = np.zeros(self.n, np.int64)
        L.check(L.lib().mrg_batch_get_info(h, C.byref(info), self.node_off.ctypes.data_as(C.c_void_p),
                                           self.nnz_off.ctypes.data_as(C.c_void_p)), "mrg_batch_get_info")
        self.info = info
        self.u = torch.zeros(info.n_nodes, dtype=torch.float64, device="cuda")
        self.J = torch.zeros(info.nnz, dtype=torch.float32, device="cuda")

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            L.lib().mrg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def opts(tol=1e-10, inner_tol=1e-5, max_outer=20, max_inner=2000):
        o = L.BatchOpts()
        o.tol, o.inner_tol, o.max_outer, o.max_inner = tol, inner_tol, max_outer, max_inner
        return o

    def solve(self, tol=1e-10, inner_tol=1e-5, max_outer=20, max_inner=2000, stream=None, stats=True):
        o = self.opts(tol, inner_tol, max_outer, max_inner)
        st = (L.BatchStat * self.n)() if stats else None
        L.check(L.lib().mrg_batch_solve(self._h, C.c_void_p(self.u.data_ptr()), C.c_void_p(self.J.data_ptr()),
                                        C.byref(o), st, _stream(stream)), "mrg_batch_solve")
        if stats:
            return np.array([(s.outer_iterations, s.inner_iterations, s.rel_residual, s.status) for s in st])
        return None

    def autotune(self, tol=1e-10, inner_tol=1e-5, max_outer=20, max_inner=2000, stream=None):
        o = self.opts(tol, inner_tol, max_outer, max_inner)
        L.check(L.lib().mrg_batch_autotune(self._h, C.c_void_p(self.u.data_ptr()), C.c_void_p(self.J.data_ptr()),
                                           C.byref(o), _stream(stream)), "mrg_batch_autotune")
        info = L.BatchInfo()
        L.lib().mrg_batch_get_info(self._h, C.byref(info), None, None)
        self.info = info
        return info.threads, info.ctas_per_sm

    def set_config(self, threads, ctas_per_sm):
        L.check(L.lib().mrg_batch_set_config(self._h, threads, ctas_per_sm), "mrg_batch_set_config")

    def solution(self, k):
        nx, ny, nz = (int(v) for v in self.sizes[k])
        nn = (nx + 1) * (ny + 1) * (nz + 1)
        o = int(self.node_off[k])
        return self.u[o:o + nn]
