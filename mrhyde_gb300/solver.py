"""Host-side mirror of MrHyDE's SolverManager pieces that call the assembly path.

``setDirichlet`` (src/managers/solver/solverManager_util.hpp:60-140), ``PCG``
(src/managers/solver/solverManager_solvers.hpp:812-901) and ``nonlinearSolver``
(src/managers/solver/solverManager_solvers.hpp:290-643) run on the GPU through libmrhyde_gb.so.
Settings keep the reference's names and defaults ("nonlinear TOL" 1e-6, "max nonlinear iters" 10,
"linear TOL" 1e-7; src/managers/solver/solverManager_construct.hpp:58-64).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import _lib as L
from .assembly import Problem, _ptr, _require_cuda, _stream


@dataclass
class SolveResult:
    iterations: int
    outer_iterations: int
    rel_residual: float
    abs_residual: float
    status: int


def _result(st: L.SolveStats) -> SolveResult:
    return SolveResult(st.iterations, st.outer_iterations, st.rel_residual, st.abs_residual, st.status)


class SolverManager:
    def __init__(self, problem: Problem, nonlinear_tol=1.0e-6, max_nonlinear_iters=10, linear_tol=1.0e-7,
                 linear_maxiter=100000, mixed_precision=False, reuse_jacobian=False, krylov="auto",
                 preconditioner="jacobi", gmg_full_setup=False):
        self.problem = problem
        self.NLtol = nonlinear_tol
        self.maxNLiter = max_nonlinear_iters
        self.linear_tol = linear_tol
        self.linear_maxiter = linear_maxiter
        self.mixed = mixed_precision
        self.reuse_jacobian = reuse_jacobian
        # multigrid with a re-assembled Jacobian: True rebuilds every level at every Newton step; False keeps
        # the coarse Galerkin operators while the Krylov iteration count does not grow (mrg_newton_opts)
        self.gmg_full_setup = gmg_full_setup
        self.krylov = {"auto": L.MRG_KRYLOV_AUTO, "pcg": L.MRG_KRYLOV_PCG, "bicgstab": L.MRG_KRYLOV_BICGSTAB}[krylov]
        # "jacobi": the reference's SolverManager::PCG; "gmg": geometric multigrid V-cycle (Q1 and Q2),
        # the structured-grid counterpart of the reference's Belos + MueLu option; "gmg_split": the same
        # cycle with every coarse-level step its own launch (bit-identical, for comparison).  The choice
        # is a property of the problem handle (mrg_set_preconditioner) and applies to PCG, BiCGStab and
        # Newton's Krylov solves.
        self.preconditioner = preconditioner
        prec = {"jacobi": L.MRG_PREC_JACOBI, "gmg": L.MRG_PREC_GMG, "gmg_split": L.MRG_PREC_GMG_SPLIT}[preconditioner]
        L.check(L.lib().mrg_set_preconditioner(problem.handle, prec), "mrg_set_preconditioner")

    def setDirichlet(self, u: torch.Tensor, stream=None):
        _require_cuda(u, "u", torch.float64, self.problem.info.n_dofs)
        L.check(L.lib().mrg_set_dirichlet(self.problem.handle, _ptr(u), _stream(stream)), "mrg_set_dirichlet")
        return u

    def apply(self, J: torch.Tensor, x: torch.Tensor, y: torch.Tensor, stream=None):
        """y = J x on the problem's canonical graph (CrsMatrix::apply)."""
        fp32 = J.dtype == torch.float32
        _require_cuda(J, "J", None, self.problem.info.nnz)
        L.check(L.lib().mrg_spmv(self.problem.handle, _ptr(J), int(fp32), _ptr(x), _ptr(y), _stream(stream)),
                "mrg_spmv")
        return y

    def PCG(self, J: torch.Tensor, b: torch.Tensor, x: torch.Tensor, tol: float, maxiter: int, stream=None,
            raise_on_noconv=True) -> SolveResult:
        """Preconditioned CG on J x = b (Jacobi, or multigrid when chosen); x holds the initial guess and
        receives the solution."""
        info = self.problem.info
        fp32 = J.dtype == torch.float32
        _require_cuda(J, "J", None, info.nnz)
        _require_cuda(b, "b", torch.float64, info.n_dofs)
        _require_cuda(x, "x", torch.float64, info.n_dofs)
        st = L.SolveStats()
        rc = L.lib().mrg_solve_pcg(self.problem.handle, _ptr(J), int(fp32), _ptr(b), _ptr(x), float(tol),
                                   int(maxiter), C.byref(st), _stream(stream))
        if rc != L.MRG_OK and (raise_on_noconv or rc != L.MRG_ENOCONV):
            L.check(rc, "mrg_solve_pcg")
        return _result(st)

    def BiCGStab(self, J: torch.Tensor, b: torch.Tensor, x: torch.Tensor, tol: float, maxiter: int, stream=None,
                 raise_on_noconv=True) -> SolveResult:
        """Jacobi BiCGStab on J x = b ("Belos solver: BiCGStab"); x holds the initial guess."""
        info = self.problem.info
        fp32 = J.dtype == torch.float32
        _require_cuda(J, "J", None, info.nnz)
        _require_cuda(b, "b", torch.float64, info.n_dofs)
        _require_cuda(x, "x", torch.float64, info.n_dofs)
        st = L.SolveStats()
        rc = L.lib().mrg_solve_bicgstab(self.problem.handle, _ptr(J), int(fp32), _ptr(b), _ptr(x), float(tol),
                                        int(maxiter), C.byref(st), _stream(stream))
        if rc != L.MRG_OK and (raise_on_noconv or rc != L.MRG_ENOCONV):
            L.check(rc, "mrg_solve_bicgstab")
        return _result(st)

    def nonlinearSolver(self, u: torch.Tensor, stream=None, raise_on_noconv=True) -> SolveResult:
        """Newton on F(u) = 0 with relative inf-norm test; u holds the initial guess."""
        _require_cuda(u, "u", torch.float64, self.problem.info.n_dofs)
        o = L.NewtonOpts()
        o.nl_tol = self.NLtol
        o.max_iters = self.maxNLiter
        o.mixed = int(self.mixed)
        o.lin_tol = self.linear_tol
        o.lin_maxiter = self.linear_maxiter
        o.reuse_jacobian = int(self.reuse_jacobian)
        o.krylov = self.krylov
        o.gmg_full_setup = int(self.gmg_full_setup)
        st = L.SolveStats()
        rc = L.lib().mrg_newton(self.problem.handle, _ptr(u), C.byref(o), C.byref(st), _stream(stream))
        if rc != L.MRG_OK and (raise_on_noconv or rc != L.MRG_ENOCONV):
            L.check(rc, "mrg_newton")
        return _result(st)
