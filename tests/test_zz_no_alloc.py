"""mrg_solve_pcg_noalloc: the PCG entry point for callers that cannot allocate device memory.

Such callers (a runtime that owns every byte of device memory and admits work against a fixed HBM
budget, a framework whose pool allocator must be the only one, a latency-critical loop) get a PCG
whose scratch lives in a fixed device array inside the library.  This file is collected last so that
a run stopping at the first failure has already run every other test; it also passes on its own in a
fresh process.

Checked through the C ABI: two calls in a row agree with mrg_solve_pcg (same tolerance as the other
PCG tests: 1e-9 of the solution's max norm), a call after a warm-up call leaves the device's free
memory and torch's allocator counters unchanged, and a problem above the fixed limit is rejected.
"""
import ctypes as C

import numpy as np
import pytest
import torch


def _solve_noalloc(L, P, J, b, x, tol, maxiter):
    st = L.SolveStats()
    s = torch.cuda.current_stream().cuda_stream
    rc = L.lib().mrg_solve_pcg_noalloc(P.handle, C.c_void_p(J.data_ptr()), C.c_void_p(b.data_ptr()),
                                       C.c_void_p(x.data_ptr()), tol, maxiter, C.byref(st), s)
    return rc, st


@pytest.mark.gpu
def test_noalloc_pcg_matches_allocating_pcg_twice(cuda):
    from mrhyde_gb300 import AssemblyManager, Problem, SolverManager
    from mrhyde_gb300 import _lib as L

    rng = np.random.default_rng(12)
    n = (40, 30, 20)  # 41*31*21 = 26,691 DOFs, below MRG_NOALLOC_MAX_DOFS
    P = Problem(dim=3, order=1, n=n, kappa=np.exp(0.5 * rng.standard_normal(int(np.prod(n)))),
                source=("const", 1.0, 0.0), dirichlet_faces=3)
    assert P.info.n_dofs <= L.MRG_NOALLOC_MAX_DOFS
    A, S = AssemblyManager(P), SolverManager(P)
    u, r, J = P.new_vector(), P.new_vector(), P.new_matrix_values()
    A.assembleJacRes(u, r, J, overwrite=True)
    x_ref = P.new_vector()
    ref = S.PCG(J, r, x_ref, tol=1e-10, maxiter=5000)
    xr = x_ref.cpu().numpy()
    for call in range(2):
        x = P.new_vector()
        rc, st = _solve_noalloc(L, P, J, r, x, 1e-10, 5000)
        assert rc == L.MRG_OK, L.last_error()
        assert st.rel_residual <= 1e-10
        assert st.iterations == ref.iterations
        np.testing.assert_allclose(x.cpu().numpy(), xr, rtol=0, atol=1e-9 * np.abs(xr).max())


@pytest.mark.gpu
def test_noalloc_pcg_allocates_nothing(cuda):
    """After a warm-up call (which loads the kernels and looks up the scratch array's address), a call
    changes neither the device's free memory (cudaMemGetInfo, which sees every allocation on the device,
    library or torch) nor torch's allocation counters."""
    from mrhyde_gb300 import AssemblyManager, Problem
    from mrhyde_gb300 import _lib as L

    rng = np.random.default_rng(13)
    n = (30, 30, 30)
    P = Problem(dim=3, order=1, n=n, kappa=np.exp(0.5 * rng.standard_normal(int(np.prod(n)))),
                source=("const", 1.0, 0.0), dirichlet_faces=3)
    A = AssemblyManager(P)
    u, r, J = P.new_vector(), P.new_vector(), P.new_matrix_values()
    A.assembleJacRes(u, r, J, overwrite=True)
    x0, x1 = P.new_vector(), P.new_vector()
    rc, _ = _solve_noalloc(L, P, J, r, x0, 1e-10, 5000)  # warm-up
    assert rc == L.MRG_OK, L.last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    stats0 = torch.cuda.memory_stats()
    rc, st = _solve_noalloc(L, P, J, r, x1, 1e-10, 5000)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    stats1 = torch.cuda.memory_stats()
    assert rc == L.MRG_OK, L.last_error()
    assert st.rel_residual <= 1e-10
    assert free1 == free0, (free0, free1)
    for key in ("allocation.all.allocated", "segment.all.allocated", "allocated_bytes.all.current",
                "reserved_bytes.all.current"):
        assert stats1.get(key, 0) == stats0.get(key, 0), key
    assert torch.equal(x0, x1)


@pytest.mark.gpu
def test_noalloc_pcg_rejects_problems_above_the_limit(cuda):
    from mrhyde_gb300 import Problem
    from mrhyde_gb300 import _lib as L

    P = Problem(dim=2, order=1, n=(600, 600))  # 361,201 DOFs > 2^18
    assert P.info.n_dofs > L.MRG_NOALLOC_MAX_DOFS
    J = P.new_matrix_values()
    b, x = P.new_vector(), P.new_vector()
    rc, _ = _solve_noalloc(L, P, J, b, x, 1e-10, 10)
    assert rc == L.MRG_EINVAL
    assert "MRG_NOALLOC_MAX_DOFS" in L.last_error()
