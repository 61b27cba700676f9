"""The bounded device waits run out, the kernels leave cleanly and the next call is correct.

No fault and no hang is involved: mrg_set_wait_policy shortens the limit of the device-side waits and
(testing switch) withholds the first staged copy, so the wait for it runs out after the limit.  The
kernel then raises its abort flag, lets its own copies and MMAs in flight land, frees its tensor
memory and exits; the call reports MRG_ETIMEOUT.  With the default policy restored, the next call on
the same context gives the oracle's result -- which also shows that the tensor memory was released
(the next launch allocates the same 512 TMEM columns on every SM).
"""
import numpy as np
import pytest
import torch

from mrhyde_gb300 import _lib as L
from tests.cases import gpu_problem, oracle_problem
from tests.test_gpu_assembly_parity import scaled_err

LIMIT_NS = 20_000_000  # 20 ms


@pytest.mark.gpu
def test_tensor_core_wait_runs_out_then_next_call_is_correct(cuda):
    from mrhyde_gb300 import AssemblyManager

    cfg = dict(dim=3, order=2, n=(12, 12, 12), kind="diffusion_1pu2", source=("const", 10.0, 0.0),
               dirichlet_faces=3, kappa=1.0)
    O = oracle_problem(cfg)
    u = np.random.default_rng(81).uniform(0.0, 0.3, O.ndof)
    _, Jo = O.assemble(u)
    G = gpu_problem(cfg)
    A = AssemblyManager(G)
    ud = torch.tensor(u, device="cuda")
    J = G.new_matrix_values(fp32=True)
    A.assembleJac(ud, J, fp32_jacobian=True, overwrite=True, tensor_cores=True)
    assert scaled_err(J.cpu().numpy(), Jo) <= 1e-4

    G.set_wait_policy(LIMIT_NS, withhold_copy=True)
    A.assembleJac(ud, J, fp32_jacobian=True, overwrite=True, tensor_cores=True)  # does not synchronise
    torch.cuda.synchronize()
    G.set_wait_policy(0, withhold_copy=False)
    with pytest.raises(L.MrgError) as e:  # the time-out of the previous launch is reported here
        A.assembleJac(ud, J, fp32_jacobian=True, overwrite=True, tensor_cores=True)
    assert e.value.status == L.MRG_ETIMEOUT
    for _ in range(2):
        J.fill_(np.nan)
        A.assembleJac(ud, J, fp32_jacobian=True, overwrite=True, tensor_cores=True)
        torch.cuda.synchronize()
        assert scaled_err(J.cpu().numpy(), Jo) <= 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("fp32", [False, True])
def test_pcg_staging_wait_runs_out_then_next_solve_is_identical(cuda, fp32):
    from mrhyde_gb300 import AssemblyManager, Problem, SolverManager

    rng = np.random.default_rng(82)
    n = (20, 20, 20)
    P = Problem(dim=3, order=1, n=n, kappa=np.exp(0.5 * rng.standard_normal(int(np.prod(n)))),
                source=("const", 1.0, 0.0), dirichlet_faces=3)
    A, S = AssemblyManager(P), SolverManager(P)
    u, r, J = P.new_vector(), P.new_vector(), P.new_matrix_values(fp32=fp32)
    A.assembleJacRes(u, r, J, fp32_jacobian=fp32, overwrite=True)
    tol = 1e-5 if fp32 else 1e-10
    x_ref = P.new_vector()
    ref = S.PCG(J, r, x_ref, tol=tol, maxiter=5000)

    P.set_wait_policy(LIMIT_NS, withhold_copy=True)
    x = P.new_vector()
    with pytest.raises(L.MrgError) as e:
        S.PCG(J, r, x, tol=tol, maxiter=5000)
    assert e.value.status == L.MRG_ETIMEOUT
    assert "time bound" in str(e.value)

    P.set_wait_policy(0, withhold_copy=False)
    x2 = P.new_vector()
    res = S.PCG(J, r, x2, tol=tol, maxiter=5000)
    assert res.iterations == ref.iterations
    assert torch.equal(x2, x_ref)


@pytest.mark.gpu
def test_wait_policy_rejects_bad_arguments(cuda):
    from mrhyde_gb300 import Problem

    P = Problem(dim=2, order=1, n=(4, 4))
    assert L.lib().mrg_set_wait_policy(None, 0, 0) == L.MRG_EINVAL
    with pytest.raises(L.MrgError) as e:
        P.set_wait_policy(L.MRG_WAIT_LIMIT_MAX_NS + 1)
    assert e.value.status == L.MRG_EINVAL
