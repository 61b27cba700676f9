"""Serving loop on the GPU: every result is the same alone and in the mix; admission under a budget."""
import numpy as np
import pytest
import torch


@pytest.mark.gpu
def test_results_identical_alone_and_in_the_mix(cuda):
    from mrhyde_gb300 import serving

    reqs = serving.poisson_stream(rate=400.0, count=16, edge=(8, 28), nonlinear_fraction=0.5, mixed=True, seed=11)
    srv = serving.Server(hbm_budget_bytes=80 * 10**9, slots=6, keep_solutions=True)
    out = srv.run(reqs, realtime=True)
    assert out["ok"] == 16 and out["max_rel_residual"] < 1e-10
    assert srv.peak_active >= 2  # requests overlapped on the device
    mix = {r.rid: r for r in srv.results}
    for rid in (0, 5, 11):
        res, uh, chk, dofs = serving.solve_request(reqs[rid], torch.cuda.Stream(), keep_solution=True)
        assert res.rel_residual < 1e-10
        assert torch.equal(uh, mix[rid].u), rid


@pytest.mark.gpu
def test_fp64_and_mixed_requests_agree(cuda):
    from mrhyde_gb300 import serving

    for kind in ("thermal", "nonlinear"):
        r64 = serving.Request(0, kind, 20, 123, mixed=False)
        r32 = serving.Request(1, kind, 20, 123, mixed=True)
        s = torch.cuda.Stream()
        a = serving.solve_request(r64, s, keep_solution=True)
        b = serving.solve_request(r32, s, keep_solution=True)
        assert a[0].rel_residual < 1e-10 and b[0].rel_residual < 1e-10
        ua, ub = a[1].numpy(), b[1].numpy()
        assert np.abs(ua - ub).max() <= 1e-8 * np.abs(ua).max(), kind


@pytest.mark.gpu
def test_malformed_request_does_not_stop_the_loop(cuda):
    from mrhyde_gb300 import _lib as L
    from mrhyde_gb300 import serving

    reqs = [serving.Request(0, "thermal", 12, 1), serving.Request(1, "thermal", 0, 2), serving.Request(2, "nonlinear", 12, 3)]
    srv = serving.Server(slots=2)
    out = srv.run(reqs, realtime=False)
    st = {r.rid: r.status for r in srv.results}
    assert st[1] == L.MRG_EINVAL and st[0] == 0 and st[2] == 0
