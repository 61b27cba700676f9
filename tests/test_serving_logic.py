"""Host logic of the serving loop on the CPU: FIFO admission under an HBM budget and a slot limit,
rejection of requests that can never fit, failures of single requests (injected on the host) that
do not stop the loop.  The GPU solve is replaced by a fake; no GPU is touched."""
import threading
import time

import pytest

from mrhyde_gb300 import serving


class FakeSolve:
    def __init__(self, fail_ids=()):
        self.active = 0
        self.peak = 0
        self.lock = threading.Lock()
        self.fail_ids = set(fail_ids)

    def __call__(self, req, stream, keep, preconditioner="gmg"):
        with self.lock:
            self.active += 1
            self.peak = max(self.peak, self.active)
        time.sleep(0.01)
        with self.lock:
            self.active -= 1
        if req.rid in self.fail_ids:
            from mrhyde_gb300 import _lib as L

            raise L.MrgError(L.MRG_EINVAL, "fake", "injected failure")

        class R:
            status, outer_iterations, iterations, rel_residual = 0, 2, 10, 1e-11

        return R(), None, 1.0, (req.n + 1) ** 3


@pytest.fixture
def fake(monkeypatch):
    f = FakeSolve(fail_ids={3})
    monkeypatch.setattr(serving, "solve_request", f)

    class S:
        def __init__(self):
            pass

    monkeypatch.setattr(serving.torch.cuda, "Stream", lambda: None)
    return f


def test_budget_limits_concurrency(fake):
    reqs = [serving.Request(i, "thermal", 20, i, True, 0.0) for i in range(12)]
    one = serving.estimate_bytes(reqs[0])
    srv = serving.Server(hbm_budget_bytes=2 * one + 10, slots=8)
    out = srv.run(reqs, realtime=False)
    assert fake.peak <= 2 and srv.peak_active <= 2
    assert srv.peak_bytes <= 2 * one + 10
    assert out["requests"] == 12 and out["ok"] == 11  # rid 3 failed by injection
    failed = [r for r in srv.results if r.status != 0]
    assert [r.rid for r in failed] == [3]


def test_slots_limit_concurrency_and_fifo(fake):
    reqs = [serving.Request(i, "nonlinear", 10, i, True, 0.001 * i) for i in range(16)]
    srv = serving.Server(hbm_budget_bytes=10**12, slots=3)
    srv.run(reqs, realtime=True)
    assert fake.peak <= 3
    starts = sorted(srv.results, key=lambda r: r.queue_wait + r.latency - r.latency)
    assert len(starts) == 16


def test_request_larger_than_budget_is_rejected_not_deadlocked(fake):
    big = serving.Request(0, "thermal", 96, 1, False, 0.0)
    small = serving.Request(1, "thermal", 8, 2, True, 0.0)
    srv = serving.Server(hbm_budget_bytes=serving.estimate_bytes(small) + 1, slots=2)
    out = srv.run([big, small], realtime=False)
    st = {r.rid: r.status for r in srv.results}
    from mrhyde_gb300 import _lib as L

    assert st[0] == L.MRG_ENOMEM and st[1] == 0
    assert out["ok"] == 1


def test_poisson_stream_shape():
    reqs = serving.poisson_stream(rate=200.0, count=2000, seed=1)
    ns = [r.n for r in reqs]
    assert min(ns) >= 16 and max(ns) <= 96
    t = [r.arrival for r in reqs]
    rate = len(t) / t[-1]
    assert 180 < rate < 220
    frac = sum(r.kind == "nonlinear" for r in reqs) / len(reqs)
    assert 0.45 < frac < 0.55


def test_unexpected_exception_fails_only_that_request(monkeypatch):
    """A request whose solve raises something other than MrgError is reported failed; the worker and the
    other requests carry on."""
    class Boom(FakeSolve):
        def __call__(self, req, stream, keep, preconditioner="gmg"):
            if req.rid == 2:
                raise RuntimeError("injected")
            return super().__call__(req, stream, keep, preconditioner)

    f = Boom()
    monkeypatch.setattr(serving, "solve_request", f)
    monkeypatch.setattr(serving.torch.cuda, "Stream", lambda: None)
    reqs = serving.poisson_stream(rate=1000.0, count=6, edge=(4, 6), seed=2)
    srv = serving.Server(hbm_budget_bytes=10**12, slots=2)
    out = srv.run(reqs, realtime=False)
    assert out["requests"] == 6 and out["ok"] == 5
    assert [rid for rid, _ in srv.errors] == [2]


def test_warmup_solves_each_kind_and_precision(monkeypatch):
    seen = []

    class Rec(FakeSolve):
        def __call__(self, req, stream, keep, preconditioner="gmg"):
            seen.append((req.kind, req.mixed, req.n, keep, preconditioner))
            return super().__call__(req, stream, keep, preconditioner)

    class Stream:
        def synchronize(self):
            seen.append("sync")

    monkeypatch.setattr(serving, "solve_request", Rec())
    monkeypatch.setattr(serving.torch.cuda, "Stream", Stream)
    srv = serving.Server(slots=2, preconditioner="jacobi")
    srv.warmup()
    assert sorted(seen[:-1]) == sorted((k, m, 64, False, "jacobi") for k in ("thermal", "nonlinear") for m in (True, False))
    assert seen[-1] == "sync" and srv.results == []
