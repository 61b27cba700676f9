"""Continuous-batching serving loop for steady thermal and nonlinear-diffusion solves (configuration C5).

The reference has no serving mode; this is the request loop around the GB300 path:

* requests (kind, cube edge n, seed, precision) arrive as a Poisson stream;
* admission is FIFO, gated by a free slot and by an HBM budget (the request's device bytes are
  estimated before admission and returned when it completes), so requests that arrive while others
  are running are admitted as soon as a slot and memory free up;
* every slot is a host thread with its own CUDA stream; a request's whole solve (problem creation,
  coefficient generation, Newton with multigrid-preconditioned CG or BiCGStab, or Jacobi-preconditioned
  when asked) is enqueued on that stream and runs inside library calls
  that release the GIL, so the kernels of different requests overlap on the device;
* state (mesh, coefficients, Jacobian, vectors) stays on the device for the life of the request; the
  solution is copied to the host once, at completion;
* results do not depend on what else is running: coefficients come from the request's seed (device
  generator), all reductions in the library are fixed-order, the assembly has no atomics.

Metrics: per-request latency (arrival -> result on the host), p50/p99, DOF/s and requests/s.
"""
from __future__ import annotations

import math
import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib as L
from .assembly import Problem
from .solver import SolverManager


@dataclass
class Request:
    rid: int
    kind: str          # "thermal" or "nonlinear"
    n: int             # cells per cube edge
    seed: int
    mixed: bool = True
    arrival: float = 0.0   # seconds after the stream start


@dataclass
class Result:
    rid: int
    kind: str
    n: int
    dofs: int
    latency: float
    queue_wait: float
    service: float
    newton_iters: int
    pcg_iters: int
    rel_residual: float
    status: int
    checksum: float
    u: np.ndarray | None = None
    t_setup: float = 0.0   # problem creation + coefficients on the device
    t_solve: float = 0.0   # Newton + Krylov


def poisson_stream(rate=200.0, count=400, edge=(16, 96), nonlinear_fraction=0.5, mixed=True, seed=5):
    """Poisson arrivals (mean `rate`/s); edge log-uniform in [edge0, edge1]; per-request seeds."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    lo, hi = math.log(edge[0]), math.log(edge[1])
    ns = np.floor(np.exp(rng.uniform(lo, hi, count)) + 0.5).astype(int)
    kinds = np.where(rng.uniform(0, 1, count) < nonlinear_fraction, "nonlinear", "thermal")
    seeds = rng.integers(1, 2**31 - 1, count)
    return [Request(i, str(kinds[i]), int(ns[i]), int(seeds[i]), mixed, float(t[i])) for i in range(count)]


def estimate_bytes(req: Request) -> int:
    """Device bytes a request holds while admitted (problem data, Jacobian, Newton / Krylov vectors and
    the multigrid hierarchy: coarse operators ~1/7 of the fine nonzeros, six vectors per level, CG and
    BiCGStab vectors on the fine level)."""
    n = req.n
    ndof = (n + 1) ** 3
    ncell = n ** 3
    nnz = (3 * (n + 1) - 2) ** 3
    w = 4 if req.mixed else 8
    jbytes = nnz * w
    vec = ndof * 8 * 9 + (ndof * 4 * 6 if req.mixed else 0)
    hier = int(nnz * w / 7) + int(ndof * 1.15) * 6 * w + ndof * 10 * w
    return int(jbytes + vec + hier + ncell * (8 + 4) + 4 * 1024 * 1024)


# Per serving thread: one device generator (reseeded per request: the same sequence as a fresh generator
# with that seed) and grow-only buffers for the coefficient samples and the solution, so that a request's
# setup creates no generator and allocates no tensor (the caching allocator serialises its device
# allocations on one lock shared by all serving threads).
_tls = threading.local()


def _thread_state():
    st = getattr(_tls, "state", None)
    if st is None:
        st = _tls.state = {"gen": torch.Generator(device="cuda"), "kap": None, "u": None}
    return st


def _buffer(st, key, count):
    buf = st[key]
    if buf is None or buf.numel() < count:
        # at least 2^20 values (8 MB: a 100^3 cube), then 1.25x growth, so a thread allocates rarely
        buf = st[key] = torch.empty(max(int(count * 1.25) + 1024, 1 << 20), dtype=torch.float64, device="cuda")
    return buf[:count]


def solve_request(req: Request, stream: torch.cuda.Stream, keep_solution=False, preconditioner="gmg"):
    """Runs one request to completion on `stream`; returns (Result without timing, u on host or None)."""
    n = req.n
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        st = _thread_state()
        gen = st["gen"]
        gen.manual_seed(req.seed)
        nonlinear = req.kind == "nonlinear"
        P = Problem(dim=3, order=1, n=(n, n, n), kind="diffusion_1pu2" if nonlinear else "thermal",
                    source=("const", 10.0 if nonlinear else 1.0, 0.0), kappa=1.0,
                    dirichlet_faces=L.MRG_FACE_XLO | L.MRG_FACE_XHI, stream=stream)
        try:
            u = _buffer(st, "u", P.info.n_dofs)
            if not nonlinear:
                kap = _buffer(st, "kap", n ** 3)
                torch.randn(n ** 3, generator=gen, out=kap)
                kap.exp_()
                P.set_kappa(kap, stream=stream)
                u.zero_()
            else:
                torch.rand(P.info.n_dofs, generator=gen, out=u)
                u.mul_(0.1)
            S = SolverManager(P, nonlinear_tol=1e-10, max_nonlinear_iters=30,
                              linear_tol=1e-3 if req.mixed else 1e-11, linear_maxiter=20000,
                              mixed_precision=req.mixed, preconditioner=preconditioner)
            stream.synchronize()
            t1 = time.perf_counter()
            res = S.nonlinearSolver(u, stream=stream, raise_on_noconv=False)
            t2 = time.perf_counter()
            res.t_setup, res.t_solve = t1 - t0, t2 - t1
            uh = u.to("cpu", non_blocking=False) if keep_solution else None
            checksum = float(torch.linalg.vector_norm(u, ord=1).item())  # no full-size temporary
            stream.synchronize()
        finally:
            P.close()
    return res, uh, checksum, P.info.n_dofs


class Server:
    def __init__(self, hbm_budget_bytes=80 * 10**9, slots=12, keep_solutions=False, preconditioner="gmg"):
        self.budget = int(hbm_budget_bytes)
        self.preconditioner = preconditioner
        self.slots = slots
        self.keep = keep_solutions
        self._lock = threading.Condition()
        self._in_use = 0
        self._pending: list[Request] = []
        self._closed = False
        self.results: list[Result] = []
        self.peak_bytes = 0
        self.peak_active = 0
        self._active = 0
        self.errors: list[tuple[int, str]] = []  # (request id, exception) of requests that failed outside the library

    def warmup(self, edge=64):
        """Solves one request of each kind and precision on the calling thread before traffic is admitted.
        The first launch of a kernel loads it (CUDA lazy loading) and a load may synchronise the context,
        i.e. wait for every request in flight: in a cold process the first pass over a 200 req/s stream saw
        p99 368 ms against 59-69 ms warm.  Edge 64 gives coarse levels above and below the row count where
        the Galerkin sweep changes from thread-per-row to warp-per-row, so every kernel of the path loads."""
        stream = torch.cuda.Stream()
        for kind in ("thermal", "nonlinear"):
            for mixed in (True, False):
                solve_request(Request(-1, kind, edge, 1, mixed), stream, False, self.preconditioner)
        stream.synchronize()

    # admission: FIFO head may start when a slot is free and its bytes fit in the budget
    def _take(self):
        with self._lock:
            while True:
                if self._pending:
                    req = self._pending[0]
                    need = estimate_bytes(req)
                    if need > self.budget:
                        self._pending.pop(0)
                        return req, -1
                    if self._in_use + need <= self.budget:
                        self._pending.pop(0)
                        self._in_use += need
                        self._active += 1
                        self.peak_bytes = max(self.peak_bytes, self._in_use)
                        self.peak_active = max(self.peak_active, self._active)
                        return req, need
                elif self._closed:
                    return None, 0
                self._lock.wait(timeout=0.05)

    def _release(self, need):
        with self._lock:
            self._in_use -= need
            self._active -= 1
            self._lock.notify_all()

    def _worker(self, t0):
        stream = torch.cuda.Stream()
        while True:
            req, need = self._take()
            if req is None:
                return
            start = time.perf_counter() - t0
            if need < 0:
                self.results.append(Result(req.rid, req.kind, req.n, 0, start - req.arrival, start - req.arrival, 0.0,
                                           0, 0, float("nan"), L.MRG_ENOMEM, 0.0))
                continue
            try:
                res, uh, chk, dofs = solve_request(req, stream, self.keep, self.preconditioner)
                status = res.status
            except L.MrgError as e:
                res, uh, chk, dofs, status = None, None, 0.0, 0, e.status
            except Exception as e:  # anything else fails this request alone, never the worker
                self.errors.append((req.rid, repr(e)))
                res, uh, chk, dofs, status = None, None, 0.0, 0, L.MRG_EINVAL
            finally:
                self._release(need)
            end = time.perf_counter() - t0
            self.results.append(Result(req.rid, req.kind, req.n, dofs, end - req.arrival, start - req.arrival,
                                       end - start, res.outer_iterations if res else 0,
                                       res.iterations if res else 0, res.rel_residual if res else float("nan"),
                                       status, chk, uh, getattr(res, "t_setup", 0.0), getattr(res, "t_solve", 0.0)))

    def run(self, requests, realtime=True):
        """Feeds `requests` at their arrival times (or all at t=0 if not realtime) and serves them."""
        self.results = []
        t0 = time.perf_counter()
        workers = [threading.Thread(target=self._worker, args=(t0,), daemon=True) for _ in range(self.slots)]
        for w in workers:
            w.start()
        for req in sorted(requests, key=lambda r: r.arrival):
            if realtime:
                delay = req.arrival - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
            else:
                req.arrival = 0.0
            with self._lock:
                self._pending.append(req)
                self._lock.notify_all()
        with self._lock:
            self._closed = True
            self._lock.notify_all()
        for w in workers:
            w.join()
        self.wall = time.perf_counter() - t0
        return summarize(self.results, self.wall)


def shard(requests, rank: int, world: int):
    """The requests replica `rank` of `world` serves: round-robin by request id (a front end spreading one
    Poisson stream over independent replicas; each replica sees a thinned Poisson stream)."""
    return [r for r in requests if r.rid % world == rank]


def merge(parts):
    """Whole-job summary from the replicas' (results, wall) pairs: latencies pooled, throughput over the
    longest replica wall time."""
    results = [r for res, _ in parts for r in res]
    wall = max((w for _, w in parts), default=0.0)
    return summarize(results, wall)


def summarize(results, wall):
    ok = [r for r in results if r.status == L.MRG_OK]
    lat = np.array([r.latency for r in ok]) * 1e3 if ok else np.array([np.nan])
    dofs = sum(r.dofs for r in ok)
    by_kind = {}
    for kind in ("thermal", "nonlinear"):
        rk = [r for r in ok if r.kind == kind]
        if rk:
            by_kind[kind] = {"count": len(rk), "mean_service_ms": 1e3 * float(np.mean([r.service for r in rk])),
                             "mean_setup_ms": 1e3 * float(np.mean([r.t_setup for r in rk])),
                             "mean_solve_ms": 1e3 * float(np.mean([r.t_solve for r in rk])),
                             "mean_krylov_iters": float(np.mean([r.pcg_iters for r in rk])),
                             "mean_newton_iters": float(np.mean([r.newton_iters for r in rk]))}
    return {"requests": len(results), "ok": len(ok), "wall_s": wall, "by_kind": by_kind,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(np.mean(lat)), "dof_per_s": dofs / wall, "req_per_s": len(ok) / wall,
            "max_rel_residual": float(max((r.rel_residual for r in ok), default=float("nan")))}
