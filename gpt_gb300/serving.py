"""Propagator-solve serving with continuous batching.

Requests arrive as a stream (Poisson in the benchmark).  Each asks for
propagator solves on its own gauge field: a Wilson-clover operator on an L^4
lattice with a given mass and 1-12 sources, solved to a true FP64 residual.
The server

* admits a request when its device footprint fits the free part of an HBM
  budget (requests that do not fit wait; nothing is oversubscribed),
* batches by lattice size: waiting requests of the size class of the oldest
  waiting request are dispatched together, up to a per-size concurrency cap
  (small lattices fill few SMs each, so more of them run side by side),
* runs every admitted request on its own CUDA stream from its own worker
  thread (the C ABI releases the GIL), so work of different requests
  overlaps on the device while requests that arrive meanwhile are admitted as
  slots and memory free up,
* keeps each request's gauge field, clover term and Krylov state in HBM from
  admission to completion, and reports p50/p99 latency (arrival to
  completion) and throughput.

A request's result does not depend on what else runs: every reduction has a
fixed summation order and no request shares buffers with another.
"""
import collections
import dataclasses
import gc
import math
import threading
import time

import numpy as np


@dataclasses.dataclass
class Request:
    rid: int
    L: int
    eps: float
    gauge_seed: int
    mass: float
    n_src: int
    src_seed: int
    arrival: float = 0.0
    tol: float = 1e-10


@dataclasses.dataclass
class Result:
    rid: int
    L: int
    n_src: int
    ok: bool
    latency_ms: float
    service_ms: float
    true_residual: list
    checksum: list
    error: str = ""
    solution: object = None


def poisson_stream(n, rate, seed, sizes=(8, 16, 24, 32), eps=(0.2, 0.5), mass=(0.01, 0.2), nsrc=(1, 12), tol=1e-10):
    """The benchmark request stream: exponential inter-arrival times at `rate`
    per second; L uniform in `sizes`, gauge roughness, mass and the number of
    sources uniform in their ranges; a fresh gauge seed per request."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        out.append(Request(rid=i, L=int(rng.choice(sizes)), eps=float(rng.uniform(*eps)), gauge_seed=int(rng.integers(1, 2**62)),
                           mass=float(rng.uniform(*mass)), n_src=int(rng.integers(nsrc[0], nsrc[1] + 1)),
                           src_seed=int(rng.integers(1, 2**62)), arrival=t, tol=tol))
    return out


def footprint_bytes(L, n_src, method="mixed"):
    """Upper estimate of the device bytes one request holds: FP64 operator
    (links 144 B x 4 per site, clover and inverse 1152 B, 12 workspace half
    fields), the FP32 operator of the mixed method (links 48 B x 4, clover
    576 B, workspace), the gauge field in natural layout (576 B/site) and the
    solver's full fields (source, solution, residual, temporaries)."""
    V = L ** 4
    per_rhs64 = 192 * V  # one full FP64 field per rhs
    b = V * (576 + 1152 + 576) + 6 * per_rhs64 * n_src + 12 * (per_rhs64 // 2) * n_src
    if method == "mixed":
        b += V * (192 + 576) + 12 * (96 * V // 2) * n_src + 3 * (96 * V) * n_src
    return int(b * 1.1) + (64 << 20)


class HBMBudget:
    def __init__(self, total_bytes):
        self.total = int(total_bytes)
        self.used = 0
        self.peak = 0
        self.cv = threading.Condition()

    def fits(self, n):
        return self.used + n <= self.total

    def acquire(self, n):
        with self.cv:
            self.used += n
            self.peak = max(self.peak, self.used)

    def release(self, n):
        with self.cv:
            self.used -= n
            self.cv.notify_all()


def default_caps(sizes=(8, 16, 24, 32)):
    """Concurrent requests allowed per lattice size."""
    return {8: 8, 16: 6, 24: 3, 32: 2, **{L: 2 for L in sizes if L not in (8, 16, 24, 32)}}


class Server:
    def __init__(self, executor, hbm_budget_bytes, caps=None, method="mixed", realtime=True, max_total=None):
        """executor(request, method) -> Result fields (dict); runs on the
        calling worker thread with its own CUDA stream.  caps: concurrent
        requests per lattice size; max_total: concurrent requests over all
        sizes (1 serves the stream strictly one request at a time)."""
        self.executor = executor
        self.budget = HBMBudget(hbm_budget_bytes)
        self.caps = caps or default_caps()
        self.max_total = max_total
        self.max_retries = 3
        self.retries = collections.Counter()
        self.requeue = collections.deque()
        self.method = method
        self.realtime = realtime
        self.lock = threading.Condition()
        self.running = collections.Counter()
        self.max_running = collections.Counter()
        self.results = []

    def _worker(self, req, nbytes, t0):
        start = time.perf_counter()
        try:
            fields = self.executor(req, self.method)
            ok, err = True, ""
        except Exception as e:  # a failed request releases its slot and memory
            fields, ok, err = {}, False, f"{type(e).__name__}: {e}"
            if "out of memory" in str(e) and self.retries[req.rid] < self.max_retries:
                # the footprint estimate admitted it, but the device could not
                # hold it at that moment (memory of other requests not yet
                # returned): release its share and queue it again
                self.retries[req.rid] += 1
                self.budget.release(nbytes)
                with self.lock:
                    self.running[req.L] -= 1
                    self.requeue.append(req)
                    self.lock.notify_all()
                return
        end = time.perf_counter()
        res = Result(rid=req.rid, L=req.L, n_src=req.n_src, ok=ok,
                     latency_ms=1000.0 * (end - (t0 + req.arrival)), service_ms=1000.0 * (end - start),
                     true_residual=fields.get("true_residual", []), checksum=fields.get("checksum", []), error=err,
                     solution=fields.get("solution"))
        self.budget.release(nbytes)
        with self.lock:
            self.running[req.L] -= 1
            self.results.append(res)
            self.lock.notify_all()

    def run(self, requests):
        """Serve `requests` (sorted by arrival).  Returns (results, wall seconds)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        for r in reqs:
            if footprint_bytes(r.L, r.n_src, self.method) > self.budget.total:
                raise ValueError(f"request {r.rid} (L={r.L}, {r.n_src} sources) can never fit the HBM budget")
        t0 = time.perf_counter()
        waiting = collections.deque()
        threads = []
        i = 0
        with self.lock:
            while i < len(reqs) or waiting or self.requeue or sum(self.running.values()) > 0:
                now = time.perf_counter() - t0
                while self.requeue:  # out-of-memory retries go first
                    waiting.appendleft(self.requeue.pop())
                while i < len(reqs) and (reqs[i].arrival <= now or not self.realtime):
                    waiting.append(reqs[i])
                    i += 1
                if not waiting and i >= len(reqs):
                    # only running requests left (one may still come back to retry)
                    self.lock.wait(timeout=0.05)
                    continue
                dispatched = False
                if waiting:
                    # batch by lattice size: the size class of the oldest waiting request
                    L = waiting[0].L
                    for r in list(waiting):
                        if r.L != L:
                            continue
                        nb = footprint_bytes(r.L, r.n_src, self.method)
                        total_ok = self.max_total is None or sum(self.running.values()) < self.max_total
                        if total_ok and self.running[L] < self.caps.get(L, 2) and self.budget.fits(nb):
                            waiting.remove(r)
                            self.budget.acquire(nb)
                            self.running[L] += 1
                            self.max_running[L] = max(self.max_running[L], self.running[L])
                            th = threading.Thread(target=self._worker, args=(r, nb, t0), daemon=True)
                            th.start()
                            threads.append(th)
                            dispatched = True
                        else:
                            break
                if not dispatched:
                    timeout = None
                    if i < len(reqs) and self.realtime:
                        timeout = max(0.0, reqs[i].arrival - (time.perf_counter() - t0))
                    self.lock.wait(timeout=timeout if timeout is not None else 0.05)
        for th in threads:
            th.join()
        wall = time.perf_counter() - t0
        return sorted(self.results, key=lambda r: r.rid), wall


def summarize(results, wall):
    ok = [r for r in results if r.ok]
    lat = sorted(r.latency_ms for r in ok)

    def pct(p):
        if not lat:
            return None
        return lat[min(len(lat) - 1, max(0, int(math.ceil(p / 100.0 * len(lat))) - 1))]

    solves = sum(r.n_src for r in ok)
    return {"requests": len(results), "failed": len(results) - len(ok), "solves": solves, "wall_s": wall,
            "solves_per_s": solves / wall if wall > 0 else None, "requests_per_s": len(ok) / wall if wall > 0 else None,
            "p50_ms": pct(50), "p99_ms": pct(99), "max_true_residual": max((max(r.true_residual) for r in ok if r.true_residual),
                                                                          default=None)}


# ---------------------------------------------------------------------------
# the GPU executor
# ---------------------------------------------------------------------------
def gpu_executor(keep_solution=False, inner_tol=1e-5, iterations_per_graph=0):
    """executor for Server: Wilson-clover (csw 1.0, phases [1,1,1,-1]) on a
    fresh device-generated gauge field; mixed = defect_correcting(
    mixed_precision(preconditioned(eo2_ne, cg(inner_tol))), single, double);
    plain = preconditioned(eo2_ne, cg(tol / 3)) in FP64."""
    import torch

    from . import _lib, core
    from .algorithms import inverter as inv
    from .qcd import fermion, gauge

    def run(req, method):
        try:
            return _run(req, method)
        finally:
            # operator objects sit in reference cycles (their matrix operators
            # close over them): collect them now, and hand torch's cached
            # blocks back to the device, so that the request's device memory
            # returns before the admission of the next one (the library's own
            # allocations cannot use torch's cache)
            gc.collect()
            torch.cuda.empty_cache()

    def _run(req, method):
        stream = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            grid = core.grid([req.L] * 4, core.double)
            U = gauge.random_su3_device(grid, req.eps, req.gauge_seed)
            op = fermion.wilson_clover(U, mass=req.mass, csw_r=1.0, csw_t=1.0, boundary_phases=[1, 1, 1, -1],
                                       n_rhs=req.n_src)
            V = grid.gsites
            src = op.F_lattice()
            nat = torch.empty(V * 24, dtype=torch.float64, device="cuda")
            L = _lib.load()
            for k in range(req.n_src):
                _lib.check(L.gbf_random_spinor(V * 12, (req.src_seed + 7919 * k) % (1 << 63), nat.data_ptr(), core.stream_ptr()))
                _lib.check(L.gbf_field_import(src.layout.op, nat.data_ptr(), src.ptr, k, 0, core.stream_ptr()))
            pc = fermion.preconditioner
            if method == "mixed":
                solver = inv.defect_correcting(
                    inv.mixed_precision(inv.preconditioned(pc.eo2_ne(), inv.cg({"eps": inner_tol, "maxiter": 20000,
                                                                               "iterations_per_graph": iterations_per_graph})),
                                        core.single, core.double), eps=req.tol, maxiter=100)(op)
            else:
                # eps bounds the eo2_ne normal residual; tol / 3 brings the true
                # residual of M x = b below tol (eps = tol leaves about 2 tol)
                solver = inv.preconditioned(pc.eo2_ne(), inv.cg({"eps": req.tol / 3, "maxiter": 40000,
                                                                 "iterations_per_graph": iterations_per_graph,
                                                                 "fail_if_not_converged": True}))(op)
            x = solver(src)
            r = op.F_lattice()
            op.M(r, x)
            core.axpby(r, -1.0, r, 1.0, src)
            nr = core.norm2(r)
            ns = core.norm2(src)
            nx = core.norm2(x)
            nr, ns, nx = ([v] if req.n_src == 1 else v for v in (nr, ns, nx))
            out = {"true_residual": [math.sqrt(a / b) for a, b in zip(nr, ns)], "checksum": list(nx)}
            if keep_solution:
                out["solution"] = x.tensor.clone()
            stream.synchronize()
            return out

    return run
