"""Serving loop: admission by HBM footprint, batching by lattice size,
failure isolation (CPU, fake executor) and, on the GPU, that a request gives
the same result alone and in a concurrent mix."""
import threading
import time

import numpy as np
import pytest

from gpt_gb300 import serving


class FakeExecutor:
    """Sleeps per request and records concurrent device bytes."""

    def __init__(self, fail_rids=(), oom_once=()):
        self.lock = threading.Lock()
        self.live = 0
        self.peak = 0
        self.live_sizes = []
        self.fail_rids = set(fail_rids)
        self.oom_once = set(oom_once)
        self.order = []

    def __call__(self, req, method):
        nb = serving.footprint_bytes(req.L, req.n_src, method)
        with self.lock:
            self.live += nb
            self.peak = max(self.peak, self.live)
            self.order.append(req.L)
        time.sleep(0.002 * req.L / 8)
        with self.lock:
            self.live -= nb
        if req.rid in self.fail_rids:
            raise RuntimeError("injected failure")
        with self.lock:
            if req.rid in self.oom_once:
                self.oom_once.discard(req.rid)
                raise RuntimeError("cudaMalloc of 1 bytes failed: out of memory")
        return {"true_residual": [1e-11] * req.n_src, "checksum": [float(req.rid)] * req.n_src}


def test_poisson_stream_shape():
    reqs = serving.poisson_stream(200, 20.0, seed=3)
    assert len(reqs) == 200
    gaps = np.diff([0.0] + [r.arrival for r in reqs])
    assert abs(gaps.mean() - 1 / 20.0) < 0.02
    assert {r.L for r in reqs} <= {8, 16, 24, 32}
    assert all(1 <= r.n_src <= 12 and 0.01 <= r.mass <= 0.2 and 0.2 <= r.eps <= 0.5 for r in reqs)


def test_admission_never_exceeds_budget_and_all_complete():
    reqs = serving.poisson_stream(60, 2000.0, seed=5)
    budget = serving.footprint_bytes(32, 12) + serving.footprint_bytes(16, 12)
    ex = FakeExecutor()
    srv = serving.Server(ex, budget, realtime=True)
    res, wall = srv.run(reqs)
    assert len(res) == 60 and all(r.ok for r in res)
    assert ex.peak <= budget
    assert srv.budget.used == 0 and srv.budget.peak <= budget
    for L, n in srv.max_running.items():
        assert n <= srv.caps[L]
    s = serving.summarize(res, wall)
    assert s["solves"] == sum(r.n_src for r in reqs) and s["p50_ms"] <= s["p99_ms"]


def test_request_that_can_never_fit_is_rejected_up_front():
    reqs = [serving.Request(0, 32, 0.3, 1, 0.1, 12, 2)]
    with pytest.raises(ValueError):
        serving.Server(FakeExecutor(), serving.footprint_bytes(8, 1), realtime=False).run(reqs)


def test_failed_request_releases_memory_and_others_finish():
    reqs = serving.poisson_stream(20, 5000.0, seed=9)
    ex = FakeExecutor(fail_rids={3, 11})
    srv = serving.Server(ex, 10 * serving.footprint_bytes(32, 12), realtime=False)
    res, wall = srv.run(reqs)
    bad = [r for r in res if not r.ok]
    assert sorted(r.rid for r in bad) == [3, 11] and "injected failure" in bad[0].error
    assert srv.budget.used == 0
    assert serving.summarize(res, wall)["failed"] == 2


def test_out_of_memory_is_retried_not_failed():
    # a request admitted by its footprint estimate may still meet a device
    # that cannot hold it yet: it goes back to the queue and completes later
    reqs = serving.poisson_stream(16, 5000.0, seed=11)
    ex = FakeExecutor(oom_once={2, 9})
    srv = serving.Server(ex, 10 * serving.footprint_bytes(32, 12), realtime=False)
    res, wall = srv.run(reqs)
    assert len(res) == 16 and all(r.ok for r in res)
    assert srv.retries[2] == 1 and srv.retries[9] == 1
    assert srv.budget.used == 0 and sum(srv.running.values()) == 0


def test_batching_dispatches_same_size_together():
    # all requests arrive at once: dispatch order groups lattice sizes
    reqs = [serving.Request(i, [8, 16][i % 2], 0.3, i + 1, 0.1, 1, i + 7, arrival=0.0) for i in range(12)]
    ex = FakeExecutor()
    srv = serving.Server(ex, 100 * serving.footprint_bytes(16, 1), caps={8: 6, 16: 6}, realtime=False)
    srv.run(reqs)
    # the first six dispatched share the oldest request's size
    assert ex.order[:6] == [8] * 6


@pytest.mark.gpu
def test_gpu_request_same_alone_and_in_mix():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    ex = serving.gpu_executor(keep_solution=True)
    # requests 4 and 5 share lattice size and source count (so the field
    # layout) with 0 and 1: concurrent reductions on the same layout
    reqs = [serving.Request(0, 8, 0.3, 11, 0.1, 2, 21), serving.Request(1, 16, 0.4, 12, 0.05, 3, 22),
            serving.Request(2, 8, 0.25, 13, 0.2, 1, 23), serving.Request(3, 16, 0.3, 14, 0.1, 1, 24),
            serving.Request(4, 8, 0.35, 15, 0.15, 2, 25), serving.Request(5, 16, 0.45, 16, 0.08, 3, 26)]
    alone = {}
    for r in reqs:
        res, _ = serving.Server(ex, 1 << 36, realtime=False).run([r])
        assert res[0].ok, res[0].error
        alone[r.rid] = res[0]
    mix, wall = serving.Server(ex, 1 << 36, realtime=False).run(reqs)
    for m in mix:
        assert m.ok, m.error
        a = alone[m.rid]
        assert max(m.true_residual) < 1e-10
        # the same solution alone and in the mix, bitwise: every kernel is
        # deterministic (fixed reduction order and grid), each request has its
        # own operators, workspace and stream, and the vector algebra its own
        # per-thread handle
        assert m.checksum == a.checksum
        assert torch.equal(m.solution, a.solution)


@pytest.mark.gpu
def test_gpu_random_gauge_is_su3_and_reproducible():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    import gpt_gb300 as g

    grid = g.grid([4, 4, 4, 8])
    a = g.qcd.gauge.random_su3_device(grid, 0.4, 99).host()
    b = g.qcd.gauge.random_su3_device(grid, 0.4, 99).host()
    c = g.qcd.gauge.random_su3_device(grid, 0.4, 100).host()
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    U = a.reshape(-1, 3, 3)
    assert np.abs(np.einsum("nji,njk->nik", U.conj(), U) - np.eye(3)).max() < 1e-13
    assert np.abs(np.linalg.det(U) - 1).max() < 1e-13
    p = g.qcd.gauge.plaquette(g.qcd.gauge.gauge_field(grid, a))
    q = g.qcd.gauge.plaquette(g.qcd.gauge.random_su3(grid, 0.4, 1))
    assert abs(p - q) < 0.05  # same recipe, different random numbers
