"""Serving loop: scheduling and admission on the host (fake evaluators), and
on the GPU that every result is the same alone and in the mix."""

from __future__ import annotations

import threading
import time

import numpy as np
import pytest


class _FakeEval:
    live = 0
    peak = 0
    lock = threading.Lock()

    def __init__(self, kind, norb, nelec):
        self.key = (kind, norb, nelec)
        self.nbytes = norb * 100

    def run(self, req):
        with _FakeEval.lock:
            _FakeEval.live += 1
            _FakeEval.peak = max(_FakeEval.peak, _FakeEval.live)
        time.sleep(0.01 * req.norb / 8)
        with _FakeEval.lock:
            _FakeEval.live -= 1
        return float(req.rid) * 0.5, None


def _reqs(n, norbs=(8, 10, 12)):
    from ffsim_gb300.serving import Request

    rng = np.random.default_rng(0)
    out = []
    for i in range(n):
        m = int(rng.choice(norbs))
        out.append(Request(i, "energy", m, (m // 2, m // 2), 1, np.zeros(3), None))
    return out


def test_server_overlaps_and_returns_every_result():
    from ffsim_gb300.serving import LUCJServer, latency_stats

    _FakeEval.live = _FakeEval.peak = 0
    srv = LUCJServer(workers=4, budget_bytes=10**9, make_evaluator=_FakeEval,
                     size_of=lambda k, n, ne: n * 100, use_streams=False)
    reqs = _reqs(40)
    for r in reqs:
        srv.submit(r)
    res = srv.drain(len(reqs), timeout=60)
    srv.close()
    assert [r.rid for r in res] == list(range(40))
    assert all(r.energy == r.rid * 0.5 for r in res)
    assert srv.max_concurrent > 1 and _FakeEval.peak > 1
    st = latency_stats(res)
    assert st["requests"] == 40 and st["p99_ms"] >= st["p50_ms"] > 0


def test_server_admits_by_memory_budget():
    """A budget that holds one evaluator at a time serialises the requests and
    swaps buffers between shapes."""
    from ffsim_gb300.serving import LUCJServer

    _FakeEval.live = _FakeEval.peak = 0
    srv = LUCJServer(workers=4, budget_bytes=1200, make_evaluator=_FakeEval,
                     size_of=lambda k, n, ne: n * 100, use_streams=False)
    reqs = _reqs(12)
    for r in reqs:
        srv.submit(r)
    res = srv.drain(len(reqs), timeout=60)
    srv.close()
    assert len(res) == 12
    assert _FakeEval.peak == 1


def test_server_rejects_requests_larger_than_the_budget():
    from ffsim_gb300.serving import LUCJServer

    srv = LUCJServer(workers=2, budget_bytes=500, make_evaluator=_FakeEval,
                     size_of=lambda k, n, ne: n * 100, use_streams=False)
    srv.submit(_reqs(1, norbs=(8,))[0])
    with pytest.raises(MemoryError):
        srv.drain(1, timeout=30)
    srv.close()


@pytest.mark.gpu
def test_results_alone_and_in_the_mix(cuda):
    import torch

    from ffsim_gb300.serving import LUCJServer, _Evaluator, replay, synthetic_stream

    offsets, reqs = synthetic_stream(16, rate=200.0, seed=3, norbs=(8, 10, 12), gradient_fraction=0.3)
    alone = {}
    for r in reqs:
        ev = _Evaluator(r.kind, r.norb, r.nelec, torch.complex64)
        alone[r.rid] = ev.run(r)
        del ev
    srv = LUCJServer(workers=4)
    res = replay(srv, offsets, reqs)
    srv.close()
    assert srv.max_concurrent > 1
    for r in res:
        e, g = alone[r.rid]
        assert abs(r.energy - e) <= 1e-9
        if g is not None:
            np.testing.assert_allclose(r.grad, g, rtol=0, atol=1e-9)
