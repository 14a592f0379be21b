"""Serving loop: batching, admission and failure handling on the host (fake
engines, no GPU), and on the GPU that every result is the same alone and in
the mix."""

from __future__ import annotations

import threading
import time
from concurrent.futures import CancelledError

import numpy as np
import pytest


class _FakeEngine:
    """Host-only engine: records its batches; run() returns rid / 2."""

    live = 0
    peak = 0
    made = []
    lock = threading.Lock()

    def __init__(self, kind, norb, nelec, capacity, fail_rids=(), delay=0.01):
        self.kind, self.norb, self.capacity = kind, norb, capacity
        self.nbytes = norb * 100 * capacity
        self.fail_rids = set(fail_rids)
        self.delay = delay
        self.batches = []
        self.closed = False
        with _FakeEngine.lock:
            _FakeEngine.made.append(self)

    def close(self):
        self.closed = True

    def run(self, reqs, control):
        with _FakeEngine.lock:
            _FakeEngine.live += 1
            _FakeEngine.peak = max(_FakeEngine.peak, _FakeEngine.live)
        try:
            self.batches.append([r.rid for r in reqs])
            t_end = time.perf_counter() + self.delay * reqs[0].norb / 8
            while time.perf_counter() < t_end:  # a long batch that checks its control, as the library does
                if control is not None and control._flag.value:
                    raise CancelledError("cancelled")
                time.sleep(0.001)
            if any(r.rid in self.fail_rids for r in reqs):
                raise RuntimeError("engine failed")
            return [(r.rid * 0.5, None) for r in reqs]
        finally:
            with _FakeEngine.lock:
                _FakeEngine.live -= 1


def _reset():
    _FakeEngine.live = _FakeEngine.peak = 0
    _FakeEngine.made = []


def _reqs(n, norbs=(8, 10, 12), seed=0, n_reps=1):
    from ffsim_gb300.serving import Request
    from ffsim_gb300.variational import UCJOpSpinBalanced

    rng = np.random.default_rng(seed)
    hams = {m: object() for m in norbs}
    out = []
    for i in range(n):
        m = int(rng.choice(norbs))
        out.append(Request(i, "energy", m, (m // 2, m // 2), n_reps, np.zeros(UCJOpSpinBalanced.n_params(m, n_reps)),
                           hams[m]))
    return out


def _server(workers=3, budget=10**9, max_batch=64, resident=None, **kw):
    from ffsim_gb300.serving import LUCJServer

    return LUCJServer(workers=workers, budget_bytes=budget, max_batch=max_batch,
                      make_engine=lambda k, n, ne, c: _FakeEngine(k, n, ne, c, **kw),
                      size_of=lambda k, n, ne, c: n * 100 * c, use_streams=False,
                      make_resident=(lambda: resident) if resident is not None else None)


class _FakeResident:
    """Host-only resident evaluator: `cap` requests in flight, each done
    `delay` s after submission with energy norb + 0.5; tickets of cancelled
    requests end with CancelledError; unplannable norbs raise
    NotImplementedError at submission."""

    def __init__(self, cap=1000, delay=0.005, unplannable=()):
        self.cap, self.delay, self.unplannable = cap, delay, set(unplannable)
        self.inflight = {}
        self.next = 0
        self.cancelled = set()
        self.peak = 0
        self.closed = False
        self.lock = threading.Lock()

    def submit(self, op, ham, nelec):
        with self.lock:
            if op.norb in self.unplannable:
                raise NotImplementedError("no plan")
            if len(self.inflight) >= self.cap:
                raise MemoryError("queue full")
            t = self.next
            self.next += 1
            self.inflight[t] = (op.norb, time.perf_counter() + self.delay)
            self.peak = max(self.peak, len(self.inflight))
            return t

    def poll(self, ticket):
        with self.lock:
            norb, t_done = self.inflight[ticket]
            if ticket in self.cancelled:
                del self.inflight[ticket]
                raise CancelledError("cancelled")
            if time.perf_counter() < t_done:
                return None
            del self.inflight[ticket]
            return norb + 0.5

    def submit_grad(self, params, n_reps, ham, nelec):
        class _Op:  # n_params = n_reps (2 norb^2 + norb) without a final rotation
            norb = int(round((-1 + (1 + 8 * len(params) / n_reps) ** 0.5) / 4))
        return self.submit(_Op, ham, nelec)

    def poll_grad(self, ticket):
        e = self.poll(ticket)
        return None if e is None else (e, np.full(3, e))

    def cancel(self, ticket):
        with self.lock:
            self.cancelled.add(ticket)

    def close(self):
        self.closed = True


def test_server_batches_overlaps_and_returns_every_result():
    from ffsim_gb300.serving import latency_stats

    _reset()
    srv = _server(workers=3)
    reqs = _reqs(60)
    for r in reqs:
        srv.submit(r)
    res = srv.drain(len(reqs), timeout=60)
    srv.close()
    assert [r.rid for r in res] == list(range(60))
    assert all(r.ok and r.energy == r.rid * 0.5 for r in res)
    assert max(srv.batch_sizes) > 1  # requests of one key ran together
    assert _FakeEngine.peak > 1  # batches of different keys overlapped
    # every batch holds one key only
    by_rid = {r.rid: r for r in reqs}
    for eng in _FakeEngine.made:
        for b in eng.batches:
            assert len({by_rid[i].norb for i in b}) == 1
    st = latency_stats(res)
    assert st["requests"] == 60 and st["p99_ms"] >= st["p50_ms"] > 0


def test_server_admits_by_memory_budget():
    """A budget that holds one small engine at a time runs the batches one
    after the other and swaps engines between shapes."""
    _reset()
    srv = _server(workers=4, budget=1200, max_batch=1)
    reqs = _reqs(12)
    for r in reqs:
        srv.submit(r)
    res = srv.drain(len(reqs), timeout=60)
    srv.close()
    assert all(r.ok for r in res)
    assert _FakeEngine.peak == 1
    # engines swapped out for other shapes were released at once
    assert any(e.closed for e in _FakeEngine.made)
    assert not any(e.closed for engines in srv._idle.values() for e in engines)


def test_server_shrinks_a_batch_to_the_budget():
    _reset()
    srv = _server(workers=1, budget=8 * 100 * 4, max_batch=64)
    reqs = _reqs(10, norbs=(8,))
    for r in reqs:
        srv.submit(r)
    res = srv.drain(len(reqs), timeout=60)
    srv.close()
    assert all(r.ok for r in res)
    assert max(srv.batch_sizes) <= 4


def test_request_larger_than_the_budget_fails_alone():
    _reset()
    srv = _server(workers=2, budget=900)
    big, small = _reqs(1, norbs=(12,))[0], _reqs(2, norbs=(8,))[1]
    small.rid = 1
    srv.submit(big)
    srv.submit(small)
    res = srv.drain(2, timeout=30)
    srv.close()
    assert isinstance(res[0].error, MemoryError)
    assert res[1].ok and res[1].energy == 0.5


def test_invalid_requests_fail_alone():
    from ffsim_gb300.serving import Request

    _reset()
    srv = _server()
    good = _reqs(3, norbs=(8,))
    bad_nelec = Request(10, "energy", 8, (9, 4), 1, good[0].params, good[0].ham)
    bad_params = Request(11, "gradient", 8, (4, 4), 1, np.zeros(3), good[0].ham)
    bad_kind = Request(12, "density", 8, (4, 4), 1, good[0].params, good[0].ham)
    for r in good + [bad_nelec, bad_params, bad_kind]:
        srv.submit(r)
    res = {r.rid: r for r in srv.drain(6, timeout=30)}
    srv.close()
    assert all(res[i].ok for i in range(3))
    assert all(isinstance(res[i].error, ValueError) for i in (10, 11, 12))


def test_failing_engine_fails_its_batch_only_and_is_not_reused():
    _reset()
    srv = _server(workers=2, fail_rids={3})
    reqs = _reqs(12, norbs=(8, 10))
    for r in reqs:
        srv.submit(r)
    res = {r.rid: r for r in srv.drain(12, timeout=60)}
    srv.close()
    failed = [i for i, r in res.items() if not r.ok]
    assert 3 in failed
    assert all(isinstance(res[i].error, RuntimeError) for i in failed)
    assert all(res[i].ok for i in res if i not in failed)
    # the engine that raised was dropped and released: none of the idle pool's
    # engines ran rid 3
    for engines in srv._idle.values():
        for e in engines:
            assert all(3 not in b for b in e.batches)
    assert all(e.closed for e in _FakeEngine.made if any(3 in b for b in e.batches))


def test_cancel_pending_and_running():
    _reset()
    srv = _server(workers=1, delay=0.5)
    reqs = _reqs(3, norbs=(8,), n_reps=1)
    reqs[2].n_reps = 2  # another key: waits behind the first batch
    from ffsim_gb300.variational import UCJOpSpinBalanced

    reqs[2].params = np.zeros(UCJOpSpinBalanced.n_params(8, 2))
    srv.submit(reqs[0])
    srv.submit(reqs[1])
    time.sleep(0.05)  # the first batch (rids 0, 1) is running
    srv.submit(reqs[2])
    assert srv.cancel(2)  # pending: dropped
    assert srv.cancel(0) and srv.cancel(1)  # the whole running batch: stopped early
    t0 = time.perf_counter()
    res = srv.drain(3, timeout=30)
    srv.close()
    assert time.perf_counter() - t0 < 0.4
    assert all(isinstance(r.error, CancelledError) for r in res)


def test_deadline_while_pending():
    _reset()
    srv = _server(workers=1, delay=0.3)
    reqs = _reqs(2, norbs=(8,))
    reqs[1].norb = 10  # another key
    reqs[1].nelec = (5, 5)
    from ffsim_gb300.variational import UCJOpSpinBalanced

    reqs[1].params = np.zeros(UCJOpSpinBalanced.n_params(10, 1))
    reqs[1].ham = type("H", (), {"norb": 10})()
    reqs[1].deadline = 0.05
    srv.submit(reqs[0])
    time.sleep(0.02)
    srv.submit(reqs[1])
    res = srv.drain(2, timeout=30)
    srv.close()
    assert res[0].ok
    assert isinstance(res[1].error, TimeoutError)


def test_engine_build_out_of_memory_requeues_then_fails():
    """An engine whose allocation fails (the device held less than the
    budget said) sends its batch back to the queue; a later build serves it.
    A batch whose engine fails three times gets MemoryError."""
    from ffsim_gb300.serving import LUCJServer

    _reset()
    fails = {"left": 2}

    def make(k, n, ne, c):
        if fails["left"] > 0:
            fails["left"] -= 1
            raise MemoryError("device full")
        return _FakeEngine(k, n, ne, c)

    srv = LUCJServer(workers=1, budget_bytes=10**9, max_batch=8, make_engine=make,
                     size_of=lambda k, n, ne, c: n * 100 * c, use_streams=False)
    reqs = _reqs(6, norbs=(8,))
    for r in reqs:
        srv.submit(r)
    res = srv.drain(len(reqs), timeout=30)
    srv.close()
    assert all(r.ok for r in res)
    assert srv.oom_retries == 2

    def never(k, n, ne, c):
        raise MemoryError("device full")

    srv = LUCJServer(workers=1, budget_bytes=10**9, max_batch=8, make_engine=never,
                     size_of=lambda k, n, ne, c: n * 100 * c, use_streams=False)
    reqs = _reqs(3, norbs=(8,))
    for r in reqs:
        srv.submit(r)
    res = srv.drain(len(reqs), timeout=30)
    srv.close()
    assert all(isinstance(r.error, MemoryError) for r in res)
    assert srv._in_use == 0


def _mixed(n, seed=0):
    """Energy requests of norb 6, 8 (resident) and 10 (batch), and norb-8
    gradients (resident)."""
    from ffsim_gb300.serving import Request
    from ffsim_gb300.variational import UCJOpSpinBalanced

    rng = np.random.default_rng(seed)
    hams = {m: object() for m in (6, 8, 10)}
    out = []
    for i in range(n):
        m = int(rng.choice((6, 8, 10)))
        kind = "gradient" if m == 8 and rng.random() < 0.3 else "energy"
        out.append(Request(i, kind, m, (m // 2, m // 2), 1, np.zeros(UCJOpSpinBalanced.n_params(m, 1)), hams[m]))
    return out


def _is_resident(req):
    return req.norb <= 8


def test_resident_lane_takes_small_energy_requests():
    _reset()
    fake = _FakeResident()
    srv = _server(resident=fake)
    reqs = _mixed(60)
    for r in reqs:
        srv.submit(r)
    res = srv.drain(len(reqs), timeout=60)
    srv.close()
    assert all(r.ok for r in res)
    for req, r in zip(reqs, res):
        if _is_resident(req):
            assert r.path == "resident" and r.energy == req.norb + 0.5
        else:
            assert r.path == "batch" and r.energy == req.rid * 0.5
    assert srv.resident_served == sum(_is_resident(q) for q in reqs)
    assert fake.closed


def test_resident_queue_full_waits_for_room():
    _reset()
    fake = _FakeResident(cap=3, delay=0.01)
    srv = _server(resident=fake)
    reqs = [r for r in _mixed(80, seed=1) if _is_resident(r)]
    for r in reqs:
        srv.submit(r)
    res = srv.drain(len(reqs), timeout=60)
    srv.close()
    assert all(r.ok and r.path == "resident" for r in res)
    assert fake.peak <= 3


def test_resident_cancel_and_unplannable_fallback():
    _reset()
    fake = _FakeResident(delay=0.5, unplannable={6})
    srv = _server(resident=fake)
    reqs = [r for r in _mixed(40, seed=2) if _is_resident(r)]
    eight = [r for r in reqs if r.norb == 8]
    six = [r for r in reqs if r.norb == 6]
    for r in reqs:
        srv.submit(r)
    time.sleep(0.1)
    assert srv.cancel(eight[0].rid)
    res = {r.rid: r for r in srv.drain(len(reqs), timeout=60)}
    srv.close()
    assert isinstance(res[eight[0].rid].error, CancelledError)
    assert all(res[r.rid].ok and res[r.rid].path == "resident" for r in eight[1:])
    # the resident kernel could not plan them: served by the batch path
    assert all(res[r.rid].ok and res[r.rid].path == "batch" and res[r.rid].energy == r.rid * 0.5 for r in six)


def test_resident_evaluator_that_cannot_start_sends_requests_to_the_batch_path():
    _reset()
    from ffsim_gb300.serving import LUCJServer

    def broken():
        raise RuntimeError("no device memory for the resident queue")

    srv = LUCJServer(workers=2, budget_bytes=10**9, make_engine=lambda k, n, ne, c: _FakeEngine(k, n, ne, c),
                     size_of=lambda k, n, ne, c: n * 100 * c, use_streams=False, make_resident=broken)
    reqs = _mixed(40, seed=5)
    first, rest = reqs[:20], reqs[20:]
    for r in first:
        srv.submit(r)
    time.sleep(0.2)
    for r in rest:
        srv.submit(r)
    res = srv.drain(len(reqs), timeout=60)
    srv.close()
    assert not srv.resident
    assert all(r.ok and r.path == "batch" and r.energy == r.rid * 0.5 for r in res)


def test_resident_deadline_while_pending():
    _reset()
    fake = _FakeResident(cap=1, delay=0.3)
    srv = _server(resident=fake)
    reqs = [r for r in _mixed(30, seed=4) if _is_resident(r)][:3]
    reqs[2].deadline = 0.05
    for r in reqs:
        srv.submit(r)
    res = srv.drain(len(reqs), timeout=60)
    srv.close()
    assert res[0].ok and res[1].ok
    assert isinstance(res[2].error, TimeoutError)


@pytest.mark.gpu
def test_results_alone_and_in_the_mix(cuda):
    """Each request's result through the server equals the same request run
    alone (a batch of one), energies and gradients."""
    import torch

    from ffsim_gb300.serving import LUCJServer, _Engine, replay, synthetic_stream

    offsets, reqs = synthetic_stream(24, rate=400.0, seed=3, norbs=(8, 10, 12), reps=(1, 2),
                                     gradient_fraction=0.3)
    from ffsim_gb300.resident import ResidentEvaluator, accepts
    from ffsim_gb300.variational import UCJOpSpinBalanced

    alone = {}
    ev = ResidentEvaluator(n_slots=8, n_ctas=1)
    for r in reqs:
        if accepts(r.norb, r.n_reps):  # served by the resident kernel
            if r.kind == "gradient":
                alone[r.rid] = ev.wait_grad(ev.submit_grad(r.params, r.n_reps, r.ham, r.nelec))
            else:
                op = UCJOpSpinBalanced.from_parameters(r.params, norb=r.norb, n_reps=r.n_reps)
                alone[r.rid] = (ev.wait(ev.submit(op, r.ham, r.nelec)), None)
            continue
        eng = _Engine(r.kind, r.norb, r.nelec, 1, torch.complex64)
        alone[r.rid] = eng.run([r], None)[0]
        del eng
    ev.close()
    srv = LUCJServer(workers=2)
    res = replay(srv, offsets, reqs)
    srv.close()
    assert all(r.ok for r in res)
    assert max(srv.batch_sizes) > 1
    assert srv.resident_served == sum(r.norb <= 8 for r in reqs) > 0
    for r in res:
        e, g = alone[r.rid]
        assert abs(r.energy - e) <= 1e-9, (r.rid, r.energy, e)
        if g is not None:
            np.testing.assert_allclose(r.grad, g, rtol=0, atol=1e-9)
